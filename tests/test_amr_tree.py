"""Adaptive-refinement host logic against the oracle (no GPU).

Refinement flags (CheckAllRefinement + MeshRefinement::SetRefinement with its
derefinement counter) and the tree update (Mesh::UpdateMeshBlockTree with proper
nesting) must match the oracle exactly: same flags, same new leaf list in gid order,
over several successive adaptive steps on moving refinement targets.
"""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg


def _block_centres(locs, geom, bnx):
    return geom[:, :3] + 0.5 * np.asarray(bnx)[None, :] * geom[:, 3:]


def _crit(locs, geom, bnx, centre, width, rng, noise):
    x = _block_centres(locs, geom, bnx)
    d = x - np.asarray(centre)[None, :]
    d -= np.round(d)  # periodic distance on the unit cube
    v = np.exp(-(d ** 2).sum(axis=1) / (2.0 * width ** 2))
    return v + noise * rng.random(v.shape)


CASES = [
    # nx, bnx, numlevel, derefine_count, steps, seed
    ((64, 64, 64), (16, 16, 16), 3, 1, 6, 0),
    ((64, 64, 64), (16, 16, 16), 3, 2, 8, 1),
    ((32, 32, 32), (8, 8, 8), 3, 1, 6, 2),
    ((128, 128, 128), (16, 16, 16), 2, 3, 6, 3),
]


@pytest.mark.parametrize("case", CASES, ids=["64-16-l3-c1", "64-16-l3-c2", "32-8-l3-c1", "128-16-l2-c3"])
def test_adaptive_steps_match_oracle(case):
    nx, bnx, numlevel, count, steps, seed = case
    rng = np.random.default_rng(seed)
    mesh = pg.Mesh(nx, bnx, 2)
    o = O.OracleSim(nx, bnx, 2, ncomp=1)
    mml = numlevel + mesh.root_level - 1
    saw_refine = saw_deref = False
    for step in range(steps):
        locs, geom = mesh.block_info()
        olocs, ogeom = o.block_info()
        np.testing.assert_array_equal(locs, olocs)
        np.testing.assert_array_equal(geom, ogeom)
        centre = rng.random(3)
        crit = _crit(locs, geom, bnx, centre, 0.12, rng, 0.02)
        flags = mesh.set_refinement(crit, 0.5, 0.05, mml, mml, count)
        oflags = o.set_refinement(crit, 0.5, 0.05, mml, mml, count)
        np.testing.assert_array_equal(flags, oflags)
        saw_refine |= bool((flags == 1).any())
        new = mesh.remesh(flags)
        changed = o.remesh(oflags)
        assert changed == (new is not None)
        if new is not None:
            saw_deref |= new.nblocks < mesh.nblocks + 7 * int((flags == 1).sum())
            mesh = new
    assert saw_refine
    assert saw_deref


def test_derefine_needs_all_siblings_and_count():
    # a two-level mesh: one root block refined; derefinement only after `count` tags of
    # all eight children and never at the root level
    nx, bnx = (32, 32, 32), (16, 16, 16)
    root = 1
    leaves = [(root + 1, i, j, k) for k in range(2) for j in range(2) for i in range(2)]
    leaves += [(root, i, j, k) for k in range(2) for j in range(2) for i in range(2) if (i, j, k) != (0, 0, 0)]
    mesh = pg.Mesh(nx, bnx, 2, leaves=leaves)
    o = O.OracleSim(nx, bnx, 2, leaves=leaves, ncomp=1)
    assert mesh.nblocks == 15
    mml = root + 1
    crit = np.zeros(mesh.nblocks)  # everything asks to derefine
    for rep in range(3):
        flags = mesh.set_refinement(crit, 0.5, 0.05, mml, mml, 3)
        oflags = o.set_refinement(crit, 0.5, 0.05, mml, mml, 3)
        np.testing.assert_array_equal(flags, oflags)
        locs, _ = mesh.block_info()
        fine = locs[:, 0] == root + 1
        assert (flags[~fine] == 0).all()  # root level never derefines
        assert (flags[fine] == (-1 if rep == 2 else 0)).all()
    new = mesh.remesh(flags)
    assert o.remesh(oflags)
    assert new is not None and new.nblocks == 8
    np.testing.assert_array_equal(new.block_info()[0], o.block_info()[0])
    # one child that does not ask blocks the whole group
    mesh = pg.Mesh(nx, bnx, 2, leaves=leaves)
    flags = np.where(mesh.block_info()[0][:, 0] == root + 1, -1, 0).astype(np.int32)
    flags[0] = 0
    assert mesh.remesh(flags) is None


def test_refine_keeps_proper_nesting():
    # refining a level-2 block next to level-1 blocks also refines those neighbours
    nx, bnx = (32, 32, 32), (8, 8, 8)
    mesh = pg.Mesh(nx, bnx, 2)
    o = O.OracleSim(nx, bnx, 2, ncomp=1)
    flags = np.zeros(mesh.nblocks, np.int32)
    flags[0] = 1
    m1 = mesh.remesh(flags)
    assert o.remesh(flags)
    f2 = np.zeros(m1.nblocks, np.int32)
    locs, _ = m1.block_info()
    f2[np.flatnonzero(locs[:, 0] == locs[:, 0].max())[0]] = 1
    m2 = m1.remesh(f2)
    assert o.remesh(f2)
    l2, _ = m2.block_info()
    np.testing.assert_array_equal(l2, o.block_info()[0])
    assert m2.nblocks > m1.nblocks + 7
    # 2:1 balance: leaves that touch (faces, edges, corners; periodic) differ by <= 1 level
    _, g2 = m2.block_info()
    lo = g2[:, :3]
    hi = lo + np.asarray(bnx)[None, :] * g2[:, 3:]
    for a in range(m2.nblocks):
        for b in range(a + 1, m2.nblocks):
            touch = True
            for d in range(3):
                gap = min(max(lo[b, d] + s - hi[a, d], lo[a, d] - hi[b, d] - s) for s in (-1.0, 0.0, 1.0))
                touch &= gap <= 1e-12
            if touch:
                assert abs(int(l2[a, 0]) - int(l2[b, 0])) <= 1


def test_remesh_rejects_bad_flags():
    mesh = pg.Mesh((32,) * 3, (16,) * 3, 2)
    with pytest.raises(pg.NativeError):
        mesh.remesh(np.full(mesh.nblocks, 2, np.int32))
    with pytest.raises(ValueError):
        mesh.remesh(np.zeros(3, np.int32))
