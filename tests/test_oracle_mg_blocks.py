"""Composite-grid multigrid on the CPU: the oracle's block-structured V-cycle and the
product's multigrid index maps.

On a uniform mesh the two-level composite grids are the uniform levels, so the block
restatement (oracle/gmg_blocks.hpp: block storage, ghost exchanges, per-block
restriction and prolongation) must reproduce the global-array V-cycle of oracle/gmg.hpp
bit for bit; that pins the block machinery the refined cases rely on. The gmg_same
index maps of every grid (mesh-gmg.cpp:48-201 neighbours, bnd_info.cpp ranges) are
compared record by record with the product's, as the leaf-grid maps are.
"""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import MG_CASES, gaussian_rhs


def _oracle(nx, bnx, ng, leaves, **kw):
    sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
    mg = O.OracleMgBlocks(sim, **kw)
    locs, geom = sim.block_info()
    mg.rhs()[:] = gaussian_rhs(locs, geom, bnx, ng)
    return sim, mg


def test_block_vcycle_is_the_uniform_vcycle_bitwise():
    ng, n, b = 2, 32, 8
    sim, mg = _oracle((n,) * 3, (b,) * 3, ng, None)
    rms_b = mg.run(5)
    g = O.OracleGmg(n, mg.lmax - mg.lmin)
    locs, _ = sim.block_info()
    R = g.rhs()
    rhs = mg.rhs()
    for q in range(mg.nleaf):
        l = locs[q, 1:] * b
        R[l[2]:l[2] + b, l[1]:l[1] + b, l[0]:l[0] + b] = rhs[q, ng:-ng, ng:-ng, ng:-ng]
    rms_g = g.run(5)
    # the sums of squares run in block order vs global order
    np.testing.assert_allclose(rms_b, rms_g, rtol=1e-13, atol=0)
    U, u = g.u(), mg.u()
    for q in range(mg.nleaf):
        l = locs[q, 1:] * b
        assert np.array_equal(U[l[2]:l[2] + b, l[1]:l[1] + b, l[0]:l[0] + b], u[q, ng:-ng, ng:-ng, ng:-ng])


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", MG_CASES, ids=[c[0] for c in MG_CASES])
def test_composite_index_maps_match_oracle(name, nx, bnx, ng, leaves):
    sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
    om = O.OracleMgBlocks(sim)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    pm = pg.CompositeMultigrid(m)
    assert (pm.lmin, pm.lmax, pm.nslots, pm.nleaf) == (om.lmin, om.lmax, om.nslots, om.nleaf)
    assert pm.ngrids == om.lmax - om.lmin + 1
    for level in range(om.lmin, om.lmax + 1):
        a, b = om.boundaries(level), pm.boundaries(level)
        assert a.shape == b.shape, level
        assert np.array_equal(a, b), level


def test_refined_vcycle_converges():
    # diagonal_alpha > 0 makes the periodic problem non-singular; without flux
    # correction the refined periodic Poisson operator is not conservative, so
    # alpha = 0 stalls at the consistency error of the coarse/fine faces
    _, mg = _oracle((32,) * 3, (8,) * 3, 2, MG_CASES[1][4], alpha=10.0)
    rms = mg.run(8)
    assert np.all(np.diff(rms) < 0)
    assert rms[-1] < 1e-4 * rms[0]


def test_coarsening_limit():
    leaves = MG_CASES[1][4]
    sim = O.OracleSim((32,) * 3, (8,) * 3, 2, leaves=leaves)
    m = pg.Mesh((32,) * 3, (8,) * 3, 2, leaves=leaves)
    # two grids: the coarsest holds only blocks of its own level
    assert pg.CompositeMultigrid(m, max_coarsenings=1).lmin == O.OracleMgBlocks(sim, max_coarsenings=1).lmin == 2
    # one grid would hold leaves of a coarser level: rejected by both
    with pytest.raises(pg.NativeError):
        pg.CompositeMultigrid(m, max_coarsenings=0)
    with pytest.raises(RuntimeError):
        O.OracleMgBlocks(sim, max_coarsenings=0)


def test_invalid_parameters_rejected():
    m = pg.Mesh((32,) * 3, (8,) * 3, 2)
    with pytest.raises(pg.NativeError):
        pg.CompositeMultigrid(m, stages=4)
    with pytest.raises(pg.NativeError):
        pg.CompositeMultigrid(m, stages=0)
    with pytest.raises(pg.NativeError):
        pg.CompositeMultigrid(m, coarse_sweeps=-1)


def test_face_coefficient_constant_equals_constant_path():
    # the face-coefficient operator with D = 2 on every face is the constant-D operator
    from meshes import region_coefficient
    name, nx, bnx, ng, leaves = MG_CASES[1]
    a = O.OracleMgBlocks(O.OracleSim(nx, bnx, ng, leaves=leaves), alpha=10.0, D=2.0)
    b = O.OracleMgBlocks(O.OracleSim(nx, bnx, ng, leaves=leaves), alpha=10.0, D=1.0)
    locs, geom = a.sim.block_info()
    r = gaussian_rhs(locs, geom, bnx, ng)
    a.rhs()[:] = r
    b.rhs()[:] = r
    b.set_coefficient(region_coefficient(locs, geom, bnx, ng, inside=2.0, outside=2.0))
    assert np.array_equal(a.run(3), b.run(3))
    assert np.array_equal(a.u(), b.u())


def test_face_coefficient_converges():
    from meshes import region_coefficient
    name, nx, bnx, ng, leaves = MG_CASES[1]
    _, mg = _oracle(nx, bnx, ng, leaves, alpha=10.0)
    locs, geom = mg.sim.block_info()
    mg.set_coefficient(region_coefficient(locs, geom, bnx, ng, inside=10.0, outside=1.0))
    rms = mg.run(8)
    assert np.all(np.diff(rms) < 0) and rms[-1] < 1e-3 * rms[0]
