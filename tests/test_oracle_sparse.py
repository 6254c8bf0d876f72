"""Sparse variables in the oracle (CPU): the reference's allocation rules.

- With every variable allocated, a zero allocation threshold and a negative
  deallocation threshold, a sparse run equals the dense run bit for bit.
- Ghost exchange: an unallocated sender, or one whose packed values are all below the
  allocation threshold, sends a null buffer; the receiver allocates its variable when
  any buffer brings data, and a null buffer fills an allocated receiver's ghosts with
  the default value (boundary_communication.cpp:95-140, 216-232, 267-330).
- Flux correction: an allocated fine block always sends, so its coarse neighbour
  allocates (boundary_communication.cpp:121).
- SparseDealloc: consecutive all-below checks, deallocation after more than
  dealloc_count of them (update.cpp:143-216).
- Remesh: a new fine block allocates what its parent had, a new coarse block what any
  child had (mesh-amr_loadbalance.cpp:95-145, 187-213).
- The sparse advection package's min/max refinement tag.
"""
import numpy as np

import oracle_lib as O
from meshes import refined_cube


def _index(o):
    locs, _ = o.block_info()
    return {tuple(int(x) for x in l): b for b, l in enumerate(locs)}, locs


def test_all_allocated_sparse_run_equals_dense():
    nx, bnx, ng, nc = (32, 32, 32), (8, 8, 8), 2, 3
    leaves = refined_cube(2, 1, 3)
    rng = np.random.default_rng(3)
    runs = []
    for sparse in (False, True):
        o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=nc, physics="advection", recon=1, cfl=0.3)
        o.set_component_velocities([[1.0, -0.5, 0.25], [-1.0, 0.0, 0.5], [0.3, 0.7, -1.1]])
        if sparse:
            o.sparse_enable(0.0, -1.0, dealloc_count=1)
            o.sparse_set(np.ones((o.nblocks, nc), np.uint8))
        if not runs:
            state = rng.standard_normal(o.base().shape)
        o.base()[:] = state
        o.exchange(True, 0)
        o.init_dt()
        o.run(3)
        runs.append(np.array(o.base()))
        if sparse:
            a, c = o.sparse_alloc()
            assert a.all() and not c.any()
    assert np.array_equal(runs[0], runs[1])


def test_null_buffers_default_fill_and_allocation_on_receipt():
    nx, bnx, ng, nc = (32, 32, 32), (16, 16, 16), 2, 2
    o = O.OracleSim(nx, bnx, ng, ncomp=nc)
    dense = O.OracleSim(nx, bnx, ng, ncomp=nc)
    idx, _ = _index(o)
    lev = next(iter(idx))[0]
    b0, b1 = idx[(lev, 0, 0, 0)], idx[(lev, 1, 0, 0)]
    rng = np.random.default_rng(5)
    u = np.zeros(o.base().shape)
    # variable 0 lives on block (0,0,0) only: one value next to its +x face
    m = ng + 8
    u[b0, 0, m, m, ng + bnx[0] - 1] = 1.0
    # variable 1 is allocated everywhere with values above the threshold
    u[:, 1, ng:-ng, ng:-ng, ng:-ng] = rng.uniform(0.01, 1.0, (o.nblocks, 16, 16, 16))
    alloc = np.zeros((o.nblocks, nc), np.uint8)
    alloc[b0, 0] = 1
    alloc[:, 1] = 1
    o.sparse_enable(1e-3, 1e-6, default_value=[0.25, 0.5])
    o.sparse_set(alloc)
    o.base()[:] = u
    dense.base()[:] = u
    o.exchange(True, 0)
    dense.exchange(True, 0)
    a, _ = o.sparse_alloc()
    # only the +x neighbour received data for variable 0
    expect = alloc.copy()
    expect[b1, 0] = 1
    assert np.array_equal(a, expect)
    got, ref = np.array(o.base()), np.array(dense.base())
    assert np.array_equal(got[:, 1], ref[:, 1])
    inner = (slice(ng, -ng),) * 3
    for b in range(o.nblocks):
        g = got[b, 0]
        if b not in (b0, b1):
            assert not g.any()  # unallocated: untouched zeros
            continue
        assert np.array_equal(g[inner], u[b, 0][inner])
        ghost = np.ones(g.shape, bool)
        ghost[inner] = False
        if b == b0:
            assert np.all(g[ghost] == 0.25)  # every neighbour sent a null buffer
        else:
            # the -x face ghosts carry block (0,0,0)'s data; every other ghost the default
            face = np.zeros(g.shape, bool)
            face[ng:-ng, ng:-ng, :ng] = True
            assert np.array_equal(g[face], ref[b, 0][face])
            assert g[face].max() == 1.0
            assert np.all(g[ghost & ~face] == 0.25)


def test_flux_correction_allocates_coarse_neighbours():
    nx, bnx, ng, nc = (32, 32, 32), (8, 8, 8), 2, 1
    leaves = refined_cube(2, 1, 3)
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=nc, physics="advection", recon=0, cfl=0.3)
    # threshold so high that no ghost exchange ever carries data
    o.sparse_enable(1e300, -1.0)
    locs, _ = o.block_info()
    fine = locs[:, 0] == locs[:, 0].max()
    alloc = fine[:, None].astype(np.uint8)
    u = np.zeros(o.base().shape)
    u[fine, 0, ng:-ng, ng:-ng, ng:-ng] = 1.0
    o.sparse_set(alloc)
    o.base()[:] = u
    o.exchange(True, 0)
    o.init_dt()
    o.run(1)
    a, _ = o.sparse_alloc()
    coarse = ~fine
    # coarse blocks sharing a face with the refined region now hold the variable
    lo, hi = 1 * 8, 3 * 8  # refined region in root-cell units of the 32^3 root grid
    touch = []
    for b in np.flatnonzero(coarse):
        lv, l1, l2, l3 = locs[b]
        s = 8  # root blocks are 8 cells wide
        box = [(l1 * s, l1 * s + s), (l2 * s, l2 * s + s), (l3 * s, l3 * s + s)]
        nface = 0
        inside = 0
        for d in range(3):
            a0, a1 = box[d]
            if a1 == lo or a0 == hi:
                nface += 1
            elif a0 >= lo and a1 <= hi:
                inside += 1
        touch.append(nface == 1 and inside == 2)
    touch = np.array(touch)
    assert a[fine, 0].all()
    assert np.array_equal(a[coarse, 0].astype(bool), touch)
    assert touch.sum() == 6 * 4


def test_dealloc_counts_and_zeroes():
    nx, bnx, ng, nc = (16, 16, 16), (8, 8, 8), 2, 2
    o = O.OracleSim(nx, bnx, ng, ncomp=nc)
    o.sparse_enable(1e-3, 1e-8, dealloc_count=2)
    u = np.zeros(o.base().shape)
    u[:, 0] = 1e-9  # below the deallocation threshold everywhere
    u[:, 1] = 1e-9
    u[0, 1, 3, 3, 3] = 1.0  # block 0 keeps variable 1
    o.sparse_set(np.ones((o.nblocks, nc), np.uint8))
    o.base()[:] = u
    for call in range(1, 4):
        o.sparse_dealloc()
        a, c = o.sparse_alloc()
        if call < 3:
            assert a.all()
            assert np.all(c[:, 0] == call)
        else:
            assert not a[:, 0].any() and not c[:, 0].any()
            assert not np.array(o.base())[:, 0].any()
        assert a[0, 1] == 1 and c[0, 1] == 0
        assert np.all(c[1:, 1] == (call if call < 3 else 0))
    assert np.array(o.base())[0, 1, 3, 3, 3] == 1.0


def test_remesh_moves_allocation():
    nx, bnx, ng, nc = (32, 32, 32), (8, 8, 8), 2, 2
    leaves = refined_cube(2, 1, 2)  # root block (1,1,1) refined into 8 children
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=nc, physics="advection")
    o.sparse_enable(1e-3, -1.0)
    idx, locs = _index(o)
    fine_lev = int(locs[:, 0].max())
    root = fine_lev - 1
    alloc = np.zeros((o.nblocks, nc), np.uint8)
    # variable 0 on one child of the refined block; variable 1 on root block (0,0,0)
    child = idx[(fine_lev, 3, 2, 2)]
    alloc[child, 0] = 1
    alloc[idx[(root, 0, 0, 0)], 1] = 1
    u = np.zeros(o.base().shape)
    u[child, 0, ng:-ng, ng:-ng, ng:-ng] = 2.0
    u[idx[(root, 0, 0, 0)], 1, ng:-ng, ng:-ng, ng:-ng] = 3.0
    o.sparse_set(alloc, counts=np.full((o.nblocks, nc), 4, np.int32))
    o.base()[:] = u
    flags = np.zeros(o.nblocks, np.int32)
    flags[locs[:, 0] == fine_lev] = -1  # derefine the refined block
    flags[idx[(root, 0, 0, 0)]] = 1     # refine root block (0,0,0)
    assert o.remesh(flags)
    idx2, locs2 = _index(o)
    a, c = o.sparse_alloc()
    par = idx2[(root, 1, 1, 1)]
    assert a[par, 0] == 1 and a[par, 1] == 0 and c[par].sum() == 0
    base = np.array(o.base())
    h = bnx[0] // 2
    # the allocated child's octant holds its restricted data, the others zeros
    q = base[par, 0, ng:-ng, ng:-ng, ng:-ng]
    assert np.all(q[:h, :h, h:] == 2.0)
    assert q.sum() == 2.0 * h ** 3
    for dk in (0, 1):
        for dj in (0, 1):
            for di in (0, 1):
                ch = idx2[(fine_lev, di, dj, dk)]
                assert a[ch, 1] == 1 and a[ch, 0] == 0 and c[ch].sum() == 0
    # untouched blocks keep their counters
    other = idx2[(root, 2, 2, 2)]
    assert np.all(c[other] == 4) and not a[other].any()


def test_sparse_minmax_tag():
    nx, bnx, ng, nc = (16, 16, 16), (8, 8, 8), 1, 2
    o = O.OracleSim(nx, bnx, ng, ncomp=nc)
    o.sparse_enable(1e-5, 1e-6)
    alloc = np.zeros((o.nblocks, nc), np.uint8)
    u = np.zeros(o.base().shape)
    # block 0: variable 0 spans 0..1 -> refine; block 1: variable 1 in (0.05, 0.2) -> keep
    alloc[0, 0] = 1
    u[0, 0, 2, 2, 2] = 1.0
    alloc[1, 1] = 1
    u[1, 1] = 0.1
    # block 2: variable 0 tiny -> derefine; block 3: nothing allocated -> derefine
    alloc[2, 0] = 1
    u[2, 0] = 0.001
    # block 4: an unallocated variable's values do not count
    alloc[4, 0] = 1
    u[4, 0] = 0.1
    u[4, 1] = 5.0
    o.sparse_set(alloc)
    o.base()[:] = u
    t = o.sparse_tag(0.3, 0.03)
    assert list(t[:5]) == [1.0, 0.0, -1.0, -1.0, 0.0]
