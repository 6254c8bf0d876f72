"""Sparse variables on the GPU vs the oracle (bit-exact, exact build).

- Ghost exchange with null buffers, allocation on receipt and default fills on uniform,
  statically refined and three-level meshes: identical allocation flags and fields.
- SparseDealloc counters and zeroing; the sparse advection min/max tag.
- RK2 runs of the sparse advection problem (four fields, one velocity each, donor
  cell): a uniform mesh replayed from a CUDA graph, and an adaptive run (tagging every
  cycle, remeshes carrying the allocation, flux-correction allocation) step-locked
  with the oracle: identical tags, block lists, allocation flags, fields and dt.
"""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import refined_cube, two_level_nested

pytestmark = pytest.mark.gpu

ALLOC, DEALLOC = 1e-5, 1e-6


def _torch():
    import torch
    return torch


def _sparse_state(shape, nblocks, ncomp, ng, seed):
    """Allocation flags (about half) and values: a few O(1) spikes, some values below
    the allocation threshold, zeros elsewhere; unallocated variables all zero."""
    rng = np.random.default_rng(seed)
    alloc = (rng.random((nblocks, ncomp)) < 0.5).astype(np.uint8)
    u = np.zeros(shape)
    inner = (slice(ng, -ng),) * 3
    for b in range(nblocks):
        for v in range(ncomp):
            if not alloc[b, v]:
                continue
            q = np.zeros(shape[2:])
            n = q[inner].shape
            spikes = rng.random(n) < 0.01
            tiny = rng.random(n) < 0.2
            q[inner] = np.where(spikes, rng.standard_normal(n), np.where(tiny, 1e-7 * rng.random(n), 0.0))
            u[b, v] = q
    return alloc, u


EXCHANGE_CASES = [
    ("two-per-dim", (32, 32, 32), (16, 16, 16), 4, None),
    ("uniform-64", (64, 64, 64), (16, 16, 16), 2, None),
    ("smr", (64, 64, 64), (16, 16, 16), 4, refined_cube(2, 1, 3)),
    ("three-level", (64, 64, 64), (8, 8, 8), 4, two_level_nested(3, 2, 6, 6, 10)),
]


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", EXCHANGE_CASES, ids=[c[0] for c in EXCHANGE_CASES])
@pytest.mark.parametrize("prolongate", [True, False])
def test_sparse_exchange_bit_exact(name, nx, bnx, ng, leaves, prolongate):
    torch = _torch()
    nc = 3
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=nc)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves).upload()
    m.enable_sparse(nc, ALLOC, DEALLOC, default_value=[0.0, 0.25, -1.5])
    o.sparse_enable(ALLOC, DEALLOC, default_value=[0.0, 0.25, -1.5])
    alloc, u = _sparse_state(o.base().shape, o.nblocks, nc, ng, seed=len(name))
    o.sparse_set(alloc)
    m.set_sparse_alloc(alloc)
    o.base()[:] = u
    f = torch.tensor(u, device="cuda")
    c = m.new_coarse(nc) if m.multilevel else None
    m.exchange(f, c, prolongate=prolongate)
    o.exchange(prolongate, 0)
    a, cnt = m.sparse_alloc()
    ra, rc = o.sparse_alloc()
    assert np.array_equal(a, ra)
    assert a.sum() > alloc.sum()  # some receivers allocated
    got = f.cpu().numpy()
    ref = np.array(o.base())
    bad = np.argwhere(got != ref)
    assert bad.size == 0, (bad[:5], got[tuple(bad[0])], ref[tuple(bad[0])])
    # unallocated variables stay zero
    assert not got[a == 0].any()


def test_sparse_dealloc_and_tag_bit_exact():
    torch = _torch()
    nx, bnx, ng, nc = (32, 32, 32), (8, 8, 8), 2, 4
    o = O.OracleSim(nx, bnx, ng, ncomp=nc)
    m = pg.Mesh(nx, bnx, ng).upload()
    m.enable_sparse(nc, ALLOC, DEALLOC, dealloc_count=2)
    o.sparse_enable(ALLOC, DEALLOC, dealloc_count=2)
    alloc, u = _sparse_state(o.base().shape, o.nblocks, nc, ng, seed=9)
    # some allocated variables below the deallocation threshold everywhere
    rng = np.random.default_rng(1)
    quiet = (rng.random((o.nblocks, nc)) < 0.5) & (alloc == 1)
    u[quiet] = 1e-7 * (rng.random(u[quiet].shape) < 0.5)
    o.sparse_set(alloc)
    m.set_sparse_alloc(alloc)
    o.base()[:] = u
    f = torch.tensor(u, device="cuda")
    g = torch.tensor(u, device="cuda")  # a second container, zeroed alongside
    t = m.sparse_tag(f, 0.3, 0.03).cpu().numpy()
    assert np.array_equal(t, o.sparse_tag(0.3, 0.03))
    assert set(np.unique(t)) == {-1.0, 0.0, 1.0}
    for _ in range(3):
        m.sparse_dealloc(f, cells=[g])
        o.sparse_dealloc()
        a, cnt = m.sparse_alloc()
        ra, rc = o.sparse_alloc()
        assert np.array_equal(a, ra) and np.array_equal(cnt, rc)
    assert a.sum() < alloc.sum()
    assert np.array_equal(f.cpu().numpy(), np.array(o.base()))
    assert np.array_equal(g.cpu().numpy(), np.array(o.base()))


def _sparse_cfg(cfl, vel, exact=True):
    return pg.StageConfig("advection", "dc", cfl, exact=exact, comp_vel=vel)


def test_sparse_uniform_graph_run_matches_oracle():
    torch = _torch()
    nx, bnx, ng, nc, cfl = (32, 32, 32), (8, 8, 8), 2, 4, 0.45
    vel = pg.problems.sparse_advection_velocities()
    lo, hi = (-1.0,) * 3, (1.0,) * 3
    m = pg.Mesh(nx, bnx, ng, xmin=lo, xmax=hi)
    m.enable_sparse(nc, ALLOC, DEALLOC, dealloc_count=2)
    state, alloc = pg.problems.sparse_advection_state(m, init_size=0.3)
    drv = pg.RK2Driver(m, nc, _sparse_cfg(cfl, vel))
    drv.set_state(state, alloc)
    o = O.OracleSim(nx, bnx, ng, xmin=lo, xmax=hi, ncomp=nc, physics="advection", recon=0, cfl=cfl)
    o.set_component_velocities(vel)
    o.sparse_enable(ALLOC, DEALLOC, dealloc_count=2)
    o.sparse_set(alloc)
    o.base()[:] = state
    o.exchange(True, 0)
    o.init_dt()
    drv.run(12, graph=True)
    o.run(12)
    drv.stream.synchronize()
    a, cnt = m.sparse_alloc(drv.stream)
    ra, rc = o.sparse_alloc()
    assert np.array_equal(a, ra) and np.array_equal(cnt, rc)
    assert a.sum() > alloc.sum()  # the fields spread to new blocks
    assert np.array_equal(drv.base.cpu().numpy(), np.array(o.base()))
    assert float(drv.dt.cpu()[0]) == o.dt()


class _OracleSparseAMR:
    """AMRDriver's adaptive loop with the sparse min/max tag, restated on the oracle."""

    def __init__(self, nx, bnx, ng, nc, cfl, vel, numlevel, count, lo, hi, dealloc_count, init_size):
        self.o = O.OracleSim(nx, bnx, ng, xmin=lo, xmax=hi, ncomp=nc, physics="advection", recon=0, cfl=cfl)
        self.o.set_component_velocities(vel)
        self.o.sparse_enable(ALLOC, DEALLOC, dealloc_count=dealloc_count)
        self.ng, self.bnx, self.nc = ng, bnx, nc
        root = int(self.o.block_info()[0][:, 0].min())
        self.mml = numlevel + root - 1
        self.count = count
        self.init_size = init_size
        self.history = []

    def geometry(self):
        _, geom = self.o.block_info()
        return pg.problems.BlockGeometry(geom, self.ng, self.bnx)

    def adapt(self):
        t = self.o.sparse_tag(0.3, 0.03)
        flags = self.o.set_refinement(t, 0.5, -0.5, self.mml, self.mml, self.count)
        self.history.append((t.copy(), flags.copy()))
        if self.o.remesh(flags):
            self.o.exchange(True, 0)
            self.o.remesh_dt()

    def initialize(self):
        for _ in range(16):
            a, _ = self.o.sparse_alloc()
            state, alloc = pg.problems.sparse_advection_state(self.geometry(), np.array(self.o.base()), a,
                                                              init_size=self.init_size)
            state = np.where(alloc[:, :, None, None, None] != 0, state, 0.0)
            self.o.sparse_set(alloc)
            self.o.base()[:] = state
            self.o.exchange(True, 0)
            before = self.o.nblocks
            self.adapt()
            if self.o.nblocks == before:
                break
        self.o.init_dt()

    def run(self, ncycles):
        for _ in range(ncycles):
            self.o.run(1)
            self.adapt()


def test_sparse_advection_amr_run_matches_oracle():
    nx, bnx, ng, nc, cfl = (32, 32, 32), (8, 8, 8), 2, 4, 0.45
    lo, hi = (-1.0,) * 3, (1.0,) * 3
    vel = pg.problems.sparse_advection_velocities()
    # 60 cycles move each field across a refined block: remeshes during the run
    numlevel, count, dcount, ncycles, size = 2, 2, 2, 60, 0.2
    ref = _OracleSparseAMR(nx, bnx, ng, nc, cfl, vel, numlevel, count, lo, hi, dcount, size)
    mesh = pg.Mesh(nx, bnx, ng, xmin=lo, xmax=hi)
    mesh.enable_sparse(nc, ALLOC, DEALLOC, dealloc_count=dcount)
    crit = pg.SparseMinMaxCriterion(0.3, 0.03)
    drv = pg.AMRDriver(mesh, nc, _sparse_cfg(cfl, vel), crit, numlevel=numlevel, derefine_count=count,
                       check_interval=1)
    seen = []
    orig = drv.flags

    def spy(c):
        f = orig(c)
        seen.append((c.copy(), f.copy()))
        return f

    drv.flags = spy
    drv.initialize(lambda m, prev, a: pg.problems.sparse_advection_state(m, prev, a, init_size=size))
    ref.initialize()
    drv.run(ncycles)
    ref.run(ncycles)
    drv.stream.synchronize()
    assert len(seen) == len(ref.history)
    for (c, f), (rc, rf) in zip(seen, ref.history):
        assert np.array_equal(c, rc)
        assert np.array_equal(f, rf)
    np.testing.assert_array_equal(drv.mesh.block_info()[0], ref.o.block_info()[0])
    assert drv.mesh.multilevel and drv.nremesh >= 3
    assert len(set(drv.block_history)) >= 2
    a, cnt = drv.mesh.sparse_alloc(drv.stream)
    ra, rc = ref.o.sparse_alloc()
    assert np.array_equal(a, ra) and np.array_equal(cnt, rc)
    assert 0 < a.mean() < 0.75  # the fields stay sparse
    assert np.array_equal(drv.base.cpu().numpy(), np.array(ref.o.base()))
    assert float(drv.dt.cpu()[0]) == ref.o.dt()
