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


def test_sparse_api_errors():
    torch = _torch()
    m = pg.Mesh((32, 32, 32), (16, 16, 16), 2).upload()
    m.enable_sparse(2, ALLOC, DEALLOC)
    f = m.new_field(3)
    # field components must match the mesh's sparse variables
    with pytest.raises(pg.NativeError, match="sparse"):
        m.exchange(f)
    # the packed-buffer exchange does not take sparse variables
    with pytest.raises(pg.NativeError, match="sparse"):
        m.exchange(m.new_field(2), buffered=True)
    # flags must be 0 or 1
    with pytest.raises(pg.NativeError):
        m.set_sparse_alloc(np.full((m.nblocks, 2), 2, np.uint8))
    # Burgers declares no sparse variables
    mb = pg.Mesh((32, 32, 32), (16, 16, 16), 4).upload().enable_sparse(5, ALLOC, DEALLOC)
    with pytest.raises(pg.NativeError, match="advection only"):
        pg.RK2Driver(mb, 5, pg.StageConfig("burgers", "weno5", 0.8)).run(1, graph=False)
    del torch


def test_sparse_fast_build_within_tolerance():
    """The FMA-contracted kernels on the sparse advection problem (PLM) stay within 1e-12
    of the oracle; the allocation flags, which depend on thresholds, match exactly."""
    nx, bnx, ng, nc, cfl = (32, 32, 32), (16, 16, 16), 4, 4, 0.45
    vel = pg.problems.sparse_advection_velocities()
    lo, hi = (-1.0,) * 3, (1.0,) * 3
    leaves = refined_cube(1, 0, 1)
    m = pg.Mesh(nx, bnx, ng, xmin=lo, xmax=hi, leaves=leaves)
    m.enable_sparse(nc, ALLOC, DEALLOC, dealloc_count=2)
    state, alloc = pg.problems.sparse_advection_state(m, init_size=0.3)
    drv = pg.RK2Driver(m, nc, pg.StageConfig("advection", "plm", cfl, comp_vel=vel))
    drv.set_state(state, alloc)
    o = O.OracleSim(nx, bnx, ng, xmin=lo, xmax=hi, leaves=leaves, ncomp=nc, physics="advection", recon=1, cfl=cfl)
    o.set_component_velocities(vel)
    o.sparse_enable(ALLOC, DEALLOC, dealloc_count=2)
    o.sparse_set(alloc)
    o.base()[:] = np.where(alloc[:, :, None, None, None] != 0, state, 0.0)
    o.exchange(True, 0)
    o.init_dt()
    drv.run(6, graph=True)
    o.run(6)
    drv.stream.synchronize()
    a, cnt = m.sparse_alloc(drv.stream)
    ra, rc = o.sparse_alloc()
    assert np.array_equal(a, ra) and np.array_equal(cnt, rc)
    g = drv.base.cpu().numpy()[:, :, ng:-ng, ng:-ng, ng:-ng]
    r = np.array(o.base())[:, :, ng:-ng, ng:-ng, ng:-ng]
    scale = np.abs(r).max(axis=(0, 2, 3, 4))
    err = np.abs(g - r).max(axis=(0, 2, 3, 4)) / np.where(scale > 0, scale, 1.0)
    assert err.max() <= 1e-12, err


def test_sparse_three_level_exchange_and_flux_allocation():
    """Three-level mesh, 16^3-class boxes: one dense-like variable and one that lives only
    on the finest blocks, so the coarse face neighbours of the fine region allocate
    through flux correction in the first stage."""
    torch = _torch()
    nx, bnx, ng, nc = (64, 64, 64), (8, 8, 8), 4, 2
    leaves = two_level_nested(3, 2, 6, 6, 10)
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=nc, physics="advection", recon=0, cfl=0.3)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    locs, _ = m.block_info()
    finest = locs[:, 0] == locs[:, 0].max()
    alloc = np.zeros((m.nblocks, nc), np.uint8)
    alloc[:, 0] = 1
    alloc[finest, 1] = 1
    rng = np.random.default_rng(4)
    u = np.zeros((m.nblocks, nc) + tuple(m.N[::-1]))
    u[:, 0, ng:-ng, ng:-ng, ng:-ng] = rng.random((m.nblocks,) + (8, 8, 8))
    u[finest, 1, ng:-ng, ng:-ng, ng:-ng] = 1e-7  # below the allocation threshold
    vel = [[1.0, 0.5, -0.25], [-0.5, 1.0, 0.75]]
    m.enable_sparse(nc, ALLOC, DEALLOC, dealloc_count=3)
    drv = pg.RK2Driver(m, nc, pg.StageConfig("advection", "dc", 0.3, exact=True, comp_vel=vel))
    drv.set_state(u, alloc)
    o.set_component_velocities(vel)
    o.sparse_enable(ALLOC, DEALLOC, dealloc_count=3)
    o.sparse_set(alloc)
    o.base()[:] = u
    o.exchange(True, 0)
    o.init_dt()
    drv.run(2, graph=False)
    o.run(2)
    drv.stream.synchronize()
    a, cnt = m.sparse_alloc(drv.stream)
    ra, rc = o.sparse_alloc()
    assert np.array_equal(a, ra) and np.array_equal(cnt, rc)
    assert a[:, 1].sum() > alloc[:, 1].sum()  # flux correction allocated coarse neighbours
    assert np.array_equal(drv.base.cpu().numpy(), np.array(o.base()))
