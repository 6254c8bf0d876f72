"""Adaptive refinement on the GPU vs the oracle.

- Per-block criteria (FirstDerivative, SecondDerivative, |grad q|): bit-exact.
- Remesh data movement (same-level copy, prolongation into new fine blocks,
  restriction into new coarse blocks) and the ghost fill after it: bit-exact.
- Whole adaptive runs (initial refinement, RK2 cycles, periodic tagging, remeshes with
  refinement and derefinement) in the exact build, step-locked with the oracle:
  Burgers (no prolongation inside stages) and advection (prolongation in every stage
  exchange, flux correction); identical flags and block lists, bit-exact fields and dt.
"""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import refined_cube, two_level_nested

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _state(geom_src, nghost, bnx, ncomp):
    # four sinusoids of low wavenumber: gradients localised enough for the relative
    # criterion to refine and derefine parts of a small mesh
    locs, geom = geom_src.block_info()
    bg = pg.problems.BlockGeometry(geom, nghost, bnx)
    return pg.problems.burgers_amr_state(bg, nscalars=ncomp - 3, nmodes=4, kmax=2)


CRIT_CASES = [
    ("uniform", (32, 32, 32), (8, 8, 8), 2, None),
    ("smr", (64, 64, 64), (16, 16, 16), 4, refined_cube(2, 1, 3)),
    ("three-level", (64, 64, 64), (8, 8, 8), 4, two_level_nested(3, 2, 6, 6, 10)),
]


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", CRIT_CASES, ids=[c[0] for c in CRIT_CASES])
@pytest.mark.parametrize("method", ["first", "second", "gradient"])
def test_block_criterion_bit_exact(name, nx, bnx, ng, leaves, method):
    torch = _torch()
    ncomp = 5
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=ncomp)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves).upload()
    st = _state(m, ng, bnx, ncomp)
    o.base()[:] = st
    o.exchange(True, 0)
    f = torch.tensor(np.array(o.base()), device="cuda")
    mi = {"first": 0, "second": 1, "gradient": 2}[method]
    for comp in (0, 3):
        got = m.block_criterion(f, comp, method).cpu().numpy()
        ref = o.block_criterion(comp, mi)
        assert np.array_equal(got, ref), (comp, np.abs(got - ref).max())


TRANSFER_CASES = [
    # refine a few root blocks of a uniform mesh
    ("refine", (32, 32, 32), (8, 8, 8), 4, None, "refine"),
    # derefine the refined cube of an SMR mesh and refine one coarse block elsewhere
    ("refine+derefine", (64, 64, 64), (16, 16, 16), 4, refined_cube(2, 1, 2), "both"),
    ("three-level", (64, 64, 64), (8, 8, 8), 4, two_level_nested(3, 2, 6, 6, 10), "both"),
]


def _flags(locs, mode, root_level):
    n = locs.shape[0]
    flags = np.zeros(n, np.int32)
    lev = locs[:, 0]
    if mode in ("refine", "both"):
        coarse = np.flatnonzero(lev == lev.min())
        flags[coarse[:: max(1, len(coarse) // 3)]] = 1
    if mode == "both":
        finest = lev.max()
        if finest > root_level:
            flags[lev == finest] = -1
    return flags


@pytest.mark.parametrize("name,nx,bnx,ng,leaves,mode", TRANSFER_CASES, ids=[c[0] for c in TRANSFER_CASES])
def test_remesh_transfer_bit_exact(name, nx, bnx, ng, leaves, mode):
    torch = _torch()
    ncomp = 5
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=ncomp, physics="burgers", prolong_in_stage=False)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves).upload()
    rng = np.random.default_rng(11)
    o.base()[:] = rng.standard_normal(o.base().shape)
    o.exchange(True, 0)
    f = torch.tensor(np.array(o.base()), device="cuda")
    locs, _ = m.block_info()
    flags = _flags(locs, mode, m.root_level)
    new = m.remesh(flags)
    assert new is not None
    assert o.remesh(flags)
    np.testing.assert_array_equal(new.block_info()[0], o.block_info()[0])
    g = m.transfer(new, f)
    torch.cuda.synchronize()
    got = g.cpu().numpy()
    assert got.shape == o.base().shape
    assert np.array_equal(got, o.base())
    # ghost fill after the remesh (CommunicateBoundaries with prolongation)
    c = new.new_coarse(ncomp) if new.multilevel else None
    new.exchange(g, c, prolongate=True)
    o.exchange(True, 0)
    torch.cuda.synchronize()
    assert np.array_equal(g.cpu().numpy(), o.base())


class _OracleAMR:
    """The adaptive loop of AMRDriver restated on the oracle (same cadence)."""

    def __init__(self, nx, bnx, ng, ncomp, cfl, criterion, numlevel, count, interval, physics="burgers", recon=0,
                 pgen=None):
        self.o = O.OracleSim(nx, bnx, ng, ncomp=ncomp, physics=physics, recon=recon, cfl=cfl,
                             prolong_in_stage=(physics != "burgers"))
        self.ng, self.bnx, self.ncomp = ng, bnx, ncomp
        self.pgen = pgen if pgen is not None else (lambda src: _state(src, ng, bnx, ncomp))
        self.crit = criterion
        root = int(self.o.block_info()[0][:, 0].min())
        self.mml = numlevel + root - 1
        self.count, self.interval = count, interval
        self.ncycle = 0
        self.history = []

    def adapt(self):
        mi = {"first": 0, "second": 1, "gradient": 2}[self.crit.method]
        vals = None
        for c in self.crit.comps:
            v = self.o.block_criterion(c, mi)
            vals = v if vals is None else np.maximum(vals, v)
        rt, dt = self.crit.tolerances(vals)
        flags = self.o.set_refinement(vals, rt, dt, self.mml, self.mml, self.count)
        self.history.append((vals.copy(), flags.copy()))
        if self.o.remesh(flags):
            self.o.exchange(True, 0)
            self.o.remesh_dt()
            return True
        return False

    def initialize(self):
        for _ in range(16):
            self.o.base()[:] = self.pgen(self.o)
            self.o.exchange(True, 0)
            before = self.o.nblocks
            self.adapt()
            if self.o.nblocks == before:
                break
        self.o.init_dt()

    def run(self, ncycles):
        done = 0
        while done < ncycles:
            k = min(ncycles - done, self.interval - self.ncycle % self.interval)
            self.o.run(k)
            self.ncycle += k
            done += k
            if self.ncycle % self.interval == 0:
                self.adapt()


def test_adaptive_burgers_run_matches_oracle():
    torch = _torch()
    nx, bnx, ng, ncomp, cfl = (32, 32, 32), (8, 8, 8), 4, 5, 0.8
    crit = pg.RefinementCriterion(comps=(0, 1, 2), method="gradient", refine_tol=0.8, derefine_tol=0.75,
                                  relative=True)
    numlevel, count, interval, ncycles = 2, 1, 2, 12
    ref = _OracleAMR(nx, bnx, ng, ncomp, cfl, crit, numlevel, count, interval)
    mesh = pg.Mesh(nx, bnx, ng)
    drv = pg.AMRDriver(mesh, ncomp, pg.StageConfig("burgers", "weno5", cfl, exact=True), crit, numlevel=numlevel,
                       derefine_count=count, check_interval=interval)
    seen = []
    orig_flags = drv.flags

    def spy(c):
        f = orig_flags(c)
        seen.append((c.copy(), f.copy()))
        return f

    drv.flags = spy
    drv.initialize(lambda m: _state(m, ng, bnx, ncomp))
    ref.initialize()
    drv.run(ncycles)
    ref.run(ncycles)
    drv.stream.synchronize()
    assert len(seen) == len(ref.history)
    for (c, f), (rc, rf) in zip(seen, ref.history):
        assert np.array_equal(c, rc)
        assert np.array_equal(f, rf)
    np.testing.assert_array_equal(drv.mesh.block_info()[0], ref.o.block_info()[0])
    # initial refinement, then derefinement steps during the run
    assert drv.nremesh >= 3
    assert min(drv.block_history[2:]) < max(drv.block_history[1:])
    assert np.array_equal(drv.base.cpu().numpy(), ref.o.base())
    assert float(drv.dt.cpu()[0]) == ref.o.dt()


def _blob(src, ng, bnx):
    # advected Gaussian (sigma 0.08) off the domain centre, a function of position only
    _, geom = src.block_info()
    bg = pg.problems.BlockGeometry(geom, ng, bnx)
    xs, ys, zs = bg.cell_centers()
    r2 = ((zs - 0.3) ** 2)[:, :, None, None] + ((ys - 0.4) ** 2)[:, None, :, None] + ((xs - 0.5) ** 2)[:, None, None, :]
    out = np.zeros((bg.nblocks, 1) + tuple(bg.N[::-1]))
    out[:, 0, ng:-ng, ng:-ng, ng:-ng] = np.exp(-r2 / (2 * 0.08 ** 2))[:, ng:-ng, ng:-ng, ng:-ng]
    return out


def test_adaptive_advection_run_matches_oracle():
    # advection prolongates inside every stage exchange and corrects fluxes at
    # fine/coarse faces; the mesh follows the moving blob
    nx, bnx, ng, ncomp, cfl = (32, 32, 32), (8, 8, 8), 2, 1, 0.3
    crit = pg.RefinementCriterion(comps=(0,), method="gradient", refine_tol=0.4, derefine_tol=0.3, relative=True)
    numlevel, count, interval, ncycles = 2, 1, 4, 48
    pgen = lambda src: _blob(src, ng, bnx)  # noqa: E731
    ref = _OracleAMR(nx, bnx, ng, ncomp, cfl, crit, numlevel, count, interval, physics="advection", recon=1,
                     pgen=pgen)
    drv = pg.AMRDriver(pg.Mesh(nx, bnx, ng), ncomp, pg.StageConfig("advection", "plm", cfl, exact=True), crit,
                       numlevel=numlevel, derefine_count=count, check_interval=interval)
    drv.initialize(pgen)
    ref.initialize()
    drv.run(ncycles)
    ref.run(ncycles)
    drv.stream.synchronize()
    np.testing.assert_array_equal(drv.mesh.block_info()[0], ref.o.block_info()[0])
    # refinement and derefinement both happen while the blob moves
    assert drv.nremesh >= 5 and drv.mesh.multilevel
    assert len(set(drv.block_history)) >= 3
    assert np.array_equal(drv.base.cpu().numpy(), ref.o.base())
    assert float(drv.dt.cpu()[0]) == ref.o.dt()
