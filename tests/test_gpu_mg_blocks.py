"""Composite-grid multigrid on the GPU vs the oracle (FP64, bitwise).

The device V-cycle (csrc/mg_blocks.cu: fused Ax + Jacobi, residual and FAS kernels,
octant restriction, prolongation added into u, the gmg_same exchange of every grid,
the leaf residual) rounds every value as the oracle's restatement of
mg_solver.hpp:119-520 does, so the leaf interiors agree bit for bit after several
V-cycles; the rms residuals differ only by the order of their sums (rtol 1e-12).
"""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import MG_CASES, gaussian_rhs

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _pair(nx, bnx, ng, leaves, ncycles, exact=True, **kw):
    sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
    om = O.OracleMgBlocks(sim, **kw)
    locs, geom = sim.block_info()
    rhs = gaussian_rhs(locs, geom, bnx, ng)
    om.rhs()[:] = rhs
    rms_o = om.run(ncycles)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    pm = pg.CompositeMultigrid(m, exact=exact, **kw)
    u = torch.zeros(rhs.shape, dtype=torch.float64, device="cuda")
    r = torch.from_numpy(rhs).cuda()
    rms_p = pm.vcycles(u, r, ncycles)
    torch.cuda.synchronize()
    return om, rms_o, u.cpu().numpy(), rms_p


def _interior(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng]


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", MG_CASES, ids=[c[0] for c in MG_CASES])
def test_composite_vcycles_bitwise(name, nx, bnx, ng, leaves):
    om, rms_o, u, rms_p = _pair(nx, bnx, ng, leaves, 4, alpha=10.0)
    assert np.array_equal(_interior(u, ng), _interior(om.u(), ng))
    np.testing.assert_allclose(rms_p, rms_o, rtol=1e-12, atol=0)
    assert rms_p[-1] < 5e-2 * rms_p[0]


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", MG_CASES, ids=[c[0] for c in MG_CASES])
def test_composite_fast_build_within_rounding(name, nx, bnx, ng, leaves):
    # FMA contraction, the 7-point form and the diagonal's reciprocal: the same
    # algorithm rounded differently (tolerance on the max-norm of the interiors)
    om, rms_o, u, rms_p = _pair(nx, bnx, ng, leaves, 4, exact=False, alpha=10.0)
    ref = _interior(om.u(), ng)
    assert np.abs(_interior(u, ng) - ref).max() <= 1e-11 * np.abs(ref).max()
    np.testing.assert_allclose(rms_p, rms_o, rtol=1e-9, atol=0)


@pytest.mark.parametrize("kw", [dict(stages=3), dict(stages=1), dict(jacobi=True, stages=2, weight=0.8),
                                dict(coarse_sweeps=2, alpha=1.0), dict(D=2.0, alpha=0.5, max_coarsenings=3)],
                         ids=["srj3", "srj1", "jacobi", "coarse-sweeps", "D-alpha-3-coarsenings"])
def test_composite_smoother_variants_bitwise(kw):
    name, nx, bnx, ng, leaves = MG_CASES[1]
    om, rms_o, u, rms_p = _pair(nx, bnx, ng, leaves, 3, **kw)
    assert np.array_equal(_interior(u, ng), _interior(om.u(), ng))
    np.testing.assert_allclose(rms_p, rms_o, rtol=1e-12, atol=0)


def test_composite_solve_to_tolerance():
    name, nx, bnx, ng, leaves = MG_CASES[2]
    sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
    om = O.OracleMgBlocks(sim, alpha=10.0)
    locs, geom = sim.block_info()
    rhs = gaussian_rhs(locs, geom, bnx, ng)
    om.rhs()[:] = rhs
    r0 = om.residual()
    ocyc = 0
    while om.residual() > 1e-10 * r0 and ocyc < 40:
        om.run(1)
        ocyc += 1
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    pm = pg.CompositeMultigrid(m, alpha=10.0, exact=True)
    u = torch.zeros(rhs.shape, dtype=torch.float64, device="cuda")
    cyc, rel = pm.solve(u, torch.from_numpy(rhs).cuda(), tol=1e-10, relative=True)
    assert rel <= 1e-10
    assert cyc == ocyc
    assert np.array_equal(_interior(u.cpu().numpy(), ng), _interior(om.u(), ng))
    # the fast build reaches the tolerance in the same number of cycles
    u2 = torch.zeros(rhs.shape, dtype=torch.float64, device="cuda")
    cyc2, rel2 = pg.CompositeMultigrid(m, alpha=10.0).solve(u2, torch.from_numpy(rhs).cuda(), tol=1e-10)
    assert rel2 <= 1e-10 and abs(cyc2 - ocyc) <= 1
    assert torch.allclose(u2, u, rtol=0, atol=1e-9 * float(u.abs().max()))
    # ghosts hold the final leaf exchange: a fresh exchange changes nothing
    g = u.clone()
    m.upload()
    m.exchange(g.view(g.shape[0], 1, *g.shape[1:]), m.new_coarse(1) if m.multilevel else None, prolongate=True,
               op="linear")
    torch.cuda.synchronize()
    assert torch.equal(g, u)


def test_composite_requires_created_stream():
    name, nx, bnx, ng, leaves = MG_CASES[1]
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    pm = pg.CompositeMultigrid(m)
    N = [b + 2 * ng for b in bnx]
    u = torch.zeros((m.nblocks, N[2], N[1], N[0]), dtype=torch.float64, device="cuda")
    with pytest.raises(pg.NativeError):
        pm.vcycles(u, u.clone(), 1, stream=torch.cuda.default_stream())


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", MG_CASES, ids=[c[0] for c in MG_CASES])
def test_composite_mixed_precision_solve(name, nx, bnx, ng, leaves):
    # an FP32 V-cycle on A e = r inside FP64 iterative refinement reaches the FP64
    # tolerance and the FP64 solve's solution
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    locs, geom = m.block_info()
    r = torch.from_numpy(gaussian_rhs(locs, geom, bnx, ng)).cuda()
    u64 = torch.zeros_like(r)
    c64, rel64 = pg.CompositeMultigrid(m, alpha=10.0).solve(u64, r, tol=1e-10)
    u32 = torch.zeros_like(r)
    c32, rel32 = pg.CompositeMultigrid(m, alpha=10.0).solve(u32, r, tol=1e-10, mixed=True)
    assert rel64 <= 1e-10 and rel32 <= 1e-10
    assert c32 <= c64 + 2
    a, b = _interior(u64.cpu().numpy(), ng), _interior(u32.cpu().numpy(), ng)
    assert np.abs(a - b).max() <= 1e-8 * np.abs(a).max()


@pytest.mark.parametrize("prec", ["fp64", "fp32", None], ids=["mg-fp64", "mg-fp32", "none"])
def test_composite_bicgstab(prec):
    # BiCGSTABSolver on the leaf grid with one composite V-cycle per preconditioner
    # application, against the oracle's restatement (compensated dot products there,
    # fixed-order sums here, so iteration counts may differ by one)
    name, nx, bnx, ng, leaves = MG_CASES[1]
    sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
    om = O.OracleMgBlocks(sim, alpha=10.0)
    locs, geom = sim.block_info()
    rhs = gaussian_rhs(locs, geom, bnx, ng)
    xo, it_o, rms_o = om.bicgstab(rhs, precondition=prec is not None, rtol=1e-10, max_iters=600)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    pm = pg.CompositeMultigrid(m, alpha=10.0)
    u = torch.zeros(rhs.shape, dtype=torch.float64, device="cuda")
    it, rms = pm.bicgstab(u, torch.from_numpy(rhs).cuda(), precondition=prec, rtol=1e-10, max_iters=600)
    assert it < 600 and it_o < 600
    if prec is None:
        assert it <= 1.2 * it_o + 5
    else:
        assert abs(it - it_o) <= (1 if prec == "fp64" else 2)
    ref = _interior(xo, ng)
    tol = 1e-8 if prec is not None else 1e-7
    assert np.abs(_interior(u.cpu().numpy(), ng) - ref).max() <= tol * np.abs(ref).max()


@pytest.mark.parametrize("name,nx,bnx,ng,leaves", MG_CASES, ids=[c[0] for c in MG_CASES])
def test_composite_face_coefficient_bitwise(name, nx, bnx, ng, leaves):
    # D on the faces (the poisson_gmg package's Face field), 10 inside two boxes and 1
    # outside, restricted to every grid by the setup tasks: exact build bitwise
    from meshes import region_coefficient
    sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
    om = O.OracleMgBlocks(sim, alpha=10.0)
    locs, geom = sim.block_info()
    rhs = gaussian_rhs(locs, geom, bnx, ng)
    dcoef = region_coefficient(locs, geom, bnx, ng)
    om.rhs()[:] = rhs
    om.set_coefficient(dcoef)
    rms_o = om.run(4)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    pm = pg.CompositeMultigrid(m, alpha=10.0, exact=True)
    pm.set_coefficient(torch.from_numpy(dcoef).cuda())
    u = torch.zeros(rhs.shape, dtype=torch.float64, device="cuda")
    rms_p = pm.vcycles(u, torch.from_numpy(rhs).cuda(), 4)
    assert np.array_equal(_interior(u.cpu().numpy(), ng), _interior(om.u(), ng))
    np.testing.assert_allclose(rms_p, rms_o, rtol=1e-12, atol=0)


def test_composite_face_coefficient_fast_mixed_bicgstab():
    from meshes import region_coefficient
    name, nx, bnx, ng, leaves = MG_CASES[1]
    sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
    om = O.OracleMgBlocks(sim, alpha=10.0)
    locs, geom = sim.block_info()
    rhs = gaussian_rhs(locs, geom, bnx, ng)
    dcoef = region_coefficient(locs, geom, bnx, ng)
    om.rhs()[:] = rhs
    om.set_coefficient(dcoef)
    om.run(4)
    ref4 = _interior(om.u(), ng).copy()
    xo, it_o, _ = om.bicgstab(rhs, precondition=True, rtol=1e-10, max_iters=200)
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    r = torch.from_numpy(rhs).cuda()
    pm = pg.CompositeMultigrid(m, alpha=10.0)
    pm.set_coefficient(torch.from_numpy(dcoef).cuda())
    u = torch.zeros_like(r)
    pm.vcycles(u, r, 4)
    assert np.abs(_interior(u.cpu().numpy(), ng) - ref4).max() <= 1e-11 * np.abs(ref4).max()
    u64 = torch.zeros_like(r)
    c64, rel64 = pm.solve(u64, r, tol=1e-10)
    u32 = torch.zeros_like(r)
    c32, rel32 = pm.solve(u32, r, tol=1e-10, mixed=True)
    assert rel64 <= 1e-10 and rel32 <= 1e-10 and c32 <= c64 + 2
    ub = torch.zeros_like(r)
    it, rms = pm.bicgstab(ub, r, precondition="fp64", rtol=1e-10, max_iters=200)
    assert abs(it - it_o) <= 1
    ref = _interior(xo, ng)
    for x in (u64, u32, ub):
        assert np.abs(_interior(x.cpu().numpy(), ng) - ref).max() <= 1e-8 * np.abs(ref).max()


@pytest.mark.parametrize("case", [MG_CASES[1], MG_CASES[2], MG_CASES[4]], ids=[MG_CASES[i][0] for i in (1, 2, 4)])
def test_composite_flux_correct(case):
    # poisson/flux_correct: the leaf-grid operator (outer residual, BiCGSTAB) with flux
    # correction at coarse/fine faces. The V-cycle's own operator has none, so the
    # V-cycle iteration stalls at its fixed point while BiCGSTAB converges, at alpha = 0
    # too (the corrected operator is conservative).
    name, nx, bnx, ng, leaves = case
    for alpha in (10.0, 0.0):
        sim = O.OracleSim(nx, bnx, ng, leaves=leaves)
        om = O.OracleMgBlocks(sim, alpha=alpha, flux_correct=True)
        locs, geom = sim.block_info()
        rhs = gaussian_rhs(locs, geom, bnx, ng)
        om.rhs()[:] = rhs
        rms_o = om.run(3)
        m = pg.Mesh(nx, bnx, ng, leaves=leaves)
        r = torch.from_numpy(rhs).cuda()
        pe = pg.CompositeMultigrid(m, alpha=alpha, exact=True, flux_correct=True)
        u = torch.zeros_like(r)
        rms_p = pe.vcycles(u, r, 3)
        np.testing.assert_allclose(rms_p, rms_o, rtol=1e-12, atol=0)
        xo, it_o, _ = O.OracleMgBlocks(O.OracleSim(nx, bnx, ng, leaves=leaves), alpha=alpha,
                                       flux_correct=True).bicgstab(rhs, rtol=1e-10, max_iters=100)
        pf = pg.CompositeMultigrid(m, alpha=alpha, flux_correct=True)
        ub = torch.zeros_like(r)
        it, rms = pf.bicgstab(ub, r, precondition="fp64", rtol=1e-10, max_iters=100)
        assert it < 100 and abs(it - it_o) <= 1
        ref = _interior(xo, ng)
        if alpha == 0.0:  # defined up to a constant
            ref = ref - ref.mean()
            got = _interior(ub.cpu().numpy(), ng)
            got = got - got.mean()
        else:
            got = _interior(ub.cpu().numpy(), ng)
        assert np.abs(got - ref).max() <= 1e-7 * np.abs(ref).max()
