"""A Poisson package written against the Parthenon package interface -- its own
equation class (face fluxes D grad u and their divergence, SetDiagonal) built on
SparsePacks with type-based variables, PDOpt::WithFluxes and face fields -- solved by the
compatibility layer's MGSolver<u, rhs, Eq> and BiCGSTABSolver<u, rhs, Eq> on the
multigrid grids of the layer's mesh (mg_solver.hpp, bicgstab_solver.hpp).

The V-cycles run the package's operator on every grid and the library's transfers
between them; with the package and the layer rounding each operation in the reference's
order, the leaf solution after a fixed number of V-cycles equals the oracle's
restatement of MGSolver bit for bit. BiCGSTAB with the V-cycle as preconditioner takes
the oracle's iteration count and agrees to rounding (its dot products sum in another
order).
"""
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as O
from compat_build import ROOT, compile_objects, link
from meshes import gaussian_rhs, region_coefficient

pytestmark = pytest.mark.gpu

DECK = """
<parthenon/mesh>
nghost = {ng}
refinement = none
multigrid = true
nx1 = {n}
nx2 = {n}
nx3 = {n}
ix1_bc = periodic
ox1_bc = periodic
ix2_bc = periodic
ox2_bc = periodic
ix3_bc = periodic
ox3_bc = periodic
<parthenon/meshblock>
nx1 = {b}
nx2 = {b}
nx3 = {b}
<poisson>
solver = {solver}
diagonal_alpha = {alpha}
<poisson/solver_params>
max_iterations = {iters}
residual_tolerance = {tol}
smoother = SRJ2
do_FAS = true
precondition = true
relative_residual = {relative}
"""


@pytest.fixture(scope="module")
def app():
    src = os.path.join(ROOT, "tests", "cxx", "poisson_compat")
    objs = compile_objects([os.path.join(src, "poisson.cpp"), os.path.join(src, "main.cpp")], "compatpoisson",
                           extra=("-fmad=false",))
    return link(objs, "compat_poisson_app")


def _run(app, tmp_path, n, b, ng, solver, alpha, iters, tol, relative, rhs, coef=None):
    deck = tmp_path / "poisson.in"
    deck.write_text(DECK.format(n=n, b=b, ng=ng, solver=solver, alpha=alpha, iters=iters, tol=tol,
                                relative="true" if relative else "false"))
    prefix = str(tmp_path / "run")
    rhs_file = str(tmp_path / "rhs.bin")
    np.ascontiguousarray(rhs, np.float64).tofile(rhs_file)
    cmd = [app, "-i", str(deck), "-o", prefix, "--rhs", rhs_file]
    if coef is not None:
        coef_file = str(tmp_path / "coef.bin")
        np.ascontiguousarray(coef, np.float64).tofile(coef_file)
        cmd += ["--coef", coef_file]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-3000:]
    it, res, ms, graph = open(prefix + "_info.txt").read().split()
    u = np.fromfile(prefix + "_u.bin").reshape(rhs.shape)
    print(r.stdout.strip())
    if solver == "MG":
        assert graph == "1"  # the V-cycles after the first replay from a captured CUDA graph
    return u, int(it), float(res), float(ms)


def _setup(n, b, ng, alpha, varying_d):
    sim = O.OracleSim((n,) * 3, (b,) * 3, ng)
    om = O.OracleMgBlocks(sim, stages=2, alpha=alpha)
    locs, geom = sim.block_info()
    rhs = gaussian_rhs(locs, geom, (b,) * 3, ng)
    coef = region_coefficient(locs, geom, (b,) * 3, ng) if varying_d else None
    if coef is not None:
        om.set_coefficient(coef)
    om.rhs()[:] = rhs
    return sim, om, rhs, coef


def _interior(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng]


@pytest.mark.parametrize("varying_d", [False, True], ids=["constant-D", "region-D"])
def test_package_equation_vcycles_bitwise_oracle(app, tmp_path, varying_d):
    n, b, ng, alpha = 32, 8, 2, 10.0
    sim, om, rhs, coef = _setup(n, b, ng, alpha, varying_d)
    rms_o = om.run(4)
    u, it, res, _ = _run(app, tmp_path, n, b, ng, "MG", alpha, 4, 0.0, False, rhs, coef)
    assert it == 4
    assert np.array_equal(_interior(u, ng), _interior(om.u(), ng))
    np.testing.assert_allclose(res, rms_o[-1], rtol=1e-12)
    assert rms_o[-1] < 1e-2 * rms_o[0]


def test_package_equation_bicgstab_matches_oracle(app, tmp_path):
    n, b, ng, alpha = 32, 8, 2, 1.0
    sim, om, rhs, coef = _setup(n, b, ng, alpha, True)
    x, it_o, rms_o = om.bicgstab(rhs, precondition=True, rtol=1e-10, relative=True, max_iters=100)
    u, it, res, _ = _run(app, tmp_path, n, b, ng, "BiCGSTAB", alpha, 100, 1e-10, True, rhs, coef)
    # GetFinalIterations is the zero-based counter of the last iteration
    # (bicgstab_solver.hpp:138-143, 176-180), the oracle counts the iterations run
    assert it + 1 == it_o
    ref = _interior(x, ng)
    assert np.abs(_interior(u, ng) - ref).max() <= 1e-9 * np.abs(ref).max()
    np.testing.assert_allclose(res, rms_o, rtol=1e-6)


def test_package_equation_c4_shape_solve(app, tmp_path):
    # C4's mesh: 128^3 periodic in 16^3 blocks, V-cycles down to 1^3 blocks of 8^3 cells
    # (the coarsest grids of the layer's mesh), to an rms residual below 1e-10 of the
    # initial one; the oracle's restatement takes the same number of V-cycles
    n, b, ng, alpha = 128, 16, 2, 0.0
    sim, om, rhs, coef = _setup(n, b, ng, alpha, False)
    r0 = np.sqrt(np.mean(_interior(rhs, ng) ** 2))
    tol = 1e-10 * r0
    u, it, res, ms = _run(app, tmp_path, n, b, ng, "MG", alpha, 40, tol, False, rhs, coef)
    assert res <= tol
    rms_o = om.run(it)
    assert rms_o[-1] <= tol and (it == 1 or rms_o[-2] > tol)
    ref = _interior(om.u(), ng)
    assert np.array_equal(_interior(u, ng), ref)
    print("compat MGSolver<u, rhs, Eq> C4 solve: %d V-cycles, %.1f ms (warm)" % (it, ms))
