"""The oracle's multigrid converges (CPU): FAS V-cycles with SRJ2 or weighted Jacobi
reduce the rms residual every cycle on a periodic Poisson problem."""
import numpy as np

import oracle_lib as O
import parthenon_gb300 as pg


def test_vcycles_reduce_residual():
    n = 16
    o = O.OracleGmg(n, 2)
    o.rhs()[:] = pg.problems.poisson_rhs(n, ngauss=4, sigma=0.1, seed=1)
    r0 = o.residual()
    rms = o.run(6)
    assert np.all(np.diff(rms) < 0)
    assert rms[-1] < 1e-3 * r0


def test_jacobi_smoother_converges():
    n = 16
    o = O.OracleGmg(n, 2, stages=2, jacobi=True, weight=2.0 / 3.0, coarse_sweeps=8)
    o.rhs()[:] = pg.problems.poisson_rhs(n, ngauss=4, sigma=0.1, seed=1)
    r0 = o.residual()
    rms = o.run(8)
    assert rms[-1] < 1e-3 * r0


def test_oracle_bicgstab_converges_faster_with_multigrid():
    # right-preconditioned BiCGSTAB (bicgstab_solver.hpp): with a V-cycle per
    # application it needs far fewer iterations than without, and both reach the
    # requested relative residual
    n = 16
    o = O.OracleGmg(n, 2)
    rhs = pg.problems.poisson_rhs(n, ngauss=4, sigma=0.1, seed=1)
    x_mg, it_mg, rms_mg = o.bicgstab(rhs, precondition=True, rtol=1e-10)
    x_pl, it_pl, rms_pl = o.bicgstab(rhs, precondition=False, rtol=1e-10, max_iters=2000)
    tol = 1e-10 * np.sqrt((rhs ** 2).mean())
    assert rms_mg < tol and rms_pl < tol
    assert it_mg < it_pl / 3
    a, b = x_mg - x_mg.mean(), x_pl - x_pl.mean()
    assert np.abs(a - b).max() <= 1e-7 * np.abs(a).max()
