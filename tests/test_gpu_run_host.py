"""The host-buffer entry point (the end-to-end path of the benchmark) vs the oracle.

pgb_run_host_dt copies the field in, fills the ghosts, runs K RK2 cycles and copies the
field and each cycle's next dt back: advection in the exact build is bit-exact (field
and every dt); Burgers WENO5 in the fast build is within 1e-12 relative.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import refined_cube
from parthenon_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def _run_host(mesh, cfg, state, ncomp, ncycles):
    L = nat.lib()
    p = cfg.params()
    src = np.ascontiguousarray(state, np.float64)
    out = np.zeros_like(src)
    dt = ctypes.c_double(0.0)
    dts = (ctypes.c_double * ncycles)()
    nat.check(L.pgb_run_host_dt(mesh.handle, ctypes.byref(p), src.ctypes.data_as(ctypes.c_void_p),
                                out.ctypes.data_as(ctypes.c_void_p), ncomp, ncycles, ctypes.byref(dt), dts),
              "pgb_run_host_dt")
    return out, dt.value, np.array(dts[:])


def test_run_host_advection_exact_bit_exact():
    nx, bnx, ng, ncycles = (32, 32, 32), (8, 8, 8), 2, 5
    leaves = refined_cube(2, 1, 3)
    mesh = pg.Mesh(nx, bnx, ng, leaves=leaves).upload()
    state = pg.problems.advection_state(mesh, nscalars=0)
    cfg = pg.StageConfig("advection", "plm", 0.3, exact=True)
    out, dt, dts = _run_host(mesh, cfg, state, 1, ncycles)
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=1, physics="advection", recon=1, cfl=0.3)
    o.base()[:] = state
    o.exchange(True, 0)
    o.init_dt()
    used = o.run(ncycles)
    assert np.array_equal(out, np.array(o.base()))
    assert dt == o.dt()
    # dt after cycle c is the dt the oracle uses in cycle c + 1
    assert np.array_equal(dts[:-1], used[1:]) and dts[-1] == o.dt()


def test_run_host_burgers_fast_within_tolerance():
    nx, bnx, ng, nc, ncycles = (32, 32, 32), (16, 16, 16), 4, 5, 3
    mesh = pg.Mesh(nx, bnx, ng).upload()
    state = pg.problems.burgers_state(mesh, nscalars=2, nmodes=8, kmax=4, seed=2)
    cfg = pg.StageConfig("burgers", "weno5", 0.8)
    out, dt, dts = _run_host(mesh, cfg, state, nc, ncycles)
    o = O.OracleSim(nx, bnx, ng, ncomp=nc, physics="burgers", recon=0, cfl=0.8, prolong_in_stage=False)
    o.base()[:] = state
    o.exchange(True, 0)
    o.init_dt()
    used = o.run(ncycles)
    r = np.array(o.base())
    sl = (slice(None), slice(None)) + (slice(ng, -ng),) * 3
    err = np.abs(out[sl] - r[sl]).max(axis=(0, 2, 3, 4)) / np.abs(r[sl]).max(axis=(0, 2, 3, 4))
    assert err.max() <= 1e-12, err
    np.testing.assert_allclose(dts[:-1], used[1:], rtol=1e-12)
    np.testing.assert_allclose(dt, o.dt(), rtol=1e-12)


def test_run_host_reuses_and_releases_its_workspace():
    """A second call reuses the mesh's device buffers and gives the same result; a call
    with another component count reallocates them; after a release the next call
    allocates them again."""
    nx, bnx, ng = (32, 32, 32), (8, 8, 8), 2
    leaves = refined_cube(2, 1, 3)
    mesh = pg.Mesh(nx, bnx, ng, leaves=leaves).upload()
    cfg = pg.StageConfig("advection", "plm", 0.3, exact=True)
    s1 = pg.problems.advection_state(mesh, nscalars=0)
    s3 = pg.problems.advection_state(mesh, nscalars=2)
    a1, dta, _ = _run_host(mesh, cfg, s1, 1, 3)
    b1, dtb, _ = _run_host(mesh, cfg, s1, 1, 3)
    assert np.array_equal(a1, b1) and dta == dtb
    c3, _, _ = _run_host(mesh, cfg, s3, 3, 2)
    nat.check(nat.lib().pgb_release_host_workspace(mesh.handle), "pgb_release_host_workspace")
    d3, _, _ = _run_host(mesh, cfg, s3, 3, 2)
    assert np.array_equal(c3, d3)
    # component 0 of the three-component run is the one-component run
    e1, _, _ = _run_host(mesh, cfg, s1, 1, 2)
    assert np.array_equal(e1[:, 0], d3[:, 0])
