"""RK2 evolution on the GPU vs the oracle.

Exact build (separately rounded arithmetic in the reference's order): bit-for-bit.
Fast build (FMA contraction, shared reciprocals): within 1e-12 relative on the
interior (the FP64 tolerance of the hot path), scaled by the field's magnitude.
"""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from meshes import refined_cube

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12


def _interior(a, ng):
    return a[:, :, ng:-ng, ng:-ng, ng:-ng]


def _run(case, exact, ncycles):
    nx, bnx, ng, leaves, physics, recon, ncomp, cfl, state = case
    o = O.OracleSim(nx, bnx, ng, leaves=leaves, ncomp=ncomp, physics=physics,
                    recon={"dc": 0, "plm": 1, "weno5": 0, "linear": 1}[recon], cfl=cfl,
                    prolong_in_stage=(physics != "burgers"))
    m = pg.Mesh(nx, bnx, ng, leaves=leaves)
    host = state(m)
    u = o.base()
    u[:] = host
    o.exchange(True, 0)  # initial CommunicateBoundaries prolongates for every package
    dt0 = o.init_dt()
    dts = o.run(ncycles)
    drv = pg.RK2Driver(m, ncomp, pg.StageConfig(physics, recon, cfl, exact=exact))
    drv.set_state(host)
    drv.run(ncycles, graph=True)
    drv.stream.synchronize()
    got = drv.base.cpu().numpy()
    if physics == "burgers":
        # FillDerived after every stage: the last stage's output
        _DERIVED[(exact, id(case))] = (drv.derived.cpu().numpy()[:, 0], np.array(o.derived()))
    return got, np.array(o.base()), float(drv.dt.cpu()[0]), o.dt(), dt0, dts


_DERIVED = {}


def _advection_gaussian(m):
    return pg.problems.advection_state(m)


def _advection_smr(m):
    return pg.problems.advection_state(m, nscalars=4, seed=3)


def _burgers(m):
    return pg.problems.burgers_state(m, nscalars=8, nmodes=8, kmax=4, seed=2)


def _burgers_reference_ic(m):
    # the reference benchmark's own initial condition, centred in the unit cube
    return pg.problems.burgers_reference_state(m, nscalars=8, center=(0.5, 0.5, 0.5))


def _burgers5(m):
    return pg.problems.burgers_state(m, nscalars=2, nmodes=16, kmax=6, seed=5)


CASES = {
    "advection-dc-64": ((64,) * 3, (16,) * 3, 2, None, "advection", "dc", 1, 0.3, _advection_gaussian),
    "advection-plm-64": ((64,) * 3, (16,) * 3, 2, None, "advection", "plm", 1, 0.3, _advection_gaussian),
    "burgers-weno5": ((32,) * 3, (16,) * 3, 4, None, "burgers", "weno5", 11, 0.8, _burgers),
    "burgers-linear": ((32,) * 3, (16,) * 3, 4, None, "burgers", "linear", 11, 0.8, _burgers),
    "burgers-5comp": ((32,) * 3, (16,) * 3, 4, None, "burgers", "weno5", 5, 0.8, _burgers5),
    "smr-advection-plm": ((32,) * 3, (8,) * 3, 4, refined_cube(2, 1, 3), "advection", "plm", 5, 0.3,
                          _advection_smr),
    # one block that is its own neighbour in every direction
    "single-block-burgers": ((16,) * 3, (16,) * 3, 4, None, "burgers", "weno5", 5, 0.8, _burgers5),
    # multilevel Burgers: stored face fluxes, flux correction, divergence update
    "smr-burgers-weno5": ((32,) * 3, (8,) * 3, 4, refined_cube(2, 1, 3), "burgers", "weno5", 5, 0.8, _burgers5),
    "smr-burgers-11": ((32,) * 3, (8,) * 3, 4, refined_cube(2, 0, 2), "burgers", "weno5", 11, 0.8, _burgers),
    # the uniform Burgers benchmark's block shape: 32^3 blocks, 4 ghosts, 11 components
    "burgers-weno5-64-32cubed-blocks": ((64,) * 3, (32,) * 3, 4, None, "burgers", "weno5", 11, 0.8, _burgers),
    # one 64^3 block (its own neighbour): the fast sweep's shared-memory coefficient
    # buffers exceed the default 48 KB from n = 48 on and take the opt-in launch attribute
    "single-block-64cubed-burgers": ((64,) * 3, (64,) * 3, 4, None, "burgers", "weno5", 5, 0.8, _burgers5),
    # the reference's own Burgers initial condition: exactly constant scalars with a
    # box of +10 (jumps next to constant stretches) and tanh fronts
    "burgers-reference-ic-32": ((32,) * 3, (8,) * 3, 4, None, "burgers", "weno5", 11, 0.8, _burgers_reference_ic),
    # the static-refinement advection benchmark's own mesh: 128^3 root in 16^3 blocks,
    # central 1/8 refined once (448 + 512 blocks), 4 ghosts, 5 components, PLM
    "smr-advection-plm-128root-16cubed": ((128,) * 3, (16,) * 3, 4, refined_cube(3, 2, 6), "advection", "plm", 5,
                                          0.3, _advection_smr),
}

# cycles per case (default: 10 for advection, 3 for Burgers)
NCYCLES = {"smr-advection-plm-128root-16cubed": 2}


def _ncycles(name):
    return NCYCLES.get(name, 10 if "advection" in name else 3)


@pytest.mark.parametrize("name", list(CASES))
def test_exact_build_bit_exact(name):
    got, ref, dtg, dto, _, _ = _run(CASES[name], True, _ncycles(name))
    ng = CASES[name][2]
    assert dtg == dto
    assert np.array_equal(_interior(got, ng), _interior(ref, ng))
    if CASES[name][4] == "burgers":
        dg, do = _DERIVED.pop((True, id(CASES[name])))
        assert np.array_equal(dg[:, ng:-ng, ng:-ng, ng:-ng], do[:, ng:-ng, ng:-ng, ng:-ng])


@pytest.mark.parametrize("name", list(CASES))
def test_fast_build_within_tolerance(name):
    got, ref, dtg, dto, _, _ = _run(CASES[name], False, _ncycles(name))
    ng = CASES[name][2]
    g, r = _interior(got, ng), _interior(ref, ng)
    scale = np.abs(r).max(axis=(0, 2, 3, 4), keepdims=True)
    err = np.abs(g - r) / scale
    assert err.max() <= REL_TOL, err.max()
    assert abs(dtg - dto) <= REL_TOL * dto
    if CASES[name][4] == "burgers":
        dg, do = _DERIVED.pop((False, id(CASES[name])))
        dg, do = dg[:, ng:-ng, ng:-ng, ng:-ng], do[:, ng:-ng, ng:-ng, ng:-ng]
        assert np.abs(dg - do).max() <= REL_TOL * np.abs(do).max()
