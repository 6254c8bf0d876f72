"""The reference's own applications compile and link against the package-facing
compatibility layer and libparthenon_gb300.so without a changed line: the Burgers
benchmark (benchmarks/burgers: package, driver, problem generator, main), the
geometric-multigrid Poisson example (example/poisson_gmg: its PoissonEquation on
SparsePacks and face fields, MGSolver / BiCGSTABSolver on that equation, the driver's
task list) and the advection example (example/advection: block-level hooks and packs,
par_for_outer with team scratch and donor-cell reconstruction, a sparse pool, history
functions with Kokkos reducers, per-block time-step votes).

The reference sources are read where they lie when they are available (this is the one
test that reads them); the test is skipped elsewhere. Nothing is copied into the
repository and the binary is only built, not run (the GPU runs of the layer use the
repository's own package, tests/test_gpu_compat_burgers.py).
"""
import os

import pytest

from compat_build import compile_objects, link

REFERENCE = os.environ.get("PARTHENON_REFERENCE_DIR", "/root/reference")
BURGERS = os.path.join(REFERENCE, "benchmarks", "burgers")
POISSON = os.path.join(REFERENCE, "example", "poisson_gmg")
ADVECTION = os.path.join(REFERENCE, "example", "advection")


@pytest.mark.skipif(not os.path.isdir(BURGERS), reason="reference sources not available here")
def test_reference_burgers_app_builds_unchanged():
    srcs = [os.path.join(BURGERS, f) for f in
            ("burgers_package.cpp", "burgers_driver.cpp", "parthenon_app_inputs.cpp", "main.cpp")]
    objs = compile_objects(srcs, "refburgers", include=(BURGERS,))
    exe = link(objs, "reference_burgers_app")
    assert os.path.getsize(exe) > 0


@pytest.mark.skipif(not os.path.isdir(POISSON), reason="reference sources not available here")
def test_reference_poisson_gmg_app_builds_unchanged():
    srcs = [os.path.join(POISSON, f) for f in
            ("poisson_package.cpp", "poisson_driver.cpp", "parthenon_app_inputs.cpp", "main.cpp")]
    objs = compile_objects(srcs, "refpoisson", include=(POISSON,))
    exe = link(objs, "reference_poisson_app")
    assert os.path.getsize(exe) > 0


@pytest.mark.skipif(not os.path.isdir(ADVECTION), reason="reference sources not available here")
def test_reference_advection_app_builds_unchanged():
    srcs = [os.path.join(ADVECTION, f) for f in
            ("advection_package.cpp", "advection_driver.cpp", "parthenon_app_inputs.cpp", "main.cpp")]
    objs = compile_objects(srcs, "refadvection", include=(ADVECTION,))
    exe = link(objs, "reference_advection_app")
    assert os.path.getsize(exe) > 0
