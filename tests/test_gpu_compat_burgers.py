"""A Burgers package written against the Parthenon package interface (StateDescriptor,
Metadata, MeshData packs, par_for / par_for_outer with team scratch / par_reduce, a
TaskList per stage following benchmarks/burgers/burgers_driver.cpp:53-148) runs through
the compatibility layer on the GPU, and its state after three RK2 cycles -- fields with
ghosts, the derived field and dt -- equals the oracle's bit for bit (the package and
the layer round every operation in the reference's order).
"""
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as O
from compat_build import OUT, ROOT, compile_objects, link

pytestmark = pytest.mark.gpu

DECK = """
<parthenon/job>
problem_id = burgers
<parthenon/mesh>
nghost = 4
refinement = none
nx1 = 64
x1min = -0.5
x1max = 0.5
ix1_bc = periodic
ox1_bc = periodic
nx2 = 64
x2min = -0.5
x2max = 0.5
ix2_bc = periodic
ox2_bc = periodic
nx3 = 64
x3min = -0.5
x3max = 0.5
ix3_bc = periodic
ox3_bc = periodic
<parthenon/meshblock>
nx1 = 32
nx2 = 32
nx3 = 32
<parthenon/time>
nlim = 3
tlim = 10.0
integrator = rk2
<burgers>
cfl = 0.8
num_scalars = 8
"""


@pytest.fixture(scope="module")
def app():
    src = os.path.join(ROOT, "tests", "cxx", "burgers_compat")
    objs = compile_objects([os.path.join(src, "burgers.cpp"), os.path.join(src, "main.cpp")], "compatburgers",
                           extra=("-fmad=false",))
    return link(objs, "compat_burgers_app")


def test_compat_burgers_three_cycles_bitwise_oracle(app, tmp_path):
    deck = tmp_path / "burgers.in"
    deck.write_text(DECK)
    prefix = str(tmp_path / "run")
    r = subprocess.run([app, "-i", str(deck), "-o", prefix], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    nb, nc, N = 8, 11, 40
    init = np.fromfile(prefix + "_init.bin").reshape(nb, nc, N, N, N)
    final = np.fromfile(prefix + "_final.bin").reshape(nb, nc, N, N, N)
    derived = np.fromfile(prefix + "_derived.bin").reshape(nb, N, N, N)
    time, dt, ncycle = open(prefix + "_time.txt").read().split()
    assert int(ncycle) == 3
    o = O.OracleSim((64,) * 3, (32,) * 3, 4, xmin=(-0.5,) * 3, xmax=(0.5,) * 3, ncomp=nc, physics="burgers",
                    recon=0, cfl=0.8, prolong_in_stage=False)
    o.base()[:] = init
    o.exchange(False, 0)
    assert np.array_equal(np.array(o.base()), init)  # the layer's initial ghost fill
    o.init_dt()
    o.run(3)
    assert np.array_equal(final, np.array(o.base()))
    g = slice(4, -4)
    assert np.array_equal(derived[:, g, g, g], np.array(o.derived())[:, g, g, g])
    assert float(dt) == o.dt()
    assert float(time) == o.time()
    # the state is not trivial: the fronts moved
    assert not np.array_equal(final, init)
