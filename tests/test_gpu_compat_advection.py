"""An advection package written against the block-level Parthenon package interface
(fluxes per block from MeshBlockData packs with par_for_outer team scratch and the
donor-cell team helpers, a per-block time-step vote, block fill-derived hooks writing a
dense field and a sparse pool, Kokkos::MinMax per block, a volume-weighted history sum,
the task regions of example/advection/advection_driver.cpp:60-162) runs through the
compatibility layer on the GPU. After four RK2 cycles its state -- fields with ghosts,
dt and time -- equals the oracle's advection run (advection_package.cpp:465-647, donor
cell) bit for bit; the derived fields, block extrema and history sums are checked
against numpy on that state.
"""
import os
import subprocess

import numpy as np
import pytest

import oracle_lib as O
from compat_build import ROOT, compile_objects, link

pytestmark = pytest.mark.gpu

NC = 3
VEL = (1.0, -0.5, 0.75)
DECK = """
<parthenon/job>
problem_id = advection
<parthenon/mesh>
nghost = 2
refinement = none
nx1 = 64
x1min = -0.5
x1max = 0.5
nx2 = 64
x2min = -0.5
x2max = 0.5
nx3 = 64
x3min = -0.5
x3max = 0.5
<parthenon/meshblock>
nx1 = 16
nx2 = 16
nx3 = 16
<parthenon/time>
nlim = 4
tlim = 10.0
integrator = rk2
<Advection>
cfl = 0.45
vx = %r
vy = %r
vz = %r
num_components = %d
""" % (VEL + (NC,))


@pytest.fixture(scope="module")
def app():
    src = os.path.join(ROOT, "tests", "cxx", "advection_compat")
    objs = compile_objects([os.path.join(src, "advection.cpp"), os.path.join(src, "main.cpp")], "compatadvection",
                           extra=("-fmad=false",))
    return link(objs, "compat_advection_app")


def test_compat_advection_block_interface_matches_oracle(app, tmp_path):
    deck = tmp_path / "advection.in"
    deck.write_text(DECK)
    prefix = str(tmp_path / "run")
    r = subprocess.run([app, "-i", str(deck), "-o", prefix], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "PARTHENON ERROR" not in r.stdout + r.stderr
    ng, bn = 2, 16
    N = bn + 2 * ng
    nb = 4 * 4 * 4
    shape = (nb, NC, N, N, N)
    init = np.fromfile(prefix + "_init.bin").reshape(shape)
    final = np.fromfile(prefix + "_final.bin").reshape(shape)
    time, dt, ncycle = open(prefix + "_time.txt").read().split()
    assert int(ncycle) == 4

    o = O.OracleSim((64, 64, 64), (bn,) * 3, ng, xmin=(-0.5,) * 3, xmax=(0.5,) * 3, ncomp=NC,
                    physics="advection", recon=0, cfl=0.45, vel=VEL)
    o.base()[:] = init
    o.exchange(False, 0)
    assert np.array_equal(np.array(o.base()), init)  # the layer's initial ghost fill
    o.init_dt()
    o.run(4)
    ref = np.array(o.base())
    assert np.array_equal(final, ref)
    assert float(dt) == o.dt()
    assert float(time) == o.time()
    assert not np.array_equal(final, init)  # the profile moved

    # block fill-derived hooks on the final state (ghosts included), the sparse pool
    sq = np.fromfile(prefix + "_sq.bin").reshape(shape)
    p2 = np.fromfile(prefix + "_pow2.bin").reshape(shape)
    p5 = np.fromfile(prefix + "_pow5.bin").reshape(shape)
    assert np.array_equal(sq, final * final)
    assert np.array_equal(p2, sq)
    assert np.array_equal(p5, sq * sq * final)

    # per-block extrema of the last stage (Kokkos::MinMax through MeshBlock::par_reduce)
    mm = np.loadtxt(prefix + "_minmax.txt").reshape(nb, 2)
    assert np.array_equal(mm[:, 0], final.reshape(nb, -1).min(axis=1))
    assert np.array_equal(mm[:, 1], final.reshape(nb, -1).max(axis=1))

    # the history sum (Kokkos::Sum<Real, HostExecSpace>) before and after the run
    hist = [float(line.split()[1]) for line in open(prefix + "_hist.txt")]
    g = slice(ng, ng + bn)
    vol = (1.0 / 64) ** 3
    for h, state in zip(hist, (init, final)):
        want = float(np.sum(state[:, 0, g, g, g]) * vol)
        assert abs(h - want) <= 1e-12 * abs(want)
