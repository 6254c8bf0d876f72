"""History output: file format, octant order and the oracle's MassHistory (no GPU)."""
import numpy as np

import oracle_lib as O
import parthenon_gb300 as pg
from parthenon_gb300 import history as H


def test_octant_order_matches_package():
    # burgers_package.cpp:106-119: x1 side outermost, x3 side innermost
    r = H.octant_regions((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    assert r.shape == (8, 6)
    np.testing.assert_array_equal(r[0], [-0.5, 0.0, -0.5, 0.0, -0.5, 0.0])
    np.testing.assert_array_equal(r[1], [-0.5, 0.0, -0.5, 0.0, 0.0, 0.5])
    np.testing.assert_array_equal(r[2], [-0.5, 0.0, 0.0, 0.5, -0.5, 0.0])
    np.testing.assert_array_equal(r[4], [0.0, 0.5, -0.5, 0.0, -0.5, 0.0])
    np.testing.assert_array_equal(r[7], [0.0, 0.5, 0.0, 0.5, 0.0, 0.5])


def test_file_format_matches_history_writer(tmp_path):
    # history.cpp:177-200 with data_format "%.14e" (burgers.pin), one blank prepended
    f = H.HistoryFile(str(tmp_path / "burgers.out1.hst"), ["MS Mass 0", "MS Mass 1"], "%.14e")
    f.write(0.0, 1.25e-3, 0, 512, [0.5, 0.25])
    f.write(0.01, 1.5e-3, 7, 520, [0.5000001, 0.2499999])
    text = open(f.path).read().splitlines()
    assert text[0] == "#  History data"
    assert text[1] == "# [1]=time     [2]=dt       [3]=cycle    [4]=nbtotal  [5]=MS Mass 0 [6]=MS Mass 1"
    assert text[2] == (" 0.00000000000000e+00 1.25000000000000e-03            0          512"
                       " 5.00000000000000e-01 2.50000000000000e-01")
    assert text[3].split()[2:4] == ["7", "520"]
    d = np.loadtxt(f.path)  # what burgers_diff.py reads
    assert d.shape == (2, 6)


def test_oracle_mass_history_against_numpy():
    nx, bnx, ng = (32, 32, 32), (8, 8, 8), 2
    o = O.OracleSim(nx, bnx, ng, xmin=(-0.5,) * 3, xmax=(0.5,) * 3, ncomp=4)
    rng = np.random.default_rng(3)
    o.base()[:] = rng.standard_normal(o.base().shape)
    regions = H.octant_regions((-0.5,) * 3, (0.5,) * 3)
    got = o.history_mass(regions, 1.0)
    locs, geom = o.block_info()
    u = np.array(o.base())[:, :, ng:-ng, ng:-ng, ng:-ng]
    bg = pg.problems.BlockGeometry(geom, ng, bnx)
    xs, ys, zs = bg.cell_centers()
    x = xs[:, ng:-ng][:, None, None, :]
    y = ys[:, ng:-ng][:, None, :, None]
    z = zs[:, ng:-ng][:, :, None, None]
    vol = np.prod(geom[:, 3:], axis=1)[:, None, None, None]
    for r, bx in enumerate(regions):
        m = ((bx[0] <= x) & (x <= bx[1]) & (bx[2] <= y) & (y <= bx[3]) & (bx[4] <= z) & (z <= bx[5]))
        want = (m[:, None] * u * u * (vol / (1.0 + 1e-20))[:, None]).sum()
        assert abs(got[r] - want) <= 1e-12 * abs(want)
    # the octants tile the domain: their sum is the whole-domain sum
    total = (u * u).sum() * (1.0 / 32) ** 3
    assert abs(got.sum() - total) <= 1e-12 * total
