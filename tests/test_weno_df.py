"""The fast Burgers sweep's double-float reconstruction (weno_df.cuh) on the host.

The same header the GPU kernel compiles is built here with g++ (FP32 operations
separately rounded, no contraction) and marched along lines of cell values exactly as
the kernel marches them. Its face values must agree with WENO5-Z + MC blending
(benchmarks/burgers/recon.hpp:42-99, restated below in numpy in the reference's
operation order) to a few 1e-14 of the line's largest magnitude, whatever the line's
units, including lines with exactly constant stretches, jumps next to them, and
magnitudes far from one. The FP64 fallback expression must equal the restatement bit
for bit.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cxx", "weno_df_line.cpp")
OUT = os.path.join(ROOT, "tests", "cxx", "_build", "libweno_df_line.so")

# agreement with the reference expression, relative to the line's largest magnitude
TOL = 3e-14


@pytest.fixture(scope="module")
def lib():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-o", OUT, SRC])
    L = ctypes.CDLL(OUT)
    L.pgb_test_weno_line.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.pgb_test_weno_line.restype = ctypes.c_int
    L.pgb_test_weno_ref.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.pgb_test_df_roundtrip.argtypes = [ctypes.c_double]
    L.pgb_test_df_roundtrip.restype = ctypes.c_double
    L.pgb_test_df_op.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
    L.pgb_test_df_op.restype = ctypes.c_double
    L.pgb_test_df_roundtrip_raw.argtypes = [ctypes.c_double]
    L.pgb_test_df_roundtrip_raw.restype = ctypes.c_double
    L.pgb_test_df_pow2.argtypes = [ctypes.c_double, ctypes.c_int]
    L.pgb_test_df_pow2.restype = ctypes.c_double
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def weno5z_numpy(q):
    """recon.hpp:42-99 on every cell with a full stencil, in the reference's order."""
    q0, q1, q2, q3, q4 = q[:-4], q[1:-3], q[2:-2], q[3:-1], q[4:]
    eps = 10.0 * np.finfo(np.float64).eps
    tt = 13.0 / 3.0
    a = q0 - 2 * q1 + q2
    b = q0 - 4.0 * q1 + 3.0 * q2
    be0 = tt * a * a + b * b + eps
    a = q1 - 2.0 * q2 + q3
    b = q3 - q1
    be1 = tt * a * a + b * b + eps
    a = q2 - 2.0 * q3 + q4
    b = q4 - 4.0 * q3 + 3.0 * q2
    be2 = tt * a * a + b * b + eps
    tau = np.abs(be2 - be0)
    be0, be1, be2 = (be0 + tau) / be0, (be1 + tau) / be1, (be2 + tau) / be2

    def side(b0, b1, b2, p0, p1, p2):
        w0, w1, w2 = 0.1 * b0 + eps, 0.6 * b1 + eps, 0.3 * b2 + eps
        ws = 1.0 / (w0 + w1 + w2)
        x = w0 * p0
        x = x + w1 * p1
        x = x + w2 * p2
        x = x * ws
        al = 3.0 * ws * w0 * w1 * w2 / (0.3 * w0 * w1 + 0.6 * w0 * w2 + 0.1 * w1 * w2) + eps
        return x, al

    c = [(1.0 / 3.0, -7.0 / 6.0, 11.0 / 6.0), (-1.0 / 6.0, 5.0 / 6.0, 1.0 / 3.0), (1.0 / 3.0, 5.0 / 6.0, -1.0 / 6.0)]

    def poly(x, y, z, k):
        return c[k][0] * x + c[k][1] * y + c[k][2] * z

    xl, al = side(be0, be1, be2, poly(q0, q1, q2, 0), poly(q1, q2, q3, 1), poly(q2, q3, q4, 2))
    xr, ar = side(be2, be1, be0, poly(q4, q3, q2, 0), poly(q3, q2, q1, 1), poly(q2, q1, q0, 2))
    dm, dp = q2 - q1, q3 - q2
    dc = (dm * dp > 0.0) * 0.5 * (dm + dp)
    mn = np.where(np.abs(dp) < np.abs(dm), np.abs(dp), np.abs(dm))
    lim = np.where(2.0 * mn < np.abs(dc), 2.0 * mn, np.abs(dc))
    dq = 0.5 * np.copysign(lim, dc)
    alin = 2.0 * al * ar / (al + ar)
    return alin * xl + (1.0 - alin) * (q2 + dq), alin * xr + (1.0 - alin) * (q2 - dq)


def _lines():
    rng = np.random.default_rng(11)
    x = (np.arange(300) + 0.5) / 256
    base = {
        "sinusoids": np.sin(2 * np.pi * 3 * x) + 0.5 * np.sin(2 * np.pi * 5 * x + 1),
        "uniform-noise": rng.random(300),
        "step": np.where(x < 0.5, 1.0, 2.0),
        "constant": np.ones(300),
        "constant-with-box": np.where(np.abs(x - 0.5) < 0.1, 11.0, 1.0),
        "tanh-front": np.tanh(-20 * (x - 0.5)) * np.cos(np.pi * x) + 1.0,
        "gaussian-with-tails": np.exp(-((x - 0.5) / 0.03) ** 2),
        "zeros-with-spike": np.where(np.arange(300) == 150, 1.0, 0.0),
        "shock-on-slope": np.where(x < 0.3, 2.0, 0.1) + 0.01 * np.sin(2 * np.pi * x),
        "signed-noise": rng.standard_normal(300),
    }
    out = dict(base)
    for k in ("uniform-noise", "sinusoids", "constant-with-box"):
        out[k + "-times-1e-30"] = base[k] * 1e-30
        out[k + "-times-1e+30"] = base[k] * 1e30
    return out


LINES = _lines()


@pytest.mark.parametrize("name", list(LINES))
def test_line_matches_reference(lib, name):
    q = np.ascontiguousarray(LINES[name], np.float64)
    m = q.size
    ql, qr = np.zeros(m), np.zeros(m)
    lib.pgb_test_weno_line(_p(q), m, _p(ql), _p(qr))
    rl, rr = weno5z_numpy(q)
    scale = np.abs(q).max()
    assert np.abs(ql[2:-2] - rl).max() <= TOL * scale
    assert np.abs(qr[2:-2] - rr).max() <= TOL * scale


def _random_lines(count=100, seed=5):
    """Seeded lines of five kinds (signed noise, sinusoids of random wavenumber and
    phase, a random walk about 1, sparse spikes on 1, Gaussians of random width), each
    scaled by a random power of ten in [1e-5, 1e5]."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 1, 200)
    out = []
    for t in range(count):
        kind = t % 5
        if kind == 0:
            q = rng.standard_normal(200)
        elif kind == 1:
            q = np.sin(2 * np.pi * rng.uniform(1, 20) * x + rng.uniform(0, 6))
        elif kind == 2:
            q = np.cumsum(rng.standard_normal(200)) * 0.01 + 1.0
        elif kind == 3:
            q = np.where(rng.random(200) < 0.05, rng.standard_normal(200) * 5, 0.0) + 1.0
        else:
            q = np.exp(-((x - rng.uniform(0.2, 0.8)) / rng.uniform(0.01, 0.2)) ** 2)
        out.append(q * 10.0 ** rng.uniform(-5, 5))
    return out


def test_random_lines_match_reference(lib):
    worst = 0.0
    for q in _random_lines():
        q = np.ascontiguousarray(q, np.float64)
        ql, qr = np.zeros(q.size), np.zeros(q.size)
        lib.pgb_test_weno_line(_p(q), q.size, _p(ql), _p(qr))
        rl, rr = weno5z_numpy(q)
        scale = np.abs(q).max()
        worst = max(worst, np.abs(ql[2:-2] - rl).max() / scale, np.abs(qr[2:-2] - rr).max() / scale)
    assert worst <= TOL


@pytest.mark.parametrize("name", ["uniform-noise", "constant-with-box", "shock-on-slope"])
def test_fp64_fallback_is_the_reference_expression(lib, name):
    q = np.ascontiguousarray(LINES[name], np.float64)
    m = q.size
    ql, qr = np.zeros(m), np.zeros(m)
    lib.pgb_test_weno_ref(_p(q), m, _p(ql), _p(qr))
    rl, rr = weno5z_numpy(q)
    assert np.array_equal(ql[2:-2], rl) and np.array_equal(qr[2:-2], rr)


def test_jump_next_to_constant_takes_the_fallback(lib):
    q = np.ascontiguousarray(LINES["constant-with-box"])
    ql, qr = np.zeros(q.size), np.zeros(q.size)
    assert lib.pgb_test_weno_line(_p(q), q.size, _p(ql), _p(qr)) > 0
    q = np.ascontiguousarray(LINES["sinusoids"])
    assert lib.pgb_test_weno_line(_p(q), q.size, _p(ql), _p(qr)) == 0


def test_pair_arithmetic(lib):
    rng = np.random.default_rng(3)
    xs = rng.standard_normal(2000) * 10.0 ** rng.uniform(-20, 20, 2000)
    rt = np.array([lib.pgb_test_df_roundtrip(x) for x in xs])
    assert np.max(np.abs(rt - xs) / np.abs(xs)) < 8e-15  # 2^-47
    a, b = rng.uniform(0.1, 10, 500), rng.uniform(0.1, 10, 500)
    for op, ref, tol in [(0, a + b, 3e-14), (2, a * b, 3e-14), (3, a / b, 5e-14), (4, 1 / a, 5e-14),
                         (5, a * a, 3e-14), (6, 1 / a, 5e-14), (7, a / b, 5e-14)]:
        got = np.array([lib.pgb_test_df_op(op, x, y) for x, y in zip(a, b)])
        assert np.max(np.abs(got - ref) / np.abs(ref)) < tol, op
    # differences: absolute accuracy relative to the operands
    got = np.array([lib.pgb_test_df_op(1, x, y) for x, y in zip(a, b)])
    assert np.max(np.abs(got - (a - b)) / (np.abs(a) + np.abs(b))) < 3e-14


def test_unnormalised_conversions(lib):
    """from_double<false> keeps the value of the normalised conversion (only the split
    between the words differs); the increment conversion through 2^-off is exact."""
    rng = np.random.default_rng(5)
    xs = rng.standard_normal(2000) * 10.0 ** rng.uniform(-20, 20, 2000)
    raw = np.array([lib.pgb_test_df_roundtrip_raw(x) for x in xs])
    norm = np.array([lib.pgb_test_df_roundtrip(x) for x in xs])
    assert np.array_equal(raw, norm)
    for off in (-600, -40, 0, 3, 200, 700):
        x = xs * 2.0 ** -off  # scaled to magnitudes near 2^-off, as a line's increments are
        got = np.array([lib.pgb_test_df_pow2(v, off) for v in x])
        assert np.max(np.abs(got - x) / np.abs(x)) < 8e-15, off
