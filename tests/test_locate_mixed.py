"""The MIXED form's cell lookup (locate_mixed in srt_scheme.cuh), built for the
host: for a position given as an unevaluated float sum th + lo, the centred and
staggered cells must be exactly those of the exact sum (the cell choice is
what the cell-face guard and the FP64 re-trace rely on), and the offsets and
the distance from the nearest face must be the exact values rounded once, up
to ~1e-15 grid units (checked against rational arithmetic). Positions just
below a face under th, or th in (-1/2, 0), are the cases where a float
subtraction rounds."""
import ctypes
import math
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ULP1 = Fraction(1, 2 ** 24)  # half an ulp of 1.0: the rounding error bound on [0, 1]


@pytest.fixture(scope="module")
def loc(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    if not os.path.isfile(os.path.join(cuda_inc, "cuda_fp16.h")):
        pytest.skip("CUDA headers not found")
    out = str(tmp_path_factory.mktemp("loc") / "libscheme.so")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                        "-I" + os.path.join(ROOT, "snapshot-raytracer_gb300", "csrc"), "-I" + cuda_inc,
                        os.path.join(ROOT, "tests", "scheme_shim.cpp"), "-o", out], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("g++ failed: " + r.stderr[-300:])
    L = ctypes.CDLL(out)
    L.rsqrt1p_m1.argtypes = [ctypes.c_float]
    L.rsqrt1p_m1.restype = ctypes.c_float
    PI, PF = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_float)
    L.locate.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int, PI, PF, PI, PF, PF]

    def call(th, lo, n):
        cc, cs = ctypes.c_int(), ctypes.c_int()
        tc, ts, df = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        L.locate(th, lo, n, ctypes.byref(cc), ctypes.byref(tc), ctypes.byref(cs), ctypes.byref(ts),
                 ctypes.byref(df))
        return cc.value, tc.value, cs.value, ts.value, df.value

    call.rsqrt1p_m1 = L.rsqrt1p_m1
    return call


def check(call, th, lo, n):
    th, lo = float(np.float32(th)), float(np.float32(lo))
    cc, tc, cs, ts, df = call(th, lo, n)
    x = Fraction(th) + Fraction(lo)
    cell = math.floor(x)
    frac = x - cell
    stag = math.floor(x - Fraction(1, 2))
    fs = x - Fraction(1, 2) - stag
    where = "th=%r lo=%r n=%d" % (th, lo, n)
    assert cc == cell % n, where
    assert cs == stag % n, where
    assert 0.0 <= tc <= 1.0 and 0.0 <= ts <= 1.0, where
    assert abs(Fraction(tc) - frac) <= ULP1, where
    assert abs(Fraction(ts) - fs) <= ULP1, where
    # the distance: one rounding, plus the roundings of the remainder e
    # (~1e-15 grid units, far below the smallest guard width, ~4e-10)
    d = min(frac, 1 - frac, abs(frac - Fraction(1, 2)))
    assert abs(Fraction(df) - d) <= d / 2 ** 23 + Fraction(1, 2 ** 40), where


def test_random_positions(loc):
    rng = np.random.default_rng(11)
    for n in (16, 128, 1024, 2048):
        for _ in range(3000):
            th = np.float32(rng.uniform(-3.0, n + 3.0))
            lo = np.float32(rng.choice([0.0, 1.0]) * rng.standard_normal() * 10.0 ** rng.uniform(-12, 0))
            check(loc, th, lo, n)


def test_faces_and_half_faces(loc):
    """Positions on, and a hair either side of, the centred faces (integers)
    and the staggered faces (half-integers), where the sign of a tiny lo decides
    the cell."""
    for n in (16, 1024):
        for k in (0, 1, 7, n // 2, n - 1, n, -1):
            for base in (Fraction(k), Fraction(2 * k + 1, 2)):
                for eps in (0.0, 1e-30, 1e-12, 3e-8, 1e-6):
                    for sign in (1.0, -1.0):
                        lo = sign * eps
                        check(loc, float(base), lo, n)
                        # the same sum split differently: th one ulp off, lo compensating
                        th = np.nextafter(np.float32(float(base)), np.float32(np.inf))
                        rest = float(Fraction(float(base)) - Fraction(float(th)))
                        if np.float32(rest) == rest:
                            check(loc, th, rest + lo if np.float32(rest + lo) == rest + lo else rest, n)


def test_ray_positions_of_the_trace(loc):
    """th + lo as the trace forms them: x0 - s n0 split exactly (FMA) plus a
    small perturbation, along steps and stages of a ray."""
    rng = np.random.default_rng(12)
    n = 1024
    x0 = np.float32(n / 2)
    for _ in range(200):
        n0 = np.float32(rng.uniform(-1, 1))
        dx = rng.standard_normal() * 1e-3
        for s in (0.0, 0.5, 1.0, 37.5, 255.0, 511.5, 512.0):
            s = np.float32(s)
            p = np.float32(s * n0)
            pe = float(Fraction(float(s)) * Fraction(float(n0)) - Fraction(float(p)))  # the FMA residual
            th = np.float32(x0 - p)
            tl = float(Fraction(float(x0)) - Fraction(float(p)) - Fraction(float(th)))
            lo = np.float32(np.float32(tl - pe) + np.float32(dx))
            check(loc, th, lo, n)


def test_far_outside_the_box(loc):
    """Rays that wrapped around the periodic box many times: positions far
    outside [0, n) still give the exact cells modulo n (every tap index stays
    in range), through the integer wrap of the cell index."""
    rng = np.random.default_rng(14)
    for n in (16, 1000, 1024):
        for _ in range(2000):
            th = np.float32(rng.choice([-1.0, 1.0]) * 10.0 ** rng.uniform(1, 6.5))
            lo = np.float32(rng.standard_normal() * 1e-3)
            check(loc, th, lo, n)


def test_unresolvable_and_non_finite_positions_stay_in_range(loc):
    """Positions beyond 2^24 cells (where FP32 no longer resolves a cell) and
    non-finite positions (non-finite field values) still give cells inside
    the grid, so every tap index stays inside the halo-padded arrays; the wrap
    is exact below 2^24 cells (test_far_outside_the_box)."""
    inf, nan = float("inf"), float("nan")
    for n in (16, 1000, 1024):
        for th in (3e7, -3e7, 3e9, -3e9, 1e38, -1e38, inf, -inf, nan):
            for lo in (0.0, 1e-3, -1e-3, nan):
                cc, tc, cs, ts, df = loc(th, lo, n)
                assert 0 <= cc < n and 0 <= cs < n, (th, lo, n, cc, cs)


def test_normalisation_term_without_cancellation(loc):
    """rsqrt1p_m1(q) = (1 + q)^(-1/2) - 1, the correction that keeps a
    perturbed unit vector unit, in the closed form -q / (s (1 + s)),
    s = (1 + q)^(1/2): no cancellation for the tiny q of the perturbation
    form (|q| ~ 1e-5 and far below) nor for large q, so its relative error
    stays at a few float ulps everywhere (host build, IEEE sqrt and division;
    the GPU build's fast-math sqrt and division add ~2 ulps)."""
    rng = np.random.default_rng(3)
    qs = np.concatenate([np.float32(np.sign(rng.standard_normal(400)) * 10.0 ** rng.uniform(-30, -1, 400)),
                         np.float32(rng.uniform(-0.9, 10.0, 200)), np.float32([0.0])])
    worst = 0.0
    for q in qs:
        got = loc.rsqrt1p_m1(float(q))
        sq = math.sqrt(1.0 + float(q))  # float q is exact in double
        exact = -float(q) / (sq * (1.0 + sq))  # no cancellation: ~1e-16 relative
        if q == 0.0:
            assert got == 0.0
            continue
        worst = max(worst, abs(got - exact) / abs(exact))
    assert worst < 4 * 2.0 ** -23, worst
