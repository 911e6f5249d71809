"""The double-float arithmetic of the re-trace (srt_dd.cuh), built for the
host: sums, products, quotients, square roots and floors of random
double-floats agree with exact rational arithmetic to ~2^-44 relative."""
import ctypes
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ddlib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("dd") / "libdd.so")
    src = os.path.join(ROOT, "tests", "dd_shim.cpp")
    inc = os.path.join(ROOT, "snapshot-raytracer_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I" + inc, src, "-o",
                        out], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("g++ failed: " + r.stderr[-300:])
    L = ctypes.CDLL(out)
    P = ctypes.POINTER(ctypes.c_float)
    for n in ("dd_add", "dd_mul", "dd_div"):
        getattr(L, n).argtypes = [P, P, P]
    L.dd_sqrt_.argtypes = [P, P]
    L.dd_floor_.argtypes = [P, P]
    L.dd_from_double.argtypes = [ctypes.c_double, P]
    return L


def _dd(L, x):
    r = (ctypes.c_float * 2)()
    L.dd_from_double(float(x), r)
    return r


def _val(r):
    return Fraction(float(r[0])) + Fraction(float(r[1]))


def test_dd_operations_are_accurate(ddlib):
    L = ddlib
    rng = np.random.default_rng(1)
    out = (ctypes.c_float * 2)()
    worst = {"add": 0.0, "mul": 0.0, "div": 0.0, "sqrt": 0.0}
    for _ in range(400):
        x = rng.standard_normal() * 10.0 ** rng.integers(-6, 4)
        y = rng.standard_normal() * 10.0 ** rng.integers(-6, 4)
        a, b = _dd(L, x), _dd(L, y)
        fa, fb = _val(a), _val(b)
        # the double-float of a double keeps its leading ~48 bits
        assert abs(fa - Fraction(x)) <= abs(Fraction(x)) * Fraction(1, 2 ** 47)
        for name, fn, exact in (("add", L.dd_add, fa + fb), ("mul", L.dd_mul, fa * fb), ("div", L.dd_div, fa / fb)):
            fn(a, b, out)
            if exact != 0:
                worst[name] = max(worst[name], float(abs(_val(out) - exact) / abs(exact)))
        sa = _dd(L, abs(x))
        L.dd_sqrt_(sa, out)
        got = _val(out)
        worst["sqrt"] = max(worst["sqrt"], float(abs(got * got - _val(sa)) / _val(sa)))
    # additions of values of different signs are exact up to the final rounding
    assert worst["add"] < 2.0 ** -44, worst
    assert worst["mul"] < 2.0 ** -44, worst
    assert worst["div"] < 2.0 ** -43, worst
    assert worst["sqrt"] < 2.0 ** -43, worst


def test_dd_floor(ddlib):
    L = ddlib
    out = (ctypes.c_float * 2)()
    for v in (0.0, 1.5, -1.5, 3.0, 1e6 + 0.25, -(1e6 + 0.25), 2.0 ** 30 + 0.5, 17.0 - 2.0 ** -30, -2.0 ** -30):
        a = _dd(L, v)
        L.dd_floor_(a, out)
        assert _val(out) == Fraction(int(np.floor(float(_val(a))))), v
