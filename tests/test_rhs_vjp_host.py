"""The hand-written vjp of the right-hand side (srt_adjoint.cuh rhs_vjp, with
stage_view_fp64), built for the host in FP64 and checked without a GPU against
the right-hand side it differentiates (srt_scheme.cuh rhs_std<kFP64>,
snapshot-raytracer.cu:315-510): the state cotangent J(y)^T fb against central
differences along random directions, and the tap cotangents of the four
fields against the right-hand side's exact linearity in the field values. The
MIXED sweep runs the same template in FP32."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import srt_fields

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
N = 12


@pytest.fixture(scope="module")
def adj(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc)), "include")
    if not os.path.isfile(os.path.join(cuda_inc, "cuda_fp16.h")):
        pytest.skip("CUDA headers not found")
    out = str(tmp_path_factory.mktemp("adj") / "libadj.so")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                        "-I" + os.path.join(ROOT, "snapshot-raytracer_gb300", "csrc"), "-I" + cuda_inc,
                        os.path.join(ROOT, "tests", "adjoint_shim.cpp"), "-o", out], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("g++ failed: " + r.stderr[-300:])
    L = ctypes.CDLL(out)
    P, I = ctypes.c_void_p, ctypes.c_int
    L.rhs_fp64.argtypes = [P, P, P, P, P, P, I, I, I]
    L.rhs_vjp_fp64.argtypes = [P, P, P, P, P, P, P, P, P, P, P, I, I, I]
    return L


def padded(f):
    return np.ascontiguousarray(np.pad(f, ((1, 2), (1, 2), (1, 2)), mode="wrap"), np.float32)


def fields(seed, strength=1.0):
    phi, b = srt_fields.gaussian_fields_np(N, seed=seed)
    return [padded(b[..., c] * strength) for c in range(3)] + [padded(phi * strength)]


def rhs(L, y, F):
    dy = np.zeros(19)
    L.rhs_fp64(y.ctypes.data, dy.ctypes.data, F[3].ctypes.data, F[0].ctypes.data, F[1].ctypes.data,
               F[2].ctypes.data, N, N, N)
    return dy


def vjp(L, y, fb, F):
    yb = np.zeros(19)
    g = [np.zeros(F[0].shape) for _ in range(4)]
    L.rhs_vjp_fp64(y.ctypes.data, fb.ctypes.data, yb.ctypes.data, g[0].ctypes.data, g[1].ctypes.data,
                   g[2].ctypes.data, g[3].ctypes.data, F[3].ctypes.data, F[0].ctypes.data, F[1].ctypes.data,
                   F[2].ctypes.data, N, N, N)
    return yb, g


def random_state(rng, dA):
    """A ray state away from every cell face (centred and staggered)."""
    frac = rng.choice([rng.uniform(0.1, 0.4), rng.uniform(0.6, 0.9)], size=3)
    x = rng.integers(0, N, 3) + frac
    n = rng.standard_normal(3)
    n /= np.linalg.norm(n)
    a = np.cross(n, rng.standard_normal(3))
    a /= np.linalg.norm(a)
    b = np.cross(n, a)
    y = np.concatenate([x, -n * 1.01, a * 0.99, -b, [dA, -1.0 + 1e-3 * rng.standard_normal()],
                        1e-3 * rng.standard_normal(4), [1e-4 * rng.standard_normal()]])
    return y


@pytest.mark.parametrize("dA", [0.3, 7.5], ids=["before-the-switch", "after-the-switch"])
def test_state_cotangent_against_central_differences(adj, dA):
    rng = np.random.default_rng(31)
    F = fields(3, strength=300.0)  # strong fields, so every term of the right-hand side counts
    for _ in range(20):
        y = random_state(rng, dA)
        fb = rng.standard_normal(19)
        yb, _ = vjp(adj, y, fb, F)
        for _ in range(3):
            v = rng.standard_normal(19)
            eps = 1e-6
            fd = fb @ (rhs(adj, y + eps * v, F) - rhs(adj, y - eps * v, F)) / (2 * eps)
            assert abs(yb @ v - fd) <= 1e-6 * (abs(fd) + np.abs(fb).sum() * 1e-3), (yb @ v, fd)


def test_field_cotangents_against_linearity(adj):
    """The right-hand side is affine in the field values at fixed state, so
    fb . (f(y; dF) - f(y; 0)) must equal sum(g . dF) to rounding."""
    rng = np.random.default_rng(32)
    zero = [np.zeros_like(f) for f in fields(4)]
    for _ in range(20):
        y = random_state(rng, rng.choice([0.3, 7.5]))
        fb = rng.standard_normal(19)
        F = fields(int(rng.integers(1000)))
        _, g = vjp(adj, y, fb, F)
        for c in range(4):
            dF = [z.copy() for z in zero]
            dF[c] = (rng.standard_normal(zero[c].shape) * 1e-5).astype(np.float32)
            want = fb @ (rhs(adj, y, dF) - rhs(adj, y, zero))
            got = float(np.sum(g[c] * dF[c]))
            assert abs(got - want) <= 1e-9 * (abs(want) + 1e-12), (c, got, want)
        # taps outside the ray's 4x4x4 footprints get nothing
        assert sum(int(np.count_nonzero(gc)) for gc in g) <= 4 * 64


def test_mixed_sweep_indices_stay_in_the_padded_grids(adj):
    """Index audit of the MIXED sweep's field passes, built for the host: every
    tap read and every tap-cotangent row of rhs_vjp on stage_view_mixed (the
    arithmetic of sweep_kernel_mixed) for rays in all directions at affine
    distances up to several box lengths (positions wrap around the periodic
    box), with perturbations up to a few cells, stays inside the halo-padded
    grid, and the row-pair reads inside the row-pair array. The fields are
    zero: only the indices are checked."""
    import ctypes

    adj.audit_vjp_indices_mixed.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 5
    rng = np.random.default_rng(12)
    for n0, n1, n2 in ((12, 12, 12), (16, 20, 24), (7, 5, 9)):
        count = 4000
        theta = np.arccos(rng.uniform(-1, 1, count))
        phi = rng.uniform(0, 2 * np.pi, count)
        s = np.concatenate([rng.uniform(0, 4 * max(n0, n1, n2), count - 8),
                            np.array([0, 0.5, 1, n0 / 2, n0 / 2 + 0.5, n0, 2 * n0, 3.5 * n0])]).astype(np.float32)
        d = (rng.standard_normal((count, 19)) * rng.choice([1e-6, 1e-3, 2.0], (count, 1))).astype(np.float32)
        # positions exactly on faces of both grids
        d[:16, :3] = 0
        out = np.zeros(5, np.int64)
        adj.audit_vjp_indices_mixed(n0, n1, n2, count, theta.ctypes.data, phi.ctypes.data, s.ctypes.data,
                                    d.ctypes.data, out.ctypes.data)
        lo, hi, hip, pvox, npair = (int(x) for x in out)
        assert lo >= 0, (n0, n1, n2, lo)
        assert hi < pvox, (n0, n1, n2, hi, pvox)
        assert hip < npair, (n0, n1, n2, hip, npair)
