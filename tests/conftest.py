import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "snapshot-raytracer_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _ensure_built():
    import build_srt

    if not (os.path.isfile(build_srt.LIBSRT) and os.path.isfile(build_srt.LIBORACLE)):
        build_srt.build()


_ensure_built()


@pytest.fixture(scope="session")
def srt():
    import srt as _srt

    return _srt


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as _o

    return _o


@pytest.fixture(scope="session")
def golden():
    import json

    import numpy as np

    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "golden_cases.json")) as fh:
        meta = json.load(fh)
    maps = dict(np.load(os.path.join(d, "golden_maps.npz")))
    return meta, maps


def golden_fields(meta, case):
    import numpy as np

    import srt_fields

    c = meta["cases"][case]
    phi, b = srt_fields.int_noise_fields(tuple(c["extents"]), c["seed"])
    if c["zero_fields"]:
        phi, b = np.zeros_like(phi), np.zeros_like(b)
    return phi, b


def map_errors(a, b, ulps=1):
    from oracle.oracle import map_errors as _me

    return _me(a, b, ulps)


def has_gpu():
    import srt

    try:
        return srt.device_count() > 0
    except Exception:
        return False


def linear_phi_case(n=64, g=(3e-7, -2e-7, 4e-7)):
    """A potential with constant gradient g around the box centre (B = 0) and
    the first-order analytic maps of a ray of S steps through it: dn/ds = 2 g_perp
    gives a deflection D = -S g_perp (defl1 = D.theta_hat, defl2 = D.(sin phi,
    -cos phi, 0)), dA' = 1 - 4 (n0.g) s gives dA = S - 2 (n0.g) S^2, and the
    shear and rotation stay 0 (Catmull-Rom reproduces a linear field exactly).
    Rays of S < n/2 - 3 steps never reach the box faces, where the field jumps."""
    import numpy as np

    g = np.asarray(g, np.float64)
    x0 = n / 2
    i = np.arange(n)
    phi = (g[0] * (i[None, None, :] - x0) + g[1] * (i[None, :, None] - x0) + g[2] * (i[:, None, None] - x0))
    b = np.zeros((n, n, n, 3), np.float32)

    def predict(theta, phiang, S):
        n0 = -np.array([np.sin(theta) * np.cos(phiang), np.sin(theta) * np.sin(phiang), np.cos(theta)])
        th_hat = np.array([np.cos(theta) * np.cos(phiang), np.cos(theta) * np.sin(phiang), -np.sin(theta)])
        e2 = np.array([np.sin(phiang), -np.cos(phiang), 0.0])
        D = -S * (g - n0 * np.dot(n0, g))
        return S - 2 * np.dot(n0, g) * S * S, np.dot(D, th_hat), np.dot(D, e2)

    return phi.astype(np.float32), b, predict


def check_linear_phi_maps(maps, nside, S, predict, pix2ang):
    import numpy as np

    for p in range(maps.shape[1]):
        dA, d1, d2 = predict(*pix2ang(nside, p), S)
        assert abs(maps[0, p] - dA) <= 0.02 * abs(dA - S) + 4e-6, (p, maps[0, p], dA)
        assert abs(maps[4, p] - d1) <= 2e-3 * abs(d1) + 2e-9, (p, maps[4, p], d1)
        assert abs(maps[5, p] - d2) <= 2e-3 * abs(d2) + 2e-9, (p, maps[5, p], d2)
        assert abs(maps[1, p]) < 1e-9 and abs(maps[2, p]) < 1e-9 and abs(maps[3, p]) < 1e-12, p
