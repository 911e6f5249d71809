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
