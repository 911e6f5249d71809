"""HEALPix geometry of the ray setup (replaces chealpix pix2ang_ring64,
snapshot-raytracer.cu:862-866): the product's implementation against the
oracle's independent one and against known answers of the published scheme."""
import math

import numpy as np
import pytest


@pytest.mark.parametrize("nside", [1, 2, 3, 4, 5, 8, 16, 33])
def test_pix2ang_product_vs_oracle(srt, orc, nside):
    for p in range(12 * nside * nside):
        t1, f1 = srt.pix2ang_ring(nside, p)
        t2, f2 = orc.pix2ang_ring(nside, p)
        assert abs(t1 - t2) < 4e-15 and abs(f1 - f2) < 4e-15 * max(1.0, f2), (nside, p)


def test_known_answers(srt):
    t, f = srt.pix2ang_ring(1, 0)
    assert t == pytest.approx(math.acos(2.0 / 3.0), abs=1e-15) and f == pytest.approx(math.pi / 4, abs=1e-15)
    t, f = srt.pix2ang_ring(1, 4)
    assert t == pytest.approx(math.pi / 2, abs=1e-15) and f == 0.0
    t, f = srt.pix2ang_ring(1, 11)
    assert t == pytest.approx(math.pi - math.acos(2.0 / 3.0), abs=1e-15) and f == pytest.approx(7 * math.pi / 4)
    # nside 2: first equatorial ring (ring 2) at z = 2/3, its first pixel at phi = pi/8
    t, f = srt.pix2ang_ring(2, 4)
    assert math.cos(t) == pytest.approx(2.0 / 3.0, abs=1e-15) and f == pytest.approx(math.pi / 8)


@pytest.mark.parametrize("nside", [1, 2, 4, 7, 16])
def test_ring_structure(srt, nside):
    """Rings run north to south; ring i holds min(4i, 4 nside, 4(4 nside - i))
    pixels at equal z; their phi are equally spaced."""
    zs = np.array([math.cos(srt.pix2ang_ring(nside, p)[0]) for p in range(12 * nside * nside)])
    start = 0
    for i in range(1, 4 * nside):
        cnt = min(4 * i, 4 * nside, 4 * (4 * nside - i))
        ring = zs[start:start + cnt]
        assert np.ptp(ring) < 1e-14
        if i < nside:
            assert ring[0] == pytest.approx(1 - i * i / (3.0 * nside * nside), abs=1e-15)
        elif i <= 3 * nside:
            assert ring[0] == pytest.approx(4.0 / 3 - 2.0 * i / (3.0 * nside), abs=1e-15)
        start += cnt
    assert start == 12 * nside * nside
    assert np.all(np.diff(zs) <= 1e-15)


@pytest.mark.parametrize("nside", [1, 2, 4, 8, 32])
def test_nest_ring_bijection(srt, nside):
    npix = 12 * nside * nside
    r = [srt.nest2ring(nside, p) for p in range(npix)]
    assert sorted(r) == list(range(npix))
    assert all(srt.ring2nest(nside, r[p]) == p for p in range(npix))


def test_nest_known_and_invalid(srt):
    assert srt.nest2ring(2, 0) == 13
    assert srt.nest2ring(1, 5) == 5
    assert srt.nest2ring(3, 0) == -1  # NESTED needs a power-of-two nside
    assert srt.nest2ring(4, 12 * 16) == -1


def test_nested_children_are_neighbours(srt):
    """The four NESTED children 4k..4k+3 of a parent pixel are within about one
    pixel size of each other (the locality the launch order relies on)."""
    nside = 16
    size = math.sqrt(4 * math.pi / (12 * nside * nside))
    for k in range(0, 12 * nside * nside // 4, 7):
        vecs = []
        for c in range(4):
            t, f = srt.pix2ang_ring(nside, srt.nest2ring(nside, 4 * k + c))
            vecs.append((math.sin(t) * math.cos(f), math.sin(t) * math.sin(f), math.cos(t)))
        v = np.array(vecs)
        d = np.sqrt(((v[:, None, :] - v[None, :, :]) ** 2).sum(-1)).max()
        assert d < 2.5 * size
