"""Synthetic field generators (srt_fields): the benchmark's Gaussian fields
have the requested rms, spectrum and a transverse B; the integer-noise
fixtures are exact and reproducible."""
import numpy as np

import srt_fields


def test_gaussian_fields_properties():
    n = 32
    phi, b = srt_fields.gaussian_fields_np(n, seed=5)
    assert phi.shape == (n, n, n) and b.shape == (n, n, n, 3)
    assert phi.dtype == np.float32 and b.dtype == np.float32
    assert abs(np.sqrt(np.mean(phi.astype(np.float64) ** 2)) / 1e-5 - 1) < 1e-5
    assert abs(np.sqrt(np.mean(b.astype(np.float64) ** 2)) / 1e-7 - 1) < 1e-5
    assert abs(phi.mean()) < 1e-6 * 1e-5 * n ** 3  # zero mode removed
    # divergence free: k . B(k) = 0
    kx = 2 * np.pi * np.fft.fftfreq(n)[None, None, :]
    ky = 2 * np.pi * np.fft.fftfreq(n)[None, :, None]
    kz = 2 * np.pi * np.fft.fftfreq(n)[:, None, None]
    B = [np.fft.fftn(b[..., c].astype(np.float64)) for c in range(3)]
    div = kx * B[0] + ky * B[1] + kz * B[2]
    mag = np.sqrt(sum(np.abs(x) ** 2 for x in B)) * np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    assert np.abs(div).max() < 1e-5 * mag.max()
    # spectrum: no power beyond the Nyquist sphere, P(k) ~ k^-3 inside
    F = np.abs(np.fft.fftn(phi.astype(np.float64))) ** 2
    k = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    assert F[k > np.pi * 1.0001].max() < 1e-12 * F.max()  # float32 rounding only
    lo = F[(k > 0.3) & (k < 0.4)].mean() * 0.35 ** 3
    hi = F[(k > 2.0) & (k < 2.3)].mean() * 2.15 ** 3
    assert 0.7 < lo / hi < 1.4


def test_int_noise_exact_and_reproducible():
    phi1, b1 = srt_fields.int_noise_fields(16, seed=3)
    phi2, b2 = srt_fields.int_noise_fields(16, seed=3)
    assert np.array_equal(phi1.view(np.uint32), phi2.view(np.uint32))
    assert np.array_equal(b1.view(np.uint32), b2.view(np.uint32))
    # exact multiples of the power-of-two scale
    q = phi1.astype(np.float64) * 2.0 ** 37
    assert np.array_equal(q, np.round(q))
    assert 3e-6 < phi1.std() < 3e-5 and 3e-8 < b1.std() < 3e-7
