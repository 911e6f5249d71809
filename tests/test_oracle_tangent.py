"""The oracle's forward-mode tangent (the checker of the GPU vjp): its value
equals the FP64 oracle's loss and its derivatives agree with central
differences of that loss."""
import numpy as np

import srt_fields


def test_tangent_value_and_central_differences(orc):
    phi, b = srt_fields.int_noise_fields(16, seed=3)
    nside, steps, pix = 2, 10, np.arange(48)
    w = np.random.default_rng(0).standard_normal((6, 48)).astype(np.float32)
    L, _ = orc.tangent(phi, b, nside, steps, pix, w)
    maps = orc.trace(phi, b, nside, steps, mode="fp64")
    assert abs(L - float((w.astype(np.float64) * maps).sum())) < 1e-6 * abs(L)
    rng = np.random.default_rng(1)
    dphi = rng.standard_normal(phi.shape).astype(np.float32) * np.float32(1e-5)
    db = rng.standard_normal(b.shape).astype(np.float32) * np.float32(1e-7)
    _, (d1, d2) = orc.tangent(phi, b, nside, steps, pix, w, dir_phi=[dphi, None], dir_b=[None, db])
    eps = 1e-3
    fd1 = (orc.tangent(phi + eps * dphi, b, nside, steps, pix, w)[0] -
           orc.tangent(phi - eps * dphi, b, nside, steps, pix, w)[0]) / (2 * eps)
    fd2 = (orc.tangent(phi, b + eps * db, nside, steps, pix, w)[0] -
           orc.tangent(phi, b - eps * db, nside, steps, pix, w)[0]) / (2 * eps)
    assert abs(fd1 - d1) < 1e-4 * abs(d1)
    assert abs(fd2 - d2) < 1e-4 * abs(d2)
