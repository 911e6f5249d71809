"""The GPU adjoint (srt_vjp through the C ABI) against the oracle's FP64
forward-mode tangent — the dot-product test <vjp, v> = dL/de along grid
directions v, including single voxels — and against central finite
differences of the oracle's FP64 loss; plus determinism, checkpoint-interval
invariance, accumulation and Phi-only gradients."""
import numpy as np
import pytest

import srt_fields

pytestmark = pytest.mark.gpu


def _case(n=16, nside=2, steps=10, seed=3):
    phi, b = srt_fields.int_noise_fields(n, seed=seed)
    w = np.random.default_rng(seed).standard_normal((6, 12 * nside * nside)).astype(np.float32)
    return phi, b, nside, steps, w


def _dot(g, v):
    return float(np.dot(g.astype(np.float64).ravel(), v.astype(np.float64).ravel()))


@pytest.mark.parametrize("precision,tol", [("fp64", 2e-6), ("mixed", 2e-4)])
def test_vjp_dot_product_with_tangent(srt, orc, precision, tol):
    phi, b, nside, steps, w = _case()
    with srt.Fields(phi, b) as f:
        gphi, gb, st = f.vjp(nside, steps, w, precision=precision, ckpt_every=3)
    assert st.kernels >= 3 and st.ray_steps == 48 * steps
    rng = np.random.default_rng(7)
    dirs_phi = [rng.standard_normal(phi.shape).astype(np.float32) if k % 2 == 0 else None for k in range(8)]
    dirs_b = [rng.standard_normal(b.shape).astype(np.float32) if k % 2 == 1 or k == 4 else None for k in range(8)]
    _, dL = orc.tangent(phi, b, nside, steps, np.arange(48), w, dirs_phi, dirs_b)
    for k in range(8):
        got = (_dot(gphi, dirs_phi[k]) if dirs_phi[k] is not None else 0.0) + \
              (_dot(gb, dirs_b[k]) if dirs_b[k] is not None else 0.0)
        assert abs(got - dL[k]) <= tol * abs(dL[k]) + 1e-9, (k, got, dL[k])


def test_vjp_single_voxels_fp64(srt, orc):
    """Gradient entries at seeded voxels (16 in phi, 16 in B) against exact
    tangent derivatives along the corresponding unit directions."""
    phi, b, nside, steps, w = _case(n=16, nside=2, steps=12, seed=5)
    with srt.Fields(phi, b) as f:
        gphi, gb, _ = f.vjp(nside, steps, w, precision="fp64", deterministic=True)
    rng = np.random.default_rng(11)
    # voxels the rays actually pass near: pick among the largest gradient entries and random ones
    big = np.argsort(-np.abs(gphi.ravel()))[:8]
    vox = np.concatenate([big, rng.choice(phi.size, 8, replace=False)])
    for chunk in (vox[:8], vox[8:]):
        dirs = []
        for v in chunk:
            d = np.zeros(phi.shape, np.float32)
            d.ravel()[v] = 1.0
            dirs.append(d)
        _, dL = orc.tangent(phi, b, nside, steps, np.arange(48), w, dirs, [])
        for v, want in zip(chunk, dL):
            got = float(gphi.ravel()[v])
            assert abs(got - want) <= 1e-5 * max(abs(want), 1e-3 * np.abs(gphi).max()), (v, got, want)
    bvox = np.argsort(-np.abs(gb.ravel()))[:8]
    dirs = []
    for v in bvox:
        d = np.zeros(b.shape, np.float32)
        d.ravel()[v] = 1.0
        dirs.append(d)
    _, dL = orc.tangent(phi, b, nside, steps, np.arange(48), w, [], dirs)
    for v, want in zip(bvox, dL):
        got = float(gb.ravel()[v])
        assert abs(got - want) <= 1e-5 * abs(want), (v, got, want)


def test_vjp_central_differences(srt, orc):
    """Central differences of the oracle's FP64 loss with eps = 1e-3 x field
    rms at seeded voxels agree with the vjp to 1e-4 relative."""
    phi, b, nside, steps, w = _case(n=16, nside=2, steps=12, seed=9)
    with srt.Fields(phi, b) as f:
        gphi, gb, _ = f.vjp(nside, steps, w, precision="fp64")
    eps_phi = 1e-3 * float(np.sqrt(np.mean(phi.astype(np.float64) ** 2)))
    eps_b = 1e-3 * float(np.sqrt(np.mean(b.astype(np.float64) ** 2)))
    pix = np.arange(48)
    for v in np.argsort(-np.abs(gphi.ravel()))[:6]:
        p1, p2 = phi.copy(), phi.copy()
        p1.ravel()[v] += np.float32(eps_phi)
        p2.ravel()[v] -= np.float32(eps_phi)
        h = float(p1.ravel()[v]) - float(p2.ravel()[v])
        fd = (orc.tangent(p1, b, nside, steps, pix, w)[0] - orc.tangent(p2, b, nside, steps, pix, w)[0]) / h
        assert abs(fd - gphi.ravel()[v]) <= 1e-4 * abs(fd), (v, fd, gphi.ravel()[v])
    for v in np.argsort(-np.abs(gb.ravel()))[:6]:
        b1, b2 = b.copy(), b.copy()
        b1.ravel()[v] += np.float32(eps_b)
        b2.ravel()[v] -= np.float32(eps_b)
        h = float(b1.ravel()[v]) - float(b2.ravel()[v])
        fd = (orc.tangent(phi, b1, nside, steps, pix, w)[0] - orc.tangent(phi, b2, nside, steps, pix, w)[0]) / h
        assert abs(fd - gb.ravel()[v]) <= 1e-4 * abs(fd), (v, fd, gb.ravel()[v])


def test_vjp_deterministic_and_checkpoint_invariant(srt):
    phi, b, nside, steps, w = _case(n=24, nside=4, steps=14, seed=2)
    with srt.Fields(phi, b) as f:
        runs = [f.vjp(nside, steps, w, precision="fp64", deterministic=True, ckpt_every=c)[:2] for c in (1, 4, 14, 4)]
        mixed = [f.vjp(nside, steps, w, precision="mixed", deterministic=True, ckpt_every=c)[:2] for c in (2, 5)]
        atomic = f.vjp(nside, steps, w, precision="fp64")[:2]
    for g in runs[1:]:
        assert np.array_equal(g[0].view(np.uint32), runs[0][0].view(np.uint32))
        assert np.array_equal(g[1].view(np.uint32), runs[0][1].view(np.uint32))
    assert np.array_equal(mixed[0][0].view(np.uint32), mixed[1][0].view(np.uint32))
    for a, d in zip(atomic, runs[0]):
        scale = np.abs(d).max()
        assert np.abs(a - d).max() <= 1e-6 * scale
    for a, d in zip(mixed[0], runs[0]):
        scale = np.abs(d).max()
        assert np.abs(a - d).max() <= 1e-3 * scale


def test_vjp_accumulate_phi_only_and_ranges(srt):
    phi, b, nside, steps, w = _case(n=16, nside=2, steps=8, seed=4)
    with srt.Fields(phi, b) as f:
        g1, b1, _ = f.vjp(nside, steps, w, precision="fp64", deterministic=True)
        g2, b2, _ = f.vjp(nside, steps, w, precision="fp64", deterministic=True, dphi=g1.copy(), db_xyz=b1.copy(),
                          accumulate=True)
        assert np.allclose(g2, 2 * g1, rtol=1e-6, atol=0) and np.allclose(b2, 2 * b1, rtol=1e-6, atol=0)
        # phi only: no B gradient buffer, same phi gradient
        import ctypes
        gphi = np.zeros_like(phi)
        rows = (ctypes.c_void_p * 6)(*[w.ctypes.data + 4 * w.shape[1] * m for m in range(6)])
        rc = srt.lib().srt_vjp(f.handle, nside, 0, 48, steps, 0, rows, gphi.ctypes.data, None, 0, 16, None, None)
        assert rc == 0 and np.array_equal(gphi.view(np.uint32), g1.view(np.uint32))
        # the same through the Python face (wrt), in the MIXED deterministic mode
        gp_only, gb_none, _ = f.vjp(nside, steps, w, precision="mixed", deterministic=True, wrt=("phi",))
        gfull, _, _ = f.vjp(nside, steps, w, precision="mixed", deterministic=True)
        assert gb_none is None and np.array_equal(gp_only.view(np.uint32), gfull.view(np.uint32))
        gp_none, gb_only, _ = f.vjp(nside, steps, w, precision="mixed", deterministic=True, wrt=("b",))
        _, gbfull, _ = f.vjp(nside, steps, w, precision="mixed", deterministic=True)
        assert gp_none is None and np.array_equal(gb_only.view(np.uint32), gbfull.view(np.uint32))
        # disjoint pixel ranges add up to the full-sky gradient
        acc = np.zeros_like(phi)
        for lo, hi in ((0, 13), (13, 40), (40, 48)):
            gp, _, _ = f.vjp(nside, steps, np.ascontiguousarray(w[:, lo:hi]), pix_begin=lo, pix_count=hi - lo,
                             precision="fp64", deterministic=True)
            acc += gp
        assert np.allclose(acc, g1, rtol=1e-5, atol=1e-6 * np.abs(g1).max())
        # zero weights give a zero gradient; REF16 has no adjoint
        gz, bz, _ = f.vjp(nside, steps, np.zeros_like(w), precision="mixed")
        assert not np.any(gz) and not np.any(bz)
        with pytest.raises(srt.SrtError):
            f.vjp(nside, steps, w, precision="ref16")


def test_forward_tape_vjp_pair(srt):
    """srt_forward_tape gives srt_forward's maps and keeps the checkpoints;
    srt_vjp_tape then gives srt_vjp's gradient (bit for bit in the
    deterministic mode) without a forward pass, as often as wanted."""
    phi, b, nside, steps, w = _case(n=24, nside=4, steps=14, seed=2)
    lo, cnt = 37, 120
    wpart = np.ascontiguousarray(w[:, lo:lo + cnt])
    with srt.Fields(phi, b) as f:
        m, _ = f.forward(nside, steps, lo, cnt, precision="mixed")
        mt, tape, st = f.forward_tape(nside, steps, lo, cnt, ckpt_every=5)
        assert np.array_equal(mt.view(np.uint32), m.view(np.uint32))
        assert tape.nbytes >= (14 // 5 + 2) * 38 * 4 * cnt
        g1, b1, _ = f.vjp(nside, steps, wpart, lo, cnt, precision="mixed", deterministic=True, ckpt_every=5)
        g2, b2, s2 = tape.vjp(wpart, deterministic=True)
        assert np.array_equal(g2.view(np.uint32), g1.view(np.uint32))
        assert np.array_equal(b2.view(np.uint32), b1.view(np.uint32))
        assert s2.kernels < 2 * (14 // 5 + 1) + 8
        g3, _, _ = tape.vjp(2 * wpart, deterministic=True, wrt=("phi",))
        assert np.allclose(g3, 2 * g1, rtol=1e-6, atol=1e-6 * np.abs(g1).max())
        ga, ba, _ = tape.vjp(wpart)  # FP32 atomics
        assert np.abs(ga - g1).max() <= 1e-4 * np.abs(g1).max()
        tape.close()


def test_vjp_deterministic_range_overflow_is_an_error(srt):
    """The deterministic mode's 64-bit fixed point holds |gradient| < 2^30 per
    voxel; weights that drive the gradient past it make srt_vjp fail with
    SRT_ERR_OVERFLOW (-8) instead of returning wrapped sums, while the FP32
    accumulation of the same call stays finite, and a call within range after
    it succeeds."""
    phi, b, nside, steps, w = _case(n=16, nside=2, steps=10, seed=3)
    big = (w * np.float32(1e20)).astype(np.float32)
    with srt.Fields(phi, b) as f:
        with pytest.raises(srt.SrtError) as ei:
            f.vjp(nside, steps, big, precision="mixed", deterministic=True)
        assert ei.value.code == -8 and "fixed-point range" in str(ei.value)
        with pytest.raises(srt.SrtError) as ei:
            f.vjp(nside, steps, big, precision="fp64", deterministic=True)
        assert ei.value.code == -8
        g, gb, _ = f.vjp(nside, steps, big, precision="mixed")
        assert np.all(np.isfinite(g)) and np.abs(g).max() > 2.0 ** 31
        g1, _, _ = f.vjp(nside, steps, w, precision="mixed", deterministic=True)
        assert np.all(np.isfinite(g1)) and np.abs(g1).max() < 2.0 ** 30
