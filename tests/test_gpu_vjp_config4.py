"""The adjoint at the named adjoint configuration, checked by central finite
differences: 256^3 Gaussian fields (P(k) ~ k^-3, phi rms 1e-5, transverse B
rms 1e-7, numpy generator seed 256), nside 128 (196,608 rays), 128 steps,
checkpoints every 12 steps; loss L = sum over the six maps of seeded N(0, 1)
pixel weights times the map values. At 64 seeded voxels (32 of phi, 32 of a B
component, 30 to 100 cells from the observer) the gradient of srt_vjp (FP64
form, deterministic accumulation; and the MIXED form) is compared with
(L(f + eps e_v) - L(f - eps e_v)) / (2 eps), eps = 1e-3 x the field's rms, L
evaluated by the FP64 host oracle (the maps before their float cast).

Only rays whose tap footprints can reach the voxel depend on it: a stage
position x reads taps floor(x) - 1 .. floor(x) + 2 on each axis (B staggered
by 1/2), so the voxel must lie within 2.5 cells of the ray on every axis,
i.e. within 2.5 sqrt(3) < 4.4 cells. The rays are straight to ~1e-3 cells at
these field strengths, so the oracle's loss is restricted to the pixels
whose straight ray passes within 5 cells of the voxel; the other pixels'
terms cancel exactly in the difference.

The scheme is only C1: Catmull-Rom's Hessian jumps across cell faces, so the
loss is piecewise smooth in a voxel value, and a perturbation that moves
some stage position of some ray across a face adds a jump to the difference
(measured at eps = 1e-3 x rms: a phi voxel whose forward difference was 10x
its backward one). The vjp is the derivative of the smooth piece. So each
voxel's central difference is taken where the loss is smooth on [-eps, eps]:
its forward and backward differences agree to 2e-4 (a jump J shifts the
central difference by half of their gap J/eps); otherwise eps shrinks tenfold
(once, to 1e-4 x rms) and the voxel is counted. The FP64 loss itself carries
rounding noise that matters for the small B gradients (B's eps is 1e-10):
the gap between the one-sided differences, which for a smooth loss is that
noise plus an O(eps) curvature term, is added to the 1e-4 tolerance."""
import numpy as np
import pytest

import srt_fields

pytestmark = pytest.mark.gpu

N, NSIDE, STEPS, C, SEED = 256, 128, 128, 12, 256
NVOX = 64
RADIUS = 5.0


def _near_pixels(dirs, x0, p, steps):
    """RING pixels whose straight ray from x0 along dirs (unit, (npix, 3))
    passes within RADIUS cells of the point p over affine distance [0, steps]."""
    d = p - x0
    t = dirs @ d
    perp = np.sqrt(np.maximum(d @ d - t * t, 0.0))
    return np.nonzero((t > -RADIUS) & (t < steps + RADIUS) & (perp < RADIUS))[0]


@pytest.fixture(scope="module")
def config4(srt, orc):
    phi, b = srt_fields.gaussian_fields_np(N, seed=SEED)
    npix = 12 * NSIDE * NSIDE
    w = np.random.default_rng(SEED + 1).standard_normal((6, npix)).astype(np.float32)
    with srt.Fields(phi, b) as f:
        g64 = f.vjp(NSIDE, STEPS, w, precision="fp64", deterministic=True, ckpt_every=C)[:2]
        gmx = f.vjp(NSIDE, STEPS, w, precision="mixed", ckpt_every=C)[:2]
    th, ph = orc.pix2ang_ring_range(NSIDE, 0, npix)
    dirs = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
    x0 = np.array([N / 2, N / 2, N / 2])
    rng = np.random.default_rng(SEED + 2)
    vox = []
    while len(vox) < NVOX:
        q = rng.integers(0, N, 3)
        r = np.linalg.norm(q - x0)
        if 30 <= r <= 100:
            field = "phi" if len(vox) < NVOX // 2 else "b%d" % rng.integers(0, 3)
            vox.append((field, int(q[0]), int(q[1]), int(q[2])))
    # finite differences of the oracle's FP64 loss
    eps = {"phi": 1e-3 * float(np.sqrt(np.mean(phi.astype(np.float64) ** 2))),
           "b": 1e-3 * float(np.sqrt(np.mean(b.astype(np.float64) ** 2)))}
    fd, npx, shrunk = [], [], 0
    threads = orc.max_threads()
    for field, i, j, k in vox:
        pix = _near_pixels(dirs, x0, np.array([i, j, k], np.float64), STEPS)
        npx.append(len(pix))
        wp = np.ascontiguousarray(w[:, pix])
        if field == "phi":
            arr, idx, e = phi, (k, j, i), eps["phi"]
        else:
            arr, idx, e = b, (k, j, i, int(field[1])), eps["b"]
        old = arr[idx]
        L0 = orc.tangent(phi, b, NSIDE, STEPS, pix, wp, threads=threads)[0]
        for attempt in range(2):
            arr[idx] = old + np.float32(e)
            hi_v = float(arr[idx])
            Lp = orc.tangent(phi, b, NSIDE, STEPS, pix, wp, threads=threads)[0]
            arr[idx] = old - np.float32(e)
            lo_v = float(arr[idx])
            Lm = orc.tangent(phi, b, NSIDE, STEPS, pix, wp, threads=threads)[0]
            arr[idx] = old
            fwd, bwd = (Lp - L0) / (hi_v - float(old)), (L0 - Lm) / (float(old) - lo_v)
            if abs(fwd - bwd) <= 2e-4 * max(abs(fwd), abs(bwd)):
                break
            if attempt == 0:
                e *= 0.1  # a stage crossed a cell face within [-eps, eps]
                shrunk += 1
        fd.append(((Lp - Lm) / (hi_v - lo_v), abs(fwd - bwd)))
    assert shrunk <= 16, "%d of %d voxels met a cell face within eps = 1e-3 x rms" % (shrunk, NVOX)
    return vox, np.array(fd), np.array(npx), g64, gmx


def _grad_at(g, field, i, j, k):
    gphi, gb = g
    return float(gphi[k, j, i]) if field == "phi" else float(gb[k, j, i, int(field[1])])


def test_config4_vjp_fp64_central_differences(config4):
    vox, fd, npx, g64, _ = config4
    assert len(vox) == NVOX and npx.min() > 0
    for (field, i, j, k), (want, gap) in zip(vox, fd):
        got = _grad_at(g64, field, i, j, k)
        assert abs(got - want) <= 1e-4 * abs(want) + gap, (field, i, j, k, got, want, gap)


def test_config4_vjp_mixed_central_differences(config4):
    vox, fd, _, _, gmx = config4
    vals = fd[:, 0]
    scale = {"phi": np.sqrt(np.mean(vals[:NVOX // 2] ** 2)), "b": np.sqrt(np.mean(vals[NVOX // 2:] ** 2))}
    for (field, i, j, k), (want, gap) in zip(vox, fd):
        got = _grad_at(gmx, field, i, j, k)
        # relative 1e-4, with a floor of 1e-5 of the rms gradient of the voxel set for the
        # few voxels whose gradient nearly cancels (FP32 accumulation)
        floor = 1e-5 * scale["phi" if field == "phi" else "b"]
        assert abs(got - want) <= 1e-4 * abs(want) + gap + floor, (field, i, j, k, got, want, gap)
