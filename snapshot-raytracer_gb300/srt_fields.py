"""Synthetic Weyl-potential (phi) and shift (B) fields for tests and benchmarks.

Array convention (that of the tracer and of the reference's HDF5 reads,
snapshot-raytracer.cu:89-91, :216-256): a scalar field of extents
(n0, n1, n2) is a C-contiguous float32 array of shape (n2, n1, n0), so voxel
(i, j, k) with i the x axis is at flat index i + n0 * (j + n1 * k); the B field
is shaped (n2, n1, n0, 3) with B_x, B_y, B_z interleaved per voxel.

Two generators:
  * gaussian_* — the benchmark fields: a Gaussian random field with power
    spectrum P(k) proportional to k^-3 for 0 < |k| <= pi (the Nyquist
    wavenumber in radians per grid unit), zero mode removed, rescaled to a
    real-space rms (phi: 1e-5); B has the same spectrum, is projected
    transverse to k (divergence free) and rescaled to an rms over all
    components (1e-7). numpy on the CPU, torch (cuFFT) on a GPU for 1024^3.
  * int_noise_* — bit-reproducible fields for parity fixtures: integer white
    noise from a counter hash, smoothed with integer [1, 2, 1] passes and
    scaled by a power of two, so every value is an exact float32 on any
    platform, with no FFT or libm in the way.
"""
import numpy as np

PHI_RMS = 1e-5
B_RMS = 1e-7


# ----------------------------------------------------------------- integer noise

def _splitmix64(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(0xFFFFFFFFFFFFFFFF)
    z = x
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def int_noise_scalar(shape, seed, log2_scale, passes=2):
    """Exact float32 field of `shape` (n2, n1, n0): integers in [-2048, 2048)
    from a hash of (seed, index), `passes` periodic [1, 2, 1] smoothings per
    axis, times 2**log2_scale."""
    n = int(np.prod(shape))
    with np.errstate(over="ignore"):
        idx = np.arange(n, dtype=np.uint64) + np.uint64(seed) * np.uint64(0x100000001B3)
        h = _splitmix64(idx)
    v = ((h >> np.uint64(52)).astype(np.int64) - 2048).reshape(shape)
    for ax in range(3):
        for _ in range(passes):
            v = np.roll(v, 1, ax) + 2 * v + np.roll(v, -1, ax)
    assert np.abs(v).max() < 2 ** 24
    return (v.astype(np.float32) * np.float32(2.0 ** log2_scale)).astype(np.float32)


def int_noise_fields(n, seed=1, phi_log2=-37, b_log2=-44):
    """(phi, b_xyz) for an n^3 grid (n may be a 3-tuple (n0, n1, n2)); the
    default scales give phi rms ~ 1e-5 and B rms ~ 1e-7."""
    n0, n1, n2 = (n, n, n) if np.isscalar(n) else n
    shape = (n2, n1, n0)
    phi = int_noise_scalar(shape, seed, phi_log2)
    b = np.stack([int_noise_scalar(shape, seed * 7 + 1 + c, b_log2) for c in range(3)], axis=-1)
    return np.ascontiguousarray(phi), np.ascontiguousarray(b)


# -------------------------------------------------------------- Gaussian fields

def _kgrid_np(n0, n1, n2):
    kx = 2 * np.pi * np.fft.rfftfreq(n0)[None, None, :]
    ky = 2 * np.pi * np.fft.fftfreq(n1)[None, :, None]
    kz = 2 * np.pi * np.fft.fftfreq(n2)[:, None, None]
    return kx, ky, kz


def _amplitude_np(k2):
    amp = np.zeros_like(k2)
    m = (k2 > 0) & (k2 <= np.pi ** 2)
    amp[m] = k2[m] ** (-0.75)  # sqrt(P) with P ~ k^-3
    return amp


def gaussian_fields_np(n, seed=0, phi_rms=PHI_RMS, b_rms=B_RMS):
    """numpy generator (small grids): returns (phi, b_xyz) float32."""
    n0, n1, n2 = (n, n, n) if np.isscalar(n) else n
    rng = np.random.default_rng(seed)
    kx, ky, kz = _kgrid_np(n0, n1, n2)
    k2 = kx * kx + ky * ky + kz * kz
    amp = _amplitude_np(k2)
    w = np.fft.rfftn(rng.standard_normal((n2, n1, n0)))
    phi = np.fft.irfftn(w * amp, s=(n2, n1, n0), axes=(0, 1, 2))
    phi *= phi_rms / np.sqrt(np.mean(phi * phi))
    W = [np.fft.rfftn(rng.standard_normal((n2, n1, n0))) for _ in range(3)]
    with np.errstate(invalid="ignore", divide="ignore"):
        kdotw = (kx * W[0] + ky * W[1] + kz * W[2]) / np.where(k2 > 0, k2, 1.0)
    ks = (kx, ky, kz)
    comps = [np.fft.irfftn((W[c] - ks[c] * kdotw) * amp, s=(n2, n1, n0), axes=(0, 1, 2)) for c in range(3)]
    b = np.stack(comps, axis=-1)
    b *= b_rms / np.sqrt(np.mean(b * b))
    return np.ascontiguousarray(phi.astype(np.float32)), np.ascontiguousarray(b.astype(np.float32))


def gaussian_fields_torch(n, seed=0, phi_rms=PHI_RMS, b_rms=B_RMS, device="cuda"):
    """torch / cuFFT generator for large grids. Returns (phi, b_xyz) as float32
    tensors on `device`, shaped (n2, n1, n0) and (n2, n1, n0, 3).

    Memory-lean for 2048^3 on one GPU: the three white-noise spectra of B are
    drawn one at a time (their generator states are kept, so each is drawn
    again when its component is formed), the rms normalisations are summed
    slice by slice in float64, and above 2^32 voxels phi is parked in host
    memory while B is formed. Peak: b and three complex half-spectra."""
    import torch

    n0, n1, n2 = (n, n, n) if np.isscalar(n) else n
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    kx = (2 * np.pi * torch.fft.rfftfreq(n0, device=device)).view(1, 1, -1)
    ky = (2 * np.pi * torch.fft.fftfreq(n1, device=device)).view(1, -1, 1)
    kz = (2 * np.pi * torch.fft.fftfreq(n2, device=device)).view(-1, 1, 1)

    def k2_of():
        return kx * kx + ky * ky + kz * kz

    def amp_of(k2):  # in place on k2: k^-3/2 for 0 < k <= k_Nyquist, else 0
        m = (k2 > 0) & (k2 <= np.pi ** 2)
        k2.masked_fill_(~m, 1.0)
        k2.pow_(-0.75)
        k2.mul_(m)
        return k2

    def noise_spectrum():
        return torch.fft.rfftn(torch.randn((n2, n1, n0), generator=g, device=device, dtype=torch.float32))

    def rms(x):
        acc = torch.zeros((), dtype=torch.float64, device=x.device)
        for z in range(x.shape[0]):
            sl = x[z].double()
            acc += (sl * sl).sum()
        return torch.sqrt(acc / x.numel()).float()

    w = noise_spectrum()
    w *= amp_of(k2_of())
    phi = torch.fft.irfftn(w, s=(n2, n1, n0))
    del w
    phi *= phi_rms / rms(phi)
    # above 2^32 voxels (2048^3: 32 GiB a field) phi waits in host memory while
    # B is formed, so that B's spectra and cuFFT's workspace fit beside b
    park = n0 * n1 * n2 > (1 << 32) and phi.is_cuda
    if park:
        phi = phi.cpu()
        torch.cuda.empty_cache()
    # transverse projection: B_c = (W_c - k_c (k.W) / k^2) amp
    states, kdotw = [], None
    for kc in (kx, ky, kz):
        states.append(g.get_state())
        wc = noise_spectrum()
        wc *= kc
        if kdotw is None:
            kdotw = wc
        else:
            kdotw += wc
            del wc
    kdotw /= torch.where(k2_of() > 0, k2_of(), torch.ones((), device=device))
    b = torch.empty((n2, n1, n0, 3), device=device, dtype=torch.float32)
    for c, kc in enumerate((kx, ky, kz)):
        g.set_state(states[c])
        wc = noise_spectrum()
        wc.addcmul_(kdotw, kc.to(wc.dtype), value=-1)  # wc -= kc kdotw, no temporary
        wc *= amp_of(k2_of())
        b[..., c] = torch.fft.irfftn(wc, s=(n2, n1, n0))
        del wc
    del kdotw
    b *= b_rms / rms(b)
    if park:
        torch.cuda.empty_cache()
        phi = phi.to(device)
    return phi.contiguous(), b.contiguous()
