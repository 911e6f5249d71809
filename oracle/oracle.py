"""ctypes binding of the CPU oracle (oracle/liboracle.so), of the reference's
own host code (oracle/_ref/libsrt_ref.so) and of the reference's own GPU build
(oracle/_ref/ref_kernel.cubin through oracle/librefgpu.so); the oracle/_ref
files exist only where the reference sources were available to build them.

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs, as the checker or the timed CPU
baseline — never by the product path.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORACLE = os.path.join(HERE, "liboracle.so")
LIBREF = os.path.join(HERE, "_ref", "libsrt_ref.so")
LIBREFGPU = os.path.join(HERE, "librefgpu.so")
REFCUBIN = os.path.join(HERE, "_ref", "ref_kernel.cubin")

MODE = {"fp64": 0, "ref16": 2}
_P, _I64 = ctypes.c_void_p, ctypes.c_int64
_lib = None
_ref = None
_refgpu = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.isfile(LIBORACLE):
            raise RuntimeError("oracle not built: %s" % LIBORACLE)
        L = ctypes.CDLL(LIBORACLE)
        L.srto_trace.argtypes = [_P, _P, _I64, _I64, _I64, _I64, _I64, _I64, ctypes.c_int, ctypes.c_int, _P,
                                 ctypes.c_int]
        L.srto_trace_pixels.argtypes = [_P, _P, _I64, _I64, _I64, _I64, _P, _I64, ctypes.c_int, ctypes.c_int, _P,
                                        ctypes.c_int]
        L.srto_pix2ang_ring.argtypes = [_I64, _I64, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
        L.srto_pix2ang_ring.restype = None
        L.srto_pix2ang_ring_range.argtypes = [_I64, _I64, _I64, _P, _P]
        L.srto_pix2ang_ring_range.restype = None
        L.srto_interp.argtypes = [_P, _P, _I64, _I64, _I64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_double, _P]
        L.srto_float_to_half.argtypes = [ctypes.c_float]
        L.srto_float_to_half.restype = ctypes.c_uint16
        L.srto_half_to_float.argtypes = [ctypes.c_uint16]
        L.srto_half_to_float.restype = ctypes.c_float
        L.srto_max_threads.restype = ctypes.c_int
        L.srto_fields_new.argtypes = [_P, _P, _I64, _I64, _I64, ctypes.c_int]
        L.srto_fields_new.restype = _P
        L.srto_fields_delete.argtypes = [_P]
        L.srto_fields_delete.restype = None
        L.srto_trace_pixels_h.argtypes = [_P, _I64, _P, _I64, ctypes.c_int, _P, ctypes.c_int]
        _lib = L
    return _lib


def ref_available():
    return os.path.isfile(LIBREF)


def ref_lib():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference host library not built (needs the reference sources): %s" % LIBREF)
        L = ctypes.CDLL(LIBREF)
        L.srtref_trace_angles.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _I64, ctypes.c_int,
                                          _P, ctypes.c_int]
        L.srtref_fields_new.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.srtref_fields_new.restype = _P
        L.srtref_fields_delete.argtypes = [_P]
        L.srtref_fields_delete.restype = None
        L.srtref_trace_angles_h.argtypes = [_P, _P, _P, _I64, ctypes.c_int, _P, ctypes.c_int]
        L.srtref_interp.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_double, _P]
        _ref = L
    return _ref


def _dims(phi, b):
    phi = np.ascontiguousarray(phi, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    n2, n1, n0 = phi.shape
    assert b.shape == (n2, n1, n0, 3)
    return phi, b, n0, n1, n2


def max_threads():
    return lib().srto_max_threads()


def trace(phi, b, nside, n_steps, pix_begin=0, pix_count=None, mode="fp64", threads=0):
    """(6, count) maps of RING pixels [pix_begin, pix_begin + count)."""
    phi, b, n0, n1, n2 = _dims(phi, b)
    if pix_count is None:
        pix_count = 12 * nside * nside - pix_begin
    out = np.zeros((6, pix_count), np.float32)
    rc = lib().srto_trace(phi.ctypes.data, b.ctypes.data, n0, n1, n2, nside, pix_begin, pix_count, n_steps,
                          MODE[mode], out.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError("srto_trace failed (%d)" % rc)
    return out


def trace_pixels(phi, b, nside, n_steps, pixels, mode="fp64", threads=0):
    """(6, len(pixels)) maps of an arbitrary list of RING pixels."""
    phi, b, n0, n1, n2 = _dims(phi, b)
    pix = np.ascontiguousarray(pixels, np.int64)
    out = np.zeros((6, len(pix)), np.float32)
    rc = lib().srto_trace_pixels(phi.ctypes.data, b.ctypes.data, n0, n1, n2, nside, pix.ctypes.data, len(pix),
                                 n_steps, MODE[mode], out.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError("srto_trace_pixels failed (%d)" % rc)
    return out


class Fields:
    """Fields laid out once for repeated oracle traces (FP64 or REF16 mode);
    the reference's own host code instead when reference=True (oracle/_ref)."""

    def __init__(self, phi, b, mode="fp64", reference=False):
        self.phi, self.b, self.n0, self.n1, self.n2 = _dims(phi, b)
        self.reference = reference
        if reference:
            self._h = ref_lib().srtref_fields_new(self.phi.ctypes.data, self.b.ctypes.data, self.n0, self.n1, self.n2)
        else:
            self._h = lib().srto_fields_new(self.phi.ctypes.data, self.b.ctypes.data, self.n0, self.n1, self.n2,
                                            MODE[mode])
        if not self._h:
            raise RuntimeError("oracle fields: allocation failed")

    def trace_pixels(self, nside, n_steps, pixels, threads=0):
        """Maps (6, len(pixels)) of the listed RING pixels."""
        pixels = np.ascontiguousarray(pixels, np.int64)
        out = np.zeros((6, len(pixels)), np.float32)
        if self.reference:
            th = np.zeros(len(pixels))
            ph = np.zeros(len(pixels))
            for i, p in enumerate(pixels):
                th[i], ph[i] = pix2ang_ring(nside, int(p))
            rc = ref_lib().srtref_trace_angles_h(self._h, th.ctypes.data, ph.ctypes.data, len(pixels), n_steps,
                                                 out.ctypes.data, threads)
        else:
            rc = lib().srto_trace_pixels_h(self._h, nside, pixels.ctypes.data, len(pixels), n_steps,
                                           out.ctypes.data, threads)
        if rc != 0:
            raise RuntimeError("oracle trace failed (%d)" % rc)
        return out

    def close(self):
        if self._h:
            (ref_lib().srtref_fields_delete if self.reference else lib().srto_fields_delete)(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def pix2ang_ring_range(nside, begin, count):
    """theta, phi (float64 arrays) of RING pixels [begin, begin + count)."""
    th = np.zeros(count)
    ph = np.zeros(count)
    lib().srto_pix2ang_ring_range(nside, begin, count, th.ctypes.data, ph.ctypes.data)
    return th, ph


def pix2ang_ring(nside, pix):
    t, p = ctypes.c_double(), ctypes.c_double()
    lib().srto_pix2ang_ring(nside, pix, ctypes.byref(t), ctypes.byref(p))
    return t.value, p.value


def interp(phi, b, field, x, y, z, mode="fp64"):
    phi, b, n0, n1, n2 = _dims(phi, b)
    out = np.zeros(10, np.float64)
    lib().srto_interp(phi.ctypes.data, b.ctypes.data, n0, n1, n2, MODE[mode], field, x, y, z, out.ctypes.data)
    return out


def float_to_half_bits(x):
    return lib().srto_float_to_half(float(x))


def half_bits_to_float(h):
    return lib().srto_half_to_float(int(h))


def ref_trace(phi, b, nside, n_steps, pix_begin=0, pix_count=None, threads=0):
    """The reference's own host code (oracle/_ref) on RING pixels
    [pix_begin, pix_begin + count), ray angles from the oracle's pix2ang."""
    phi, b, n0, n1, n2 = _dims(phi, b)
    if pix_count is None:
        pix_count = 12 * nside * nside - pix_begin
    th, ph = pix2ang_ring_range(nside, pix_begin, pix_count)
    out = np.zeros((6, pix_count), np.float32)
    ref_lib().srtref_trace_angles(phi.ctypes.data, b.ctypes.data, n0, n1, n2, th.ctypes.data, ph.ctypes.data,
                                  pix_count, n_steps, out.ctypes.data, threads)
    return out


def ref_interp(phi, b, field, x, y, z):
    phi, b, n0, n1, n2 = _dims(phi, b)
    out = np.zeros(10, np.float64)
    ref_lib().srtref_interp(phi.ctypes.data, b.ctypes.data, n0, n1, n2, field, x, y, z, out.ctypes.data)
    return out


def map_errors(a, b, ulps=1):
    """Per map m: (rms error, max error) of maps `a` against the checker `b`,
    relative to the rms of b's signal — for dA (map 0), the rms of its
    fluctuation about the mean, since dA ~ n_steps. Differences of up to
    `ulps` float32 spacings of b are the resolution of float32 maps and are
    not counted."""
    out = []
    for m in range(6):
        bm = np.asarray(b[m], np.float32)
        d = np.asarray(a[m], np.float64) - bm.astype(np.float64)
        d = np.sign(d) * np.maximum(np.abs(d) - ulps * np.spacing(np.abs(bm)).astype(np.float64), 0.0)
        r = bm.astype(np.float64)
        if m == 0:
            r = r - r.mean()
        s = float(np.sqrt(np.mean(r * r))) if r.size else 0.0
        s = s if s > 0 else 1.0
        out.append((float(np.sqrt(np.mean(d * d))) / s if d.size else 0.0, float(np.abs(d).max()) / s if d.size else 0.0))
    return out


def tangent(phi, b, nside, n_steps, pixels, weights, dir_phi=(), dir_b=(), threads=0):
    """FP64 loss L = sum_m sum_i weights[m, i] map_m(pixels[i]) (maps before the
    float cast) and its derivatives along grid directions (forward mode, up to
    8 per call): dir_phi[k] shaped like phi, dir_b[k] like b (None = zero).
    Returns (L, [dL_k])."""
    L_ = lib()
    if not hasattr(L_, "_tangent_sig"):
        L_.srto_tangent.argtypes = [_P, _P, _I64, _I64, _I64, _I64, _P, _I64, ctypes.c_int, _P, _P, _P, ctypes.c_int,
                                    _P, _P, ctypes.c_int]
        L_._tangent_sig = True
    phi, b, n0, n1, n2 = _dims(phi, b)
    pix = np.ascontiguousarray(pixels, np.int64)
    w = np.ascontiguousarray(weights, np.float32).reshape(6, len(pix))
    nd = max(len(dir_phi), len(dir_b))
    if nd > 8:
        raise ValueError("at most 8 directions per call")
    keep = []

    def arr(lst, shape):
        ptrs = (ctypes.c_void_p * max(nd, 1))()
        for k in range(nd):
            a = lst[k] if k < len(lst) else None
            if a is not None:
                a = np.ascontiguousarray(a, np.float32)
                assert a.shape == shape
                keep.append(a)
                ptrs[k] = a.ctypes.data
        return ptrs

    pp = arr(list(dir_phi), phi.shape)
    pb = arr(list(dir_b), b.shape)
    out = ctypes.c_double()
    dl = np.zeros(max(nd, 1), np.float64)
    rc = L_.srto_tangent(phi.ctypes.data, b.ctypes.data, n0, n1, n2, nside, pix.ctypes.data, len(pix), n_steps,
                         w.ctypes.data, ctypes.cast(pp, _P), ctypes.cast(pb, _P), nd, ctypes.byref(out),
                         dl.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError("srto_tangent failed (%d)" % rc)
    return out.value, list(dl[:nd])


def ref_gpu_available():
    return os.path.isfile(REFCUBIN) and os.path.isfile(LIBREFGPU)


def _refgpu_lib():
    global _refgpu
    if _refgpu is None:
        if not ref_gpu_available():
            raise RuntimeError("reference GPU build not available (needs the reference sources): %s" % REFCUBIN)
        L = ctypes.CDLL(LIBREFGPU)
        L.srtrefgpu_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.srtrefgpu_trace.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _I64, _I64,
                                      ctypes.c_int, _P, ctypes.c_int, _P, ctypes.c_char_p, ctypes.c_size_t]
        err = ctypes.create_string_buffer(512)
        if L.srtrefgpu_load(REFCUBIN.encode(), err, 512) != 0:
            raise RuntimeError(err.value.decode())
        _refgpu = L
    return _refgpu


def ref_gpu_trace(phi_dev, b_dev, nside, n_steps, pix_begin=0, pix_count=None, reps=1):
    """The reference's own GPU build (its vector3_to_half and
    raytracing_kernel, staged as its main() does) on RING pixels
    [pix_begin, pix_begin + count). phi_dev / b_dev: contiguous float32 CUDA
    tensors shaped (n2, n1, n0) and (n2, n1, n0, 3). Returns (maps as a
    (6, count) CUDA tensor, per-launch kernel milliseconds)."""
    import torch
    n2, n1, n0 = phi_dev.shape
    if pix_count is None:
        pix_count = 12 * nside * nside - pix_begin
    th, ph = pix2ang_ring_range(nside, pix_begin, pix_count)
    maps = torch.zeros(6, pix_count, dtype=torch.float32, device=phi_dev.device)
    ms = (ctypes.c_float * reps)()
    err = ctypes.create_string_buffer(512)
    torch.cuda.synchronize(phi_dev.device)
    rc = _refgpu_lib().srtrefgpu_trace(phi_dev.data_ptr(), b_dev.data_ptr(), n0, n1, n2, th.ctypes.data,
                                       ph.ctypes.data, pix_count, nside, n_steps, maps.data_ptr(), reps, ms, err, 512)
    if rc != 0:
        raise RuntimeError("reference GPU build: " + err.value.decode())
    return maps, list(ms)
