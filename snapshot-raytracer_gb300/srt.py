"""Python binding of libsrt (include/srt.h) over ctypes.

This is the Python face of the drop-in boundary: it calls the C ABI with plain
pointers (numpy arrays for host memory, torch CUDA tensors or raw integers for
device memory) and raises SrtError with the library's message on any failure.
The library must have been built (snapshot-raytracer_gb300/build_srt.py); there
is no fallback implementation.

Map order everywhere is MAP_NAMES, the reference's output order
(snapshot-raytracer.cu:941-987).
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libsrt.so")

MAP_NAMES = ("dA", "ellipticity1", "ellipticity2", "rotation", "deflection1", "deflection2")
PRECISION = {"fp64": 0, "mixed": 1, "ref16": 2}

SRT_INPUT_DEVICE = 1
SRT_OUTPUT_DEVICE = 2
SRT_ASYNC = 4
SRT_ACCUMULATE = 8
SRT_DETERMINISTIC = 16
SRT_FIELDS_NO_PAIRS = 32
SRT_MIXED_NO_REFINE = 64
SRT_NESTED_RANGE = 128
SRT_FIELDS_STAGED = 256

ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "I/O error",
          -5: "format error", -6: "no CUDA device", -7: "unsupported", -8: "overflow", -9: "cancelled"}


class SrtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "error"), code, msg))
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("trace_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("rays", ctypes.c_int64),
                ("ray_steps", ctypes.c_int64), ("kernels", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64),
                ("d2h_bytes", ctypes.c_int64), ("refined_rays", ctypes.c_int64), ("retrace_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class LoadStats(ctypes.Structure):
    _fields_ = [("read_phi_ms", ctypes.c_double), ("read_b_ms", ctypes.c_double), ("layout_ms", ctypes.c_double),
                ("after_read_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("h2d_bytes", ctypes.c_int64),
                ("n", ctypes.c_int64 * 3)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "n"}
        d["n"] = tuple(self.n)
        return d


SRT_LOAD_XYZ_HDF5 = 512

_lib = None
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_FP6 = ctypes.c_void_p * 6


def lib():
    """The loaded libsrt (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise RuntimeError("libsrt.so is not built (%s); run snapshot-raytracer_gb300/build_srt.py" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        sig = {
            "srt_abi_version": (ctypes.c_int, []),
            "srt_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
            "srt_device_count": (ctypes.c_int, []),
            "srt_fields_create": (ctypes.c_int, [_P, _P, _I64, _I64, _I64, ctypes.c_uint, _P, ctypes.POINTER(_P)]),
            "srt_fields_destroy": (ctypes.c_int, [_P]),
            "srt_fields_bytes": (_I64, [_P]),
            "srt_forward": (ctypes.c_int, [_P, _I64, _I64, _I64, ctypes.c_int, ctypes.c_int, _FP6, ctypes.c_uint, _P,
                                           ctypes.POINTER(Stats)]),
            "srt_vjp": (ctypes.c_int, [_P, _I64, _I64, _I64, ctypes.c_int, ctypes.c_int, _FP6, _P, _P, ctypes.c_int,
                                       ctypes.c_uint, _P, ctypes.POINTER(Stats)]),
            "srt_forward_tape": (ctypes.c_int, [_P, _I64, _I64, _I64, ctypes.c_int, ctypes.c_int, _FP6, ctypes.c_uint,
                                                _P, ctypes.POINTER(Stats), ctypes.POINTER(_P)]),
            "srt_vjp_tape": (ctypes.c_int, [_P, _FP6, _P, _P, ctypes.c_uint, _P, ctypes.POINTER(Stats)]),
            "srt_tape_bytes": (_I64, [_P]),
            "srt_tape_destroy": (ctypes.c_int, [_P]),
            "srt_probe_peak": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
            "srt_pix2ang_ring": (ctypes.c_int, [_I64, _I64, ctypes.POINTER(ctypes.c_double),
                                                ctypes.POINTER(ctypes.c_double)]),
            "srt_nest2ring": (_I64, [_I64, _I64]),
            "srt_ring2nest": (_I64, [_I64, _I64]),
            "srt_h5_read_scalar": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_P),
                                                  ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_int)]),
            "srt_h5_read_vector3": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_P),
                                                   ctypes.POINTER(_I64)]),
            "srt_h5_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, _P, ctypes.POINTER(_I64), ctypes.c_int,
                                            ctypes.c_int]),
            "srt_fits_write_map": (ctypes.c_int, [ctypes.c_char_p, _P, _I64, ctypes.c_int, ctypes.c_char_p,
                                                  ctypes.c_int]),
            "srt_fits_read_map": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P), ctypes.POINTER(_I64),
                                                 ctypes.POINTER(_I64), ctypes.POINTER(ctypes.c_int)]),
            "srt_free": (None, [_P]),
            "srt_release_cached_memory": (ctypes.c_int, []),
            "srt_fields_load_h5": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_uint,
                                                  ctypes.c_double, ctypes.c_double, _P, _P, ctypes.POINTER(_P),
                                                  ctypes.POINTER(LoadStats)]),
            "srt_debug_fail_alloc": (ctypes.c_int, [_I64]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def release_cached_memory():
    """Return the field memory pool's unused memory to the device."""
    _check(lib().srt_release_cached_memory())


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().srt_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _check(rc):
    if rc != 0:
        raise SrtError(rc, last_error())
    return rc


def device_count():
    return lib().srt_device_count()


def probe_peak(kind):
    """Measured FMA rate of the current GPU in FLOP/s; kind 'fp32', 'fp64' or
    'fp32x2' (packed FFMA2 pairs)."""
    v = ctypes.c_double()
    _check(lib().srt_probe_peak({"fp32": 0, "fp64": 1, "fp32x2": 2}[kind], ctypes.byref(v)))
    return v.value


# --------------------------------------------------------------------- memory

def _is_torch(x):
    return type(x).__module__.startswith("torch")


def _ptr(x, want_device):
    """(pointer, is_device) of a numpy array, torch tensor or raw int."""
    if x is None:
        return None, want_device
    if isinstance(x, int):
        return x, want_device
    if _is_torch(x):
        if not x.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return x.data_ptr(), x.is_cuda
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return x.ctypes.data, False
    raise TypeError("unsupported buffer type %r" % type(x))


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


class Fields:
    """Laid-out phi and B on the GPU (srt_fields_create). phi: (n2, n1, n0)
    float32; b_xyz: (n2, n1, n0, 3) float32; numpy (host) or CUDA tensors.
    Host arrays in pinned memory are read by the layout kernel directly unless
    staged=True (copied through a device slab, as pageable memory is)."""

    def __init__(self, phi, b_xyz, stream=None, async_=False, pairs=True, staged=False):
        shape = tuple(phi.shape)
        if len(shape) != 3 or tuple(b_xyz.shape) != shape + (3,):
            raise ValueError("phi must be (n2, n1, n0) and b_xyz (n2, n1, n0, 3); got %r and %r"
                             % (shape, tuple(b_xyz.shape)))
        for a in (phi, b_xyz):
            if str(a.dtype).split(".")[-1] != "float32":
                raise TypeError("fields must be float32")
        p_phi, dev_phi = _ptr(phi, False)
        p_b, dev_b = _ptr(b_xyz, False)
        if dev_phi != dev_b:
            raise ValueError("phi and b_xyz must both be on the host or both on the device")
        self.n = (shape[2], shape[1], shape[0])
        flags = (SRT_INPUT_DEVICE if dev_phi else 0) | (SRT_ASYNC if async_ else 0) | \
            (0 if pairs else SRT_FIELDS_NO_PAIRS) | (SRT_FIELDS_STAGED if staged else 0)
        h = _P()
        _check(lib().srt_fields_create(p_phi, p_b, self.n[0], self.n[1], self.n[2], flags, _stream_ptr(stream),
                                       ctypes.byref(h)))
        self._h = h

    @classmethod
    def load_h5(cls, phi_path, b_path, dset="/data", xyz_order="reference", phi_scale=1.0, b_scale=1.0, pairs=True):
        """Fields read from the reference's two HDF5 files and laid out on the
        device while they are read (srt_fields_load_h5). Returns (Fields,
        LoadStats dict)."""
        self = cls.__new__(cls)
        h = _P()
        st = LoadStats()
        flags = (SRT_LOAD_XYZ_HDF5 if xyz_order == "hdf5" else 0) | (0 if pairs else SRT_FIELDS_NO_PAIRS)
        _check(lib().srt_fields_load_h5(phi_path.encode(), b_path.encode(), dset.encode(), flags, phi_scale, b_scale,
                                        None, None, ctypes.byref(h), ctypes.byref(st)))
        self._h = h
        self.n = tuple(st.n)
        return self, st.as_dict()

    @property
    def handle(self):
        return self._h

    @property
    def nbytes(self):
        return lib().srt_fields_bytes(self._h)

    def close(self):
        if getattr(self, "_h", None):
            lib().srt_fields_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def forward(self, nside, n_steps, pix_begin=0, pix_count=None, precision="mixed", out=None, stream=None,
                async_=False, refine=True, nested=False):
        """Six maps of RING pixels [pix_begin, pix_begin + pix_count) (NESTED
        pixels when nested=True; base pixel b is [b nside^2, (b+1) nside^2)).
        out: None (returns a new (6, count) float32 numpy array), a (6, count)
        numpy array, or a (6, count) CUDA tensor (device output). Returns
        (maps, Stats)."""
        npix = 12 * nside * nside
        if pix_count is None:
            pix_count = npix - pix_begin
        if out is None:
            out = np.zeros((6, max(pix_count, 0)), np.float32)
        p, dev = _ptr(out, False)
        if tuple(out.shape) != (6, pix_count):
            raise ValueError("out must have shape (6, %d)" % pix_count)
        rows = _FP6(*[p + m * pix_count * 4 for m in range(6)])
        st = Stats()
        flags = (SRT_OUTPUT_DEVICE if dev else 0) | (SRT_ASYNC if async_ else 0) | \
            (0 if refine else SRT_MIXED_NO_REFINE) | (SRT_NESTED_RANGE if nested else 0)
        _check(lib().srt_forward(self._h, nside, pix_begin, pix_count, n_steps, PRECISION[precision], rows, flags,
                                 _stream_ptr(stream), ctypes.byref(st)))
        return out, st

    def vjp(self, nside, n_steps, weights, pix_begin=0, pix_count=None, precision="mixed", dphi=None, db_xyz=None,
            ckpt_every=0, accumulate=False, deterministic=False, stream=None, wrt=("phi", "b")):
        """Gradient of sum(weights * maps) w.r.t. phi and B (srt_vjp).
        weights: (6, count) float32 (numpy or CUDA tensor). dphi / db_xyz:
        outputs shaped like phi / b_xyz (numpy or CUDA tensors); new numpy
        arrays when None. wrt: which gradients to form ("phi", "b"); the other
        is neither computed nor returned (None). Returns (dphi, db_xyz, Stats)."""
        npix = 12 * nside * nside
        if pix_count is None:
            pix_count = npix - pix_begin
        dphi, db_xyz, rows, pg, pb, flags = _grad_args(self.n, weights, pix_count, dphi, db_xyz, wrt, accumulate,
                                                       deterministic)
        st = Stats()
        _check(lib().srt_vjp(self._h, nside, pix_begin, pix_count, n_steps, PRECISION[precision], rows, pg, pb,
                             ckpt_every, flags, _stream_ptr(stream), ctypes.byref(st)))
        return dphi, db_xyz, st

    def forward_tape(self, nside, n_steps, pix_begin=0, pix_count=None, ckpt_every=0, out=None, stream=None):
        """The MIXED forward keeping its checkpoints (srt_forward_tape): the
        maps of forward() and a Tape whose vjp() needs no forward pass of its
        own. Returns (maps, Tape, Stats)."""
        npix = 12 * nside * nside
        if pix_count is None:
            pix_count = npix - pix_begin
        if out is None:
            out = np.zeros((6, max(pix_count, 0)), np.float32)
        p, dev = _ptr(out, False)
        if tuple(out.shape) != (6, pix_count):
            raise ValueError("out must have shape (6, %d)" % pix_count)
        rows = _FP6(*[p + m * pix_count * 4 for m in range(6)])
        st = Stats()
        h = _P()
        _check(lib().srt_forward_tape(self._h, nside, pix_begin, pix_count, n_steps, ckpt_every, rows,
                                      SRT_OUTPUT_DEVICE if dev else 0, _stream_ptr(stream), ctypes.byref(st),
                                      ctypes.byref(h)))
        return out, Tape(self, h, pix_count), st


def _grad_args(n, weights, pix_count, dphi, db_xyz, wrt, accumulate, deterministic):
    """Gradient buffers, weight rows, pointers and flags of a vjp call."""
    wrt = tuple(wrt)
    if not wrt or any(w not in ("phi", "b") for w in wrt):
        raise ValueError("wrt must name 'phi' and/or 'b', got %r" % (wrt,))
    n0, n1, n2 = n
    if "phi" not in wrt:
        dphi = None
    elif dphi is None:
        dphi = np.zeros((n2, n1, n0), np.float32)
    if "b" not in wrt:
        db_xyz = None
    elif db_xyz is None:
        db_xyz = np.zeros((n2, n1, n0, 3), np.float32)
    pw, wdev = _ptr(weights, False)
    pg, gdev = _ptr(dphi, False) if dphi is not None else (None, wdev)
    pb, bdev = _ptr(db_xyz, False) if db_xyz is not None else (None, wdev)
    if not (wdev == gdev == bdev):
        raise ValueError("weights and gradients must all be host or all be device buffers")
    rows = _FP6(*[pw + m * pix_count * 4 for m in range(6)])
    flags = (SRT_OUTPUT_DEVICE if wdev else 0) | (SRT_ACCUMULATE if accumulate else 0) | \
        (SRT_DETERMINISTIC if deterministic else 0)
    return dphi, db_xyz, rows, pg, pb, flags


class Tape:
    """Checkpoints of a Fields.forward_tape() call (srt_tape); vjp() sweeps
    them back. Keeps its Fields alive."""

    def __init__(self, fields, h, pix_count):
        self.fields, self._h, self.pix_count = fields, h, pix_count

    @property
    def nbytes(self):
        return lib().srt_tape_bytes(self._h)

    def vjp(self, weights, dphi=None, db_xyz=None, accumulate=False, deterministic=False, stream=None,
            wrt=("phi", "b")):
        """srt_vjp_tape: as Fields.vjp with the tape's arguments (MIXED)."""
        dphi, db_xyz, rows, pg, pb, flags = _grad_args(self.fields.n, weights, self.pix_count, dphi, db_xyz, wrt,
                                                       accumulate, deterministic)
        st = Stats()
        _check(lib().srt_vjp_tape(self._h, rows, pg, pb, flags, _stream_ptr(stream), ctypes.byref(st)))
        return dphi, db_xyz, st

    def close(self):
        if self._h:
            lib().srt_tape_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def trace(phi, b_xyz, nside, n_steps, batch=None, precision="mixed"):
    """The CLI's computation (snapshot-raytracer.cu:708-717, :939-987): full
    12*nside^2 RING maps, zero outside the batch's pixel range when batch is
    given (batch b covers RING pixels [b*nside^2, (b+1)*nside^2))."""
    npix = 12 * nside * nside
    if batch is None:
        begin, count = 0, npix
    else:
        if batch < 0 or batch * nside * nside >= npix:
            raise ValueError("invalid batch %r" % batch)
        begin, count = batch * nside * nside, nside * nside
    with Fields(phi, b_xyz) as f:
        part, _ = f.forward(nside, n_steps, begin, count, precision)
    full = np.zeros((6, npix), np.float32)
    full[:, begin:begin + count] = part
    return full


# -------------------------------------------------------------------- HEALPix

def pix2ang_ring(nside, pix):
    t, p = ctypes.c_double(), ctypes.c_double()
    _check(lib().srt_pix2ang_ring(nside, pix, ctypes.byref(t), ctypes.byref(p)))
    return t.value, p.value


def nest2ring(nside, ipnest):
    return lib().srt_nest2ring(nside, ipnest)


def ring2nest(nside, ipring):
    return lib().srt_ring2nest(nside, ipring)


# ---------------------------------------------------------------------- files

def _take_floats(ptr, count):
    try:
        arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctypes.c_float)), shape=(count,)).copy()
    finally:
        lib().srt_free(ptr)
    return arr


def h5_read_scalar(path, dset="/data"):
    """Float dataset of any rank as a numpy array shaped like the file's dims."""
    p, dims, rank = _P(), (_I64 * 8)(), ctypes.c_int()
    _check(lib().srt_h5_read_scalar(os.fsencode(path), dset.encode(), ctypes.byref(p), dims, ctypes.byref(rank)))
    shape = tuple(dims[i] for i in range(rank.value))
    return _take_floats(p, int(np.prod(shape))).reshape(shape)


def h5_read_vector3(path, dset="/data"):
    """Rank-3 dataset of array[3]-of-float elements as (d0, d1, d2, 3)."""
    p, dims = _P(), (_I64 * 3)()
    _check(lib().srt_h5_read_vector3(os.fsencode(path), dset.encode(), ctypes.byref(p), dims))
    shape = (dims[0], dims[1], dims[2])
    return _take_floats(p, 3 * int(np.prod(shape))).reshape(shape + (3,))


def h5_write(path, data, dset="/data", vector3=False):
    """Write float32 `data` as dataset `dset`; vector3 writes the last axis
    (length 3) as an array[3] element type over the leading dims."""
    a = np.ascontiguousarray(data, dtype=np.float32)
    shape = a.shape[:-1] if vector3 else a.shape
    if vector3 and a.shape[-1] != 3:
        raise ValueError("vector3 data must end in an axis of length 3")
    dims = (_I64 * len(shape))(*shape)
    _check(lib().srt_h5_write(os.fsencode(path), dset.encode(), a.ctypes.data, dims, len(shape), int(vector3)))


def fits_write_map(path, m, nside, nest=False, coordsys="C", overwrite=False):
    a = np.ascontiguousarray(m, dtype=np.float32)
    _check(lib().srt_fits_write_map(os.fsencode(path), a.ctypes.data, nside, int(nest), coordsys.encode(),
                                    int(overwrite)))


def fits_read_map(path):
    """(map, nside, nest) of a HEALPix FITS map."""
    p, npix, nside, nest = _P(), _I64(), _I64(), ctypes.c_int()
    _check(lib().srt_fits_read_map(os.fsencode(path), ctypes.byref(p), ctypes.byref(npix), ctypes.byref(nside),
                                   ctypes.byref(nest)))
    return _take_floats(p, npix.value), nside.value, bool(nest.value)
