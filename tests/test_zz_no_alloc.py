"""srt_forward_noalloc, the forward for callers that cannot allocate device
memory while tracing (their memory is reserved up front by their own pool, or
they cannot take the synchronisation an allocation may imply): called through
the C ABI it must give the maps srt_forward gives, on two calls in a row (its
scratch array is shared and keeps the previous call's contents), for RING and
NESTED ranges and with or without the FP64 re-trace, and refuse ranges beyond
its fixed scratch size and flags it does not act on. Kept in a file of its own
that pytest collects last."""
import ctypes

import numpy as np
import pytest

import srt_fields
from conftest import map_errors

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 20
SRT_ASYNC, SRT_MIXED_NO_REFINE, SRT_NESTED_RANGE, SRT_ACCUMULATE = 4, 64, 128, 8


def _rows(t, count):
    return (ctypes.c_void_p * 6)(*[t.data_ptr() + 4 * count * m for m in range(6)])


def _noalloc(srt):
    L = srt.lib()
    L.srt_forward_noalloc.restype = ctypes.c_int
    L.srt_forward_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p * 6, ctypes.c_uint, ctypes.c_void_p]
    return L.srt_forward_noalloc


@pytest.mark.parametrize("precision,mode", [("mixed", 1), ("fp64", 0)])
def test_noalloc_matches_forward_twice(srt, precision, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    fwd = _noalloc(srt)
    phi, b = srt_fields.gaussian_fields_np(64, seed=31)
    nside, steps = 16, 40
    tol = {"mixed": (1e-5, 1e-4), "fp64": (1e-9, 1e-7)}[precision]
    # (RING range, flags), (NESTED range: base pixels 2..4), MIXED without re-trace
    cases = [(100, 2900, 0, {}), (2 * 256, 3 * 256, SRT_NESTED_RANGE, {"nested": True})]
    if precision == "mixed":
        cases.append((700, 1500, SRT_MIXED_NO_REFINE, {"refine": False}))
    with srt.Fields(phi, b) as f:
        for begin, count, flags, kw in cases:
            want = torch.zeros((6, count), dtype=torch.float32, device="cuda")
            f.forward(nside, steps, begin, count, precision=precision, out=want, **kw)
            torch.cuda.synchronize()
            ref = want.cpu().numpy()
            for call in range(2):
                got = torch.full((6, count), np.nan, dtype=torch.float32, device="cuda")
                rc = fwd(f.handle, nside, begin, count, steps, mode, _rows(got, count), flags, None)
                assert rc == 0, srt.last_error()
                g = got.cpu().numpy()
                assert np.all(np.isfinite(g)), (flags, call)
                for m, (rms, mx) in enumerate(map_errors(g, ref)):
                    assert rms <= tol[0] and mx <= tol[1], (flags, call, m, rms, mx)
        # sizes beyond the fixed scratch are refused; REF16 (allocates its planes) is refused
        big = 12 * 512 * 512
        assert big > MAX_RAYS
        rows = _rows(torch.zeros((6, 1), dtype=torch.float32, device="cuda"), 0)
        assert fwd(f.handle, 512, 0, big, 4, mode, rows, 0, None) == -1
        assert "at most" in srt.last_error()
        assert fwd(f.handle, nside, 0, 10, 4, 2, rows, 0, None) == -7
        # a flag it does not act on is refused, not ignored; NESTED needs a power-of-two nside
        assert fwd(f.handle, nside, 0, 10, 4, mode, rows, SRT_ACCUMULATE, None) == -7
        assert "not supported" in srt.last_error()
        assert fwd(f.handle, 12, 0, 10, 4, mode, rows, SRT_NESTED_RANGE, None) == -1
