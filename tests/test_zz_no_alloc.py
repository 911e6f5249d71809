"""srt_forward_noalloc, the forward for callers that cannot allocate device
memory while tracing (their memory is reserved up front by their own pool, or
they cannot take the synchronisation an allocation may imply): called through
the C ABI it must give the maps srt_forward gives, on two calls in a row (its
scratch array is shared and keeps the previous call's contents), and reject
ranges beyond its fixed scratch size. Kept in a file of its own that pytest
collects last."""
import ctypes

import numpy as np
import pytest

import srt_fields
from conftest import map_errors

pytestmark = pytest.mark.gpu

MAX_RAYS = 1 << 20


def _rows(t, count):
    return (ctypes.c_void_p * 6)(*[t.data_ptr() + 4 * count * m for m in range(6)])


@pytest.mark.parametrize("precision,mode", [("mixed", 1), ("fp64", 0)])
def test_noalloc_matches_forward_twice(srt, precision, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    L = srt.lib()
    L.srt_forward_noalloc.restype = ctypes.c_int
    L.srt_forward_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p * 6, ctypes.c_uint, ctypes.c_void_p]
    phi, b = srt_fields.gaussian_fields_np(64, seed=31)
    nside, steps, begin, count = 16, 40, 100, 2900
    with srt.Fields(phi, b) as f:
        want = torch.zeros((6, count), dtype=torch.float32, device="cuda")
        f.forward(nside, steps, begin, count, precision=precision, out=want)
        torch.cuda.synchronize()
        ref = want.cpu().numpy()
        tol = {"mixed": (1e-5, 1e-4), "fp64": (1e-9, 1e-7)}[precision]
        for call in range(2):
            got = torch.full((6, count), np.nan, dtype=torch.float32, device="cuda")
            rc = L.srt_forward_noalloc(f.handle, nside, begin, count, steps, mode, _rows(got, count), 0, None)
            assert rc == 0, srt.last_error()
            g = got.cpu().numpy()
            assert np.all(np.isfinite(g)), call
            for m, (rms, mx) in enumerate(map_errors(g, ref)):
                assert rms <= tol[0] and mx <= tol[1], (call, m, rms, mx)
        # sizes beyond the fixed scratch are refused; REF16 (allocates its planes) is refused
        big = 12 * 512 * 512
        assert big > MAX_RAYS
        rows = _rows(torch.zeros((6, 1), dtype=torch.float32, device="cuda"), 0)
        assert L.srt_forward_noalloc(f.handle, 512, 0, big, 4, mode, rows, 0, None) == -1
        assert "at most" in srt.last_error()
        assert L.srt_forward_noalloc(f.handle, nside, 0, 10, 4, 2, rows, 0, None) == -7
