"""The C ABI library: loads without a GPU, exports every function that
include/srt.h declares, and validates arguments before touching a device."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu


def declared_functions():
    text = open(os.path.join(ROOT, "include", "srt.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(srt_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(srt):
    L = srt.lib()
    names = declared_functions()
    assert "srt_forward" in names and "srt_fields_create" in names and "srt_vjp" in names
    for n in names:
        assert hasattr(L, n), n


def test_abi_version(srt):
    assert srt.lib().srt_abi_version() == 3


def test_forward_rejects_bad_arguments(srt):
    L = srt.lib()
    rows = (ctypes.c_void_p * 6)()
    assert L.srt_forward(None, 4, 0, 10, 8, 1, rows, 0, None, None) == -1
    assert "fields is NULL" in srt.last_error()


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_is_reported(srt):
    phi = np.zeros((4, 4, 4), np.float32)
    b = np.zeros((4, 4, 4, 3), np.float32)
    with pytest.raises(srt.SrtError) as e:
        srt.Fields(phi, b)
    assert e.value.code == -6


def test_fields_create_validates_shapes(srt):
    with pytest.raises(ValueError):
        srt.Fields(np.zeros((4, 4, 4), np.float32), np.zeros((4, 4, 4), np.float32))
    L = srt.lib()
    h = ctypes.c_void_p()
    assert L.srt_fields_create(None, None, 4, 4, 4, 0, None, ctypes.byref(h)) == -1
    buf = np.zeros(16, np.float32)
    assert L.srt_fields_create(buf.ctypes.data, buf.ctypes.data, 0, 4, 4, 0, None, ctypes.byref(h)) == -1
    assert "bad grid extents" in srt.last_error()
