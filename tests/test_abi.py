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
    assert srt.lib().srt_abi_version() == 4


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


def test_plain_c_caller_links_and_runs(tmp_path):
    """The header compiles as C99 and a C program links against libsrt the way
    the reference's main() would call it: without a GPU the first call reports
    SRT_ERR_NO_DEVICE with a message, and nothing exits."""
    import subprocess

    import build_srt

    src = tmp_path / "use_srt.c"
    src.write_text(r'''
#include "srt.h"
#include <stdio.h>
int main(void) {
  char msg[256];
  srt_fields* F = NULL;
  float phi[8] = {0}, b[24] = {0};
  int rc = srt_fields_create(phi, b, 2, 2, 2, 0, NULL, &F);
  srt_last_error(msg, sizeof msg);
  printf("%d %d %s\n", srt_abi_version(), rc, msg);
  if (rc == SRT_OK) srt_fields_destroy(F);
  return 0;
}
''')
    exe = tmp_path / "use_srt"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src),
                        "-L" + build_srt.LIBDIR, "-lsrt", "-Wl,-rpath," + build_srt.LIBDIR, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    ver, rc, msg = r.stdout.split(" ", 2)
    assert int(ver) == 4
    if has_gpu():
        assert int(rc) == 0
    else:
        assert int(rc) == -6 and "no CUDA device" in msg
