"""The C ABI library: loads, exports every entry point include/htgpu.h
declares, and reports argument errors with htool's messages.  No compute
call needs a GPU here."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import htool_gb300 as H


def test_every_declared_symbol_is_exported():
    names = H.exported_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(H.lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", H.LIB_PATH], capture_output=True, text=True).stdout
    for n in names:
        assert (" T " + n) in out, n


def test_version_and_null_arguments():
    a, b = C.c_int(), C.c_int()
    assert H.lib.htgpu_version(C.byref(a), C.byref(b)) == 0
    assert (a.value, b.value) >= (0, 1)
    assert H.lib.htgpu_version(None, C.byref(b)) == 1
    assert "major is null" in H.lib.htgpu_last_error().decode()
    assert H.lib.htgpu_hmatrix_mvprod(None, None, None, 1, 0, None) == 1
    assert "Htool error" in H.lib.htgpu_last_error().decode()


def test_cluster_build_errors_are_status_codes():
    pts = np.zeros((10, 3))
    h = C.c_void_p()
    assert H.lib.htgpu_cluster_build(10, pts.ctypes.data_as(C.c_void_p), 0, 2, C.byref(h)) == 1
    assert "MinClusterSize" in H.lib.htgpu_last_error().decode()
    assert H.lib.htgpu_cluster_build(1, pts.ctypes.data_as(C.c_void_p), 10, 2, C.byref(h)) == 1


def test_header_compiles_as_c():
    hdr = os.path.join(os.path.dirname(H.LIB_PATH), "..", "include", "htgpu.h")
    src = '#include "%s"\nint main(void){return htgpu_version(0,0) == 0;}\n' % os.path.abspath(hdr)
    r = subprocess.run(["gcc", "-x", "c", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-"], input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
