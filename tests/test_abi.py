"""The C ABI: libgcvt_gb300.so loads without a GPU and exports every function
include/*.h declares (plus the reference's C++ symbol gCVT).  No compute calls
here -- those need a GPU and live in the gpu-marked tests."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT


def header_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(inc, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:extern\s+)?[A-Za-z_][\w\s\*]*?\b(gcvt_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_api():
    names = header_functions()
    for must in ("gcvt_ctx_create", "gcvt_ctx_label", "gcvt_ctx_run", "gcvt_compute",
                 "gcvt_label_grid"):
        assert must in names


def test_library_exports_every_declared_symbol(gcvt_lib):
    lib = ctypes.CDLL(gcvt_lib.LIB_PATH)
    for name in header_functions():
        assert hasattr(lib, name), name
    # the binding covers the whole header
    assert set(header_functions()) <= set(gcvt_lib.SIGNATURES)
    out = subprocess.run(["nm", "-D", "--defined-only", gcvt_lib.LIB_PATH],
                         capture_output=True, text=True).stdout
    for sym in gcvt_lib.CPP_SYMBOLS.values():
        assert sym in out, sym


def test_status_strings_without_gpu(gcvt_lib):
    lib = gcvt_lib.load_library()
    assert lib.gcvt_status_string(0) == b"ok"
    assert lib.gcvt_status_string(4).startswith(b"site grid")
    assert lib.gcvt_version() >= 10000


def test_argument_errors_without_gpu(gcvt_lib):
    lib = gcvt_lib.load_library()
    # null pointers and bad sizes are rejected before any CUDA call
    assert lib.gcvt_compute(None, None, None, 256, 1, 10) == 1
    assert lib.gcvt_label_grid(None, None, 256, 0) == 1
    cnt = ctypes.c_int(0)
    assert lib.gcvt_ctx_delaunay(None, None, 0, ctypes.byref(cnt), 0) == 1
    assert lib.gcvt_ctx_extract_points(None, 1.0, 0.0, 0.0, None, 0, ctypes.byref(cnt), 0) == 1
    h = ctypes.c_void_p()
    assert lib.gcvt_ctx_create(100, ctypes.byref(h)) == 2
    assert lib.gcvt_ctx_create(16384 + 256, ctypes.byref(h)) == 2
