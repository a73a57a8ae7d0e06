"""CPU: the C-ABI library loads and exports every symbol include/jx.h declares; argument
checks that need no GPU return their status codes."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jx_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_header_symbols(jx):
    L = jx.lib()
    names = declared("jx.h")
    assert "jx_jaccard" in names and "jx_rowsum" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_and_version(jx):
    L = jx.lib()
    assert L.jx_version() >= 10000
    assert L.jx_status_string(0) == b"ok"
    assert L.jx_status_string(1) == b"invalid argument"


def test_invalid_arguments_rejected_without_gpu(jx):
    L = jx.lib()
    assert L.jx_jaccard(None, None, None, 0, None) == 1
    g = jx._Csr(-1, 0, None, None)
    assert L.jx_jaccard(ctypes.byref(g), None, None, 0, None) == 1
    g = jx._Csr(10, 5, None, None)
    assert L.jx_jaccard_ws(ctypes.byref(g), None, None, 0, None, 0, None) == 1
    g = jx._Csr(0, 0, None, None)  # empty graph: nothing to do
    assert L.jx_jaccard(ctypes.byref(g), None, None, 0, None) == 0
    assert L.jx_fill(-1, None, 0.0, None) == 1
    assert L.jx_rowsum(-1, 0, None, None, None, None, None) == 1
    assert L.jx_jaccard_host(4, 2, None, None, None, None, 0) == 1


def test_cpp_header_compiles():
    src = '#include "jx_sygraph.hpp"\nint main(){ sygraph::GraphCSRView<int32_t,int32_t,float> g; (void)g; return 0; }\n'
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-x", "c++", "-"],
                       input=src, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_dropin_driver_builds_and_links(jx, tmp_path):
    """The C++ caller of the drop-in header compiles with g++ and links against libjx.so
    (it runs in the GPU tests)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "dropin"))
    import driver_build
    jx.lib()
    exe = driver_build.build_driver(str(tmp_path), jx._build.LIBJX)
    assert os.path.exists(exe)
