"""The reference's binary CSR file format, version 2 (readMtxToCSR.hpp:44-64,
readMtxToCSR.cpp:285-395), through the host library (``include/jx_io.h``)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import graphgen

WEIGHTED, ZERO_INDEXED, DIRECTED, REVERSE_EDGES = 1, 2, 4, 8
VERTEX_T64, EDGE_T64, WEIGHT_T64 = 16, 32, 64
_ERR = {1: "cannot open", 2: "file too short", 3: "not a version-2 CSR file",
        4: "value does not fit int32", 5: "invalid argument", 6: "write failed"}


def _lib():
    L = graphgen._lib()
    if not getattr(L, "_jxio_ready", False):
        L.jxio_csr_read_header.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64),
                                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint64)]
        L.jxio_csr_read.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.jxio_csr_write.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
        L._jxio_ready = True
    return L


def _check(rc, what):
    if rc != 0:
        raise OSError(f"{what}: {_ERR.get(rc, rc)}")


def read_header(path: str):
    nv, ne, fl = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_uint64()
    _check(_lib().jxio_csr_read_header(path.encode(), ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(fl)), path)
    return nv.value, ne.value, fl.value


def read_csr(path: str):
    """Returns (row_ptr int32, col_idx int32, edge_weights float32 or None, flags)."""
    nv, ne, fl = read_header(path)
    rp = np.empty(nv + 1, np.int32)
    col = np.empty(ne, np.int32)
    w = np.empty(ne, np.float32) if fl & WEIGHTED else None
    _check(_lib().jxio_csr_read(path.encode(), rp.ctypes.data, col.ctypes.data,
                                None if w is None else w.ctypes.data), path)
    return rp, col, w, fl


def write_csr(path: str, row_ptr, col_idx, edge_weights=None, flags: int = REVERSE_EDGES | ZERO_INDEXED):
    rp = np.ascontiguousarray(row_ptr, np.int32)
    col = np.ascontiguousarray(col_idx, np.int32)
    w = None if edge_weights is None else np.ascontiguousarray(edge_weights, np.float32)
    _check(_lib().jxio_csr_write(path.encode(), len(rp) - 1, len(col), rp.ctypes.data, col.ctypes.data,
                                 None if w is None else w.ctypes.data, flags), path)
