"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only the tests, the smoke check of ``__graft_entry__`` and the CPU-baseline leg of
``bench.py`` import this module.  It wraps:

* ``libjxoracle.so``: the C restatement of the reference algorithm (``jx_oracle.c``);
* ``_ref/libjxref.so``: the reference's own ``jaccard.cpp`` run through the host SYCL
  subset (``ref_driver.cpp``), when it could be built.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build_ref

_I32 = ctypes.POINTER(ctypes.c_int32)
_F32 = ctypes.POINTER(ctypes.c_float)
_F64 = ctypes.POINTER(ctypes.c_double)

_oracle = None
_ref = None


def _p(a, t):
    return None if a is None else a.ctypes.data_as(t)


def lib():
    global _oracle
    if _oracle is None:
        build_ref.build_oracle()
        L = ctypes.CDLL(build_ref.ORACLE_SO)
        L.jxo_rowsum.argtypes = [ctypes.c_int32, _I32, _I32, _F32, _F32, ctypes.c_int]
        L.jxo_intersect_rows.argtypes = [ctypes.c_int32, ctypes.c_int32, _I32, _I32, _F32, _F32,
                                         _F32, _F32, ctypes.c_int]
        L.jxo_weight.argtypes = [ctypes.c_int64, _F32, _F32, _F32]
        L.jxo_ec_scan.argtypes = [ctypes.c_int32, _I32, _I32, _F32]
        L.jxo_ec_edges.argtypes = [ctypes.c_int64, ctypes.c_int64, _I32, _I32, _I32, _F32,
                                   ctypes.c_int]
        L.jxo_jaccard_rows.argtypes = [ctypes.c_int, ctypes.c_int32, _I32, _I32, _F32,
                                       ctypes.c_int32, ctypes.c_int32, _F32, _F32, ctypes.c_int]
        L.jxo_jaccard_rows.restype = ctypes.c_int
        L.jxo_counts_rows.argtypes = [ctypes.c_int32, ctypes.c_int32, _I32, _I32, _I32,
                                      ctypes.c_int]
        L.jxo_jaccard_f64_rows.argtypes = [ctypes.c_int32, _I32, _I32, _F32, ctypes.c_int32,
                                           ctypes.c_int32, _F64, ctypes.c_int]
        L.jxo_jaccard_list.argtypes = [ctypes.c_int32, _I32, _I32, _F32, ctypes.c_int64, _I32, _I32,
                                       _F32, ctypes.c_int]
        L.jxo_row_work.argtypes = [ctypes.c_int32, _I32, _I32, _F64, ctypes.c_int]
        L.jxo_group_work.argtypes = [ctypes.c_int, ctypes.c_int32, _I32, _I32, _F64, ctypes.c_int]
        L.jxo_group_work.restype = ctypes.c_int64
        _oracle = L
    return _oracle


def ref_lib():
    """The reference via the SYCL subset, or None when its sources are not available."""
    global _ref
    if _ref is None:
        so = build_ref.build_ref()
        if so is None:
            if os.path.exists(build_ref.REF_SO):
                so = build_ref.REF_SO
            else:
                return None
        L = ctypes.CDLL(so)
        L.jxref_set_threads.argtypes = [ctypes.c_int]
        L.jxref_set_group_sample.argtypes = [ctypes.c_longlong, ctypes.c_longlong]
        L.jxref_set_group_mask.argtypes = [ctypes.c_void_p, ctypes.c_longlong]
        L.jxref_jaccard.argtypes = [ctypes.c_int, ctypes.c_int32, ctypes.c_int32, _I32, _I32, _F32,
                                    _F32]
        L.jxref_rowsum.argtypes = [ctypes.c_int32, ctypes.c_int32, _I32, _I32, _F32, _F32]
        L.jxref_fill.argtypes = [ctypes.c_int64, _F32, ctypes.c_float]
        L.jxref_intersect.argtypes = [ctypes.c_int32, ctypes.c_int32, _I32, _I32, _F32, _F32, _F32,
                                      _F32]
        L.jxref_weight.argtypes = [ctypes.c_int32, _F32, _F32, _F32]
        L.jxref_ec_scan.argtypes = [ctypes.c_int32, ctypes.c_int32, _I32, _I32, _F32]
        L.jxref_ec_unweighted.argtypes = [ctypes.c_int32, ctypes.c_int32, _I32, _I32, _I32, _F32]
        L.jxref_csr_write.argtypes = [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int32, _I32, _I32, _F32,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.jxref_csr_header.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint64)]
        L.jxref_csr_read.argtypes = [ctypes.c_char_p, _I32, _I32, _F32]
        L.jxref_remove_reverse.argtypes = [ctypes.c_int32, ctypes.c_int32, _I32, _I32, _F32, _I32, _I32,
                                           _F32, ctypes.c_int64]
        L.jxref_remove_reverse.restype = ctypes.c_int64
        _ref = L
    return _ref


# ---------------------------------------------------------------- C restatement wrappers

def rowsum(row_ptr, ind, w=None, threads=0):
    n = len(row_ptr) - 1
    out = np.empty(n, np.float32)
    lib().jxo_rowsum(n, _p(row_ptr, _I32), _p(ind, _I32), _p(w, _F32), _p(out, _F32), threads)
    return out


def intersect(row_ptr, col, w, work, weight_i, threads=0):
    """Jaccard_IsKernel over all rows; weight_i (float32[E]) accumulates in place."""
    n = len(row_ptr) - 1
    ws = np.empty(len(col), np.float32)
    lib().jxo_intersect_rows(0, n, _p(row_ptr, _I32), _p(col, _I32), _p(w, _F32), _p(work, _F32),
                             _p(weight_i, _F32), _p(ws, _F32), threads)
    return ws


def weight(weight_i, weight_s):
    out = np.empty(len(weight_i), np.float32)
    lib().jxo_weight(len(weight_i), _p(weight_i, _F32), _p(weight_s, _F32), _p(out, _F32))
    return out


def jaccard(row_ptr, col, w=None, edge_centric=False, rows=None, threads=0):
    """sygraph::jaccard restated; `rows=(r0, r1)` limits the output to those rows' edges."""
    n = len(row_ptr) - 1
    r0, r1 = rows if rows is not None else (0, n)
    out = np.empty(int(row_ptr[r1]) - int(row_ptr[r0]), np.float32)
    rc = lib().jxo_jaccard_rows(1 if edge_centric else 0, n, _p(row_ptr, _I32), _p(col, _I32),
                                _p(w, _F32), r0, r1, None, _p(out, _F32), threads)
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return out


def jaccard_rows_with_sums(row_ptr, col, w, S, rows, threads=0):
    """Weighted VC oracle for rows [r0, r1) with the row sums S (float32[n]) given, so that
    several row ranges of one big graph share one row-sum pass."""
    n = len(row_ptr) - 1
    r0, r1 = rows
    out = np.empty(int(row_ptr[r1]) - int(row_ptr[r0]), np.float32)
    rc = lib().jxo_jaccard_rows(0, n, _p(row_ptr, _I32), _p(col, _I32), _p(w, _F32), r0, r1,
                                _p(S, _F32), _p(out, _F32), threads)
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return out


def row_work(row_ptr, col, threads=0):
    """Per-row cost proxy of the reference's IS kernel (float64[n]): sum over the row's edges
    of min(d_u, d_v) * (1 + log2(max(d_u, d_v)))."""
    n = len(row_ptr) - 1
    out = np.empty(n, np.float64)
    lib().jxo_row_work(n, _p(row_ptr, _I32), _p(col, _I32), _p(out, _F64), threads)
    return out


def group_work(row_ptr, col, edge_centric=False, threads=0):
    """Cost proxy per work-group of the reference's dominant kernel (Jaccard_IsKernel, or
    Jaccard_ec_unweighted when edge_centric), float64[G] with G its number of work-groups."""
    n = len(row_ptr) - 1
    out = np.empty(65535, np.float64)
    G = lib().jxo_group_work(1 if edge_centric else 0, n, _p(row_ptr, _I32), _p(col, _I32), _p(out, _F64),
                             threads)
    return out[:G].copy()


def check_rows(row_ptr, hubs=5, cta_degree=21000, band=2000, tail=3000):
    """Row ranges that a parity check of a large skewed graph samples: the `hubs` largest rows
    (ties by id), the row whose degree is closest to `cta_degree`, a band of `band` rows in
    the middle of the id range and the last `tail` rows.  Returns [(name, r0, r1), ...]."""
    n = len(row_ptr) - 1
    d = np.diff(row_ptr.astype(np.int64))
    out = [(f"hub{k}_deg{int(d[h])}", int(h), int(h) + 1)
           for k, h in enumerate(np.argsort(-d, kind="stable")[:hubs])]
    c = int(np.argmin(np.abs(d - cta_degree)))
    out.append((f"row_deg{int(d[c])}", c, c + 1))
    m = n // 2
    out.append(("middle_band", m, min(n, m + band)))
    out.append(("tail", max(0, n - tail), n))
    return out


def counts(row_ptr, col, rows=None, threads=0):
    n = len(row_ptr) - 1
    r0, r1 = rows if rows is not None else (0, n)
    out = np.empty(int(row_ptr[r1]) - int(row_ptr[r0]), np.int32)
    lib().jxo_counts_rows(r0, r1, _p(row_ptr, _I32), _p(col, _I32), _p(out, _I32), threads)
    return out


def jaccard_f64(row_ptr, col, w=None, rows=None, threads=0):
    n = len(row_ptr) - 1
    r0, r1 = rows if rows is not None else (0, n)
    out = np.empty(int(row_ptr[r1]) - int(row_ptr[r0]), np.float64)
    lib().jxo_jaccard_f64_rows(n, _p(row_ptr, _I32), _p(col, _I32), _p(w, _F32), r0, r1,
                               _p(out, _F64), threads)
    return out


# ---------------------------------------------------------------- reference (via SYCL subset)

def ref_jaccard(row_ptr, col, w=None, edge_centric=False, threads=0, group_sample=1,
                group_residue=0, group_mask=None):
    """Run sygraph::jaccard of the reference; with group_sample=K only work-groups whose id is
    group_residue modulo K execute, with group_mask (uint8 array) only the groups g with
    group_mask[g] != 0 (timing samples: the results are then incomplete)."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference sources unavailable")
    L.jxref_set_threads(threads)
    L.jxref_set_group_sample(group_sample, group_residue)
    if group_mask is not None:
        group_mask = np.ascontiguousarray(group_mask, np.uint8)
        L.jxref_set_group_mask(group_mask.ctypes.data, len(group_mask))
    n = len(row_ptr) - 1
    out = np.zeros(len(col), np.float32)
    try:
        L.jxref_jaccard(1 if edge_centric else 0, n, len(col), _p(row_ptr, _I32), _p(col, _I32),
                        _p(w, _F32), _p(out, _F32))
    finally:
        L.jxref_set_group_mask(None, 0)
        L.jxref_set_group_sample(1, 0)
    return out


def ref_rowsum(row_ptr, ind, w=None, threads=0):
    L = ref_lib()
    L.jxref_set_threads(threads)
    n = len(row_ptr) - 1
    out = np.empty(n, np.float32)
    L.jxref_rowsum(n, len(ind), _p(row_ptr, _I32), _p(ind, _I32), _p(w, _F32), _p(out, _F32))
    return out


def ref_intersect(row_ptr, col, w, work, weight_i, threads=0):
    L = ref_lib()
    L.jxref_set_threads(threads)
    n = len(row_ptr) - 1
    ws = np.empty(len(col), np.float32)
    L.jxref_intersect(n, len(col), _p(row_ptr, _I32), _p(col, _I32), _p(w, _F32), _p(work, _F32),
                      _p(weight_i, _F32), _p(ws, _F32))
    return ws


def ref_weight(weight_i, weight_s):
    out = np.empty(len(weight_i), np.float32)
    ref_lib().jxref_weight(len(weight_i), _p(weight_i, _F32), _p(weight_s, _F32), _p(out, _F32))
    return out


def ref_ec_scan(row_ptr, e):
    n = len(row_ptr) - 1
    dest = np.empty(e, np.int32)
    wj = np.full(e, np.nan, np.float32)
    ref_lib().jxref_ec_scan(e, n, _p(row_ptr, _I32), _p(dest, _I32), _p(wj, _F32))
    return dest, wj


def ref_ec_unweighted(row_ptr, col, dest, weight_j):
    n = len(row_ptr) - 1
    ref_lib().jxref_ec_unweighted(len(col), n, _p(row_ptr, _I32), _p(col, _I32), _p(dest, _I32),
                                  _p(weight_j, _F32))
    return weight_j


def jaccard_list(row_ptr, col, first, second, w=None, threads=0):
    n = len(row_ptr) - 1
    first = np.ascontiguousarray(first, np.int32)
    second = np.ascontiguousarray(second, np.int32)
    out = np.empty(len(first), np.float32)
    lib().jxo_jaccard_list(n, _p(row_ptr, _I32), _p(col, _I32), _p(w, _F32), len(first),
                           _p(first, _I32), _p(second, _I32), _p(out, _F32), threads)
    return out


def ref_csr_write(path, row_ptr, col, w, zero_indexed=True, directed=False, reverse_edges=True):
    rc = ref_lib().jxref_csr_write(path.encode(), len(row_ptr) - 1, len(col), _p(row_ptr, _I32),
                                   _p(col, _I32), _p(w, _F32), int(zero_indexed), int(directed),
                                   int(reverse_edges))
    if rc != 0:
        raise OSError(f"reference CSRToFile failed ({rc})")


def ref_csr_read(path):
    nv, ne, fl = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_uint64()
    L = ref_lib()
    if L.jxref_csr_header(path.encode(), ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(fl)) != 0:
        raise OSError(path)
    rp = np.empty(nv.value + 1, np.int32)
    col = np.empty(ne.value, np.int32)
    w = np.empty(ne.value, np.float32) if fl.value & 1 else None
    if L.jxref_csr_read(path.encode(), _p(rp, _I32), _p(col, _I32), _p(w, _F32)) != 0:
        raise OSError(path)
    return rp, col, w, fl.value


def ref_remove_reverse(row_ptr, col, values):
    e = len(col)
    src = np.empty(e, np.int32)
    dst = np.empty(e, np.int32)
    val = np.empty(e, np.float32)
    values = np.ascontiguousarray(values, np.float32)
    k = ref_lib().jxref_remove_reverse(len(row_ptr) - 1, e, _p(row_ptr, _I32), _p(col, _I32),
                                       _p(values, _F32), _p(src, _I32), _p(dst, _I32), _p(val, _F32), e)
    return src[:k], dst[:k], val[:k]


def ref_csr_from_edges(src, dst, symmetrize=True, keep_self=False):
    """The reference's own graph preparation (main.cpp:99-118: MTX set, invertDirection,
    mtxSetToCSR) on a zero-based edge list.  Returns (row_ptr, col) of the CSR it builds,
    whose rows run from the first source vertex to the last (readMtxToCSR.cpp:158-179)."""
    src = np.ascontiguousarray(src, np.int32)
    dst = np.ascontiguousarray(dst, np.int32)
    m = len(src)
    cap = 2 * m + 1
    nv_cap = int(max(src.max(), dst.max())) + 2 if m else 1
    offsets = np.empty(nv_cap + 1, np.int32)
    indices = np.empty(cap, np.int32)
    nv = ctypes.c_int32()
    L = ref_lib()
    L.jxref_csr_from_edges.restype = ctypes.c_int64
    L.jxref_csr_from_edges.argtypes = [ctypes.c_int64, _I32, _I32, ctypes.c_int, ctypes.c_int, _I32,
                                       ctypes.c_int64, _I32, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32)]
    e = L.jxref_csr_from_edges(m, _p(src, _I32), _p(dst, _I32), int(symmetrize), int(keep_self),
                               _p(offsets, _I32), nv_cap + 1, _p(indices, _I32), cap, ctypes.byref(nv))
    if e < 0:
        raise RuntimeError(f"reference CSR build failed ({e})")
    return offsets[: nv.value + 1].copy(), indices[:e].copy()


def csr_build(n, src, dst, symmetrize=True, keep_self=False):
    """Restatement of the graph preparation with every vertex of [0, n) keeping its row: the
    set of (u, v) pairs (and (v, u) when symmetrising, main.cpp:99-111, readMtxToCSR.cpp:117-132)
    in ascending order, self loops dropped unless kept (readMtxToCSR.cpp:174), as a CSR."""
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    if symmetrize:
        src, dst = np.concatenate([src, dst]), np.concatenate([dst, src])
    if not keep_self:
        keep = src != dst
        src, dst = src[keep], dst[keep]
    keys = np.unique(src * n + dst)
    rows = keys // n
    col = (keys % n).astype(np.int32)
    row_ptr = np.zeros(n + 1, np.int64)
    np.add.at(row_ptr, rows + 1, 1)
    return np.cumsum(row_ptr).astype(np.int32), col
