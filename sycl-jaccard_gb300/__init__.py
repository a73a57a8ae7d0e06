"""jx: GB300-native Jaccard engine -- Python host mirror of the reference operator surface.

The compute path is ``csrc/libjx.so`` (hand-written sm_103a CUDA kernels behind a C ABI,
``include/jx.h``).  This module binds it with ctypes and mirrors the reference's API
(vtsynergy/SYCL-Jaccard, ``standalone_algorithms.hpp:67-87``, ``jaccard.hpp``):

* :class:`GraphCSRView` -- ``standalone_csr.hpp:44-105`` over device tensors;
* :func:`jaccard` -- ``sygraph::jaccard<edge_centric>(graph, [weights,] result, q)``;
* :func:`rowsum`, :func:`fill`, :func:`intersect`, :func:`weight`, :func:`ec_scan`,
  :func:`ec_unweighted` -- the kernel-level ``invoke`` statics of ``jaccard.hpp``;
* :func:`jaccard_host` -- the same operator on host (numpy) arrays, like the reference's
  buffers that wrap host memory.

PyTorch supplies device memory and streams only.  There is no CPU fallback: if the native
library is missing or no GPU is present, calls raise.

The package directory name contains a hyphen, so import it with
``importlib.import_module("sycl-jaccard_gb300")``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build
from . import csrfile  # noqa: F401  (binary CSR files)
from . import graphgen  # noqa: F401  (synthetic graphs)

__all__ = ["GraphCSRView", "JxError", "HostArray", "jaccard", "jaccard_host", "jaccard_noalloc", "jaccard_list",
           "count_above", "remove_reverse_edges", "csrfile", "Batch", "Server", "csr_build", "rowsum", "fill", "intersect",
           "weight", "ec_scan", "ec_unweighted", "csr_check", "lib", "launch_count",
           "launch_count_reset", "graphgen"]

JX_OK = 0
_STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory",
           4: "invalid CSR graph", 5: "unsupported request", 6: "size above the supported maximum",
           7: "request cancelled"}
ALGO_VERTEX_CENTRIC = 0
ALGO_EDGE_CENTRIC = 1

CSR_FLAGS = {0x1: "offsets_bad", 0x2: "index_range", 0x4: "unsorted", 0x8: "duplicate",
             0x10: "self_loop", 0x20: "asymmetric"}


class JxError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        msg = f"{what}: {_STATUS.get(status, 'unknown status')} ({status})"
        if status == 2 and _lib is not None:
            msg += f", cudaError {_lib.jx_last_cuda_error()}"
        super().__init__(msg)


class _HostGraph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("e", ctypes.c_int32), ("row_ptr", ctypes.c_void_p),
                ("col_idx", ctypes.c_void_p), ("vertex_w", ctypes.c_void_p)]





class _Request(ctypes.Structure):
    _fields_ = [("graph_id", ctypes.c_int32), ("graph", ctypes.POINTER(_HostGraph)), ("algo", ctypes.c_int),
                ("weighted", ctypes.c_int32), ("host_out", ctypes.c_void_p), ("arrival_ns", ctypes.c_int64)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64), ("passes", ctypes.c_uint64),
                ("folded_requests", ctypes.c_uint64), ("kernels", ctypes.c_uint64), ("edges", ctypes.c_int64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("max_ms", ctypes.c_double), ("span_s", ctypes.c_double), ("peak_reserved", ctypes.c_size_t),
                ("cancelled", ctypes.c_uint64)]


class _Schedule(ctypes.Structure):
    _fields_ = [("persistent", ctypes.c_int32), ("lane_max", ctypes.c_int32), ("warp_max", ctypes.c_int32),
                ("cta_max", ctypes.c_int32), ("hub_unit", ctypes.c_int32), ("hub_batch", ctypes.c_int32),
                ("hub_beside", ctypes.c_int32), ("hub_cluster", ctypes.c_int32), ("relabel", ctypes.c_int32)]


class _ServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget", ctypes.c_size_t), ("slots", ctypes.c_int32), ("fold_edges", ctypes.c_int64),
                ("fold_max_edges", ctypes.c_int64), ("schedule", _Schedule)]


class _Csr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("e", ctypes.c_int32), ("row_ptr", ctypes.c_void_p),
                ("col_idx", ctypes.c_void_p)]


_lib = None
_VP = ctypes.c_void_p


def lib() -> ctypes.CDLL:
    """Load libjx.so (building it first if sources are newer); raise if it cannot load."""
    global _lib
    if _lib is None:
        so = _build.LIBJX
        if not os.path.exists(so):
            try:
                _build.build_engine()
            except Exception as exc:  # pragma: no cover - depends on the machine
                raise RuntimeError(f"jx native library missing and could not be built: {exc}") from exc
        L = ctypes.CDLL(so)
        i32, i64, f32, u32p = ctypes.c_int32, ctypes.c_int64, ctypes.c_float, ctypes.POINTER(ctypes.c_uint32)
        sig = {
            "jx_jaccard": ([ctypes.POINTER(_Csr), _VP, _VP, ctypes.c_int, _VP], ctypes.c_int),
            "jx_jaccard_ws": ([ctypes.POINTER(_Csr), _VP, _VP, ctypes.c_int, _VP, ctypes.c_size_t, _VP], ctypes.c_int),
            "jx_jaccard_workspace_size": ([ctypes.POINTER(_Csr), ctypes.c_int, ctypes.c_int], ctypes.c_size_t),
            "jx_jaccard_host": ([i32, i32, _VP, _VP, _VP, _VP, ctypes.c_int], ctypes.c_int),
            "jx_jaccard_schedule": ([ctypes.POINTER(_Csr), _VP, _VP, ctypes.c_int, ctypes.POINTER(_Schedule), _VP,
                                     ctypes.c_size_t, _VP], ctypes.c_int),
            "jx_jaccard_schedule_workspace_size": ([ctypes.POINTER(_Csr), ctypes.c_int, ctypes.c_int,
                                                    ctypes.POINTER(_Schedule)], ctypes.c_size_t),
            "jx_host_release": ([], ctypes.c_int),
            "jx_host_alloc": ([ctypes.c_size_t, ctypes.POINTER(_VP)], ctypes.c_int),
            "jx_host_free": ([_VP], ctypes.c_int),
            "jx_jaccard_noalloc": ([ctypes.POINTER(_Csr), _VP, _VP, ctypes.c_int, _VP], ctypes.c_int),
            "jx_rowsum": ([i32, i32, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
            "jx_fill": ([i64, _VP, f32, _VP], ctypes.c_int),
            "jx_intersect": ([i32, i32, _VP, _VP, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
            "jx_weight": ([i32, _VP, _VP, _VP, _VP], ctypes.c_int),
            "jx_ec_scan": ([i32, i32, _VP, _VP, _VP, _VP], ctypes.c_int),
            "jx_ec_unweighted": ([i32, i32, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
            "jx_csr_check": ([ctypes.POINTER(_Csr), u32p, _VP], ctypes.c_int),
            "jx_jaccard_list": ([ctypes.POINTER(_Csr), _VP, i64, _VP, _VP, _VP, _VP], ctypes.c_int),
            "jx_count_above": ([i64, _VP, f32, _VP, _VP], ctypes.c_int),
            "jx_csr_build": ([i32, i64, _VP, _VP, ctypes.c_uint32, _VP, _VP, i64, ctypes.POINTER(ctypes.c_int64),
                              _VP], ctypes.c_int),
            "jx_remove_reverse_edges": ([ctypes.POINTER(_Csr), _VP, _VP, _VP, _VP, _VP, _VP], ctypes.c_int),
            "jx_batch_create": ([ctypes.POINTER(_HostGraph), i32, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.POINTER(_VP)], ctypes.c_int),
            "jx_batch_run": ([_VP, _VP], ctypes.c_int),
            "jx_batch_result": ([_VP, i32, ctypes.POINTER(_VP), ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
            "jx_batch_download": ([_VP, i32, _VP, _VP], ctypes.c_int),
            "jx_batch_info": ([_VP, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                               ctypes.POINTER(ctypes.c_uint64), ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
            "jx_batch_destroy": ([_VP], None),
            "jx_server_create": ([ctypes.POINTER(_ServerConfig), ctypes.POINTER(_VP)], ctypes.c_int),
            "jx_server_add_graph": ([_VP, ctypes.POINTER(_HostGraph), i32, ctypes.POINTER(ctypes.c_int32)],
                                    ctypes.c_int),
            "jx_server_submit": ([_VP, ctypes.POINTER(_Request), ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
            "jx_server_wait": ([_VP, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
            "jx_server_drain": ([_VP], ctypes.c_int),
            "jx_server_get_stats": ([_VP, ctypes.POINTER(_ServerStats)], ctypes.c_int),
            "jx_server_reset_stats": ([_VP], None),
            "jx_server_clock_ns": ([], ctypes.c_int64),
            "jx_server_destroy": ([_VP], None),
            "jx_server_set_paused": ([_VP, i32], ctypes.c_int),
            "jx_server_cancel": ([_VP, ctypes.c_uint64], ctypes.c_int),
            "jx_server_inject_alloc_failures": ([_VP, i32], ctypes.c_int),
            "jx_status_string": ([ctypes.c_int], ctypes.c_char_p),
            "jx_version": ([], ctypes.c_int),
            "jx_last_cuda_error": ([], ctypes.c_int),
            "jx_launch_count": ([], ctypes.c_uint64),
            "jx_profile_begin": ([], None),
            "jx_profile_end": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_int),
            "jx_launch_count_reset": ([], None),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _check(status: int, what: str) -> None:
    if status != JX_OK:
        raise JxError(status, what)


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("jx needs a CUDA GPU: torch.cuda.is_available() is False")
    return torch


def _stream(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t, dtype, n, what):
    if t is None:
        return None
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{what} must be a CUDA tensor")
    if t.dtype != dtype or not t.is_contiguous() or t.numel() < n:
        raise TypeError(f"{what} must be a contiguous {dtype} tensor with at least {n} elements")
    return ctypes.c_void_p(t.data_ptr())


class GraphCSRView:
    """Non-owning CSR view over device tensors (``standalone_csr.hpp:44-105``).

    ``offsets``: int32[V+1] (device), ``indices``: int32[E] (device), each row sorted
    ascending; ``edge_data`` is kept for surface parity and unused by Jaccard.
    """

    def __init__(self, offsets, indices, edge_data=None, number_of_vertices=None,
                 number_of_edges=None):
        torch = _torch()
        self.offsets = offsets
        self.indices = indices
        self.edge_data = edge_data
        self.number_of_vertices = int(number_of_vertices if number_of_vertices is not None
                                      else offsets.numel() - 1)
        self.number_of_edges = int(number_of_edges if number_of_edges is not None
                                   else indices.numel())
        _ptr(offsets, torch.int32, self.number_of_vertices + 1, "offsets")
        _ptr(indices, torch.int32, self.number_of_edges, "indices")

    @classmethod
    def from_numpy(cls, row_ptr: np.ndarray, col_idx: np.ndarray, device="cuda"):
        torch = _torch()
        return cls(torch.from_numpy(np.ascontiguousarray(row_ptr, np.int32)).to(device),
                   torch.from_numpy(np.ascontiguousarray(col_idx, np.int32)).to(device))

    def _c(self) -> _Csr:
        return _Csr(self.number_of_vertices, self.number_of_edges, self.offsets.data_ptr(),
                    self.indices.data_ptr())


def _schedule(sch: dict | None):
    """jx_schedule from a dict with any of its field names (missing fields: defaults)."""
    if sch is None:
        return None
    unknown = set(sch) - {f for f, _ in _Schedule._fields_}
    if unknown:
        raise ValueError(f"unknown schedule fields {sorted(unknown)}")
    return _Schedule(**{k: int(v) for k, v in sch.items()})


def jaccard(graph: GraphCSRView, weights=None, result=None, edge_centric: bool = False,
            stream=None, workspace=None, schedule: dict | None = None):
    """``sygraph::jaccard<edge_centric>(graph, [weights,] result, q)``.

    ``weights``: float32[V] device tensor of per-vertex weights, or None (unweighted).  The
    edge-centric algorithm ignores weights, as the reference does.  ``result``: float32[E]
    device tensor (allocated when None).  Asynchronous on ``stream``.  Returns ``result``.
    ``schedule``: launch schedule (``jx_schedule`` fields: persistent, lane_max, warp_max,
    cta_max, hub_unit, hub_batch, hub_beside, hub_cluster); results do not depend on it.
    """
    torch = _torch()
    E = graph.number_of_edges
    if result is None:
        result = torch.empty(E, dtype=torch.float32, device=graph.indices.device)
    wp = _ptr(weights, torch.float32, graph.number_of_vertices, "weights")
    rp = _ptr(result, torch.float32, E, "result")
    algo = ALGO_EDGE_CENTRIC if edge_centric else ALGO_VERTEX_CENTRIC
    g = graph._c()
    L = lib()
    if schedule is not None:
        sch = _schedule(schedule)
        if workspace is None:
            nbytes = L.jx_jaccard_schedule_workspace_size(ctypes.byref(g), int(weights is not None), algo,
                                                          ctypes.byref(sch))
            workspace = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=graph.indices.device)
        _check(L.jx_jaccard_schedule(ctypes.byref(g), wp, rp, algo, ctypes.byref(sch),
                                     ctypes.c_void_p(workspace.data_ptr()),
                                     workspace.numel() * workspace.element_size(), _stream(stream)),
               "jx_jaccard_schedule")
        return result
    if workspace is None:
        _check(L.jx_jaccard(ctypes.byref(g), wp, rp, algo, _stream(stream)), "jx_jaccard")
    else:
        _check(L.jx_jaccard_ws(ctypes.byref(g), wp, rp, algo, ctypes.c_void_p(workspace.data_ptr()),
                               workspace.numel() * workspace.element_size(), _stream(stream)),
               "jx_jaccard_ws")
    return result


def jaccard_noalloc(graph: GraphCSRView, weights=None, result=None, edge_centric: bool = False,
                    stream=None):
    """:func:`jaccard` through ``jx_jaccard_noalloc``: no device allocation inside the call
    (graphs of at most 2**20 vertices; calls sharing the library's fixed workspace must not
    overlap on the GPU)."""
    torch = _torch()
    E = graph.number_of_edges
    if result is None:
        result = torch.empty(E, dtype=torch.float32, device=graph.indices.device)
    g = graph._c()
    _check(lib().jx_jaccard_noalloc(ctypes.byref(g), _ptr(weights, torch.float32, graph.number_of_vertices, "weights"),
                                    _ptr(result, torch.float32, E, "result"),
                                    ALGO_EDGE_CENTRIC if edge_centric else ALGO_VERTEX_CENTRIC, _stream(stream)),
           "jx_jaccard_noalloc")
    return result


def workspace_size(graph: GraphCSRView, weighted: bool, edge_centric: bool = False,
                   schedule: dict | None = None) -> int:
    g = graph._c()
    algo = ALGO_EDGE_CENTRIC if edge_centric else ALGO_VERTEX_CENTRIC
    if schedule is not None:
        return int(lib().jx_jaccard_schedule_workspace_size(ctypes.byref(g), int(weighted), algo,
                                                             ctypes.byref(_schedule(schedule))))
    return int(lib().jx_jaccard_workspace_size(ctypes.byref(g), int(weighted), algo))


class HostArray:
    """A numpy array in pinned host memory from the library's runtime (jx_host_alloc), for the
    host arrays of :func:`jaccard_host` / ``jx_jaccard_host``.  ``.array`` is the numpy view;
    the memory is freed by :meth:`free` (or when the object is collected)."""

    def __init__(self, shape, dtype):
        dtype = np.dtype(dtype)
        count = int(np.prod(shape))
        p = ctypes.c_void_p()
        _check(lib().jx_host_alloc(max(1, count * dtype.itemsize), ctypes.byref(p)), "jx_host_alloc")
        self._p = p
        buf = (ctypes.c_char * max(1, count * dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=count).reshape(shape)

    @classmethod
    def copy_of(cls, a):
        h = cls(np.shape(a), np.asarray(a).dtype)
        h.array[...] = a
        return h

    def free(self):
        if self._p:
            self.array = None
            lib().jx_host_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def jaccard_host(row_ptr: np.ndarray, col_idx: np.ndarray, weights: np.ndarray | None = None,
                 edge_centric: bool = False, out: np.ndarray | None = None) -> np.ndarray:
    """Host-array form: copies in, computes on the GPU, copies out (synchronous)."""
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col_idx = np.ascontiguousarray(col_idx, np.int32)
    n, e = len(row_ptr) - 1, len(col_idx)
    if out is None:
        out = np.empty(e, np.float32)
    w = None if weights is None else np.ascontiguousarray(weights, np.float32)
    algo = ALGO_EDGE_CENTRIC if edge_centric else ALGO_VERTEX_CENTRIC
    _check(lib().jx_jaccard_host(n, e, row_ptr.ctypes.data, col_idx.ctypes.data,
                                 None if w is None else w.ctypes.data, out.ctypes.data, algo),
           "jx_jaccard_host")
    return out


# ------------------------------------------------------------------ stage-level surface

def rowsum(n, e, offsets, indices, weights, work, stream=None):
    """``Jaccard_RowSumKernel<weighted>::invoke`` (jaccard.cpp:263-313)."""
    torch = _torch()
    _check(lib().jx_rowsum(n, e, _ptr(offsets, torch.int32, n + 1, "offsets"),
                           _ptr(indices, torch.int32, e, "indices") if e > 0 else None,
                           _ptr(weights, torch.float32, 1, "weights"),
                           _ptr(work, torch.float32, n, "work"), _stream(stream)), "jx_rowsum")
    return work


def fill(x, value: float, n=None, stream=None):
    """``FillKernel<float>::invoke`` (jaccard.cpp:161-182)."""
    torch = _torch()
    n = x.numel() if n is None else n
    _check(lib().jx_fill(n, _ptr(x, torch.float32, n, "x"), float(value), _stream(stream)), "jx_fill")
    return x


def intersect(n, e, offsets, indices, weights, work, weight_i, weight_s, stream=None):
    """``Jaccard_IsKernel<weighted>::invoke`` (jaccard.cpp:402-458); weight_i accumulates."""
    torch = _torch()
    _check(lib().jx_intersect(n, e, _ptr(offsets, torch.int32, n + 1, "offsets"),
                              _ptr(indices, torch.int32, e, "indices"),
                              _ptr(weights, torch.float32, n, "weights"),
                              _ptr(work, torch.float32, n, "work"),
                              _ptr(weight_i, torch.float32, e, "weight_i"),
                              _ptr(weight_s, torch.float32, e, "weight_s"), _stream(stream)),
           "jx_intersect")


def weight(e, weight_i, weight_s, weight_j, stream=None):
    """``Jaccard_JwKernel::invoke`` (jaccard.cpp:622-653)."""
    torch = _torch()
    _check(lib().jx_weight(e, _ptr(weight_i, torch.float32, e, "weight_i"),
                           _ptr(weight_s, torch.float32, e, "weight_s"),
                           _ptr(weight_j, torch.float32, e, "weight_j"), _stream(stream)), "jx_weight")


def ec_scan(e, n, offsets, dest_ind, weight_j, stream=None):
    """``Jaccard_ec_scan::invoke`` (jaccard.cpp:666-700)."""
    torch = _torch()
    _check(lib().jx_ec_scan(e, n, _ptr(offsets, torch.int32, n + 1, "offsets"),
                            _ptr(dest_ind, torch.int32, e, "dest_ind"),
                            _ptr(weight_j, torch.float32, e, "weight_j"), _stream(stream)), "jx_ec_scan")


def ec_unweighted(e, n, offsets, indices, dest_ind, weight_j, stream=None):
    """``Jaccard_ec_unweighted::invoke`` (jaccard.cpp:745-782)."""
    torch = _torch()
    _check(lib().jx_ec_unweighted(e, n, _ptr(offsets, torch.int32, n + 1, "offsets"),
                                  _ptr(indices, torch.int32, e, "indices"),
                                  _ptr(dest_ind, torch.int32, e, "dest_ind"),
                                  _ptr(weight_j, torch.float32, e, "weight_j"), _stream(stream)),
           "jx_ec_unweighted")


def jaccard_list(graph: GraphCSRView, first, second, weights=None, result=None, stream=None):
    """``jaccard_list(graph, [weights,] num_pairs, first, second, result, q)``
    (standalone_algorithms.hpp:109-133): J for the vertex pairs (first[p], second[p])."""
    torch = _torch()
    npairs = first.numel()
    if result is None:
        result = torch.empty(npairs, dtype=torch.float32, device=first.device)
    g = graph._c()
    _check(lib().jx_jaccard_list(ctypes.byref(g), _ptr(weights, torch.float32, graph.number_of_vertices, "weights"),
                                 npairs, _ptr(first, torch.int32, npairs, "first"),
                                 _ptr(second, torch.int32, npairs, "second"),
                                 _ptr(result, torch.float32, npairs, "result"), _stream(stream)),
           "jx_jaccard_list")
    return result


def count_above(values, thresh: float = 1e-5, stream=None) -> int:
    """The reference's edge-centric driver (detail::jaccard) count of results above `thresh` (jaccard.cpp:810-819)."""
    torch = _torch()
    c = torch.zeros(1, dtype=torch.int64, device=values.device)
    _check(lib().jx_count_above(values.numel(), _ptr(values, torch.float32, values.numel(), "values"),
                                float(thresh), ctypes.c_void_p(c.data_ptr()), _stream(stream)), "jx_count_above")
    return int(c.item())


BUILD_SYMMETRIZE = 0x1
BUILD_KEEP_SELF_LOOPS = 0x2


def csr_build(n: int, src, dst, symmetrize: bool = True, keep_self: bool = False, stream=None) -> GraphCSRView:
    """The reference program's graph preparation on the device (main.cpp:99-118, readMtxToCSR.cpp:117-208):
    int32 device edge lists `src`, `dst` (zero-based) -> a CSR with sorted, duplicate-free rows,
    reverse edges added when `symmetrize`, self loops dropped unless `keep_self`."""
    torch = _torch()
    m = src.numel()
    if dst.numel() != m:
        raise ValueError("src and dst differ in length")
    dev = src.device if m else torch.device("cuda")
    cap = max(1, 2 * m if symmetrize else m)
    row_ptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
    col = torch.empty(cap, dtype=torch.int32, device=dev)
    e = ctypes.c_int64()
    flags = (BUILD_SYMMETRIZE if symmetrize else 0) | (BUILD_KEEP_SELF_LOOPS if keep_self else 0)
    _check(lib().jx_csr_build(n, m, _ptr(src, torch.int32, m, "src") if m else None,
                              _ptr(dst, torch.int32, m, "dst") if m else None, flags,
                              ctypes.c_void_p(row_ptr.data_ptr()), ctypes.c_void_p(col.data_ptr()), cap,
                              ctypes.byref(e), _stream(stream)), "jx_csr_build")
    return GraphCSRView(row_ptr, col[: e.value].clone(), None, n, e.value)


def remove_reverse_edges(graph: GraphCSRView, values, stream=None):
    """The reference program's reverse-edge removal before MTX output (main.cpp:307-309): returns the
    surviving (src, dst, value) device tensors in CSR order."""
    torch = _torch()
    E = graph.number_of_edges
    dev = graph.indices.device
    src = torch.empty(max(E, 1), dtype=torch.int32, device=dev)
    dst = torch.empty_like(src)
    val = torch.empty(max(E, 1), dtype=torch.float32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    g = graph._c()
    _check(lib().jx_remove_reverse_edges(ctypes.byref(g), _ptr(values, torch.float32, E, "values"),
                                         ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                                         ctypes.c_void_p(val.data_ptr()), ctypes.c_void_p(cnt.data_ptr()),
                                         _stream(stream)), "jx_remove_reverse_edges")
    k = int(cnt.item())
    return src[:k], dst[:k], val[:k]


class Batch:
    """Batched mode (``jx_batch_*``): host CSRs packed into one device super-CSR, one replayed
    CUDA graph per pass over all graphs.  ``graphs``: list of (row_ptr, col_idx[, weights])
    numpy arrays."""

    def __init__(self, graphs, edge_centric: bool = False, weighted: bool = False, tune: bool = False):
        keep = []
        arr = (_HostGraph * len(graphs))()
        for i, gr in enumerate(graphs):
            rp = np.ascontiguousarray(gr[0], np.int32)
            col = np.ascontiguousarray(gr[1], np.int32)
            w = np.ascontiguousarray(gr[2], np.float32) if weighted else None
            keep.append((rp, col, w))
            arr[i] = _HostGraph(len(rp) - 1, len(col), rp.ctypes.data, col.ctypes.data,
                                None if w is None else w.ctypes.data)
        self._h = ctypes.c_void_p()
        self.ngraphs = len(graphs)
        self.edges = [len(k[1]) for k in keep]
        _check(lib().jx_batch_create(arr, len(graphs), ALGO_EDGE_CENTRIC if edge_centric else ALGO_VERTEX_CENTRIC,
                                     int(weighted), int(tune), ctypes.byref(self._h)), "jx_batch_create")

    def run(self, stream=None):
        _check(lib().jx_batch_run(self._h, _stream(stream)), "jx_batch_run")

    def result(self, g):
        """Device pointer and length of graph g's results."""
        p, n = ctypes.c_void_p(), ctypes.c_int64()
        _check(lib().jx_batch_result(self._h, g, ctypes.byref(p), ctypes.byref(n)), "jx_batch_result")
        return p.value, n.value

    def download(self, g, out=None, stream=None) -> np.ndarray:
        """Graph g's results on the host (g = -1: every graph's, concatenated)."""
        if out is None:
            out = np.empty(sum(self.edges) if g < 0 else self.edges[g], np.float32)
        _check(lib().jx_batch_download(self._h, g, out.ctypes.data, _stream(stream)), "jx_batch_download")
        return out

    def info(self) -> dict:
        nv, ne, k = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_uint64()
        buf = ctypes.create_string_buffer(256)
        _check(lib().jx_batch_info(self._h, ctypes.byref(nv), ctypes.byref(ne), ctypes.byref(k), buf, 256),
               "jx_batch_info")
        return {"vertices": nv.value, "edges": ne.value, "kernels_per_run": k.value, "plan": buf.value.decode()}

    def close(self):
        if self._h:
            lib().jx_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop (``jx_server_*``): admission by a device-memory budget, resident graphs
    with their row sums, folding of queued small requests into one pass, `slots` passes in
    flight on their own streams.  Requests score every edge of a graph; results land in the
    host array given at submit."""

    def __init__(self, memory_budget: int, slots: int = 4, fold_edges: int = 1 << 21,
                 fold_max_edges: int = 1 << 26, schedule: dict | None = None):
        _torch()  # a CUDA device must be present
        cfg = _ServerConfig(memory_budget, slots, fold_edges, fold_max_edges, _schedule(schedule or {}))
        self._h = ctypes.c_void_p()
        _check(lib().jx_server_create(ctypes.byref(cfg), ctypes.byref(self._h)), "jx_server_create")
        self._keep = {}  # ticket -> host objects that must outlive the request
        self.edges = {}  # resident graph id -> edge count

    @staticmethod
    def _host_graph(rp, col, w):
        rp = np.ascontiguousarray(rp, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        w = None if w is None else np.ascontiguousarray(w, np.float32)
        hg = _HostGraph(len(rp) - 1, len(col), rp.ctypes.data, col.ctypes.data,
                        None if w is None else w.ctypes.data)
        return hg, (rp, col, w)

    def add_graph(self, row_ptr, col_idx, weights=None) -> int:
        hg, _keep = self._host_graph(row_ptr, col_idx, weights)
        gid = ctypes.c_int32()
        _check(lib().jx_server_add_graph(self._h, ctypes.byref(hg), int(weights is not None), ctypes.byref(gid)),
               "jx_server_add_graph")
        self.edges[gid.value] = len(col_idx)
        return gid.value

    def submit(self, graph, out: np.ndarray, weighted: bool = False, edge_centric: bool = False,
               arrival_ns: int = 0) -> int:
        """graph: a resident id, or (row_ptr, col_idx[, weights]) host arrays to upload.
        out: float32 host array of the graph's edge count."""
        keep = [out]
        if isinstance(graph, (int, np.integer)):
            req = _Request(int(graph), None, ALGO_EDGE_CENTRIC if edge_centric else ALGO_VERTEX_CENTRIC,
                           int(weighted), out.ctypes.data, arrival_ns)
        else:
            hg, arrays = self._host_graph(graph[0], graph[1], graph[2] if len(graph) > 2 else None)
            keep += [hg, arrays]
            req = _Request(-1, ctypes.pointer(hg), ALGO_EDGE_CENTRIC if edge_centric else ALGO_VERTEX_CENTRIC,
                           int(weighted), out.ctypes.data, arrival_ns)
        t = ctypes.c_uint64()
        _check(lib().jx_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)), "jx_server_submit")
        self._keep[t.value] = keep
        return t.value

    def wait(self, ticket: int) -> float:
        """Latency (ms, arrival -> results in host memory) of one request; raises on failure."""
        lat = ctypes.c_double()
        st = lib().jx_server_wait(self._h, ticket, ctypes.byref(lat))
        self._keep.pop(ticket, None)
        _check(st, "jx_server_wait")
        return lat.value

    def drain(self):
        _check(lib().jx_server_drain(self._h), "jx_server_drain")

    def pause(self, paused: bool = True):
        """Hold (or, with False, resume) admission; passes already started run on."""
        _check(lib().jx_server_set_paused(self._h, int(paused)), "jx_server_set_paused")

    def cancel(self, ticket: int) -> bool:
        """Cancel a request that has not started: True if cancelled (its wait raises JxError
        with status 7), False if it had already started or finished."""
        st = lib().jx_server_cancel(self._h, ticket)
        if st == 5:
            return False
        _check(st, "jx_server_cancel")
        return True

    def inject_alloc_failures(self, count: int):
        """Test hook: the next `count` device allocations of passes fail as out of memory."""
        _check(lib().jx_server_inject_alloc_failures(self._h, count), "jx_server_inject_alloc_failures")

    def stats(self) -> dict:
        st = _ServerStats()
        _check(lib().jx_server_get_stats(self._h, ctypes.byref(st)), "jx_server_get_stats")
        return {k: getattr(st, k) for k, _ in _ServerStats._fields_}

    def reset_stats(self):
        lib().jx_server_reset_stats(self._h)

    @staticmethod
    def clock_ns() -> int:
        return lib().jx_server_clock_ns()

    def close(self):
        if self._h:
            lib().jx_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def csr_check(graph: GraphCSRView, stream=None) -> set:
    """Validate the CSR on the device; returns the set of problems found (empty = valid)."""
    flags = ctypes.c_uint32(0)
    g = graph._c()
    _check(lib().jx_csr_check(ctypes.byref(g), ctypes.byref(flags), _stream(stream)), "jx_csr_check")
    return {name for bit, name in CSR_FLAGS.items() if flags.value & bit}


def launch_count() -> int:
    return int(lib().jx_launch_count())


def launch_count_reset() -> None:
    lib().jx_launch_count_reset()
