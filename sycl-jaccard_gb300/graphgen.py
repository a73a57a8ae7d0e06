"""Synthetic graphs of the shapes the benchmark configurations name.

Binds ``csrc/gen/libjxgen.so`` (host C++/OpenMP).  Every draw is a function of the seed
only (``csrc/jx_rng.h``), so a graph is identical on any machine and thread count.  All
graphs are symmetric, self-loop free, deduplicated, with each row sorted ascending -- the
form the reference's driver hands to the operator (main.cpp:99-120).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_gen = None


def _lib():
    global _gen
    if _gen is None:
        if not os.path.exists(_build.LIBGEN):
            _build.build_generator()
        L = ctypes.CDLL(_build.LIBGEN)
        L.jxg_rmat.restype = ctypes.c_void_p
        L.jxg_rmat.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                               ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int]
        L.jxg_er_gnp.restype = ctypes.c_void_p
        L.jxg_er_gnp.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_uint64, ctypes.c_int]
        L.jxg_er_gnm.restype = ctypes.c_void_p
        L.jxg_er_gnm.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_uint64, ctypes.c_int]
        for f in ("jxg_num_vertices", "jxg_num_edges"):
            getattr(L, f).restype = ctypes.c_int64
            getattr(L, f).argtypes = [ctypes.c_void_p]
        L.jxg_export.restype = ctypes.c_int
        L.jxg_export.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.jxg_free.argtypes = [ctypes.c_void_p]
        L.jxg_uniform_weights.argtypes = [ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_int]
        _gen = L
    return _gen


def _take(h):
    L = _lib()
    if not h:
        raise MemoryError("graph generation failed")
    try:
        n, e = L.jxg_num_vertices(h), L.jxg_num_edges(h)
        rp = np.empty(n + 1, np.int32)
        col = np.empty(e, np.int32)
        if L.jxg_export(h, rp.ctypes.data, col.ctypes.data) != 0:
            raise ValueError("graph has 2^31 or more edges; int32 CSR impossible")
        return rp, col
    finally:
        L.jxg_free(h)


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 0, threads: int = 0, permute: int = 0):
    """R-MAT(scale, edge_factor, a, b, c), symmetrised / deduplicated / loop-free int32 CSR.
    permute != 0 relabels the vertices by a bijection of [0, 2^scale) seeded by it (the same
    graph with hub ids scattered over the id range)."""
    return _take(_lib().jxg_rmat(scale, edge_factor, a, b, c, seed, permute, threads))


def er_gnp(n: int, p: float, seed: int = 0, threads: int = 0):
    """Erdos-Renyi G(n, p) (every pair tested; n <= 2^20)."""
    return _take(_lib().jxg_er_gnp(n, p, seed, threads))


def er_gnm(n: int, m: int, seed: int = 0, threads: int = 0):
    """Erdos-Renyi G(n, m)-style: m uniform undirected samples, symmetrised/deduplicated."""
    return _take(_lib().jxg_er_gnm(n, m, seed, threads))


def uniform_weights(n: int, seed: int = 0, threads: int = 0) -> np.ndarray:
    """Per-vertex float32 weights uniform on the 2^-24 grid of (0, 1]."""
    out = np.empty(n, np.float32)
    _lib().jxg_uniform_weights(n, seed, out.ctypes.data, threads)
    return out


def stats(row_ptr: np.ndarray, col: np.ndarray) -> dict:
    """V, E, degree facts and sum_e min(d_u, d_v) (the byte model's must-read term)."""
    n = len(row_ptr) - 1
    deg = np.diff(row_ptr).astype(np.int64)
    # per-edge min(d_u, d_v) without materialising an int64 copy of the source array
    sum_min = 0
    step = 1 << 20
    for s in range(0, n, step):
        e0, e1 = int(row_ptr[s]), int(row_ptr[min(n, s + step)])
        src_deg = np.repeat(deg[s:min(n, s + step)], deg[s:min(n, s + step)])
        sum_min += int(np.minimum(src_deg, deg[col[e0:e1]]).sum())
    return {"V": int(n), "E": int(len(col)), "isolated": int((deg == 0).sum()),
            "max_degree": int(deg.max()) if n else 0, "sum_min": int(sum_min)}


# Named configurations (the benchmark's workload shapes).
def config_graph(name: str, threads: int = 0, permute: int = 0):
    """Returns (row_ptr, col_idx, vertex_weights or None, description).  permute != 0 relabels
    the vertices of the R-MAT configurations (see rmat)."""
    if permute and name.startswith("rmat"):
        rp, col, w, desc = _config_graph(name, threads, permute)
        return rp, col, w, desc + f", vertex ids relabelled by a bijection seeded {permute}"
    return _config_graph(name, threads, 0)


def _config_graph(name: str, threads: int, permute: int):
    if name == "er4096":
        rp, col = er_gnp(4096, 16.0 / 4095.0, seed=1, threads=threads)
        return rp, col, np.ones(4096, np.float32), "ER G(4096, 16/4095) seed 1, unit weights"
    if name == "rmat20":
        rp, col = rmat(20, 16, 0.57, 0.19, 0.19, seed=2, threads=threads, permute=permute)
        return rp, col, None, "RMAT scale 20 ef 16 (.57,.19,.19,.05) seed 2, unweighted"
    if name == "rmat22w":  # the headline shape at a quarter of the size (profiling captures)
        rp, col = rmat(22, 16, 0.57, 0.19, 0.19, seed=3, threads=threads, permute=permute)
        w = uniform_weights(len(rp) - 1, seed=4, threads=threads)
        return rp, col, w, "RMAT scale 22 ef 16 (.57,.19,.19,.05) seed 3, vertex weights U(0,1] seed 4"
    if name == "rmat24w":
        rp, col = rmat(24, 16, 0.57, 0.19, 0.19, seed=3, threads=threads, permute=permute)
        w = uniform_weights(len(rp) - 1, seed=4, threads=threads)
        return rp, col, w, "RMAT scale 24 ef 16 (.57,.19,.19,.05) seed 3, vertex weights U(0,1] seed 4"
    raise KeyError(name)


def batch_graphs(count: int = 2000, seed: int = 5, threads: int = 0, vmin: int = 256, vmax: int = 262144):
    """The batched workload: `count` graphs, vertex counts log-uniform in [vmin, vmax], half
    Erdos-Renyi (G(n, m) with m = n * avg_degree / 2, avg degree uniform in [4, 64]) and half
    R-MAT (scale round(log2 n), edge factor uniform in [8, 32], a = .57, b = c = .19), each
    symmetrised / deduplicated / sorted int32 CSR.  Graph i uses seed `seed * 1000003 + i`.
    Returns a list of (row_ptr, col_idx, description)."""
    rng = np.random.default_rng(seed)
    nv = np.exp(rng.uniform(np.log(vmin), np.log(vmax), count)).round().astype(np.int64)
    kind = rng.permutation(np.arange(count) % 2)  # 0 = ER, 1 = RMAT, half each
    deg = rng.uniform(4.0, 64.0, count)
    ef = rng.integers(8, 33, count)
    out = []
    for i in range(count):
        s = seed * 1000003 + i
        if kind[i] == 0:
            n = int(nv[i])
            rp, col = er_gnm(n, int(round(n * deg[i] / 2)), seed=s, threads=threads)
            out.append((rp, col, f"ER n={n} deg={deg[i]:.1f}"))
        else:
            sc = int(np.clip(np.round(np.log2(nv[i])), 8, 18))
            rp, col = rmat(sc, int(ef[i]), 0.57, 0.19, 0.19, seed=s, threads=threads)
            out.append((rp, col, f"RMAT scale={sc} ef={int(ef[i])}"))
    return out


def served_pools(seed: int = 6, resident: int = 64, uploads: int = 32, threads: int = 0):
    """The served workload's graphs.  Resident pool: `resident` R-MAT graphs, scale uniform in
    [14, 20], edge factor 16, (a, b, c) = (.57, .19, .19).  Upload pool: `uploads` graphs with
    vertex counts log-uniform in [1e3, 1e6], half Erdos-Renyi (avg degree uniform in [4, 64]),
    half R-MAT (scale round(log2 n), edge factor 16).  Every graph carries per-vertex float32
    weights uniform in (0, 1].  Returns two lists of (row_ptr, col_idx, weights, description)."""
    rng = np.random.default_rng(seed)
    res = []
    for i, sc in enumerate(rng.integers(14, 21, resident)):
        s = seed * 1000003 + i
        rp, col = rmat(int(sc), 16, 0.57, 0.19, 0.19, seed=s, threads=threads)
        res.append((rp, col, uniform_weights(len(rp) - 1, seed=s + 500000, threads=threads),
                    f"RMAT scale={int(sc)} ef=16"))
    up = []
    nv = np.exp(rng.uniform(np.log(1e3), np.log(1e6), uploads)).round().astype(np.int64)
    deg = rng.uniform(4.0, 64.0, uploads)
    for i in range(uploads):
        s = seed * 1000003 + 700000 + i
        n = int(nv[i])
        if i % 2 == 0:
            rp, col = er_gnm(n, int(round(n * deg[i] / 2)), seed=s, threads=threads)
            d = f"ER n={n} deg={deg[i]:.1f}"
        else:
            sc = int(np.round(np.log2(n)))
            rp, col = rmat(sc, 16, 0.57, 0.19, 0.19, seed=s, threads=threads)
            d = f"RMAT scale={sc} ef=16"
        up.append((rp, col, uniform_weights(len(rp) - 1, seed=s + 500000, threads=threads), d))
    return res, up


def poisson_trace(count: int, rate: float, resident: int, uploads: int, seed: int = 6,
                  resident_share: float = 0.7):
    """Arrival times (s, from 0) of a Poisson stream of `count` requests at `rate` per second,
    and their targets: ("resident", k) with probability resident_share, else ("upload", k)."""
    rng = np.random.default_rng(seed + 1)
    t = np.cumsum(rng.exponential(1.0 / rate, count))
    is_res = rng.random(count) < resident_share
    k_res = rng.integers(0, resident, count)
    k_up = rng.integers(0, uploads, count)
    return t - t[0], [("resident", int(a)) if r else ("upload", int(b)) for r, a, b in zip(is_res, k_res, k_up)]
