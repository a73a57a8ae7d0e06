"""GPU: the allocation-free entry point jx_jaccard_noalloc.

Some callers cannot allocate device memory while they run -- services that reserve their
whole device budget up front without an allocator of their own, or pipelines where an
allocation call (and the synchronisation it may bring) is not acceptable between launches.
jx_jaccard_noalloc serves them from a fixed workspace array inside the library.  This test
calls it through the C ABI, twice in a row, and checks each result bit for bit against the
ordinary entry point jx_jaccard (the tolerance the other parity tests use).  It also checks
that a graph above the stated vertex limit is refused.

The file name sorts last so that a run stopping at the first failure has run every other test
first; it passes both alone and after the others.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_VERTICES = 1 << 20  # JX_NOALLOC_MAX_VERTICES in include/jx.h
TOO_LARGE = 6           # JX_ERR_TOO_LARGE


def _graph(jx, scale, seed):
    rp, col = jx.graphgen.rmat(scale, 16, 0.57, 0.19, 0.19, seed=seed)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=seed + 1)
    return rp, col, w


@pytest.mark.parametrize("mode", ["ec", "vc", "vcw"])
def test_noalloc_matches_jx_jaccard_twice(jx, mode):
    import torch
    L = jx.lib()
    # a skewed graph whose largest rows take the hub path, so every kernel runs
    rp, col, w = _graph(jx, 18, 71)
    assert len(rp) - 1 <= MAX_VERTICES
    g = jx.GraphCSRView.from_numpy(rp, col)
    wt = torch.from_numpy(w).cuda() if mode == "vcw" else None
    algo = 1 if mode == "ec" else 0
    ref = torch.empty(len(col), dtype=torch.float32, device="cuda")
    c = g._c()
    wp = ctypes.c_void_p(wt.data_ptr()) if wt is not None else None
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert L.jx_jaccard(ctypes.byref(c), wp, ctypes.c_void_p(ref.data_ptr()), algo, stream) == 0
    want = ref.cpu().numpy().view(np.uint32)
    for _ in range(2):
        out = torch.full((len(col),), float("nan"), dtype=torch.float32, device="cuda")
        rc = L.jx_jaccard_noalloc(ctypes.byref(c), wp, ctypes.c_void_p(out.data_ptr()), algo, stream)
        assert rc == 0, rc
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        bad = np.flatnonzero(got != want)
        assert bad.size == 0, f"{bad.size} results differ, first at {bad[:5]}"


def test_noalloc_rejects_graph_above_limit(jx):
    import torch
    L = jx.lib()
    n = MAX_VERTICES + 1
    rp = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    rp[1:] = 2  # row 0 holds two edges; the call is refused before any of it is read
    col = torch.tensor([1, 2], dtype=torch.int32, device="cuda")
    out = torch.empty(2, dtype=torch.float32, device="cuda")
    c = jx._Csr(n, 2, rp.data_ptr(), col.data_ptr())
    assert L.jx_jaccard_noalloc(ctypes.byref(c), None, ctypes.c_void_p(out.data_ptr()), 0, None) == TOO_LARGE
