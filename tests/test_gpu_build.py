"""GPU: the device CSR builder (the reference program's graph preparation) against the oracle's
restatement, which tests/test_build.py pins to the reference's own set-based code."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def skewed_edges(n, m, seed):
    rng = np.random.default_rng(seed)
    # power-law-ish endpoints (many repeats, hubs), plus self loops and reversed copies
    src = np.minimum((rng.pareto(1.2, m) * 3).astype(np.int64), n - 1).astype(np.int32)
    dst = rng.integers(0, n, m).astype(np.int32)
    src = np.concatenate([src, dst[: m // 5], np.arange(min(n, 7), dtype=np.int32)])
    dst = np.concatenate([dst, src[: m // 5], np.arange(min(n, 7), dtype=np.int32)])
    return src.astype(np.int32), dst.astype(np.int32)


@pytest.mark.parametrize("n,m", [(1, 1), (3, 10), (1000, 20000), (100_000, 1_000_000), (1 << 24, 50_000)])
@pytest.mark.parametrize("symmetrize,keep_self", [(True, False), (False, False), (True, True)])
def test_build_matches_restatement(jx, O, n, m, symmetrize, keep_self):
    import torch
    src, dst = skewed_edges(n, m, seed=n + m)
    g = jx.csr_build(n, torch.from_numpy(src).cuda(), torch.from_numpy(dst).cuda(), symmetrize, keep_self)
    rp, col = O.csr_build(n, src, dst, symmetrize, keep_self)
    assert g.number_of_vertices == n and g.number_of_edges == len(col)
    assert np.array_equal(g.offsets.cpu().numpy(), rp)
    assert np.array_equal(g.indices.cpu().numpy(), col)


def test_built_graph_scores_like_host_graph(jx):
    """An R-MAT graph rebuilt on the device from its own edge list (one direction, shuffled,
    with repeats) is the same CSR, and its Jaccard values are the same bits."""
    import torch
    rp, col = jx.graphgen.rmat(16, 16, seed=31)
    n = len(rp) - 1
    src = np.repeat(np.arange(n, dtype=np.int32), np.diff(rp))
    half = src < col
    s, d = src[half], col[half]
    perm = np.random.default_rng(5).permutation(len(s))
    s = np.concatenate([s[perm], s[:1000]])
    d = np.concatenate([d[perm], d[:1000]])
    g = jx.csr_build(n, torch.from_numpy(s).cuda(), torch.from_numpy(d).cuda())
    assert np.array_equal(g.offsets.cpu().numpy(), rp) and np.array_equal(g.indices.cpu().numpy(), col)
    assert jx.csr_check(g) == set()
    J1 = jx.jaccard(g).cpu().numpy()
    J2 = jx.jaccard(jx.GraphCSRView.from_numpy(rp, col)).cpu().numpy()
    assert np.array_equal(J1.view(np.uint32), J2.view(np.uint32))


def test_build_errors(jx):
    import torch
    L = jx.lib()
    src = torch.tensor([0, 1, 5], dtype=torch.int32, device="cuda")
    dst = torch.tensor([1, 2, 0], dtype=torch.int32, device="cuda")
    with pytest.raises(jx.JxError) as e:
        jx.csr_build(5, src, dst)  # vertex 5 outside [0, 5)
    assert e.value.status == 1
    rp = torch.empty(7, dtype=torch.int32, device="cuda")
    col = torch.empty(2, dtype=torch.int32, device="cuda")
    cnt = ctypes.c_int64()
    st = L.jx_csr_build(6, 3, ctypes.c_void_p(src.data_ptr()), ctypes.c_void_p(dst.data_ptr()), 1,
                        ctypes.c_void_p(rp.data_ptr()), ctypes.c_void_p(col.data_ptr()), 2, ctypes.byref(cnt),
                        None)
    assert st == 6 and cnt.value == 6  # JX_ERR_TOO_LARGE: 6 edges for a capacity of 2
    g = jx.csr_build(4, torch.empty(0, dtype=torch.int32, device="cuda"),
                     torch.empty(0, dtype=torch.int32, device="cuda"))
    assert g.number_of_edges == 0 and np.array_equal(g.offsets.cpu().numpy(), np.zeros(5, np.int32))
