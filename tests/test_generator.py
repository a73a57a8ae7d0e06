"""CPU: the synthetic graphs are deterministic, symmetric, sorted, loop and duplicate free."""
import numpy as np
import pytest


def check_csr(rp, col):
    n = len(rp) - 1
    assert rp[0] == 0 and rp[-1] == len(col) and np.all(np.diff(rp) >= 0)
    assert col.min(initial=0) >= 0 and col.max(initial=-1) < n
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
    assert not np.any(src == col), "self loop"
    key = src * n + col
    same_row = src[1:] == src[:-1]
    assert np.all(col[1:][same_row] > col[:-1][same_row]), "unsorted or duplicate"
    rkey = col.astype(np.int64) * n + src
    assert np.array_equal(np.sort(key), np.sort(rkey)), "not symmetric"


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_rmat_deterministic(jx, threads):
    a = jx.graphgen.rmat(12, 16, seed=2, threads=threads)
    b = jx.graphgen.rmat(12, 16, seed=2, threads=1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    check_csr(*a)


def test_er_shapes(jx):
    rp, col = jx.graphgen.er_gnp(4096, 16 / 4095, seed=1)
    check_csr(rp, col)
    assert len(rp) == 4097 and 60000 < len(col) < 70000
    rp, col = jx.graphgen.er_gnm(10000, 80000, seed=3)
    check_csr(rp, col)
    assert len(col) > 150000


def test_weights_grid(jx):
    w = jx.graphgen.uniform_weights(100000, seed=4)
    assert w.min() > 0 and w.max() <= 1
    assert np.all(np.float32(w * 16777216) == np.round(w * 16777216))
    assert np.array_equal(w, jx.graphgen.uniform_weights(100000, seed=4, threads=2))


def test_stats(jx):
    rp, col = jx.graphgen.rmat(10, 16, seed=1)
    st = jx.graphgen.stats(rp, col)
    d = np.diff(rp)
    src = np.repeat(np.arange(len(d)), d)
    assert st["sum_min"] == int(np.minimum(d[src], d[col]).sum())
    assert st["V"] == 1024 and st["E"] == len(col)


def test_rmat_permuted_is_the_same_graph_relabelled(jx, O):
    """A relabelled R-MAT has the same degree sequence and, edge for edge, the same Jaccard
    values as a multiset; its hub no longer sits at vertex 0."""
    rp, col = jx.graphgen.rmat(11, 16, seed=9)
    rq, cq = jx.graphgen.rmat(11, 16, seed=9, permute=77)
    assert len(cq) == len(col) and len(rq) == len(rp)
    d, dq = np.diff(rp), np.diff(rq)
    assert np.array_equal(np.sort(d), np.sort(dq))
    assert int(np.argmax(dq)) != int(np.argmax(d))
    check_csr(rq, cq)
    J, Jq = O.jaccard(rp, col), O.jaccard(rq, cq)
    assert np.array_equal(np.sort(J.view(np.uint32)), np.sort(Jq.view(np.uint32)))
    assert not np.array_equal(rp, rq)
