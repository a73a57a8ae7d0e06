"""GPU: the operators next to the path -- pair-list Jaccard, the reference driver's non-zero count and
its reverse-edge removal -- against the oracle and the reference's own post-processing."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same_values(got, want):
    """Bit-equal, except that a NaN (a pair of two isolated vertices: 0 / 0, as in the
    reference) matches any NaN -- its bit pattern is the platform's default NaN, which differs
    between x86, Arm and the GPU."""
    got, want = np.asarray(got, np.float32), np.asarray(want, np.float32)
    gn, wn = np.isnan(got), np.isnan(want)
    return np.array_equal(gn, wn) and np.array_equal(bits(got[~gn]), bits(want[~wn]))


@pytest.fixture(scope="module")
def g14(jx):
    rp, col = jx.graphgen.rmat(14, 16, seed=51)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=52)
    return rp, col, w


@pytest.mark.parametrize("weighted", [False, True])
def test_pair_list(jx, O, g14, weighted):
    import torch
    rp, col, w = g14
    n = len(rp) - 1
    rng = np.random.default_rng(7)
    src = np.repeat(np.arange(n, dtype=np.int32), np.diff(rp))
    # a mix of stored edges, random (mostly non-adjacent) pairs, self pairs and isolated vertices
    pick = rng.integers(0, len(col), 4000)
    first = np.concatenate([src[pick], rng.integers(0, n, 4000).astype(np.int32), np.arange(50, dtype=np.int32)])
    second = np.concatenate([col[pick], rng.integers(0, n, 4000).astype(np.int32), np.arange(50, dtype=np.int32)])
    ww = w if weighted else None
    want = O.jaccard_list(rp, col, first, second, ww)
    g = jx.GraphCSRView.from_numpy(rp, col)
    got = jx.jaccard_list(g, torch.from_numpy(first).cuda(), torch.from_numpy(second).cuda(),
                          None if ww is None else torch.from_numpy(ww).cuda()).cpu().numpy()
    assert same_values(got, want)
    # stored edges: equal to the all-edges operator
    allJ = jx.jaccard(g, None if ww is None else torch.from_numpy(ww).cuda()).cpu().numpy()
    assert np.array_equal(bits(got[:4000]), bits(allJ[pick]))


def test_count_above(jx, g14):
    import torch
    rp, col, w = g14
    g = jx.GraphCSRView.from_numpy(rp, col)
    J = jx.jaccard(g, edge_centric=True)
    Jh = J.cpu().numpy()
    assert jx.count_above(J, 1e-5) == int((Jh > np.float32(1e-5)).sum())
    assert jx.count_above(J, 2.0) == 0


@pytest.mark.parametrize("weighted", [False, True])
def test_remove_reverse_edges(jx, O, g14, weighted):
    import torch
    if O.ref_lib() is None:
        pytest.skip("reference sources unavailable")
    rp, col, w = g14
    g = jx.GraphCSRView.from_numpy(rp, col)
    J = jx.jaccard(g, torch.from_numpy(w).cuda() if weighted else None)
    src, dst, val = jx.remove_reverse_edges(g, J)
    a, b, c = O.ref_remove_reverse(rp, col, J.cpu().numpy())
    assert np.array_equal(src.cpu().numpy(), a) and np.array_equal(dst.cpu().numpy(), b)
    assert np.array_equal(bits(val.cpu().numpy()), bits(c))


def _mixed_graphs(jx, count, seed):
    rng = np.random.default_rng(seed)
    gs = []
    for i in range(count):
        if i % 2 == 0:
            n = int(rng.integers(50, 3000))
            rp, col = jx.graphgen.er_gnm(n, int(n * rng.integers(2, 20)), seed=seed * 1000 + i)
        else:
            rp, col = jx.graphgen.rmat(int(rng.integers(6, 13)), int(rng.integers(4, 17)), seed=seed * 1000 + i)
        gs.append((rp, col, jx.graphgen.uniform_weights(len(rp) - 1, seed=seed * 1000 + 500 + i)))
    gs.insert(3, (np.zeros(4, np.int32), np.zeros(0, np.int32), np.ones(3, np.float32)))  # edgeless graph
    return gs


@pytest.mark.parametrize("mode", ["ec", "vc", "vcw"])
def test_batch_equals_per_graph(jx, O, mode):
    """Every graph's slice of a mixed batch equals the oracle on that graph alone, bit for bit,
    and equals the engine's own plain call on it, on two replays of the captured pass."""
    import torch
    gs = _mixed_graphs(jx, 24, 3)
    b = jx.Batch(gs, edge_centric=(mode == "ec"), weighted=(mode == "vcw"), tune=(mode == "vc"))
    info = b.info()
    assert info["edges"] == sum(len(g[1]) for g in gs) and info["kernels_per_run"] > 0
    oracle = [O.jaccard(rp, col, w if mode == "vcw" else None, edge_centric=(mode == "ec")) if len(col) else None
              for rp, col, w in gs]
    for rep in range(2):  # the captured graph replays to the same results
        b.run()
        torch.cuda.synchronize()
        for i, (rp, col, w) in enumerate(gs):
            if len(col) == 0:
                continue
            got = b.download(i)
            ora = oracle[i]
            bad = np.nonzero(bits(got) != bits(ora))[0]
            if len(bad):
                d = np.diff(rp)
                src = np.repeat(np.arange(len(rp) - 1), d)
                info = [(int(k), int(src[k]), int(col[k]), int(d[src[k]]), int(d[col[k]]), float(got[k]),
                         float(ora[k])) for k in bad[:6]]
                raise AssertionError(f"rep {rep} graph {i}: {len(bad)} differ from the oracle; "
                                     f"(k,u,v,du,dv,batch,oracle) {info}")
            if rep == 0:
                g = jx.GraphCSRView.from_numpy(rp, col)
                plain = jx.jaccard(g, torch.from_numpy(w).cuda() if mode == "vcw" else None,
                                   edge_centric=(mode == "ec")).cpu().numpy()
                assert np.array_equal(bits(plain), bits(ora)), f"graph {i}: plain call differs from the oracle"
    b.close()
