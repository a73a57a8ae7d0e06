"""CPU: hand-checked known answers for the oracle (and the shapes the GPU tests reuse)."""
import numpy as np
import pytest


def csr_from_edges(n, edges):
    adj = [set() for _ in range(n)]
    for a, b in edges:
        if a != b:
            adj[a].add(b)
            adj[b].add(a)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(s) for s in adj])
    col = np.array([v for s in adj for v in sorted(s)], np.int32)
    return rp, col


def clique(n):
    return csr_from_edges(n, [(i, j) for i in range(n) for j in range(i + 1, n)])


@pytest.mark.parametrize("n", [2, 3, 4, 7, 33, 70])
@pytest.mark.parametrize("ec", [False, True])
def test_clique(O, n, ec):
    rp, col = clique(n)
    J = O.jaccard(rp, col, None, edge_centric=ec)
    assert np.all(J == np.float32(n - 2) / np.float32(n))


def test_star_path_disjoint(O):
    rp, col = csr_from_edges(9, [(0, i) for i in range(1, 6)] + [(6, 7)])
    assert not np.any(O.jaccard(rp, col, None))
    rp, col = csr_from_edges(5, [(0, 1), (1, 2), (2, 3), (3, 4)])
    assert not np.any(O.jaccard(rp, col, None, edge_centric=True))


def test_weighted_triangle(O):
    rp, col = clique(3)
    w = np.array([0.25, 0.5, 0.125], np.float32)
    J = O.jaccard(rp, col, w)
    # edge (0,1): I = w2, S0 = w1 + w2, S1 = w0 + w2 -> J = w2 / (w0 + w1 + w2)
    assert J[0] == np.float32(0.125) / np.float32(0.875)


def test_unit_weights_equal_unweighted(O, jx):
    rp, col = jx.graphgen.rmat(11, 16, seed=9)
    ones = np.ones(len(rp) - 1, np.float32)
    a = O.jaccard(rp, col, ones)
    b = O.jaccard(rp, col, None)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_isolated_vertices_and_empty(O):
    rp, col = csr_from_edges(6, [(1, 2), (2, 3), (1, 3)])
    J = O.jaccard(rp, col, None)
    assert np.allclose(J, 1 / 3) and len(J) == 6
    rp = np.zeros(5, np.int32)
    assert len(O.jaccard(rp, np.zeros(0, np.int32), None)) == 0


def test_zero_padding_of_an_ordered_sum():
    """The engine adds the last partial group of a weighted fold with +0.0 padding.  That is
    exact: a sequential float32 sum that starts at +0.0 is never -0.0 (round-to-nearest gives
    -0.0 only for -0.0 + -0.0), so each padding add returns the sum bit for bit -- for weights
    of both signs, signed zeros, infinities and NaNs alike."""
    rng = np.random.default_rng(61)
    pool = np.concatenate([rng.standard_normal(400).astype(np.float32) * np.float32(1e3),
                           np.float32([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45])])
    with np.errstate(invalid="ignore"):  # inf + -inf is part of the domain
        for _ in range(300):
            chain = rng.choice(pool, size=int(rng.integers(1, 40)))
            s = np.float32(0.0)
            for v in chain:
                s = np.float32(v + s)
                assert not (s == 0 and np.signbit(s))
            padded = s
            for _ in range(3):
                padded = np.float32(np.float32(0.0) + padded)
            assert np.asarray(padded).view(np.uint32) == np.asarray(s).view(np.uint32)
