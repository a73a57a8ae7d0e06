"""The operator at the int32 limit: a graph of 2,147,235,072 stored edges, 248,575 short of
2^31 - 1, the largest edge count GraphCSRView<int32_t, int32_t, float> can hold
(standalone_csr.hpp:44-105).

512 disjoint cliques of 2048 vertices (every row a CTA-bin row, every pair a degree tie) and
2 stars of 200,000 leaves (hub rows; their offsets sit above 2^31 - 2^24) whose Jaccard values
are known in closed form: an edge of a clique K_m shares m - 2 neighbours out of m, so
J = (m - 2) / m exactly in float (2046 / 2048 = 1 - 2^-10); a star edge shares none, J = 0.
With unit vertex weights the weighted operator gives the same values.  The CPU test pins the
closed form to the oracle (the reference's algorithm) on a small instance of the same shape; the
GPU test checks every edge of the full-size graph, VC unweighted, VC weighted and EC.
"""
import numpy as np
import pytest


def cliques_and_stars(torch, device, m, cliques, stars, leaves):
    """row_ptr (int32[V+1]), col_idx (int32[E]) and the number of clique edges: `cliques`
    copies of K_m on vertices [0, cliques*m), then `stars` stars, each a centre followed by
    its `leaves` leaves.  Rows are sorted ascending."""
    nv = cliques * m + stars * (leaves + 1)
    deg = torch.empty(nv, dtype=torch.int64, device=device)
    deg[: cliques * m] = m - 1
    star_deg = torch.ones(leaves + 1, dtype=torch.int64, device=device)
    star_deg[0] = leaves
    deg[cliques * m:] = star_deg.repeat(stars)
    row_ptr = torch.zeros(nv + 1, dtype=torch.int64, device=device)
    row_ptr[1:] = torch.cumsum(deg, 0)
    e = int(row_ptr[-1])
    assert e < 2 ** 31
    col = torch.empty(e, dtype=torch.int32, device=device)
    a = torch.arange(m, dtype=torch.int32, device=device)
    block = a.repeat(m).view(m, m)[~torch.eye(m, dtype=torch.bool, device=device)]  # row i: all but i
    per = m * (m - 1)
    for k in range(cliques):
        col[k * per:(k + 1) * per] = block + k * m
    base_e = cliques * per
    for s in range(stars):
        c = cliques * m + s * (leaves + 1)
        seg = col[base_e + s * 2 * leaves: base_e + (s + 1) * 2 * leaves]
        seg[:leaves] = torch.arange(c + 1, c + leaves + 1, dtype=torch.int32, device=device)
        seg[leaves:] = c
    return row_ptr.to(torch.int32), col, base_e


def expected(m, nclique_edges, e):
    j = np.float32(m - 2) / np.float32(m)
    want = np.zeros(e, np.float32)
    want[:nclique_edges] = j
    return want


def test_closed_form_matches_oracle(O):
    """Small instance: the oracle (the reference's order and expressions) gives the closed form."""
    import torch
    m, cl, st, lv = 8, 3, 2, 50
    rp, col, nce = cliques_and_stars(torch, "cpu", m, cl, st, lv)
    rp, col = rp.numpy(), col.numpy()
    want = expected(m, nce, len(col)).view(np.uint32)
    w = np.ones(len(rp) - 1, np.float32)
    for ww, ec in ((None, False), (w, False), (None, True)):
        assert np.array_equal(O.jaccard(rp, col, ww, edge_centric=ec).view(np.uint32), want)


@pytest.mark.gpu
def test_int32_edge_limit(jx):
    import torch
    m, cl, st, lv = 2048, 512, 2, 200_000
    rp, col, nce = cliques_and_stars(torch, "cuda", m, cl, st, lv)
    e = col.numel()
    assert e == 2_147_235_072 and int(rp[cl * m]) == nce and nce > 2 ** 31 - 2 ** 24
    g = jx.GraphCSRView(rp, col)
    j = np.float32(m - 2) / np.float32(m)
    jbits = int(np.array([j], np.float32).view(np.int32)[0])
    w = torch.ones(rp.numel() - 1, dtype=torch.float32, device="cuda")
    for ww, ec in ((None, False), (w, False), (None, True)):
        out = jx.jaccard(g, ww, edge_centric=ec)
        torch.cuda.synchronize()
        ob = out.view(torch.int32)
        bad_clique = int((ob[:nce] != jbits).sum())
        bad_star = int((ob[nce:] != 0).sum())
        assert bad_clique == 0 and bad_star == 0, (ww is not None, ec, bad_clique, bad_star)
        del out, ob
        torch.cuda.empty_cache()
