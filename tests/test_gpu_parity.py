"""GPU parity: the CUDA engine against the oracle and the reference's golden vectors.

Bar: bit-exact for every mode (counts and unweighted J trivially; weighted J too, because
the engine reproduces the reference's accumulation order), and bitwise deterministic.
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
MODES = [("ec", None), ("vc", None), ("vcw", "w")]


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def assert_bitwise(got, want, what=""):
    g, w = bits(got), bits(want)
    bad = np.flatnonzero(g != w)
    assert bad.size == 0, f"{what}: {bad.size} mismatches, first at {bad[:5]}: {np.asarray(got)[bad[:5]]} vs {np.asarray(want)[bad[:5]]}"


def run(jx, rp, col, w=None, ec=False):
    import torch
    g = jx.GraphCSRView.from_numpy(rp, col)
    wt = None if w is None else torch.from_numpy(w).cuda()
    out = jx.jaccard(g, wt, edge_centric=ec)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("mode", ["J_ec", "J_vc", "J_vcw"])
def test_fused_matches_golden(jx, path, mode):
    gd = np.load(path)
    w = gd["w"] if mode == "J_vcw" else None
    assert_bitwise(run(jx, gd["row_ptr"], gd["col_idx"], w, ec=(mode == "J_ec")), gd[mode], mode)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_stages_match_golden(jx, path):
    import torch
    gd = np.load(path)
    rp, col, w = gd["row_ptr"], gd["col_idx"], gd["w"]
    n, e = len(rp) - 1, len(col)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    trp, tcol, tw = d(rp), d(col), d(w)
    S = torch.empty(n, dtype=torch.float32, device="cuda")
    jx.rowsum(n, e, trp, tcol, tw, S)
    assert_bitwise(S.cpu().numpy(), gd["S_w"], "rowsum weighted")
    Su = torch.empty_like(S)
    jx.rowsum(n, e, trp, tcol, None, Su)
    assert_bitwise(Su.cpu().numpy(), gd["S_u"], "rowsum unweighted")
    wi = torch.empty(e, dtype=torch.float32, device="cuda")
    jx.fill(wi, 0.0)
    ws = torch.empty_like(wi)
    jx.intersect(n, e, trp, tcol, tw, S, wi, ws)
    assert_bitwise(wi.cpu().numpy(), gd["Wi_w"], "weight_i")
    assert_bitwise(ws.cpu().numpy(), gd["Ws_w"], "weight_s")
    wj = torch.empty_like(wi)
    jx.weight(e, wi, ws, wj)
    assert_bitwise(wj.cpu().numpy(), gd["J_vcw"], "jw")
    dest = torch.empty(e, dtype=torch.int32, device="cuda")
    wj2 = torch.full((e,), float("nan"), device="cuda")
    jx.ec_scan(e, n, trp, dest, wj2)
    assert np.array_equal(dest.cpu().numpy(), gd["dest_ind"])
    assert not torch.any(wj2 != 0)
    jx.ec_unweighted(e, n, trp, tcol, dest, wj2)
    assert_bitwise(wj2.cpu().numpy(), gd["J_ec"], "ec_unweighted")


@pytest.mark.parametrize("scale,seed", [(12, 21), (14, 22), (16, 23)])
@pytest.mark.parametrize("mode", ["ec", "vc", "vcw"])
def test_fused_vs_oracle_rmat(jx, O, scale, seed, mode):
    rp, col = jx.graphgen.rmat(scale, 16, 0.57, 0.19, 0.19, seed=seed)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=seed + 100) if mode == "vcw" else None
    want = O.jaccard(rp, col, w, edge_centric=(mode == "ec"))
    assert_bitwise(run(jx, rp, col, w, ec=(mode == "ec")), want, f"rmat{scale} {mode}")


@pytest.mark.parametrize("mode", ["ec", "vc", "vcw"])
def test_fused_er_config(jx, O, mode):
    """The small plain configuration: ER G(4096, 16/4095) seed 1 with unit weights."""
    rp, col, w, _ = jx.graphgen.config_graph("er4096")
    ww = w if mode == "vcw" else None
    want = O.jaccard(rp, col, ww, edge_centric=(mode == "ec"))
    got = run(jx, rp, col, ww, ec=(mode == "ec"))
    assert_bitwise(got, want, mode)
    if mode == "vcw":  # unit weights: weighted == unweighted, bit for bit
        assert_bitwise(got, O.jaccard(rp, col, None), "unit weights")


def test_deterministic(jx):
    rp, col = jx.graphgen.rmat(15, 16, seed=31)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=32)
    a = run(jx, rp, col, w)
    b = run(jx, rp, col, w)
    assert_bitwise(a, b, "repeat")


def csr_from_edges(n, edges, symmetric=True):
    adj = [set() for _ in range(n)]
    for a, b in edges:
        adj[a].add(b)
        if symmetric:
            adj[b].add(a)
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum([len(s) for s in adj])
    col = np.array([v for s in adj for v in sorted(s)], np.int32)
    return rp, col


def with_repeats(rp, col, rows_every, both_ways):
    """The CSR with the first neighbour of every `rows_every`-th non-empty row listed twice
    (rows stay sorted); with both_ways the reverse entry is repeated too.  The reference takes
    such CSRs without validation and counts every stored position."""
    n = len(rp) - 1
    adj = [list(col[rp[u]:rp[u + 1]]) for u in range(n)]
    for u in range(0, n, rows_every):
        if adj[u]:
            v = adj[u][0]
            adj[u].insert(0, v)
            if both_ways:
                adj[v].insert(adj[v].index(u), u)
    out = np.zeros(n + 1, np.int32)
    out[1:] = np.cumsum([len(a) for a in adj])
    return out, np.array([x for a in adj for x in a], np.int32)


@pytest.mark.parametrize("mode", ["ec", "vc", "vcw"])
def test_edge_cases(jx, O, mode):
    rng = np.random.default_rng(5)
    cases = {
        "single_edge": csr_from_edges(2, [(0, 1)]),
        "isolated_tail": csr_from_edges(10, [(1, 2), (2, 3), (1, 3)]),
        "star": csr_from_edges(70, [(0, i) for i in range(1, 70)]),
        "clique40": csr_from_edges(40, [(i, j) for i in range(40) for j in range(i + 1, 40)]),
        "regular_ties": csr_from_edges(64, [(i, (i + k) % 64) for i in range(64) for k in (1, 2, 5)]),
        # not symmetric: edges only one way -> every edge goes through the fix-up pass
        "directed": csr_from_edges(300, [(int(a), int(b)) for a, b in rng.integers(0, 300, (3000, 2)) if a != b],
                                   symmetric=False),
    }
    # repeated neighbours (each stored position counts, like the reference's binary searches),
    # on a graph with rows in every degree bin: lane, warp and CTA rows and a hub row
    hubby = csr_from_edges(30000, [(0, i) for i in range(1, 26000)] + [(1, i) for i in range(2, 600)] +
                           [(int(a), int(b)) for a, b in rng.integers(2, 30000, (60000, 2)) if a != b])
    cases["repeats_both_ways"] = with_repeats(*hubby, rows_every=7, both_ways=True)
    cases["repeats_one_way"] = with_repeats(*hubby, rows_every=5, both_ways=False)
    cases["repeats_small"] = with_repeats(*csr_from_edges(40, [(i, j) for i in range(40) for j in range(i + 1, 40)]),
                                          rows_every=3, both_ways=True)
    for name, (rp, col) in cases.items():
        w = jx.graphgen.uniform_weights(len(rp) - 1, seed=7) if mode == "vcw" else None
        want = O.jaccard(rp, col, w, edge_centric=(mode == "ec"))
        assert_bitwise(run(jx, rp, col, w, ec=(mode == "ec")), want, f"{name} {mode}")


def test_empty_graphs(jx):
    import torch
    for n in (0, 5):
        g = jx.GraphCSRView(torch.zeros(n + 1, dtype=torch.int32, device="cuda"),
                            torch.zeros(0, dtype=torch.int32, device="cuda"))
        out = jx.jaccard(g)
        torch.cuda.synchronize()
        assert out.numel() == 0


def test_host_entry_point(jx, O):
    """Host arrays in and out; the device memory kept between calls is reused, released, and
    the next call after the release maps it again -- same results every time."""
    rp, col = jx.graphgen.rmat(13, 16, seed=41)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=42)
    for rep in range(2):
        for ec, ww in ((True, None), (False, None), (False, w)):
            assert_bitwise(jx.jaccard_host(rp, col, ww, edge_centric=ec), O.jaccard(rp, col, ww, edge_centric=ec))
        assert jx.lib().jx_host_release() == 0
    rp2, col2 = jx.graphgen.rmat(9, 8, seed=43)  # a smaller graph in the same pool
    assert_bitwise(jx.jaccard_host(rp2, col2), O.jaccard(rp2, col2))
    # host arrays in the library's pinned memory (jx_host_alloc / jx_host_free)
    hrp, hcol, hw = jx.HostArray.copy_of(rp), jx.HostArray.copy_of(col), jx.HostArray.copy_of(w)
    hout = jx.HostArray((len(col),), np.float32)
    jx.jaccard_host(hrp.array, hcol.array, hw.array, out=hout.array)
    assert_bitwise(hout.array, O.jaccard(rp, col, w))
    for h in (hrp, hcol, hw, hout):
        h.free()


def test_csr_check(jx):
    import torch
    rp, col = jx.graphgen.rmat(10, 8, seed=1)
    g = jx.GraphCSRView.from_numpy(rp, col)
    assert jx.csr_check(g) == set()
    bad = col.copy()
    r = int(np.argmax(np.diff(rp)))
    bad[rp[r]], bad[rp[r] + 1] = bad[rp[r] + 1], bad[rp[r]]
    assert "unsorted" in jx.csr_check(jx.GraphCSRView.from_numpy(rp, bad))
    rp2, col2 = csr_from_edges(5, [(0, 1), (1, 2)], symmetric=False)
    assert jx.csr_check(jx.GraphCSRView.from_numpy(rp2, col2)) == {"asymmetric"}


def test_launch_counter(jx):
    rp, col = jx.graphgen.rmat(10, 8, seed=1)
    jx.launch_count_reset()
    run(jx, rp, col)
    assert jx.launch_count() >= 3


def parse_profile(L):
    import ctypes
    buf = ctypes.create_string_buffer(4096)
    n = L.jx_profile_end(buf, 4096)
    parts = [p.split("=") for p in buf.value.decode().split(";") if p]
    return n, [(k, float(v)) for k, v in parts]


def test_profiler(jx):
    """jx_profile_begin/end name every timed launch of a call, with non-negative times, and
    record nothing outside a begin/end pair."""
    import torch
    L = jx.lib()
    rp, col = jx.graphgen.rmat(12, 16, seed=2)
    w = torch.from_numpy(jx.graphgen.uniform_weights(len(rp) - 1, seed=3)).cuda()
    g = jx.GraphCSRView.from_numpy(rp, col)
    L.jx_profile_begin()
    jx.jaccard(g, w)
    n, marks = parse_profile(L)
    names = [k for k, _ in marks]
    assert n == len(marks) > 0
    for k in ("plan", "rowsum", "sentinel_fill", "cta_rows", "warp_rows", "lane_rows", "fixup"):
        assert k in names, (k, names)
    assert all(ms >= 0.0 for _, ms in marks)
    jx.jaccard(g, w)  # not between begin and end
    L.jx_profile_begin()
    jx.jaccard_host(rp, col, jx.graphgen.uniform_weights(len(rp) - 1, seed=3))
    n, marks = parse_profile(L)
    names = [k for k, _ in marks]
    for k in ("h2d", "plan", "fixup", "d2h"):
        assert k in names, (k, names)
    assert n == len(marks)


def test_signed_zero_and_infinite_weights(jx, O):
    """Weights of both signs over seven decades, signed zeros and a few infinities: the engine
    reproduces the reference's order bit for bit (J = NaN compared as NaN)."""
    rp, col = jx.graphgen.rmat(16, 16, 0.57, 0.19, 0.19, seed=51)
    n = len(rp) - 1
    rng = np.random.default_rng(52)
    w = (rng.standard_normal(n) * 10.0 ** rng.integers(-3, 4, n)).astype(np.float32)
    w[rng.random(n) < 0.05] = 0.0
    w[rng.random(n) < 0.05] = -0.0
    deg1 = np.flatnonzero(np.diff(rp) == 1)  # infinities on a few leaves, so most J stay finite
    w[deg1[:3]] = np.inf
    w[deg1[3:5]] = -np.inf
    got = run(jx, rp, col, w)
    want = O.jaccard(rp, col, w)
    gn, wn = np.isnan(got), np.isnan(want)
    assert np.array_equal(gn, wn)
    assert_bitwise(got[~gn], want[~wn], "special weights")


SCHEDULES = [
    {"persistent": 1},
    {"hub_beside": 1},
    {"hub_cluster": 4, "cta_max": 4096, "hub_unit": 1000},
    {"persistent": 1, "hub_beside": 1, "lane_max": 16, "warp_max": 128, "cta_max": 2048, "hub_unit": 700,
     "hub_batch": 8},
    {"persistent": 0, "hub_beside": -1, "lane_max": 8, "warp_max": 64, "cta_max": 1024, "hub_unit": 300,
     "hub_batch": 1},
    {"persistent": 1, "hub_beside": 1, "hub_cluster": 4, "lane_max": 1, "warp_max": 1, "cta_max": 1},  # all hub rows
    {"relabel": 1},  # vertex ids renumbered by degree
    {"relabel": 1, "persistent": 1, "hub_cluster": 8, "cta_max": 4096, "hub_unit": 1000},
]


@pytest.mark.parametrize("sch", SCHEDULES, ids=[f"sch{i}" for i in range(len(SCHEDULES))])
@pytest.mark.parametrize("mode", ["ec", "vc", "vcw"])
def test_schedules_match_oracle(jx, O, sch, mode):
    """Every launch schedule -- the persistent row kernel, the hub kernel beside or before the
    rows, bin limits that move rows between the lane, warp, CTA and hub paths, and vertex ids
    renumbered by degree -- gives the oracle's results bit for bit, on a skewed graph and on one
    with repeated neighbours."""
    import torch
    rng = np.random.default_rng(5)
    graphs = [jx.graphgen.rmat(14, 16, 0.57, 0.19, 0.19, seed=77)]
    hubby = csr_from_edges(30000, [(0, i) for i in range(1, 26000)] + [(1, i) for i in range(2, 600)] +
                           [(int(a), int(b)) for a, b in rng.integers(2, 30000, (60000, 2)) if a != b])
    graphs.append(with_repeats(*hubby, rows_every=7, both_ways=True))
    if sch.get("cta_max") == 1:
        graphs = [jx.graphgen.rmat(10, 8, seed=78)]
    for rp, col in graphs:
        w = jx.graphgen.uniform_weights(len(rp) - 1, seed=79) if mode == "vcw" else None
        g = jx.GraphCSRView.from_numpy(rp, col)
        got = jx.jaccard(g, None if w is None else torch.from_numpy(w).cuda(), edge_centric=(mode == "ec"),
                         schedule=sch).cpu().numpy()
        assert_bitwise(got, O.jaccard(rp, col, w, edge_centric=(mode == "ec")), f"{sch} {mode}")
