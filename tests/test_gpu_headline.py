"""GPU: the headline configuration checked against the oracle bit for bit.

R-MAT scale 24, edge factor 16, (a,b,c,d) = (.57,.19,.19,.05), seed 3, vertex weights U(0,1]
seed 4 (V = 16,777,216, E = 520,759,968): the graph every headline number is measured on.
The whole output is far too large for the oracle, so it is compared on sampled row ranges
(oracle.check_rows): the five largest hubs -- rows of up to 406,291 neighbours whose tasks are
split into hub work units (of 65,536 tasks on this graph) and whose hub-to-hub intersections of more than
65,536 matches overflow the 8,192-entry class streams and resume from the adjacency list --,
the row of degree nearest 21,000 (a CTA row whose hash table leaves no room for slot weights),
a band of 2,000 rows in the middle of the id range and the last 3,000 rows.  Weighted VC,
unweighted VC and EC, the reference computations of jaccard.cpp:315-400, 607-620 and 703-743.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def headline(jx):
    import torch
    rp, col, w, _ = jx.graphgen.config_graph("rmat24w")
    g = jx.GraphCSRView.from_numpy(rp, col)
    wd = torch.from_numpy(w).cuda()
    return rp, col, w, g, wd


def test_headline_exercises_hub_units_and_overflow(O, headline):
    """The sampled hubs reach the paths the small test graphs never do."""
    rp, col = headline[0], headline[1]
    d = np.diff(rp.astype(np.int64))
    ranges = O.check_rows(rp)
    hub0 = ranges[0][1]
    assert d[hub0] > 65536  # more tasks than one hub work unit
    c = O.counts(rp, col, rows=(hub0, hub0 + 1))
    assert c.max() > 8 * 8192  # some class of that task holds more than a hub class stream
    cta = ranges[5][1]
    assert 10700 < d[cta] <= 24576  # a CTA-bin row too large for slot weights


@pytest.mark.parametrize("mode", ["vcw", "vc", "ec"])
def test_headline_sampled_rows(jx, O, headline, mode):
    import torch
    rp, col, w, g, wd = headline
    ww = w if mode == "vcw" else None
    out = jx.jaccard(g, wd if mode == "vcw" else None, edge_centric=(mode == "ec"))
    torch.cuda.synchronize()
    got = bits(out.cpu().numpy())
    del out
    S = O.rowsum(rp, col, w) if mode == "vcw" else None
    for name, r0, r1 in O.check_rows(rp):
        if S is not None:
            want = O.jaccard_rows_with_sums(rp, col, ww, S, (r0, r1))
        else:
            want = O.jaccard(rp, col, None, edge_centric=(mode == "ec"), rows=(r0, r1))
        lo, hi = int(rp[r0]), int(rp[r1])
        bad = np.flatnonzero(got[lo:hi] != bits(want))
        assert bad.size == 0, f"{mode} {name}: {bad.size} of {hi - lo} differ, first at edge {lo + bad[:5]}"
