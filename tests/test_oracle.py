"""CPU: the oracle restatement is pinned to the reference's own outputs.

Golden vectors (tests/golden/*.npz) were produced by the reference's jaccard.cpp compiled
unmodified against the host SYCL subset (tests/golden/make_golden.py).  The oracle must
reproduce them bit for bit, and must equal the live reference build whenever its sources
are available.
"""
import glob
import os

import numpy as np
import pytest

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module", params=GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def golden(request):
    return dict(np.load(request.param))


def test_generator_reproduces_fixture_graph(golden, jx):
    rp, col = golden["row_ptr"], golden["col_idx"]
    name = str(golden["desc"])
    if name.startswith("ER"):
        grp, gcol = jx.graphgen.er_gnp(4096, 16.0 / 4095.0, seed=1)
    else:
        grp, gcol = jx.graphgen.rmat(11, 16, 0.57, 0.19, 0.19, seed=7)
    assert np.array_equal(grp, rp) and np.array_equal(gcol, col)


@pytest.mark.parametrize("mode", ["J_ec", "J_vc", "J_vcw"])
def test_oracle_matches_golden(golden, O, mode):
    rp, col, w = golden["row_ptr"], golden["col_idx"], golden["w"]
    out = O.jaccard(rp, col, w if mode == "J_vcw" else None, edge_centric=(mode == "J_ec"))
    assert np.array_equal(bits(out), bits(golden[mode]))


def test_oracle_stages_match_golden(golden, O):
    rp, col, w = golden["row_ptr"], golden["col_idx"], golden["w"]
    S = O.rowsum(rp, col, w)
    assert np.array_equal(bits(S), bits(golden["S_w"]))
    assert np.array_equal(bits(O.rowsum(rp, col, None)), bits(golden["S_u"]))
    wi = np.zeros(len(col), np.float32)
    ws = O.intersect(rp, col, w, S, wi)
    assert np.array_equal(bits(wi), bits(golden["Wi_w"]))
    assert np.array_equal(bits(ws), bits(golden["Ws_w"]))
    assert np.array_equal(bits(O.weight(wi, ws)), bits(golden["J_vcw"]))


def test_golden_has_teeth(golden, O):
    """The weighted order matters: a natural-order sum differs somewhere (RMAT fixture)."""
    if "RMAT" not in str(golden["desc"]):
        pytest.skip("only the skewed fixture has long weighted intersections")
    rp, col, w = golden["row_ptr"], golden["col_idx"], golden["w"]
    J64 = O.jaccard_f64(rp, col, w)
    assert np.any(golden["J_vcw"].astype(np.float64) != J64.astype(np.float32).astype(np.float64))


@pytest.mark.parametrize("ec", [False, True])
@pytest.mark.parametrize("weighted", [False, True])
def test_oracle_equals_live_reference(O, jx, ec, weighted):
    if O.ref_lib() is None:
        pytest.skip("reference sources unavailable on this machine")
    rp, col = jx.graphgen.rmat(12, 16, 0.57, 0.19, 0.19, seed=11)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=12) if weighted else None
    r = O.ref_jaccard(rp, col, w, edge_centric=ec)
    o = O.jaccard(rp, col, w, edge_centric=ec)
    assert np.array_equal(bits(r), bits(o))


def test_reference_ec_stages(O, jx):
    if O.ref_lib() is None:
        pytest.skip("reference sources unavailable on this machine")
    rp, col = jx.graphgen.rmat(10, 8, seed=3)
    dest, wj = O.ref_ec_scan(rp, len(col))
    assert np.array_equal(dest, np.repeat(np.arange(len(rp) - 1, dtype=np.int32), np.diff(rp)))
    assert not np.any(wj)
    O.ref_ec_unweighted(rp, col, dest, wj)
    assert np.array_equal(bits(wj), bits(O.jaccard(rp, col, None, edge_centric=True)))


def test_oracle_row_subset(O, jx):
    rp, col = jx.graphgen.rmat(11, 16, seed=5)
    full = O.jaccard(rp, col, None)
    r0, r1 = 100, 700
    part = O.jaccard(rp, col, None, rows=(r0, r1))
    assert np.array_equal(bits(part), bits(full[rp[r0]:rp[r1]]))
    c = O.counts(rp, col)
    d = np.diff(rp)
    src = np.repeat(np.arange(len(d)), d)
    expect = (c / ((d[src] + d[col]) - c)).astype(np.float32)
    assert np.array_equal(bits(expect), bits(full))
