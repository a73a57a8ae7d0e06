"""CPU: the binary CSR format (version 2) and the reference program's result post-processing against
the reference's own code (readMtxToCSR.cpp, through the host SYCL subset)."""
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def graph(jx):
    rp, col = jx.graphgen.rmat(11, 8, seed=13)
    w = jx.graphgen.uniform_weights(len(col), seed=14)  # per-edge weights for the file
    return rp, col, w


def test_csr_roundtrip(jx, tmp_path, graph):
    rp, col, w = graph
    p = str(tmp_path / "g.csr")
    jx.csrfile.write_csr(p, rp, col, w)
    r2, c2, w2, fl = jx.csrfile.read_csr(p)
    assert np.array_equal(r2, rp) and np.array_equal(c2, col) and np.array_equal(w2, w)
    assert fl == (jx.csrfile.WEIGHTED | jx.csrfile.ZERO_INDEXED | jx.csrfile.REVERSE_EDGES)
    assert os.path.getsize(p) == 32 + 4 * (len(rp) + 2 * len(col))
    jx.csrfile.write_csr(p, rp, col, None, flags=jx.csrfile.DIRECTED)
    r3, c3, w3, fl3 = jx.csrfile.read_csr(p)
    assert w3 is None and fl3 == jx.csrfile.DIRECTED and np.array_equal(c3, col)


def test_csr_matches_reference_files(jx, O, tmp_path, graph):
    if O.ref_lib() is None:
        pytest.skip("reference sources unavailable")
    rp, col, w = graph
    ours, theirs = str(tmp_path / "ours.csr"), str(tmp_path / "theirs.csr")
    jx.csrfile.write_csr(ours, rp, col, w)
    O.ref_csr_write(theirs, rp, col, w, zero_indexed=True, directed=False, reverse_edges=True)
    assert open(ours, "rb").read() == open(theirs, "rb").read()
    # the reference reads our file, we read the reference's
    r2, c2, w2, fl = O.ref_csr_read(ours)
    assert np.array_equal(r2, rp) and np.array_equal(c2, col) and np.array_equal(w2, w)
    r3, c3, w3, fl3 = jx.csrfile.read_csr(theirs)
    assert np.array_equal(r3, rp) and np.array_equal(c3, col) and np.array_equal(w3, w)


def test_csr_errors(jx, tmp_path):
    p = str(tmp_path / "bad.csr")
    open(p, "wb").write(b"\x01" + b"\x00" * 40)
    with pytest.raises(OSError):
        jx.csrfile.read_csr(p)
    with pytest.raises(OSError):
        jx.csrfile.read_csr(str(tmp_path / "missing.csr"))


def remove_reverse_restated(rp, col, v):
    """Survivors of main.cpp:307-309 / readMtxToCSR.cpp:134-147 in CSR order."""
    n = len(rp) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp))
    lookup = {(int(a), int(b)): float(x) for a, b, x in zip(src, col, v)}
    keep = []
    for a, b, x in zip(src, col, v):
        a, b = int(a), int(b)
        if a > b:
            keep.append(True)
        elif a == b:
            keep.append(False)
        else:
            y = lookup.get((b, a))
            keep.append(not (y is not None and (y == x or np.isnan(x) or np.isnan(y))))
    keep = np.array(keep, bool)
    return src[keep].astype(np.int32), col[keep], v[keep]


def test_remove_reverse_restatement_matches_reference(jx, O):
    if O.ref_lib() is None:
        pytest.skip("reference sources unavailable")
    rp, col = jx.graphgen.rmat(9, 8, seed=3)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=5)
    J = O.jaccard(rp, col, w)  # weighted VC: ties may make J(u,v) != J(v,u)
    J[::97] = np.float32(0.5)  # break some symmetric pairs
    a = remove_reverse_restated(rp, col, J)
    b = O.ref_remove_reverse(rp, col, J)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_pair_list_oracle_consistent(jx, O):
    rp, col = jx.graphgen.rmat(10, 8, seed=21)
    w = jx.graphgen.uniform_weights(len(rp) - 1, seed=22)
    n = len(rp) - 1
    src = np.repeat(np.arange(n, dtype=np.int32), np.diff(rp))
    for ww in (None, w):
        # pairs equal to the stored edges give the vertex-centric result
        assert np.array_equal(O.jaccard_list(rp, col, src, col, ww).view(np.uint32),
                              O.jaccard(rp, col, ww).view(np.uint32))
