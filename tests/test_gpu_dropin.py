"""GPU: the C++ drop-in boundary end to end.  A C++ program built with g++ against
include/jx_sygraph.hpp and linked with libjx.so makes the reference driver's hot-path calls
(main.cpp:205-282: EC, row sums of the edge data over pseudo indices as vertex weights,
weighted VC, unweighted VC), then drives the stage kernels as detail::jaccard does
(jaccard.cpp:784-897) and takes one error path; every result is compared bit for bit with the
oracle driven the same way."""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "dropin"))

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_cpp_dropin_replays_reference_driver(jx, O, tmp_path):
    import driver_build
    exe = driver_build.build_driver(str(tmp_path), jx._build.LIBJX)
    rp, col = jx.graphgen.rmat(13, 16, 0.57, 0.19, 0.19, seed=61)
    n, e = len(rp) - 1, len(col)
    rng = np.random.default_rng(62)
    edge_data = rng.uniform(0.01, 1.0, e).astype(np.float32)
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array([n, e], np.int32).tofile(f)
        rp.astype(np.int32).tofile(f)
        col.astype(np.int32).tofile(f)
        edge_data.tofile(f)
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "jx error during VC Jaccard" in r.stderr  # the error call was reported, not fatal
    raw = np.fromfile(outp, np.float32)
    parts = {}
    off = 0
    for name, size in (("ec", e), ("vw", n), ("vcw", e), ("vc", e), ("stages_vcw", e), ("stages_ec", e)):
        parts[name] = raw[off:off + size]
        off += size
    st_err, st_next = raw[off:off + 2].view(np.int32)
    assert st_err == 1 and st_next == 0  # JX_ERR_INVALID, then JX_OK
    # the oracle driven as main.cpp drives the reference
    vw = O.rowsum(rp, np.arange(e, dtype=np.int32), edge_data)
    assert np.array_equal(bits(parts["vw"]), bits(vw))
    want_ec = O.jaccard(rp, col, None, edge_centric=True)
    want_vcw = O.jaccard(rp, col, vw)
    assert np.array_equal(bits(parts["ec"]), bits(want_ec))
    assert np.array_equal(bits(parts["vcw"]), bits(want_vcw))
    assert np.array_equal(bits(parts["vc"]), bits(O.jaccard(rp, col, None)))
    assert np.array_equal(bits(parts["stages_vcw"]), bits(want_vcw))
    assert np.array_equal(bits(parts["stages_ec"]), bits(want_ec))
