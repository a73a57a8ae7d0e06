"""CPU: the CSR-building restatement in the oracle against the reference's own graph
preparation (MTX set, invertDirection, mtxSetToCSR) run through the host SYCL subset."""
import numpy as np
import pytest


def edge_list(n, m, seed):
    rng = np.random.default_rng(seed)
    src = rng.integers(0, n, m).astype(np.int32)
    dst = rng.integers(0, n, m).astype(np.int32)
    # duplicates, both directions, self loops; and an edge (0, n-1) so that the reference's
    # rows (first source .. last source) cover every vertex
    src = np.concatenate([src, src[:m // 4], dst[:m // 8], np.arange(5, dtype=np.int32), [0]]).astype(np.int32)
    dst = np.concatenate([dst, dst[:m // 4], src[:m // 8], np.arange(5, dtype=np.int32), [n - 1]]).astype(np.int32)
    return src, dst


@pytest.mark.parametrize("keep_self", [False, True])
@pytest.mark.parametrize("seed", [1, 2])
def test_restatement_equals_reference(O, keep_self, seed):
    if O.ref_lib() is None:
        pytest.skip("reference sources unavailable on this machine")
    n = 500
    src, dst = edge_list(n, 3000, seed)
    rp_ref, col_ref = O.ref_csr_from_edges(src, dst, symmetrize=True, keep_self=keep_self)
    rp, col = O.csr_build(n, src, dst, symmetrize=True, keep_self=keep_self)
    assert np.array_equal(rp, rp_ref) and np.array_equal(col, col_ref)


def test_restatement_directed(O):
    if O.ref_lib() is None:
        pytest.skip("reference sources unavailable on this machine")
    n = 300
    src, dst = edge_list(n, 2000, 3)
    # the reference keeps rows from the first to the last source only: give every vertex an
    # outgoing edge so both sides have n rows
    src = np.concatenate([src, np.arange(n, dtype=np.int32)])
    dst = np.concatenate([dst, (np.arange(n, dtype=np.int32) + 1) % n])
    rp_ref, col_ref = O.ref_csr_from_edges(src, dst, symmetrize=False)
    rp, col = O.csr_build(n, src, dst, symmetrize=False)
    assert np.array_equal(rp, rp_ref) and np.array_equal(col, col_ref)
