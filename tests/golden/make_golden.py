"""Generate the committed golden vectors from the reference itself.

Runs the reference's own ``jaccard.cpp`` (vtsynergy/SYCL-Jaccard), compiled unmodified
against the host SYCL subset (``oracle/syclshim``, built by ``oracle/build_ref.py``), on
small synthetic graphs and stores inputs and outputs in ``tests/golden/*.npz``.  Needs the
reference sources: a checkout named by ``JX_REFERENCE_DIR``, or the ``baseline/_ref/src`` copy
that ``oracle/build_ref.py --install`` makes; the GPU machine only reads the committed
``.npz`` files.

    JX_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

jx = importlib.import_module("sycl-jaccard_gb300")
gg = jx.graphgen


def csr_digest(rp, col):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rp, np.int32).tobytes())
    h.update(np.ascontiguousarray(col, np.int32).tobytes())
    return h.hexdigest()


def outputs(rp, col, w):
    e = len(col)
    out = {}
    out["J_ec"] = O.ref_jaccard(rp, col, None, edge_centric=True)
    out["J_vc"] = O.ref_jaccard(rp, col, None, edge_centric=False)
    out["J_vcw"] = O.ref_jaccard(rp, col, w, edge_centric=False)
    # stage level (kernel-level invoke calls, as main.cpp:255-257 drives them)
    out["S_w"] = O.ref_rowsum(rp, col, w)
    out["S_u"] = O.ref_rowsum(rp, col, None)
    wi = np.zeros(e, np.float32)
    out["Ws_w"] = O.ref_intersect(rp, col, w, out["S_w"], wi)
    out["Wi_w"] = wi
    dest, wj = O.ref_ec_scan(rp, e)
    out["dest_ind"] = dest
    return out


def make(name, rp, col, w, desc):
    o = outputs(rp, col, w)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, row_ptr=rp, col_idx=col, w=w, desc=np.array(desc),
                        digest=np.array(csr_digest(rp, col)), **o)
    print(f"{path}: V={len(rp) - 1} E={len(col)} {os.path.getsize(path) / 1024:.0f} KiB")


def main():
    if O.ref_lib() is None:
        raise SystemExit("reference sources unavailable: cannot regenerate golden vectors")
    # The small plain configuration: ER G(4096, 16/4095), seed 1.  The weighted outputs use
    # U(0,1] vertex weights (seed 4) so the accumulation order is exercised; with the
    # configuration's unit weights the weighted result equals the unweighted one.
    rp, col = gg.er_gnp(4096, 16.0 / 4095.0, seed=1)
    make("er4096_seed1", rp, col, gg.uniform_weights(4096, seed=4), "ER G(4096,16/4095) seed 1; w seed 4")
    # A skewed graph with hubs and long intersections: RMAT scale 11, edge factor 16, seed 7.
    rp, col = gg.rmat(11, 16, 0.57, 0.19, 0.19, seed=7)
    make("rmat11_seed7", rp, col, gg.uniform_weights(len(rp) - 1, seed=8), "RMAT(11,16) seed 7; w seed 8")


if __name__ == "__main__":
    main()
