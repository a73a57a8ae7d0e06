"""Build recipe for the oracle side -- TEST INFRASTRUCTURE ONLY.

Builds two host libraries with gcc/g++ (no GPU, no cmake):

* ``oracle/libjxoracle.so`` -- the plain-C restatement of the reference algorithm
  (``oracle/jx_oracle.c``).
* ``oracle/_ref/libjxref.so`` -- the reference's own ``jaccard.cpp`` compiled unmodified
  against the host SYCL subset in ``oracle/syclshim`` (``oracle/ref_driver.cpp`` includes it).

The reference sources are read from the directory given by ``--reference-dir`` or the
environment variable ``JX_REFERENCE_DIR`` (a checkout of vtsynergy/SYCL-Jaccard, read-only),
else from the git-ignored copy in ``baseline/_ref/src`` that ``--install`` makes from such a
checkout; that copy is what machines without a checkout build from.
Only the files the path and its data formats need are used: jaccard.cpp, jaccard.hpp,
standalone_algorithms.hpp, standalone_csr.hpp, and the CSR/MTX I/O of readMtxToCSR.cpp/.hpp
and filetypes.cpp/.hpp.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
REF_COPY = os.path.join(ROOT, "baseline", "_ref", "src")
REF_FILES = ["jaccard.cpp", "jaccard.hpp", "standalone_algorithms.hpp", "standalone_csr.hpp",
             "readMtxToCSR.cpp", "readMtxToCSR.hpp", "filetypes.cpp", "filetypes.hpp"]
ORACLE_SO = os.path.join(HERE, "libjxoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libjxref.so")
# The reference's shipped configuration (Makefile:33, Makefile:387, ICX flags Makefile:74).
REF_DEFINES = ["-DSTANDALONE", "-DSYCL_1_2_1", "-DDISABLE_DP_WEIGHT", "-DDISABLE_LIST",
               "-DDISABLE_DP_INDEX"]


def _has_sources(d: str | None) -> bool:
    return bool(d) and all(os.path.isfile(os.path.join(d, f)) for f in REF_FILES)


def ref_source_dir(reference_dir: str | None = None) -> str | None:
    """The first of: reference_dir, $JX_REFERENCE_DIR, baseline/_ref/src that holds the files."""
    for d in (reference_dir, os.environ.get("JX_REFERENCE_DIR"), REF_COPY):
        if _has_sources(d):
            return d
    return None


def install_copy(reference_dir: str) -> str:
    """Copy the hot-path sources of the reference checkout into the git-ignored
    baseline/_ref/src."""
    if not _has_sources(reference_dir):
        raise FileNotFoundError(f"no reference sources ({', '.join(REF_FILES)}) in {reference_dir!r}")
    os.makedirs(REF_COPY, exist_ok=True)
    for f in REF_FILES:
        shutil.copy2(os.path.join(reference_dir, f), os.path.join(REF_COPY, f))
    return REF_COPY


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: str, inputs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in inputs if os.path.exists(i))


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "jx_oracle.c")
    if force or _stale(ORACLE_SO, [src]):
        _run(["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-o", ORACLE_SO, src, "-lm"])
    return ORACLE_SO


def build_ref(force: bool = False, reference_dir: str | None = None) -> str | None:
    d = ref_source_dir(reference_dir)
    if d is None:
        return None
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(HERE, "syclshim", "syclshim.cpp"),
            os.path.join(d, "readMtxToCSR.cpp"), os.path.join(d, "filetypes.cpp")]
    deps = srcs + [os.path.join(HERE, "syclshim", "CL", "sycl.hpp")] + [os.path.join(d, f) for f in REF_FILES]
    if force or _stale(REF_SO, deps):
        _run(["g++", "-O3", "-std=c++20", "-fopenmp", "-fPIC", "-shared", "-w",
              "-U_FORTIFY_SOURCE", "-D_FORTIFY_SOURCE=0",
              "-I", os.path.join(HERE, "syclshim"), "-I", d, *REF_DEFINES,
              "-o", REF_SO, *srcs])
    return REF_SO


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-dir", default=os.environ.get("JX_REFERENCE_DIR"),
                    help="a checkout of the reference (default: $JX_REFERENCE_DIR)")
    ap.add_argument("--install", action="store_true",
                    help="copy the reference's hot-path sources from --reference-dir into baseline/_ref/src")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    if a.install:
        print("copied reference sources to", install_copy(a.reference_dir))
    print("oracle:", build_oracle(a.force))
    print("reference:", build_ref(a.force, a.reference_dir) or "unavailable (no reference sources)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
