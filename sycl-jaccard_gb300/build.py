"""Build the engine's native libraries in-tree.

* ``csrc/libjx.so``       -- the CUDA engine (all ``csrc/*.cu``), sm_103a only.
* ``csrc/gen/libjxgen.so`` -- host code: the synthetic-graph generator (C++/OpenMP) and the
  binary CSR file reader/writer (``include/jx_io.h``).

nvcc cross-compiles without a GPU, so this runs on a CPU-only build machine as well as on
the GPU machine.  Translation units compile in parallel; the link is a single nvcc call.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
LIBJX = os.path.join(CSRC, "libjx.so")
LIBGEN = os.path.join(CSRC, "gen", "libjxgen.so")
BUILD_DIR = os.path.join(CSRC, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# IEEE division and no FMA contraction: results must match the reference bit for bit.
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(out, inputs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(i) > t for i in inputs)


def build_engine(force: bool = False, verbose: bool = False) -> str:
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                  glob.glob(os.path.join(ROOT, "include", "*.h")))
    if not force and not _stale(LIBJX, srcs + hdrs):
        return LIBJX
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        out = _run([nvcc, *ARCH, *NVCC_FLAGS, "-Xptxas", "-v" if verbose else "-O3", "-c", src, "-o", obj])
        return obj, out

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        for obj, out in ex.map(compile_one, srcs):
            objs.append(obj)
            if verbose:
                print(out)
    tmp = LIBJX + ".tmp"
    _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIBJX)
    return LIBJX


def build_generator(force: bool = False) -> str:
    srcs = [os.path.join(CSRC, "gen", "jxgen.cpp"), os.path.join(CSRC, "gen", "jxio.cpp")]
    deps = srcs + [os.path.join(CSRC, "jx_rng.h"), os.path.join(ROOT, "include", "jx_io.h")]
    if force or _stale(LIBGEN, deps):
        tmp = LIBGEN + ".tmp"
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", tmp, *srcs])
        os.replace(tmp, LIBGEN)
    return LIBGEN


def build(force: bool = False, verbose: bool = False) -> None:
    build_generator(force)
    build_engine(force, verbose)


if __name__ == "__main__":
    import sys
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIBJX)
    print(LIBGEN)
