"""Compile tests/dropin/sygraph_driver.cpp with g++ against include/jx_sygraph.hpp and link it
with libjx.so and the CUDA runtime: a C++ caller of the drop-in header, as a user's program
would be built."""
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def build_driver(out_dir, libjx):
    cuda = cuda_home()
    exe = os.path.join(out_dir, "sygraph_driver")
    libdir = os.path.dirname(libjx)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(HERE, "sygraph_driver.cpp"), "-o", exe, "-L", libdir, "-ljx", "-L", os.path.join(cuda, "lib64"),
           "-lcudart", f"-Wl,-rpath,{libdir}:{os.path.join(cuda, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("g++ failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return exe
