"""Builds libclotho_gpu.so (the C-ABI of include/clotho_gpu.h) in-tree.

nvcc compiles each CUDA translation unit for sm_103a in parallel, then links
one shared library next to this file (clotho_gb300/_lib/).  No cmake, no
torch extension machinery: the library has a plain C ABI.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libclotho_gpu.so")
DRIVER_PATH = os.path.join(OUT_DIR, "qtlsim_gb300")
CPP_DIR = os.path.join(HERE, "cpp")
SOURCES = ["capi.cu", "k_freespace.cu", "k_step.cu", "k_generation.cu", "k_noalloc.cu", "k_analysis.cu"]
HEADERS = ["engine.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libclotho_gpu.so")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    nv = nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "clotho_gpu.h")]
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nv, *ARCH, *NVCC_FLAGS, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)

    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB_PATH, objs):
        run([nv, *ARCH, "-shared", "-cudart", "static", "-o", LIB_PATH, *objs])
    # C++ driver over the policy adapters (host code only, linked to the library)
    drv_src = [os.path.join(CPP_DIR, "qtlsim_gb300.cpp"), os.path.join(CPP_DIR, "clotho_gb300.hpp")]
    if force or _stale(DRIVER_PATH, drv_src + [LIB_PATH]):
        cxx = os.environ.get("CXX", "g++")
        run([cxx, "-O2", "-std=c++17", drv_src[0], "-o", DRIVER_PATH, "-L", OUT_DIR, "-lclotho_gpu",
             "-Wl,-rpath,$ORIGIN"])
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
