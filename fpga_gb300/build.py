"""Builds libgbilu.so in-tree with nvcc for sm_103a (no torch involved).

The library is compiled from fpga_gb300/csrc/ into fpga_gb300/_lib/: the host
analysis (gbilu_host.cpp) and the CUDA kernels + C ABI (gbilu_api.cu) are
compiled in parallel and linked with -shared. Host code is compiled with
-ffp-contract=off so its floating-point results (the ILU0 factors) are the
same on x86-64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(LIBDIR, "libgbilu.so")
SOURCES = ["gbilu_host.cpp", "gbilu_api.cu", "gbilu_noalloc.cu", "gbilu_fpga_compat.cpp",
           "gbilu_fpga_export.cpp", "gbilu_color.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbilu.so")


def _flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]


def _sources_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "gbilu.h"))
    return max(os.path.getmtime(f) for f in files)


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compiles libgbilu.so if it is missing or older than its sources."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + _flags() + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        return obj

    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))
