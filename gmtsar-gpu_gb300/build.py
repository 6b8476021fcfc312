"""Build recipe of the package: the CUDA library, the xcorr program.

    python gmtsar-gpu_gb300/build.py            # library + program

Outputs (git-ignored, in-tree):
    gmtsar-gpu_gb300/lib/libxcorr_gb300.so   kernels + C ABI, sm_103a only
    gmtsar-gpu_gb300/bin/xcorr               the drop-in command-line program
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INC = os.path.join(ROOT, "include")
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIB_DIR = os.path.join(PKG, "lib")
BIN_DIR = os.path.join(PKG, "bin")
LIB = os.path.join(LIB_DIR, "libxcorr_gb300.so")
CLI = os.path.join(BIN_DIR, "xcorr")

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INC, "-I" + CSRC]
def _cuda_home():
    import shutil
    nv = shutil.which(NVCC) or NVCC
    home = os.environ.get("CUDA_HOME") or os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    return home


CU_SOURCES = ["xcorr_kernels.cu", "xcorr_api.cu", "xcorr_noalloc.cu", "xcorr_stack.cu", "refiner.cu", "refiner_api.cu", "fit_offsets.cu", "time_corr.cu", "tc_dft.cu", "peak_probe.cu", "segment_rows.cu"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_lib(force=False):
    os.makedirs(LIB_DIR, exist_ok=True)
    objdir = os.path.join(LIB_DIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INC, "xcorr_gb300.h"))
    objs, jobs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(objdir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([NVCC] + NVFLAGS + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(len(jobs)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_cli(force=False):
    os.makedirs(BIN_DIR, exist_ok=True)
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".c")) if os.path.isdir(HOST) else []
    if not srcs:
        return None
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] + [LIB]
    if force or _stale(CLI, deps):
        cuda = _cuda_home()
        culib = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"))
                      if os.path.isdir(d)), os.path.join(cuda, "lib64"))
        _run(["gcc", "-O2", "-std=gnu11", "-Wall", "-I" + INC, "-I" + HOST, "-I" + os.path.join(cuda, "include")] +
             srcs + ["-L" + LIB_DIR, "-lxcorr_gb300", "-Wl,-rpath,$ORIGIN/../lib", "-L" + culib, "-lcudart",
                     "-Wl,-rpath," + culib, "-lpthread", "-lm", "-o", CLI])
    return CLI


def build_all(force=False):
    build_lib(force)
    build_cli(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
