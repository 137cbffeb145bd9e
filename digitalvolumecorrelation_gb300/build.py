"""Build libdvcgpu.so (CUDA, sm_103a) and the drop-in host programs.

    python -m digitalvolumecorrelation_gb300.build

Outputs (git-ignored, rebuilt on each machine):
    digitalvolumecorrelation_gb300/lib/libdvcgpu.so
    digitalvolumecorrelation_gb300/bin/dvc, .../bin/strain
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(CSRC, "host")
LIB_DIR = os.path.join(PKG, "lib")
BIN_DIR = os.path.join(PKG, "bin")
OBJ_DIR = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(LIB_DIR, "libdvcgpu.so")

CUDA_SOURCES = ["dvc_engine.cu", "dvc_strain.cu", "dvc_synth.cu", "dvc_cnn.cu", "dvc_knn.cu", "dvc_io.cu"]
# the strain fit follows the FP64 oracle operation by operation: no FMA
# contraction, so its results are bit-identical to the oracle's
EXTRA_FLAGS = {"dvc_strain.cu": ["-fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-diag-suppress", "128", "-I", os.path.join(ROOT, "include")]
HOST_SOURCES = ["input_read.cpp", "data_cloud.cpp"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build_library(force=False, verbose=False):
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "dvc_gpu.h"))
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + EXTRA_FLAGS.get(src, []) + ["-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=len(CUDA_SOURCES)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and r.stderr:
                print(r.stderr, file=sys.stderr)
    if force or jobs or not _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_host(force=False):
    """The drop-in `dvc` and `strain` programs (C++17 host code over the C ABI)."""
    os.makedirs(BIN_DIR, exist_ok=True)
    common = [os.path.join(HOST, s) for s in HOST_SOURCES]
    headers = [os.path.join(HOST, h) for h in os.listdir(HOST) if h.endswith(".h")]
    headers.append(os.path.join(ROOT, "include", "dvc_gpu.h"))
    cxx = os.environ.get("CXX", "g++")
    # -ffp-contract=off: the neighbour distances are formed as in the
    # reference, without fused multiply-adds (ties must compare the same)
    flags = ["-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
             "-I", HOST]
    link = ["-L", LIB_DIR, "-ldvcgpu", "-Wl,-rpath,$ORIGIN/../lib"]
    jobs = []
    for prog in ("dvc", "strain"):
        main = os.path.join(HOST, f"{prog}_main.cpp")
        out = os.path.join(BIN_DIR, prog)
        if force or not _newer(out, [main] + common + headers + [LIB]):
            jobs.append([cxx] + flags + [main] + common + ["-o", out] + link)
    with ThreadPoolExecutor(max_workers=2) as ex:
        list(ex.map(_run, jobs))
    return BIN_DIR


def build(force=False):
    build_library(force=force)
    if os.path.isdir(HOST):
        build_host(force=force)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
