"""Builds the native library sw2d-gpu_gb300/_build/libsw2d.so for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library that exports the C ABI of include/sw2d.h.  The FP64 step
kernels are compiled with --fmad=false (bit-reproducible FP64 arithmetic),
the FP32 ones with --use_fast_math.

    python sw2d-gpu_gb300/build_native.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsw2d.so")
DRIVER = os.path.join(OUT_DIR, "sw2d_run")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-I", os.path.join(ROOT, "include"), "-I", CSRC]

UNITS = {
    "step_f64.cu": ["--fmad=false"],
    "step_f32.cu": ["--use_fast_math"],
    # the one device function here (the per-launch plan) must round like the
    # oracle: no contraction in device or host code
    "sw2d_api.cu": ["--fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "sw2d_noalloc.cu": ["--fmad=false"],
    # same flags as step_f32.cu: a batched scenario advances bit for bit as alone
    "sw2d_batch.cu": ["--use_fast_math"],
    # the serving loop over the batch: host C++ only
    "sw2d_serve.cpp": [],
}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsw2d.so")
    return exe


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "sw2d.h"), __file__]


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(DRIVER):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(DRIVER))
    return all(os.path.getmtime(p) <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()

    def compile_one(item):
        src, flags = item
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [cc, *ARCH, *COMMON, *flags, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS.items()))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    # the reference-format host driver: plain C++ on top of the C ABI
    cxx = shutil.which("g++") or "g++"
    # no FMA contraction (gcc contracts by default where the target has FMA,
    # as the Arm hosts do): the driver's host arithmetic rounds the same on
    # every machine
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           os.path.join(CSRC, "sw2d_driver.cpp"), "-o", DRIVER + ".tmp", "-L", OUT_DIR, "-lsw2d",
           "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(DRIVER + ".tmp", DRIVER)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
