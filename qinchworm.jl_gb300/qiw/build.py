"""Builds libqiw.so in-tree for sm_103a (nvcc, one -gencode, translation units in parallel)."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # qinchworm.jl_gb300/
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libqiw.so")
INCLUDE = os.path.join(REPO, "include")

SOURCES = ["qiw_kernels.cu", "qiw_kernels_x.cu", "qiw_batch_kernels.cu", "qiw_api.cu", "qiw_noalloc.cu",
           "qiw_warp.cu", "qiw_batch.cu", "qiw_plan.cpp"]
HEADERS = ["qiw_internal.hpp", "qiw_kernels.hpp", "qiw_plan.hpp", "qiw_ctx.hpp", "qiw_eval.cuh", "qiw_dispatch.hpp"]
PLAN_LIB = os.path.join(BUILD, "libqiw_plan_host.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS] + [os.path.join(INCLUDE, "qiw.h")]
    return any(os.path.getmtime(p) > t for p in deps)


def build_plan_host(force: bool = False) -> str:
    """Host-only planner library (g++, no CUDA) used by the CPU tests of the planner."""
    srcs = [os.path.join(CSRC, "qiw_plan.cpp"), os.path.join(CSRC, "qiw_plan_capi.cpp")]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "qiw.h")]
    if not force and os.path.exists(PLAN_LIB) and all(os.path.getmtime(d) <= os.path.getmtime(PLAN_LIB) for d in deps):
        return PLAN_LIB
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", INCLUDE, "-I", CSRC, "-o", PLAN_LIB + ".tmp"] + srcs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"g++ failed for the host planner:\n{r.stdout}\n{r.stderr}")
    os.replace(PLAN_LIB + ".tmp", PLAN_LIB)
    return PLAN_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [cc] + common + ARCH + ["-lineinfo", "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared"] + ARCH + ["-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_plan_host(force="--force" in sys.argv))
