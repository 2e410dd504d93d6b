"""Builds the native library shiro_gb300/libshiro_gpu.so in tree.

Every CUDA translation unit under shiro_gb300/csrc is compiled for sm_103a
only (``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked
with the static CUDA runtime.  The whole backend is compiled with
``-fmad=false`` (no contraction of multiply-adds, so results follow the
reference's float expressions) and host code with ``-ffp-contract=off`` (x86
and Arm hosts evaluate the importance tables identically).
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libshiro_gpu.so")
BACKEND_DIR = os.path.join(HERE, "backend")
BACKEND_LIB = os.path.join(HERE, "libshiro_backend.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-fno-strict-aliasing",
                  "--diag-suppress", "177"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps() -> list:
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + [
        os.path.join(ROOT, "include", "shiro_gpu.h")]


def _stale(target: str, sources: list) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def _run(cmd: list, verbose: bool):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd[:3])} ...")
    return r


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    # CUDA translation units and the host-only ones (the image reader)
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    deps = _deps()
    objs = []
    jobs = []
    for src in cu:
        obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + deps):
            jobs.append([nvcc()] + NVFLAGS + ["-c", src, "-o", obj])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs, verbose)
    return LIB


def build_backend(verbose: bool = False) -> str:
    """The C++ RenderBackend adapter (GpuBackend) over the C ABI, plus a small
    C entry point used by the tests to drive it."""
    srcs = sorted(glob.glob(os.path.join(BACKEND_DIR, "*.cpp")))
    if not srcs:
        return ""
    hdrs = glob.glob(os.path.join(BACKEND_DIR, "**", "*.h"), recursive=True)
    if _stale(BACKEND_LIB, srcs + hdrs + [LIB]):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", os.path.join(BACKEND_DIR, "include"),
              "-I", os.path.join(ROOT, "include"), "-o", BACKEND_LIB] + srcs +
             ["-L", HERE, "-lshiro_gpu", "-Wl,-rpath,$ORIGIN", "-pthread"], verbose)
    return BACKEND_LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
    print(build_backend(verbose=True))
