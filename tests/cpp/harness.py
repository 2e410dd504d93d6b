"""Builds the C++ adapter harness (tests/cpp/backend_harness.cpp) into
tests/cpp/_build/libshiro_backend_harness.so.

TEST AND MEASUREMENT INFRASTRUCTURE: the harness drives the product's C++
adapter (shiro::backend::gb300::GpuBackend in shiro_gb300/libshiro_backend.so)
the way Shiro's Renderer does, for the adapter tests and for bench.py's
end-to-end timing through the adapter.  It is not part of the product
library.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libshiro_backend_harness.so")
SRC = os.path.join(HERE, "backend_harness.cpp")

_P = C.c_void_p
_U = C.c_uint32


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources if os.path.exists(s))


def build_harness() -> str:
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from shiro_gb300 import build

    build.build()
    backend = build.build_backend()
    pkg = os.path.dirname(backend)
    inc = os.path.join(pkg, "backend", "include")
    hdrs = [os.path.join(pkg, "backend", "GpuBackend.h")]
    if _stale(LIB, [SRC, backend] + hdrs):
        os.makedirs(BUILD, exist_ok=True)
        cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
               "-I", inc, "-I", os.path.join(pkg, "backend"), "-I", os.path.join(ROOT, "include"),
               "-o", LIB, SRC, "-L", pkg, "-lshiro_backend", "-lshiro_gpu", f"-Wl,-rpath,{pkg}", "-pthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("harness build failed:\n" + r.stdout + r.stderr)
    return LIB


def load_harness():
    lib = C.CDLL(build_harness())
    lib.shiro_backend_selftest.argtypes = [_P, _P, _U, _P, _U, _U]
    lib.shiro_backend_selftest.restype = C.c_int
    lib.shiro_harness_time_render.argtypes = [_P, _P, _U, _U, C.POINTER(C.c_double), _P]
    lib.shiro_harness_time_render.restype = C.c_int
    lib.shiro_harness_cancel_midframe.argtypes = [_P, _P, C.c_double, _U, _P, C.POINTER(C.c_int),
                                                  C.POINTER(C.c_double)]
    lib.shiro_harness_cancel_midframe.restype = C.c_int
    lib.shiro_harness_edit_in_place.argtypes = [_P, _P, _P, _P, _P, C.POINTER(C.c_uint64)]
    lib.shiro_harness_edit_in_place.restype = C.c_int
    return lib


if __name__ == "__main__":
    print(build_harness())
