"""CPU checkers for the GB300 path tracer.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package; the product (shiro_gb300) never does.

* ``load_port()`` - oracle/libshiro_oracle.so, this project's C++
  restatement of the reference CPU path tracer (oracle/port/shiro_oracle.cpp).
  It is pinned against the golden vectors in tests/golden, which the
  reference itself produced.
* ``load_ref()``  - oracle/_ref/libshiro_ref.so, the reference integrator
  compiled from its own sources (only where the reference tree exists).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "libshiro_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libshiro_ref.so")
REF_TREE = "/root/reference"

_P = C.c_void_p
_U = C.c_uint32


def build_port() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref() -> str | None:
    if not os.path.isdir(REF_TREE):
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)
    return REF_LIB


def _common(lib, prefix: str):
    fn = lambda name: getattr(lib, f"{prefix}_{name}")  # noqa: E731
    fn("sampler").argtypes = [_U, _P, _P, _P, _P, _P]
    fn("camera_rays").argtypes = [_P, _P, _P]
    fn("trace_rays").argtypes = [_P, _P, _P, _P, _U, _P, _P, _P]
    fn("primary_hits").argtypes = [_P, _P, _P, _P]
    fn("bsdf").argtypes = [_P, _U, _P, _P, _P, _P, _P, _P]
    fn("env_tables").argtypes = [_U, _U, _P, _P, _P]
    fn("env_query").argtypes = [_U, _U, _P, _U, _U, _P, _P, _P, _P, _P, _P, _P]
    fn("render").argtypes = [_P, _P, _P]
    for n in ("sampler", "camera_rays", "trace_rays", "primary_hits", "bsdf", "env_tables", "env_query",
              "render"):
        fn(n).restype = C.c_int
    return lib


_port = None
_ref = None


def load_port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        lib = C.CDLL(PORT_LIB)
        _common(lib, "oracle")
        lib.oracle_render_paths.argtypes = [_P, _P, _P, _U, _P, _P, _P, _P]
        lib.oracle_render_paths.restype = C.c_int
        lib.oracle_set_threads.argtypes = [_U]
        lib.oracle_set_threads.restype = None
        lib.oracle_supports_scene.argtypes = [_P]
        lib.oracle_supports_scene.restype = C.c_int
        lib.oracle_trace_rays_bruteforce.argtypes = [_P, _P, _P, _P, _U, _P, _P, _P]
        lib.oracle_trace_rays_bruteforce.restype = C.c_int
        lib.oracle_scene_create.argtypes = [_P, _P]
        lib.oracle_scene_create.restype = C.c_int
        lib.oracle_scene_destroy.argtypes = [_P]
        lib.oracle_scene_destroy.restype = None
        lib.oracle_scene_render_row_list.argtypes = [_P, _P, _P, _U, _P]
        lib.oracle_scene_render_row_list.restype = C.c_int64
        lib.oracle_scene_render_paths.argtypes = [_P, _P, _P, _U, _P, _P]
        lib.oracle_scene_render_paths.restype = C.c_int
        lib.oracle_scene_set_env_alias.argtypes = [_P, _U, _P, _P, _U]
        lib.oracle_scene_set_env_alias.restype = C.c_int
        lib.oracle_env_alias.argtypes = [_U, _U, _P, _P, _P]
        lib.oracle_env_alias.restype = C.c_int
        _port = lib
    return _port


def load_ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_LIB):
            if build_ref() is None:
                return None
        lib = C.CDLL(REF_LIB)
        _common(lib, "ref")
        _ref = lib
    return _ref


class Checker:
    """Uniform numpy-level wrapper over either library."""

    def __init__(self, lib, prefix: str):
        self.lib = lib
        self.prefix = prefix

    def fn(self, name):
        return getattr(self.lib, f"{self.prefix}_{name}")


def port_checker() -> Checker:
    return Checker(load_port(), "oracle")


def ref_checker() -> Checker | None:
    lib = load_ref()
    return None if lib is None else Checker(lib, "ref")
