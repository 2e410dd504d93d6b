"""numpy-level calls into a CPU checker (port or reference).  TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C

import numpy as np

from shiro_gb300.abi import FrameBuffer, MarshalledScene, MaterialDesc, render_desc

from . import Checker


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def sampler(ck: Checker, px, py, index, branch) -> np.ndarray:
    px, py, index, branch = (np.ascontiguousarray(a, np.uint32) for a in (px, py, index, branch))
    out = np.zeros((px.size, 2), np.float32)
    ck.fn("sampler")(px.size, _p(px), _p(py), _p(index), _p(branch), _p(out))
    return out


def camera_rays(ck: Checker, camera, settings, sample_start=0):
    req = render_desc(camera, settings, sample_start, 1)
    n = settings.width * settings.height
    o = np.zeros((n, 3), np.float32)
    d = np.zeros((n, 3), np.float32)
    ck.fn("camera_rays")(C.byref(req), _p(o), _p(d))
    return o, d


def trace_rays(ck: Checker, scene, origins, dirs, tmax=None, bruteforce=False):
    ms = MarshalledScene(scene) if not isinstance(scene, MarshalledScene) else scene
    o = np.ascontiguousarray(origins, np.float32)
    d = np.ascontiguousarray(dirs, np.float32)
    n = o.shape[0]
    tm = np.full(n, np.finfo(np.float32).max, np.float32) if tmax is None else np.ascontiguousarray(tmax, np.float32)
    prim = np.zeros(n, np.uint32)
    t = np.zeros(n, np.float32)
    occ = np.zeros(n, np.uint32)
    f = ck.lib.oracle_trace_rays_bruteforce if bruteforce else ck.fn("trace_rays")
    f(ms.ref(), _p(o), _p(d), _p(tm), n, _p(prim), _p(t), _p(occ))
    return prim, t, occ


def primary_hits(ck: Checker, scene, camera, settings, sample_start=0):
    ms = MarshalledScene(scene) if not isinstance(scene, MarshalledScene) else scene
    req = render_desc(camera, settings, sample_start, 1)
    n = settings.width * settings.height
    prim = np.zeros(n, np.uint32)
    t = np.zeros(n, np.float32)
    ck.fn("primary_hits")(ms.ref(), C.byref(req), _p(prim), _p(t))
    return prim, t


def bsdf(ck: Checker, material, normals, views, lights):
    md = material.to_desc() if not isinstance(material, MaterialDesc) else material
    n_ = np.ascontiguousarray(normals, np.float32)
    v = np.ascontiguousarray(views, np.float32)
    li = np.ascontiguousarray(lights, np.float32)
    n = n_.shape[0]
    f = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    w = np.zeros(8, np.float32)
    ck.fn("bsdf")(C.byref(md), n, _p(n_), _p(v), _p(li), _p(f), _p(pdf), _p(w))
    return f, pdf, w


def env_tables(ck: Checker, env):
    env = np.ascontiguousarray(env, np.float32)
    h, w = env.shape[:2]
    row = np.zeros(h + 1, np.float32)
    cond = np.zeros(h * (w + 1), np.float32)
    ck.fn("env_tables")(w, h, _p(env), _p(row), _p(cond))
    return row, cond


def env_alias(ck: Checker, env):
    """The GPU backend's alias table by the port's sequential sweep:
    (threshold bits, alias index), each h * w."""
    env = np.ascontiguousarray(env, np.float32)
    h, w = env.shape[:2]
    thr = np.zeros(h * w, np.uint32)
    al = np.zeros(h * w, np.uint32)
    rc = ck.lib.oracle_env_alias(w, h, _p(env), _p(thr), _p(al))
    if rc != 0:
        raise RuntimeError(f"oracle_env_alias failed: {rc}")
    return thr, al


def env_query(ck: Checker, env, u2, dirs, layout=1):
    env = np.ascontiguousarray(env, np.float32)
    h, w = env.shape[:2]
    u2 = np.ascontiguousarray(u2, np.float32)
    dirs = np.ascontiguousarray(dirs, np.float32)
    n = u2.shape[0]
    sd = np.zeros((n, 3), np.float32)
    sp = np.zeros(n, np.float32)
    sc = np.zeros((n, 3), np.float32)
    pdf = np.zeros(n, np.float32)
    rgb = np.zeros((n, 3), np.float32)
    ck.fn("env_query")(w, h, _p(env), layout, n, _p(u2), _p(dirs), _p(sd), _p(sp), _p(sc), _p(pdf), _p(rgb))
    return dict(sample_dir=sd, sample_pdf=sp, sample_rgb=sc, pdf=pdf, rgb=rgb)


def render(ck: Checker, scene, camera, settings, sample_start=0, sample_count=None) -> FrameBuffer:
    ms = MarshalledScene(scene) if not isinstance(scene, MarshalledScene) else scene
    count = settings.samples_per_pixel if sample_count is None else sample_count
    req = render_desc(camera, settings, sample_start, count)
    fb = FrameBuffer(settings.width, settings.height)
    aovs = fb.aovs()
    rc = ck.fn("render")(ms.ref(), C.byref(req), C.byref(aovs))
    if rc != 0:
        raise RuntimeError(f"{ck.prefix}_render failed: {rc}")
    return fb


def render_batches(ck: Checker, scene, camera, settings, sample_start, sample_count, batches) -> FrameBuffer:
    """The last of `batches` consecutive batches rendered by ONE reference
    tracer (reference checker only), as a progressive render issues them."""
    ms = MarshalledScene(scene) if not isinstance(scene, MarshalledScene) else scene
    req = render_desc(camera, settings, sample_start, sample_count)
    fb = FrameBuffer(settings.width, settings.height)
    aovs = fb.aovs()
    f = ck.lib.ref_render_batches
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    f.restype = C.c_int
    rc = f(ms.ref(), C.byref(req), batches, C.byref(aovs))
    if rc != 0:
        raise RuntimeError(f"ref_render_batches failed: {rc}")
    return fb


def render_paths(ck: Checker, scene, camera, settings, sample_start, pixels, sample_index):
    """Per-path results of the port: radiance (n,3), albedo (n,3), normal
    (n,3), depth (n,) for paths (pixel index, sample index)."""
    ms = MarshalledScene(scene) if not isinstance(scene, MarshalledScene) else scene
    req = render_desc(camera, settings, sample_start, 1)
    px = np.ascontiguousarray(pixels, np.uint32)
    si = np.ascontiguousarray(sample_index, np.uint32)
    n = px.size
    out = np.zeros((n, 10), np.float32)
    ck.lib.oracle_render_paths(ms.ref(), C.byref(req), _p(px), n, _p(si), _p(out), None, None)
    return out


class PortScene:
    """A scene built once in the port (oracle_scene_*), for repeated renders
    of row lists and path lists.  ``set_alias`` gives a dome texture the GPU
    backend's alias table, so that renders without SHIRO_RENDER_ENV_CDF pick
    dome-sample texels exactly as the backend's default (timed) sampler does."""

    def __init__(self, ck: Checker, scene):
        self.lib = ck.lib
        self.ms = MarshalledScene(scene) if not isinstance(scene, MarshalledScene) else scene
        self.h = C.c_void_p()
        rc = self.lib.oracle_scene_create(self.ms.ref(), C.byref(self.h))
        if rc != 0:
            raise RuntimeError(f"oracle_scene_create failed: {rc}")

    def set_alias(self, dome: int, threshold_bits, alias):
        thr = np.ascontiguousarray(threshold_bits, np.uint32)
        al = np.ascontiguousarray(alias, np.uint32)
        rc = self.lib.oracle_scene_set_env_alias(self.h, dome, _p(thr), _p(al), thr.size)
        if rc != 0:
            raise RuntimeError(f"oracle_scene_set_env_alias failed: {rc}")

    def render_rows(self, camera, settings, rows, sample_start=0, sample_count=None, flags=0) -> FrameBuffer:
        count = settings.samples_per_pixel if sample_count is None else sample_count
        req = render_desc(camera, settings, sample_start, count, flags)
        fb = FrameBuffer(settings.width, settings.height)
        aovs = fb.aovs()
        r = np.ascontiguousarray(rows, np.uint32)
        n = self.lib.oracle_scene_render_row_list(self.h, C.byref(req), _p(r), r.size, C.byref(aovs))
        if n < 0:
            raise RuntimeError(f"oracle_scene_render_row_list failed: {n}")
        return fb

    def render_paths(self, camera, settings, pixels, sample_index, flags=0) -> np.ndarray:
        req = render_desc(camera, settings, 0, 1, flags)
        px = np.ascontiguousarray(pixels, np.uint32)
        si = np.ascontiguousarray(sample_index, np.uint32)
        out = np.zeros((px.size, 10), np.float32)
        rc = self.lib.oracle_scene_render_paths(self.h, C.byref(req), _p(px), px.size, _p(si), _p(out))
        if rc != 0:
            raise RuntimeError(f"oracle_scene_render_paths failed: {rc}")
        return out

    def close(self):
        if self.h:
            self.lib.oracle_scene_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        self.close()
