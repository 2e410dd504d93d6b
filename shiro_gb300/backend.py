"""Python mirror of shiro::backend::RenderBackend over the GB300 C ABI.

``GpuBackend`` follows the reference's backend interface
(include/shiro/backend/RenderBackend.h:28-34 and OptixBackend.h:10-27):

* ``get_status()``            -> BackendStatus          (RenderBackend.h:32)
* ``supports_scene(scene)``   -> bool                   (OptixBackend.h:16)
* ``render_sample_batch(req)``-> FrameBuffer            (RenderBackend.h:33)

with the same error convention: a failed batch logs to stderr and returns a
cleared, sized FrameBuffer (OptixBackend.cpp:1142-1155), and a failed
runtime marks the backend unavailable.  ``render()`` is the strict variant
that raises.  There is no CPU fallback inside the backend: without the
native library or a device the backend is unavailable and rendering raises.
"""
from __future__ import annotations

import ctypes as C
import os
import sys
import weakref
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import abi
from .abi import (Aovs, BackendStatus, Camera, FrameBuffer, MarshalledScene, RenderDesc, RenderSettings, RenderStats,
                  Scene, WavefrontConfig, render_desc)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libshiro_gpu.so")

_P = C.c_void_p
_U = C.c_uint32


def load_environment_file(path: str) -> np.ndarray:
    """An environment image (Radiance .hdr or OpenEXR .exr) read by the native
    library's reader (shiro_hdri_load, the counterpart of EnvironmentMap::Load
    for hosts without OpenImageIO) as (height, width, 3) float32 texels, row 0
    at the top.  Raises ShiroGpuError with the reader's reason on failure."""
    lib = load_library()
    w, h = C.c_uint32(), C.c_uint32()
    px = C.POINTER(C.c_float)()
    err = C.create_string_buffer(256)
    rc = lib.shiro_hdri_load(os.fsencode(path), C.byref(w), C.byref(h), C.byref(px), err, 256)
    if rc != 0:
        raise ShiroGpuError(rc, err.value.decode())
    try:
        n = w.value * h.value * 3
        return np.ctypeslib.as_array(px, shape=(n,)).copy().reshape(h.value, w.value, 3)
    finally:
        lib.shiro_hdri_free(C.cast(px, C.c_void_p))


class ShiroGpuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libshiro_gpu.so (built by shiro_gb300.build / __graft_entry__.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ShiroGpuError(abi.SHIRO_ERR_NO_DEVICE,
                            f"native library missing: {path} (run __graft_entry__.build())")
    lib = C.CDLL(path)
    sig = {
        "shiro_gpu_status": ([_P], C.c_int),
        "shiro_gpu_create": ([C.c_int, _P], C.c_int),
        "shiro_gpu_destroy": ([_P], None),
        "shiro_gpu_last_error": ([_P], C.c_char_p),
        "shiro_gpu_set_stream": ([_P, _P], C.c_int),
        "shiro_gpu_supports_scene": ([_P, C.c_char_p, C.c_size_t], C.c_int),
        "shiro_gpu_upload_scene": ([_P, _P], C.c_int),
        "shiro_gpu_render": ([_P, _P, _P, _P], C.c_int),
        "shiro_gpu_render_batch": ([_P, _P, _U, _P, _P], C.c_int),
        "shiro_gpu_render_batch_ready": ([_P, _P, _U, _P, _P, abi.PixelsReady, _P], C.c_int),
        "shiro_gpu_get_wavefront_config": ([_P, _P], C.c_int),
        "shiro_gpu_set_wavefront_config": ([_P, _P], C.c_int),
        "shiro_gpu_autotune": ([_P, _P, _P], C.c_int),
        "shiro_gpu_set_params": ([_P, _P, _P, _P, _P], C.c_int),
        "shiro_gpu_adjoint": ([_P, _P, _P, _P, _P, _P, _P], C.c_int),
        "shiro_gpu_primary_hits": ([_P, _P, _P, _P, _U], C.c_int),
        "shiro_gpu_sample": ([_P, _P, _P, _P, _P, _U, _P], C.c_int),
        "shiro_gpu_trace_rays": ([_P, _P, _P, _P, _U, _P, _P, _P], C.c_int),
        "shiro_gpu_last_stats": ([_P, _P], C.c_int),
        "shiro_gpu_count_work": ([_P, _P, _U, _P], C.c_int),
        "shiro_gpu_render_frozen": ([_P, _P, _P, _P, _P, _P, _P], C.c_int),
        "shiro_gpu_set_bvh_width": ([_P, _U], C.c_int),
        "shiro_gpu_set_bvh_build": ([_P, _U], C.c_int),
        "shiro_gpu_set_adjoint_form": ([_P, _U], C.c_int),
        "shiro_gpu_env_tables": ([_P, _U, _P, _P, _P, _P, _P, _P, _P], C.c_int),
        "shiro_gpu_scene_signature": ([_P, _P], C.c_int),
        "shiro_gpu_host_alloc": ([C.c_size_t, _P], C.c_int),
        "shiro_gpu_host_free": ([_P], None),
        "shiro_hdri_load": ([C.c_char_p, _P, _P, _P, C.c_char_p, C.c_size_t], C.c_int),
        "shiro_hdri_decode": ([C.c_char_p, C.c_size_t, _P, _P, _P, C.c_char_p, C.c_size_t], C.c_int),
        "shiro_hdri_free": ([_P], None),
        "shiro_gpu_env_sample": ([_P, _U, _U, _P, _U, _P, _P], C.c_int),
        "shiro_gpu_render_paths": ([_P, _P, _P, _U, _P, _P], C.c_int),
        "shiro_gpu_accum_create": ([_P, _P], C.c_int),
        "shiro_gpu_accum_destroy": ([_P], None),
        "shiro_gpu_accum_reset": ([_P, _U, _U], C.c_int),
        "shiro_gpu_accum_add": ([_P, _P, _U, _U, _U], C.c_int),
        "shiro_gpu_accum_render": ([_P, _P, _P, _U], C.c_int),
        "shiro_gpu_accum_resolve": ([_P, _P], C.c_int),
        "shiro_gpu_accum_info": ([_P, _P, _P, _P], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


@dataclass
class RenderRequest:
    """shiro::backend::RenderRequest (RenderBackend.h:12-19)."""

    scene: Scene
    camera: Camera
    settings: RenderSettings
    sample_start: int = 0
    sample_count: int = 1
    cancel: Optional[C.c_int] = None  # set .value = 1 to cancel
    flags: int = 0


class GpuBackend:
    """The GB300 backend.  One instance owns one device context; calls are
    serialised by the caller (as the reference's mutex does)."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        self._ctx = C.c_void_p()
        rc = self.lib.shiro_gpu_create(int(device), C.byref(self._ctx))
        if rc != 0:
            raise ShiroGpuError(rc, self.lib.shiro_gpu_last_error(None).decode())
        self._scene_key = None
        self._marshalled: Optional[MarshalledScene] = None
        self._scene_ref = None
        self._structure_key = None
        self.last_error = ""
        self._accumulators = weakref.WeakSet()

    # -- lifetime ----------------------------------------------------------
    def close(self):
        if self._ctx:
            for acc in list(self._accumulators):  # they use the context: free them first
                acc.close()
            self.lib.shiro_gpu_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- RenderBackend -----------------------------------------------------
    @staticmethod
    def get_status() -> dict:
        lib = load_library()
        st = BackendStatus()
        lib.shiro_gpu_status(C.byref(st))
        return dict(kind=st.kind, name=st.name.decode(), available=bool(st.available), uses_gpu=bool(st.uses_gpu),
                    device_count=st.device_count, device_name=st.device_name.decode(),
                    compute=(st.compute_major, st.compute_minor))

    def supports_scene(self, scene: Scene) -> bool:
        buf = C.create_string_buffer(256)
        return bool(self.lib.shiro_gpu_supports_scene(MarshalledScene(scene).ref(), buf, 256))

    def _err(self, rc: int) -> ShiroGpuError:
        msg = self.lib.shiro_gpu_last_error(self._ctx).decode()
        self.last_error = msg
        return ShiroGpuError(rc, msg)

    def upload_scene(self, scene: Scene, force: bool = False):
        """Uploads the scene snapshot unless the device already holds one of
        the same content: the cache key is the object and the native content
        signature (shiro_gpu_scene_signature: every material field, the mesh
        arrays, lights, dome frames and texels), so a scene edited in place -
        a light, a vertex - is uploaded again (the OptiX backend compares
        ComputeSceneSignature the same way, OptixBackend.cpp:150-232)."""
        skey = abi.scene_structure_key(scene)
        ms = self._marshalled
        if (ms is None or self._scene_ref is not scene or self._structure_key != skey or not ms.aliased):
            ms = MarshalledScene(scene)
        sig = C.c_uint64(0)
        self.lib.shiro_gpu_scene_signature(ms.ref(), C.byref(sig))
        key = (id(scene), sig.value)
        self._marshalled = ms
        self._scene_ref = scene
        self._structure_key = skey
        if not force and self._scene_key == key:
            return
        self._params_on_device = None  # the upload restores the scene's own parameters
        rc = self.lib.shiro_gpu_upload_scene(self._ctx, ms.ref())
        if rc != 0:
            self._scene_key = None
            raise self._err(rc)
        self._scene_key = key

    def render(self, scene: Scene, camera: Camera, settings: RenderSettings, sample_start: int = 0,
               sample_count: Optional[int] = None, flags: int = 0, cancel: Optional[C.c_int] = None,
               out: Optional[FrameBuffer] = None) -> FrameBuffer:
        """Strict RenderSampleBatch: raises on failure."""
        self.upload_scene(scene)
        count = settings.samples_per_pixel if sample_count is None else sample_count
        req = render_desc(camera, settings, sample_start, count, flags)
        fb = out if out is not None else FrameBuffer(settings.width, settings.height)
        aovs = fb.aovs()
        rc = self.lib.shiro_gpu_render(self._ctx, C.byref(req), C.byref(cancel) if cancel is not None else None,
                                       C.byref(aovs))
        if rc != 0:
            raise self._err(rc)
        return fb

    def render_sample_batch(self, request: RenderRequest) -> FrameBuffer:
        """RenderBackend::RenderSampleBatch with the reference's error
        convention (cleared FrameBuffer + stderr message on failure), on the
        wavefront form (frames bit-identical to ``render``'s)."""
        try:
            (fb,) = self.render_batch(request.scene, [(request.camera, request.settings, request.sample_start,
                                                       request.sample_count)], request.flags, request.cancel)
            return fb
        except ShiroGpuError as e:
            sys.stderr.write(f"shiro gb300 backend: {e}\n")
            return FrameBuffer(request.settings.width, request.settings.height)

    # -- wavefront ---------------------------------------------------------
    def render_batch(self, scene: Scene, requests: Sequence[tuple], flags: int = 0,
                     cancel: Optional[C.c_int] = None, outs_fb: Optional[Sequence[FrameBuffer]] = None,
                     ready=None) -> List[FrameBuffer]:
        """requests: (camera, settings[, sample_start[, sample_count]]);
        outs_fb: frame buffers to fill (reused across calls), else new ones;
        ready(request, first_pixel, pixel_count): told of finished pixel
        ranges during the render (shiro_gpu_render_batch_ready)."""
        self.upload_scene(scene)
        n = len(requests)
        descs = (RenderDesc * max(1, n))()
        fbs = []
        outs = (Aovs * max(1, n))()
        for i, r in enumerate(requests):
            cam, st = r[0], r[1]
            start = r[2] if len(r) > 2 else 0
            count = r[3] if len(r) > 3 else st.samples_per_pixel
            descs[i] = render_desc(cam, st, start, count, flags)
            fb = outs_fb[i] if outs_fb is not None else FrameBuffer(st.width, st.height)
            fbs.append(fb)
            outs[i] = fb.aovs()
        flag = C.byref(cancel) if cancel is not None else None
        if ready is None:
            rc = self.lib.shiro_gpu_render_batch(self._ctx, descs, n, flag, outs)
        else:
            cb = abi.PixelsReady(lambda user, r, first, count: ready(r, first, count))
            rc = self.lib.shiro_gpu_render_batch_ready(self._ctx, descs, n, flag, outs, cb, None)
        if rc != 0:
            raise self._err(rc)
        return fbs

    def set_bvh_width(self, width: int):
        """2: the binary BVH everywhere; 8: the compressed wide BVH everywhere;
        0 (default): the wide BVH in the wavefront form, the binary one in the
        one-thread-per-path kernels.  Hits are identical."""
        rc = self.lib.shiro_gpu_set_bvh_width(self._ctx, int(width))
        if rc != 0:
            raise ShiroGpuError(rc, "bvh width must be 0, 2 or 8")

    def set_bvh_build(self, sah_cluster_triangles: int):
        """Binary BVHs of the next upload: > 1 rebuilds the tree above Morton
        clusters of at most that many triangles by binned SAH; 0 keeps the
        Morton hierarchy.  Hits are identical.  Forces the next upload."""
        rc = self.lib.shiro_gpu_set_bvh_build(self._ctx, int(sah_cluster_triangles))
        if rc != 0:
            raise ShiroGpuError(rc, "cluster size must be 0 or in [2, 65536]")
        self._scene_key = None

    def set_adjoint_form(self, wavefront: bool):
        """True (default): the adjoint replays paths with the wavefront stages;
        False: one thread per path."""
        rc = self.lib.shiro_gpu_set_adjoint_form(self._ctx, 1 if wavefront else 0)
        if rc != 0:
            raise self._err(rc)

    def wavefront_config(self) -> dict:
        c = WavefrontConfig()
        self.lib.shiro_gpu_get_wavefront_config(self._ctx, C.byref(c))
        return {name: int(getattr(c, name)) for name, _ in WavefrontConfig._fields_}

    def set_wavefront_config(self, **kw):
        c = WavefrontConfig()
        for k, v in kw.items():
            setattr(c, k, int(v))
        rc = self.lib.shiro_gpu_set_wavefront_config(self._ctx, C.byref(c))
        if rc != 0:
            raise self._err(rc)

    def autotune(self, scene: Scene, camera: Camera, settings: RenderSettings, sample_count: Optional[int] = None) -> dict:
        self.upload_scene(scene)
        req = render_desc(camera, settings, 0, settings.samples_per_pixel if sample_count is None else sample_count)
        c = WavefrontConfig()
        rc = self.lib.shiro_gpu_autotune(self._ctx, C.byref(req), C.byref(c))
        if rc != 0:
            raise self._err(rc)
        return self.wavefront_config()

    # -- probes --------------------------------------------------------------
    def sample(self, px, py, index, branch) -> np.ndarray:
        """OpenQmcSampler::Next2D of the device sampler for each tuple: (n, 2)."""
        px, py, index, branch = (np.ascontiguousarray(a, np.uint32) for a in (px, py, index, branch))
        out = np.zeros((px.size, 2), np.float32)
        rc = self.lib.shiro_gpu_sample(self._ctx, _ptr(px), _ptr(py), _ptr(index), _ptr(branch), px.size, _ptr(out))
        if rc != 0:
            raise self._err(rc)
        return out

    def primary_hits(self, scene: Scene, camera: Camera, settings: RenderSettings, sample_start: int = 0):
        self.upload_scene(scene)
        req = render_desc(camera, settings, sample_start, 1)
        n = settings.width * settings.height
        prim = np.zeros(n, np.uint32)
        t = np.zeros(n, np.float32)
        rc = self.lib.shiro_gpu_primary_hits(self._ctx, C.byref(req), _ptr(prim), _ptr(t), 0)
        if rc != 0:
            raise self._err(rc)
        return prim, t

    def trace_rays(self, scene: Scene, origins, dirs, tmax=None):
        self.upload_scene(scene)
        o = np.ascontiguousarray(origins, np.float32)
        d = np.ascontiguousarray(dirs, np.float32)
        n = o.shape[0]
        tm = (np.full(n, np.finfo(np.float32).max, np.float32) if tmax is None
              else np.ascontiguousarray(tmax, np.float32))
        prim = np.zeros(n, np.uint32)
        t = np.zeros(n, np.float32)
        occ = np.zeros(n, np.uint32)
        rc = self.lib.shiro_gpu_trace_rays(self._ctx, _ptr(o), _ptr(d), _ptr(tm), n, _ptr(prim), _ptr(t), _ptr(occ))
        if rc != 0:
            raise self._err(rc)
        return prim, t, occ

    def count_work(self, scene: Scene, camera: Camera, settings: RenderSettings, stride: int = 64,
                   sample_start: int = 0, sample_count: Optional[int] = None, flags: int = 0) -> dict:
        """Work counts of every `stride`-th path (node visits, triangle
        tests, environment lookups ...), for the algorithmic-bytes roofline."""
        from .abi import WorkCounts

        self.upload_scene(scene)
        req = render_desc(camera, settings, sample_start,
                          settings.samples_per_pixel if sample_count is None else sample_count, flags)
        wc = WorkCounts()
        rc = self.lib.shiro_gpu_count_work(self._ctx, C.byref(req), int(stride), C.byref(wc))
        if rc != 0:
            raise self._err(rc)
        return {k: getattr(wc, k) for k, _ in WorkCounts._fields_}

    # -- progressive accumulation ---------------------------------------------
    def accumulator(self) -> "DeviceAccumulator":
        """A device-resident Renderer::FrameAccumulator on this context."""
        return DeviceAccumulator(self)

    # -- differentiable form -------------------------------------------------
    @staticmethod
    def _dptr(t):
        """Device pointer of a contiguous float32 CUDA tensor (None -> NULL)."""
        if t is None:
            return None
        if not (t.is_cuda and t.dtype.is_floating_point and t.is_contiguous()):
            raise ValueError("expected a contiguous float32 CUDA tensor")
        return C.c_void_p(t.data_ptr())

    def set_params(self, base_color=None, roughness=None, metallic=None, env=None):
        """Overwrites the uploaded scene's base colour [M,3], roughness [M],
        metalness [M] and dome-0 texels [H,W,3] (CUDA float32 tensors).

        A group whose values equal (bit for bit, compared on the device) what
        the last call wrote is not written again: an environment write
        rebuilds the dome's importance tables, and a multi-view optimisation
        sets the same parameters before every view's render."""
        import torch

        new = (base_color, roughness, metallic, env)
        last = getattr(self, "_params_on_device", None) or (None, None, None, None)
        def same(o, t):  # bit for bit (float equality would take -0.0 for 0.0)
            return o is not None and o.shape == t.shape and torch.equal(o.view(torch.int32), t.view(torch.int32))

        send = [t if t is not None and not same(o, t) else None for t, o in zip(new, last)]
        if all(t is None for t in send):
            return
        rc = self.lib.shiro_gpu_set_params(self._ctx, *(self._dptr(t) for t in send))
        if rc != 0:
            self._params_on_device = None
            raise self._err(rc)
        self._params_on_device = tuple(t.detach().clone() if t is not None else o for t, o in zip(send, last))

    def render_device(self, camera: Camera, settings: RenderSettings, sample_start: int = 0,
                      sample_count: Optional[int] = None, flags: int = 0, wavefront: bool = False,
                      also_start: Optional[int] = None):
        """Renders the uploaded scene into CUDA tensors; returns beauty [H,W,4].
        also_start (wavefront form): the same view's `sample_count` samples
        from that index are rendered in the same call as a second request
        (its image is discarded); with RENDER_KEEP_PATHS in flags both
        requests' paths are kept for an adjoint of either."""
        import torch

        from .abi import Aovs

        count = settings.samples_per_pixel if sample_count is None else sample_count
        n = settings.width * settings.height
        starts = [sample_start] + ([] if also_start is None else [also_start])
        nreq = len(starts)
        planes = [[torch.empty(n * c, dtype=torch.float32, device="cuda") for c in (4, 3, 3, 1)] for _ in starts]
        aovs = (Aovs * nreq)(*[Aovs(*[C.cast(C.c_void_p(p.data_ptr()), C.POINTER(C.c_float)) for p in pl], 1, 0)
                               for pl in planes])
        reqs = (RenderDesc * nreq)(*[render_desc(camera, settings, s, count, flags) for s in starts])
        if wavefront:
            rc = self.lib.shiro_gpu_render_batch(self._ctx, reqs, nreq, None, aovs)
        elif nreq == 1:
            rc = self.lib.shiro_gpu_render(self._ctx, reqs, None, aovs)
        else:
            raise ValueError("also_start needs the wavefront form")
        if rc != 0:
            raise self._err(rc)
        return planes[0][0].view(settings.height, settings.width, 4)

    def adjoint(self, camera: Camera, settings: RenderSettings, d_beauty, grads: dict, sample_start: int = 0,
                sample_count: Optional[int] = None, flags: int = 0):
        """Adds d(sum d_beauty . beauty)/d(params) into grads['base_color'],
        ['roughness'], ['metallic'], ['env'] (CUDA float32 tensors)."""
        count = settings.samples_per_pixel if sample_count is None else sample_count
        req = render_desc(camera, settings, sample_start, count, flags)
        rc = self.lib.shiro_gpu_adjoint(self._ctx, C.byref(req), self._dptr(d_beauty.contiguous()),
                                        self._dptr(grads.get("base_color")), self._dptr(grads.get("roughness")),
                                        self._dptr(grads.get("metallic")), self._dptr(grads.get("env")))
        if rc != 0:
            raise self._err(rc)

    def render_frozen(self, camera: Camera, settings: RenderSettings, base_color=None, roughness=None, metallic=None,
                      env=None, sample_start: int = 0, sample_count: Optional[int] = None, flags: int = 0):
        """Beauty with sampling from the scene's parameters and values from the
        given ones (the quantity whose finite differences the adjoint estimates)."""
        import torch

        count = settings.samples_per_pixel if sample_count is None else sample_count
        out = torch.empty(settings.height * settings.width * 4, dtype=torch.float32, device="cuda")
        req = render_desc(camera, settings, sample_start, count, flags)
        rc = self.lib.shiro_gpu_render_frozen(self._ctx, C.byref(req), self._dptr(base_color), self._dptr(roughness),
                                              self._dptr(metallic), self._dptr(env), C.c_void_p(out.data_ptr()))
        if rc != 0:
            raise self._err(rc)
        return out.view(settings.height, settings.width, 4)

    # -- diagnostics -----------------------------------------------------
    def env_tables(self, env: int = 0) -> dict:
        """The device importance tables of dome texture `env`: row_cdf,
        cond_cdf (h, w + 1), mass (h, w), alias_threshold (float32 view of the
        threshold bits) and alias_index (h * w)."""
        w, h = C.c_uint32(), C.c_uint32()
        rc = self.lib.shiro_gpu_env_tables(self._ctx, env, C.byref(w), C.byref(h), None, None, None, None, None)
        if rc != 0:
            raise self._err(rc)
        w, h = w.value, h.value
        row = np.zeros(h + 1, np.float32)
        cond = np.zeros(h * (w + 1), np.float32)
        mass = np.zeros(h * w, np.float32)
        thr = np.zeros(h * w, np.uint32)
        al = np.zeros(h * w, np.uint32)
        p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        rc = self.lib.shiro_gpu_env_tables(self._ctx, env, None, None, p(row), p(cond), p(mass), p(thr), p(al))
        if rc != 0:
            raise self._err(rc)
        return dict(width=w, height=h, row_cdf=row, cond_cdf=cond.reshape(h, w + 1), mass=mass.reshape(h, w),
                    alias_threshold_bits=thr, alias_threshold=thr.view(np.float32), alias_index=al)

    def env_sample(self, u2, env: int = 0, flags: int = 0):
        """(texel index, pdf) the kernels' dome sampler gives each 2-D point."""
        u2 = np.ascontiguousarray(u2, np.float32).reshape(-1, 2)
        n = u2.shape[0]
        texel = np.zeros(n, np.uint32)
        pdf = np.zeros(n, np.float32)
        p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        rc = self.lib.shiro_gpu_env_sample(self._ctx, env, n, p(u2), flags, p(texel), p(pdf))
        if rc != 0:
            raise self._err(rc)
        return texel, pdf

    def render_paths(self, scene: Scene, camera: Camera, settings: RenderSettings, pixels, sample_index,
                     flags: int = 0) -> np.ndarray:
        """Per-path results of the plain form, (n, 10): radiance, albedo,
        normal, depth of path (pixel index, sample index)."""
        self.upload_scene(scene)
        req = render_desc(camera, settings, 0, 1, flags)
        px = np.ascontiguousarray(pixels, np.uint32)
        si = np.ascontiguousarray(sample_index, np.uint32)
        out = np.zeros((px.size, 10), np.float32)
        p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        rc = self.lib.shiro_gpu_render_paths(self._ctx, C.byref(req), p(px), px.size, p(si), p(out))
        if rc != 0:
            raise self._err(rc)
        return out

    def last_stats(self) -> dict:
        s = RenderStats()
        self.lib.shiro_gpu_last_stats(self._ctx, C.byref(s))
        out = {}
        for k, _ in RenderStats._fields_:
            v = getattr(s, k)
            out[k] = list(v) if hasattr(v, "__len__") else v
        return out

    @property
    def handle(self):
        return self._ctx


class DeviceAccumulator:
    """Renderer::FrameAccumulator (Renderer.cpp:47-110) with its running sums
    in device memory: ``reset`` / ``accumulate`` / ``resolve`` /
    ``sample_count`` follow Reset / Accumulate / Resolve / SampleCount, and
    ``render_step`` is one step of HdShiroRenderParam's progressive worker
    (RenderParam.cpp:790-806): render a batch on the device and fold it in
    there, with no host frame per batch."""

    def __init__(self, backend: GpuBackend):
        self.backend = backend
        self.lib = backend.lib
        self._h = C.c_void_p()
        if not backend._ctx:
            raise ShiroGpuError(abi.SHIRO_ERR_INVALID_ARGUMENT, "backend is closed")
        rc = self.lib.shiro_gpu_accum_create(backend._ctx, C.byref(self._h))
        if rc != 0:
            raise backend._err(rc)
        backend._accumulators.add(self)

    def close(self):
        if self._h:
            self.lib.shiro_gpu_accum_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise self.backend._err(rc)

    def reset(self, width: int, height: int):
        self._check(self.lib.shiro_gpu_accum_reset(self._h, int(width), int(height)))

    def accumulate(self, fb: FrameBuffer, sample_count: int):
        """Folds a host FrameBuffer rendered with `sample_count` samples."""
        aovs = fb.aovs()
        self._check(self.lib.shiro_gpu_accum_add(self._h, C.byref(aovs), fb.width, fb.height, int(sample_count)))

    def render_step(self, scene: Scene, camera: Camera, settings: RenderSettings, sample_start: int,
                    sample_count: int, flags: int = 0, cancel: Optional[C.c_int] = None, wavefront: bool = False):
        self.backend.upload_scene(scene)
        req = render_desc(camera, settings, sample_start, sample_count, flags)
        self._check(self.lib.shiro_gpu_accum_render(self._h, C.byref(req),
                                                    C.byref(cancel) if cancel is not None else None,
                                                    1 if wavefront else 0))

    def info(self) -> tuple:
        n, w, h = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self._check(self.lib.shiro_gpu_accum_info(self._h, C.byref(n), C.byref(w), C.byref(h)))
        return n.value, w.value, h.value

    def sample_count(self) -> int:
        return self.info()[0]

    def resolve(self, out: Optional[FrameBuffer] = None) -> FrameBuffer:
        """The accumulated frame, copied to the host once."""
        _, w, h = self.info()
        fb = out if out is not None else FrameBuffer(w, h)
        aovs = fb.aovs()
        self._check(self.lib.shiro_gpu_accum_resolve(self._h, C.byref(aovs)))
        return fb
