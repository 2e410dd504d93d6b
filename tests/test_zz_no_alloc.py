"""shiro_gpu_render_static: the render entry point for callers that must not
allocate device memory while rendering.  It takes its path-record scratch
from an array reserved in the library's device image (set up when the context
is created), so it must produce the same frame as shiro_gpu_render (same
kernels), on two calls in a row, without the device's free memory moving
across either call - the first one included.

This file is collected last on purpose (test_zz_*): a failure here leaves every
other test already run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATIC_PATHS = 1 << 20


def _device_aovs(torch, n):
    planes = {k: torch.zeros(n * c, dtype=torch.float32, device="cuda") for k, c in
              (("beauty", 4), ("albedo", 3), ("normal", 3), ("depth", 1))}
    return planes


def test_static_scratch_render_matches_render():
    torch = pytest.importorskip("torch")
    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import Aovs, render_desc

    gpu = GpuBackend(0)
    lib = gpu.lib
    lib.shiro_gpu_render_static.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.shiro_gpu_render_static.restype = C.c_int
    torch.cuda.init()
    stream = torch.cuda.current_stream()
    lib.shiro_gpu_set_stream(gpu.handle, stream.cuda_stream)

    # 192 x 128 x 48 spp = 1.18 M paths: more than one launch of the static array.
    # The context exists and has rendered once (the CUDA driver sizes the
    # kernels' thread-local memory at their first launch) before the first
    # static call; from then on the device's free memory must not move at all.
    w = scenes.sphere_workload(192, 128, 48, 8, env_width=128, env_height=64)
    ref = gpu.render(w.scene, w.camera, w.settings)
    npx = 192 * 128
    req = render_desc(w.camera, w.settings, 0, 48)
    calls = [_device_aovs(torch, npx) for _ in range(2)]
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for call, planes in enumerate(calls):
        aov = Aovs(*[C.cast(C.c_void_p(planes[k].data_ptr()), C.POINTER(C.c_float))
                     for k in ("beauty", "albedo", "normal", "depth")], 1, 0)
        rc = lib.shiro_gpu_render_static(gpu.handle, C.byref(req), None, C.byref(aov))
        assert rc == 0, lib.shiro_gpu_last_error(gpu.handle).decode()
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before, f"device memory moved during static call {call}"
        got = {k: v.cpu().numpy() for k, v in planes.items()}
        for k in ("beauty", "albedo", "normal", "depth"):
            assert np.array_equal(got[k], getattr(ref, k).reshape(-1)), (call, k)
    del calls

    # limits: more samples per pixel than the array holds, and host planes
    big = render_desc(w.camera, w.settings, 0, STATIC_PATHS + 1)
    planes = _device_aovs(torch, npx)
    aov = Aovs(*[C.cast(C.c_void_p(planes[k].data_ptr()), C.POINTER(C.c_float))
                 for k in ("beauty", "albedo", "normal", "depth")], 1, 0)
    assert lib.shiro_gpu_render_static(gpu.handle, C.byref(big), None, C.byref(aov)) == -1
    assert b"exceeds the static scratch capacity" in lib.shiro_gpu_last_error(gpu.handle)
    host = ref.aovs()
    assert lib.shiro_gpu_render_static(gpu.handle, C.byref(req), None, C.byref(host)) == -1
    gpu.close()
