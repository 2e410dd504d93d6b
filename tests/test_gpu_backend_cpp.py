"""The C++ RenderBackend adapter (shiro_gb300/backend/GpuBackend.cpp) driven
as Renderer::RenderSampleBatch drives a backend: a renderer-owned Scene
snapshot in, a FrameBuffer out.  Its frames must equal the C ABI's."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def backend_lib():
    from shiro_gb300 import build

    path = build.build_backend()
    lib = C.CDLL(path)
    lib.shiro_backend_selftest.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32]
    lib.shiro_backend_selftest.restype = C.c_int
    return lib


@pytest.fixture(scope="module")
def gpu():
    from shiro_gb300 import GpuBackend

    with GpuBackend(0) as g:
        yield g


def test_render_sample_batch_through_adapter(backend_lib, gpu):
    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer, MarshalledScene, render_desc

    w = scenes.sphere_workload(48, 40, 4, 6, env_width=128, env_height=64)
    ms = MarshalledScene(w.scene)
    req = render_desc(w.camera, w.settings, 2, 4)
    fb = FrameBuffer(48, 40)
    aov = fb.aovs()
    assert backend_lib.shiro_backend_selftest(ms.ref(), C.byref(req), 1, C.byref(aov), 0, 0) == 1
    ref = gpu.render(w.scene, w.camera, w.settings, 2, 4)
    for k in ("beauty", "albedo", "normal", "depth"):
        assert np.array_equal(getattr(fb, k), getattr(ref, k)), k


def test_batched_requests_through_adapter(backend_lib, gpu):
    from shiro_gb300 import scenes
    from shiro_gb300.abi import Aovs, FrameBuffer, MarshalledScene, RenderDesc, render_desc

    scene = scenes.sphere_scene(env_width=64, env_height=32)
    reqs = scenes.batch_requests(count=3, seed=2, lo=16, hi=32)
    ms = MarshalledScene(scene)
    descs = (RenderDesc * 3)(*[render_desc(r.camera, r.settings, 0, r.settings.samples_per_pixel) for r in reqs])
    fbs = [FrameBuffer(r.settings.width, r.settings.height) for r in reqs]
    outs = (Aovs * 3)(*[f.aovs() for f in fbs])
    assert backend_lib.shiro_backend_selftest(ms.ref(), descs, 3, outs, 0, 0) == 1
    for r, fb in zip(reqs, fbs):
        ref = gpu.render(scene, r.camera, r.settings)
        assert np.array_equal(fb.beauty, ref.beauty)


def test_emissive_scene_renders_through_adapter(backend_lib, gpu):
    """A scene with an emitter (once declined by SupportsScene) now renders on
    the GPU through the adapter and equals the direct C ABI render."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer, MarshalledScene, render_desc

    w = scenes.sphere_workload(8, 8, 1, 2, env_width=16, env_height=8)
    w.scene.materials[0].emission_strength = 2.0
    w.scene.materials[0].emission_color = (1.0, 1.0, 1.0)
    fb = FrameBuffer(8, 8)
    aov = fb.aovs()
    req = render_desc(w.camera, w.settings, 0, 1)
    assert backend_lib.shiro_backend_selftest(MarshalledScene(w.scene).ref(), C.byref(req), 1, C.byref(aov), 0, 0) == 1
    ref = gpu.render(w.scene, w.camera, w.settings, 0, 1)
    assert np.array_equal(fb.beauty, ref.beauty)


@pytest.mark.parametrize("wavefront", [0, 1])
def test_progressive_accumulation_through_adapter(backend_lib, gpu, wavefront):
    """RenderAndAccumulate steps + ResolveAccumulation (sums kept on the
    device) equal the host FrameAccumulator over the same batch frames."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer, MarshalledScene, RenderDesc, render_desc
    from shiro_gb300.replicas import FrameAccumulator

    w = scenes.sphere_workload(40, 32, 4, 6, env_width=64, env_height=32)
    batches = [(0, 4), (4, 2), (6, 6)]
    descs = (RenderDesc * 3)(*[render_desc(w.camera, w.settings, s0, c) for s0, c in batches])
    fb = FrameBuffer(40, 32)
    aov = fb.aovs()
    assert backend_lib.shiro_backend_selftest(MarshalledScene(w.scene).ref(), descs, 3, C.byref(aov), 1,
                                              wavefront) == 1
    acc = FrameAccumulator()
    for s0, c in batches:
        acc.accumulate(gpu.render(w.scene, w.camera, w.settings, s0, c), c)
    ref = acc.resolve()
    for k in ("beauty", "albedo", "normal", "depth"):
        assert np.array_equal(getattr(fb, k).view(np.uint32), getattr(ref, k).view(np.uint32)), k
