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
    from tests.cpp.harness import load_harness

    return load_harness()


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


def _cleared(fb):
    return (not fb.beauty.any() and not fb.albedo.any() and not fb.normal.any()
            and np.isinf(fb.depth).all())


def test_cancel_set_mid_frame_through_adapter(backend_lib, gpu):
    """Hydra cancels from another thread while a frame renders
    (RenderBackend.h:18, RenderParam.cpp:790-798): the adapter forwards the
    std::atomic<bool> to the device render, which stops between waves; the
    call returns early with SHIRO_ERR_CANCELLED and a cleared frame."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer, MarshalledScene, render_desc

    # 1920 x 1080 x 256 spp on the sphere scene: 16 waves of the default 32 M
    # paths; a cancel stops the render after the waves already queued (waves in
    # flight + 1)
    w = scenes.sphere_workload(1920, 1080, 256, 8, env_width=128, env_height=64)
    ms = MarshalledScene(w.scene)
    req = render_desc(w.camera, w.settings, 0, 256)
    fb = FrameBuffer(1920, 1080)
    aov = fb.aovs()
    status, elapsed = C.c_int(0), C.c_double(0.0)
    # uncancelled (flag set long after the frame) for the full duration
    assert backend_lib.shiro_harness_cancel_midframe(ms.ref(), C.byref(req), 60000.0, 0, C.byref(aov),
                                                     C.byref(status), C.byref(elapsed)) == 1
    assert status.value == 0
    full = elapsed.value
    assert not _cleared(fb)
    for mode in (0, 1):
        fb2 = FrameBuffer(1920, 1080)
        aov2 = fb2.aovs()
        assert backend_lib.shiro_harness_cancel_midframe(ms.ref(), C.byref(req), 0.1 * full, mode, C.byref(aov2),
                                                         C.byref(status), C.byref(elapsed)) == 1
        assert status.value == -6, (mode, status.value)  # SHIRO_ERR_CANCELLED; mode 1: not accumulated
        assert elapsed.value < 0.6 * full, (mode, elapsed.value, full)
        if mode == 0:
            assert _cleared(fb2)


def test_scene_edited_in_place_is_uploaded_again(backend_lib, gpu):
    """A light or a vertex changed inside the same Scene object (Hydra may
    also place a new snapshot at a freed address, RenderParam.cpp:614-659)
    must not render from the stale device copy."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer, MarshalledScene, render_desc

    from shiro_gb300.abi import DistantLight

    w = scenes.sphere_workload(40, 32, 2, 4, env_width=32, env_height=16)
    w.scene.distant_lights = [DistantLight(direction=(-0.3, -1.0, -0.4), radiance=(2.5, 2.4, 2.2))]
    ms = MarshalledScene(w.scene)
    req = render_desc(w.camera, w.settings, 0, 2)
    fbs = [FrameBuffer(40, 32) for _ in range(3)]
    from shiro_gb300.abi import Aovs
    outs = (Aovs * 3)(*[f.aovs() for f in fbs])
    uploads = (C.c_uint64 * 3)()
    rad = (C.c_float * 3)(7.0, 3.0, 1.0)
    off = (C.c_float * 3)(0.0, 0.25, 0.0)
    assert backend_lib.shiro_harness_edit_in_place(ms.ref(), C.byref(req), rad, off, outs, uploads) == 1
    assert uploads[1] == uploads[0] + 1 and uploads[2] == uploads[1] + 1
    expected = []
    expected.append(gpu.render(w.scene, w.camera, w.settings, 0, 2))
    w.scene.distant_lights[0].radiance = (7.0, 3.0, 1.0)
    expected.append(gpu.render(w.scene, w.camera, w.settings, 0, 2))
    m0 = w.scene.meshes[0]
    m0.positions = np.array(m0.positions, dtype=np.float32, copy=True)
    m0.positions[0] += np.array([0.0, 0.25, 0.0], dtype=np.float32)
    expected.append(gpu.render(w.scene, w.camera, w.settings, 0, 2))
    for k in range(3):
        for name in ("beauty", "albedo", "normal", "depth"):
            assert np.array_equal(getattr(fbs[k], name), getattr(expected[k], name)), (k, name)
    assert not np.array_equal(fbs[0].beauty, fbs[1].beauty)
