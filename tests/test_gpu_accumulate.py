"""The device-resident progressive accumulator against the host restatement of
Renderer::FrameAccumulator (Renderer.cpp:47-110).

The device applies the reference's float32 operations in the reference's
order (sum + frame * count; resolve by 1 / samples; depth over the samples
that hit), so its resolved frame must equal, bit for bit, the host
accumulation of the same batch frames.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from shiro_gb300 import GpuBackend

    with GpuBackend(0) as g:
        yield g


@pytest.fixture(scope="module")
def work():
    from shiro_gb300 import scenes

    # background hidden, so some pixels miss in every batch (depth stays +inf)
    w = scenes.sphere_workload(48, 40, 4, 6, env_width=64, env_height=32)
    w.settings.background_visible = False
    return w


def bits_equal(a, b):
    for k in ("beauty", "albedo", "normal", "depth"):
        x, y = getattr(a, k), getattr(b, k)
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32)), k


BATCHES = [(0, 4), (4, 4), (8, 8), (16, 3)]


def host_progressive(gpu, w, batches, wavefront=False):
    from shiro_gb300.replicas import FrameAccumulator

    acc = FrameAccumulator()
    for start, count in batches:
        if wavefront:
            (fb,) = gpu.render_batch(w.scene, [(w.camera, w.settings, start, count)])
        else:
            fb = gpu.render(w.scene, w.camera, w.settings, start, count)
        if start == 0 or acc.samples == 0:  # RenderParam.cpp:800-803
            acc.reset(fb.width, fb.height)
        acc.accumulate(fb, count)
    return acc.resolve(), acc.samples


@pytest.mark.parametrize("wavefront", [False, True])
def test_render_steps_equal_host_accumulation(gpu, work, wavefront):
    want, samples = host_progressive(gpu, work, BATCHES, wavefront)
    acc = gpu.accumulator()
    for start, count in BATCHES:
        acc.render_step(work.scene, work.camera, work.settings, start, count, wavefront=wavefront)
    assert acc.info() == (samples, work.settings.width, work.settings.height)
    got = acc.resolve()
    assert np.isinf(got.depth).any() and np.isfinite(got.depth).any()
    bits_equal(got, want)
    acc.close()


def test_host_frames_accumulate_like_the_reference(gpu, work):
    from shiro_gb300.replicas import FrameAccumulator

    frames = [(gpu.render(work.scene, work.camera, work.settings, s, c), c) for s, c in BATCHES]
    ref = FrameAccumulator()
    acc = gpu.accumulator()
    for fb, c in frames:
        ref.accumulate(fb, c)
        acc.accumulate(fb, c)
    bits_equal(acc.resolve(), ref.resolve())
    # an empty frame or zero samples change nothing
    acc.accumulate(frames[0][0], 0)
    assert acc.sample_count() == ref.samples


def test_restart_size_change_and_empty(gpu, work):
    from shiro_gb300.abi import FrameBuffer

    acc = gpu.accumulator()
    empty = acc.resolve()
    assert empty.width == 0 and acc.sample_count() == 0
    acc.reset(8, 4)
    cleared = acc.resolve()
    assert cleared.beauty.shape[0] == 32 and not cleared.beauty.any() and np.isinf(cleared.depth).all()
    acc.render_step(work.scene, work.camera, work.settings, 0, 4)
    acc.render_step(work.scene, work.camera, work.settings, 4, 4)
    assert acc.sample_count() == 8
    # a batch at sample 0 starts over
    acc.render_step(work.scene, work.camera, work.settings, 0, 2)
    assert acc.sample_count() == 2
    single = gpu.render(work.scene, work.camera, work.settings, 0, 2)
    got = acc.resolve()
    # one batch: sum = frame * 2, resolved as sum * (1/2)
    np.testing.assert_array_equal(got.beauty, (single.beauty * np.float32(2)) * (np.float32(1) / np.float32(2)))
    # a frame of another size resets the sums
    small = FrameBuffer(4, 4)
    small.beauty[:] = 1.0
    acc.accumulate(small, 3)
    assert acc.info() == (3, 4, 4)
    np.testing.assert_array_equal(acc.resolve().beauty, np.ones_like(small.beauty))


def test_cancelled_batch_not_accumulated(gpu, work):
    from shiro_gb300 import abi
    from shiro_gb300.backend import ShiroGpuError

    acc = gpu.accumulator()
    acc.render_step(work.scene, work.camera, work.settings, 0, 4)
    before = acc.resolve()
    cancel = C.c_int(1)
    with pytest.raises(ShiroGpuError) as e:
        acc.render_step(work.scene, work.camera, work.settings, 4, 4, cancel=cancel)
    assert e.value.code == abi.SHIRO_ERR_CANCELLED
    assert acc.sample_count() == 4
    bits_equal(acc.resolve(), before)
