"""The batched wavefront form against the plain megakernel.

Both forms evaluate every float of a path with the same integrator functions
in the same order, so the wavefront frames must be bit-identical to the plain
ones (and thereby carry the plain form's parity with the CPU oracle), for any
pool size, block sizes, graph or direct launches, and any mix of requests.
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


def same(a, b):
    for k in ("beauty", "albedo", "normal", "depth"):
        x, y = getattr(a, k), getattr(b, k)
        if not np.array_equal(x.view(np.uint32), y.view(np.uint32)):
            return False, k, int(np.count_nonzero(x.view(np.uint32) != y.view(np.uint32)))
    return True, None, 0


def test_single_request_bit_identical(gpu):
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(64, 48, 8, 8, env_width=128, env_height=64)
    plain = gpu.render(w.scene, w.camera, w.settings)
    (wave,) = gpu.render_batch(w.scene, [(w.camera, w.settings)])
    ok, k, n = same(plain, wave)
    assert ok, (k, n)


@pytest.mark.parametrize("flags", [0, 1, 2])
def test_field_scene_bit_identical(gpu, flags):
    from shiro_gb300 import scenes

    sc = scenes.field_scene(instances=16, levels=4, materials=8, env_width=256, env_height=128, seed=5, plane=14.0)
    st = scenes.RenderSettings(width=80, height=45, samples_per_pixel=6, max_depth=12, diffuse_depth=12,
                               specular_depth=12, backend=1)
    cam = scenes.look_at((0.0, 4.0, 9.0), (0.0, 0.3, 0.0), 45.0, 80 / 45)
    plain = gpu.render(sc, cam, st, 3, 6, flags=flags)
    (wave,) = gpu.render_batch(sc, [(cam, st, 3, 6)], flags=flags)
    ok, k, n = same(plain, wave)
    assert ok, (k, n)


@pytest.mark.parametrize("name", ["emissive", "opacity", "transmission"])
def test_extended_lobes_bit_identical(gpu, name):
    """Transmission and media, opacity cut-outs and emitters: the wavefront
    stages (pass-through hits, the emissive light sample with its finite
    shadow ray, medium state across bounces) match the plain form."""
    from conftest import golden
    from scene_io import camera_from_array, scene_from_arrays, settings_from_array

    g = golden(f"render_{name}.npz")
    sc, cam, st = scene_from_arrays(g), camera_from_array(g["cam"]), settings_from_array(g["settings"])
    plain = gpu.render(sc, cam, st, 0, 16)
    (wave,) = gpu.render_batch(sc, [(cam, st, 0, 16)])
    ok, k, n = same(plain, wave)
    assert ok, (name, k, n)


@pytest.mark.parametrize("pool", [0, 4096])
def test_page_locked_planes_written_in_place(gpu, pool):
    """Page-locked host planes are written by the resolve stage in place
    (wave by wave, several waves with a small pool); pageable ones go through
    device staging and one copy.  Both hold the plain frame bit for bit, in a
    batch that mixes the two kinds and a frame whose width makes the beauty
    plane's pixels of odd pixel count (so the albedo / normal planes start off
    16-byte boundaries)."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer

    w = scenes.sphere_workload(37, 23, 6, 6, env_width=64, env_height=32)
    w2 = scenes.sphere_workload(64, 48, 4, 8, env_width=64, env_height=32)
    plain = gpu.render(w.scene, w.camera, w.settings)
    plain2 = gpu.render(w.scene, w2.camera, w2.settings)  # one scene; the second request's camera / settings
    base = gpu.wavefront_config()
    if pool:
        gpu.set_wavefront_config(paths_in_flight=pool, concurrent_waves=2)
    try:
        for _ in range(2):  # again into the same (reused) buffers
            fbs = [FrameBuffer(37, 23, pinned=True), FrameBuffer(64, 48), FrameBuffer(37, 23)]
            outs = gpu.render_batch(w.scene, [(w.camera, w.settings), (w2.camera, w2.settings),
                                              (w.camera, w.settings)], outs_fb=fbs)
            for fb, ref in zip(outs, (plain, plain2, plain)):
                ok, k, n = same(ref, fb)
                assert ok, (pool, k, n)
            pinned2 = [FrameBuffer(64, 48, pinned=True)]
            (fb2,) = gpu.render_batch(w.scene, [(w2.camera, w2.settings)], outs_fb=pinned2)
            ok, k, n = same(plain2, fb2)
            assert ok, (pool, k, n)
    finally:
        gpu.set_wavefront_config(**base)


@pytest.mark.parametrize("pool", [0, 4096])
def test_ready_ranges_cover_every_pixel_once(gpu, pool):
    """shiro_gpu_render_batch_ready reports every pixel of every request once,
    the ranges of a request in increasing order: page-locked planes wave by
    wave (several ranges with a pool of 4 096 paths), pageable planes and a
    request without samples whole after the render.  A range of page-locked
    planes already holds its final values when it is reported, and the
    frames equal the plain ones bit for bit."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer

    w = scenes.sphere_workload(37, 23, 6, 6, env_width=64, env_height=32)
    w2 = scenes.sphere_workload(64, 48, 4, 8, env_width=64, env_height=32)
    plain = gpu.render(w.scene, w.camera, w.settings)
    plain2 = gpu.render(w.scene, w2.camera, w2.settings)
    fbs = [FrameBuffer(37, 23, pinned=True), FrameBuffer(64, 48), FrameBuffer(64, 48, pinned=True),
           FrameBuffer(37, 23, pinned=True)]
    reqs = [(w.camera, w.settings), (w2.camera, w2.settings), (w2.camera, w2.settings), (w.camera, w.settings, 0, 0)]
    refs = [plain, plain2, plain2, None]
    seen, final_when_reported = [], []

    def ready(r, first, count):
        seen.append((r, first, count))
        if r in (0, 2):  # page-locked planes written in place
            got = fbs[r].beauty[first:first + count].view(np.uint32)
            final_when_reported.append(np.array_equal(got, refs[r].beauty[first:first + count].view(np.uint32)))

    base = gpu.wavefront_config()
    if pool:
        gpu.set_wavefront_config(paths_in_flight=pool, concurrent_waves=2)
    try:
        outs = gpu.render_batch(w.scene, reqs, outs_fb=fbs, ready=ready)
    finally:
        gpu.set_wavefront_config(**base)
    assert final_when_reported and all(final_when_reported)
    for r, fb in enumerate(outs):
        pos = 0
        for rr, first, count in seen:
            if rr == r:
                assert first == pos and count > 0, (r, first, pos)
                pos += count
        assert pos == fb.width * fb.height, r
    count = [sum(1 for x in seen if x[0] == r) for r in range(4)]
    assert count[1] == 1 and count[3] == 1
    if pool:
        assert count[0] > 1 and count[2] > 1
    for fb, ref in zip(outs[:3], refs[:3]):
        ok, k, n = same(ref, fb)
        assert ok, (pool, k, n)
    assert not outs[3].beauty.any() and np.isinf(outs[3].depth).all()


def test_mixed_dome_samples_in_batch(gpu):
    """Requests of one batch with different dome-sample counts each use their
    own light samples."""
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(24, 16, 4, 5, env_width=64, env_height=32)
    a = w.settings
    b = scenes.RenderSettings(**{**a.__dict__, "dome_light_samples": 3})
    outs = gpu.render_batch(w.scene, [(w.camera, a), (w.camera, b)])
    assert same(outs[0], gpu.render(w.scene, w.camera, a))[0]
    assert same(outs[1], gpu.render(w.scene, w.camera, b))[0]


def test_uneven_batch_small_pool(gpu):
    """Many requests of uneven size / spp / depth, packed into waves much
    smaller than a frame (pixels of one request straddle several waves)."""
    from shiro_gb300 import scenes

    scene = scenes.sphere_scene(env_width=128, env_height=64)
    reqs = scenes.batch_requests(count=7, seed=11, lo=8, hi=40)
    gpu.set_wavefront_config(paths_in_flight=4096, extend_block=64, shade_block=256, shadow_block=128, use_graph=1)
    try:
        outs = gpu.render_batch(scene, [(r.camera, r.settings) for r in reqs])
        for r, fb in zip(reqs, outs):
            ref = gpu.render(scene, r.camera, r.settings)
            ok, k, n = same(ref, fb)
            assert ok, (r.settings.width, r.settings.samples_per_pixel, k, n)
    finally:
        gpu.set_wavefront_config(paths_in_flight=1 << 22, extend_block=128, shade_block=128, shadow_block=128,
                                 use_graph=1)


@pytest.mark.parametrize("pool", [4096, 5000])
def test_two_waves_in_flight_uneven_batch(gpu, pool):
    """Two pools, each on its own stream, take alternate waves (an odd and an
    even count of waves, requests straddling waves of both pools): frames
    equal the plain ones bit for bit, and a second call reuses both graphs."""
    from shiro_gb300 import scenes

    scene = scenes.sphere_scene(env_width=128, env_height=64)
    reqs = scenes.batch_requests(count=7, seed=11, lo=8, hi=40)
    base = gpu.wavefront_config()
    gpu.set_wavefront_config(paths_in_flight=pool, concurrent_waves=2, use_graph=1)
    try:
        for _ in range(2):
            outs = gpu.render_batch(scene, [(r.camera, r.settings) for r in reqs])
            assert gpu.last_stats()["waves"] >= 3
            for r, fb in zip(reqs, outs):
                ref = gpu.render(scene, r.camera, r.settings)
                ok, k, n = same(ref, fb)
                assert ok, (pool, r.settings.width, r.settings.samples_per_pixel, k, n)
    finally:
        gpu.set_wavefront_config(**base)
    assert gpu.wavefront_config()["concurrent_waves"] == base["concurrent_waves"]


@pytest.mark.parametrize("knobs", [dict(shade_regs=96), dict(shade_regs=80), dict(extend_steps=1, refill_idle=1),
                                   dict(extend_steps=32, refill_idle=32), dict(extend_steps=3, refill_idle=5),
                                   dict(concurrent_waves=2, paths_in_flight=2048),
                                   dict(concurrent_waves=1, paths_in_flight=2048),
                                   dict(bin_rays=1, bin_shadow=1), dict(bin_rays=1, bin_shadow=2),
                                   dict(bin_rays=2, bin_shadow=1, concurrent_waves=2, paths_in_flight=2048),
                                   dict(bin_rays=1, bin_shadow=1, use_graph=1),
                                   dict(coop_extend=1, coop_occlude=1), dict(coop_extend=1, coop_occlude=2, refill_idle=1),
                                   dict(coop_extend=2, coop_occlude=1, concurrent_waves=2, paths_in_flight=2048),
                                   dict(coop_extend=1, coop_occlude=1, bin_rays=1, bin_shadow=1, refill_idle=32),
                                   dict(extend_regs=48, occlude_regs=40), dict(extend_regs=40, occlude_regs=48),
                                   dict(occlude_refill=1), dict(occlude_refill=1, extend_steps=1, refill_idle=32),
                                   dict(occlude_refill=1, bin_shadow=1, concurrent_waves=2, paths_in_flight=2048),
                                   dict(concurrent_waves=3, paths_in_flight=2048),
                                   dict(concurrent_waves=4, paths_in_flight=1024, coop_occlude=1)])
def test_tuning_knobs_keep_frames_identical(gpu, knobs):
    """Register cap of the shade stage, the lane-refill parameters of the
    wide-BVH extend stage, the binning of the ray / occlusion queues and the
    warp-cooperative triangle tests change scheduling only."""
    from shiro_gb300 import scenes

    sc = scenes.field_scene(instances=12, levels=4, materials=6, env_width=128, env_height=64, seed=9, plane=12.0)
    st = scenes.RenderSettings(width=64, height=36, samples_per_pixel=4, max_depth=8, diffuse_depth=8,
                               specular_depth=8, backend=1)
    cam = scenes.look_at((0.0, 3.5, 8.0), (0.0, 0.3, 0.0), 45.0, 64 / 36)
    plain = gpu.render(sc, cam, st)
    base = gpu.wavefront_config()
    gpu.set_wavefront_config(**knobs)
    try:
        (wave,) = gpu.render_batch(sc, [(cam, st)])
    finally:
        gpu.set_wavefront_config(**base)
    ok, k, n = same(plain, wave)
    assert ok, (knobs, k, n)


def test_direct_launch_matches_graph_and_reports_stages(gpu):
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(40, 40, 4, 6, env_width=64, env_height=32)
    (a,) = gpu.render_batch(w.scene, [(w.camera, w.settings)])
    gpu.set_wavefront_config(use_graph=0)
    try:
        (b,) = gpu.render_batch(w.scene, [(w.camera, w.settings)])
        st = gpu.last_stats()
    finally:
        gpu.set_wavefront_config(use_graph=1)
    assert same(a, b)[0]
    assert st["stage_launches"][1] >= 6 and st["stage_ms"][1] > 0.0
    assert st["paths"] == 40 * 40 * 4


def test_zero_sample_request_in_batch(gpu):
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(16, 16, 4, 4, env_width=32, env_height=16)
    outs = gpu.render_batch(w.scene, [(w.camera, w.settings, 0, 0), (w.camera, w.settings, 0, 4)])
    assert (outs[0].beauty == 0).all() and np.isinf(outs[0].depth).all()
    assert same(outs[1], gpu.render(w.scene, w.camera, w.settings))[0]


def test_autotune_picks_a_valid_config(gpu):
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(128, 128, 16, 8, env_width=128, env_height=64)
    cfg = gpu.autotune(w.scene, w.camera, w.settings)
    assert cfg["paths_in_flight"] >= 1 << 20
    assert cfg["extend_block"] in (64, 128, 256) and cfg["shade_block"] in (64, 128, 256)
    (fb,) = gpu.render_batch(w.scene, [(w.camera, w.settings)])
    assert same(fb, gpu.render(w.scene, w.camera, w.settings))[0]


def test_cancel_batch(gpu):
    from shiro_gb300 import ShiroGpuError, scenes

    from shiro_gb300.abi import FrameBuffer

    w = scenes.sphere_workload(16, 16, 4, 4, env_width=32, env_height=16)
    fb = FrameBuffer(16, 16)
    fb.beauty[:] = 7.0
    fb.depth[:] = 1.0
    with pytest.raises(ShiroGpuError) as ei:
        gpu.render_batch(w.scene, [(w.camera, w.settings)], cancel=C.c_int(1), outs_fb=[fb])
    assert ei.value.code == -6
    # the discarded batch leaves cleared planes (FrameBuffer::Clear)
    assert not fb.beauty.any() and np.isinf(fb.depth).all()


@pytest.mark.parametrize("form", ["plain", "wavefront"])
def test_cancel_flag_set_by_another_thread_mid_frame(form):
    """The C ABI polls its cancel flag between launches / waves that have run
    (it does not queue the whole frame ahead), so a flag another host thread
    sets mid-frame stops the render: SHIRO_ERR_CANCELLED, cleared AOVs, fewer
    waves than the frame has, and an early return."""
    import ctypes as C
    import threading
    import time

    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import FrameBuffer

    w = scenes.sphere_workload(1920, 1080, 128, 8, env_width=128, env_height=64)
    with GpuBackend(0) as gpu:
        gpu.upload_scene(w.scene)
        # waves of 8 M paths: dozens per frame (a cancel takes effect after the
        # waves already queued, waves in flight + 1, so their size bounds it)
        gpu.set_wavefront_config(paths_in_flight=1 << 23)
        render = (lambda fb, cancel: gpu.render_batch(w.scene, [(w.camera, w.settings)], cancel=cancel, outs_fb=[fb])) \
            if form == "wavefront" else (lambda fb, cancel: gpu.render(w.scene, w.camera, w.settings, cancel=cancel,
                                                                        out=fb))
        fb = FrameBuffer(1920, 1080)
        t0 = time.perf_counter()
        render(fb, C.c_int(0))
        full = time.perf_counter() - t0
        full_waves = gpu.last_stats()["waves"] if form == "wavefront" else None
        flag = C.c_int(0)
        timer = threading.Timer(0.1 * full, lambda: setattr(flag, "value", 1))
        fb2 = FrameBuffer(1920, 1080)
        fb2.beauty[:] = 1.0
        timer.start()
        t0 = time.perf_counter()
        with pytest.raises(Exception) as ei:
            render(fb2, flag)
        took = time.perf_counter() - t0
        timer.join()
        assert getattr(ei.value, "code", None) == -6, ei.value
        assert took < 0.6 * full, (took, full)
        assert not fb2.beauty.any() and not fb2.albedo.any() and np.isinf(fb2.depth).all()
        if form == "wavefront":
            assert gpu.last_stats()["waves"] < full_waves
