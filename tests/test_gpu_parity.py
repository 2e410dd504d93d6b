"""GPU parity of the plain megakernel against the CPU oracle and the
reference's golden vectors, through the C ABI.

Tolerances:
* hits, t, occlusion: bit-exact (same Moller-Trumbore arithmetic, no FMA);
* camera rays: bit-exact given the same std::tan of the field of view;
* frames: a path is a deterministic function of (pixel, sample), so the GPU
  and the oracle trace the same paths; transcendental functions differ by an
  ulp or two between CUDA and glibc, which very rarely flips a discrete
  decision.  A pixel matches when every channel agrees to rtol 1e-3 /
  atol 1e-4; at least 97 % of pixels must match and the frame mean must agree
  to 1 %.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from oracle import api
from conftest import golden
from scene_io import camera_from_array, scene_from_arrays, settings_from_array

pytestmark = pytest.mark.gpu

PIX_RTOL, PIX_ATOL, MIN_MATCH, MEAN_TOL = 1e-3, 1e-4, 0.97, 0.01


@pytest.fixture(scope="module")
def gpu():
    from shiro_gb300 import GpuBackend

    with GpuBackend(0) as g:
        yield g


@pytest.fixture(scope="module")
def port():
    oracle.build_port()
    return oracle.port_checker()


def frame_match(a, b):
    close = np.isclose(a.beauty, b.beauty, rtol=PIX_RTOL, atol=PIX_ATOL).all(1)
    ma, mb = a.beauty[:, :3].mean(), b.beauty[:, :3].mean()
    return close.mean(), abs(ma - mb) / max(mb, 1e-6)


def test_status(gpu):
    st = gpu.get_status()
    assert st["available"] and st["compute"] == (10, 3), st


def test_random_rays_match_golden(gpu):
    g = golden("hits_sphere.npz")
    scene = scene_from_arrays(g)
    prim, t, occ = gpu.trace_rays(scene, g["ray_o"], g["ray_d"], g["ray_tmax"])
    assert np.array_equal(prim, g["ray_prim"])
    assert np.array_equal(t, g["ray_t"])
    assert np.array_equal(occ, g["ray_occ"])


def test_primary_hits_match_golden_and_oracle(gpu, port):
    g = golden("hits_sphere.npz")
    scene = scene_from_arrays(g)
    cam = camera_from_array(g["cam"])
    st = settings_from_array(g["settings"])
    for k in range(3):
        start = int(g[f"start{k}"])
        prim, t = gpu.primary_hits(scene, cam, st, start)
        pp, pt = api.primary_hits(port, scene, cam, st, start)
        assert np.array_equal(prim, pp) and np.array_equal(t, pt)
        assert (prim == g[f"prim{k}"]).mean() > 0.999


def test_field_rays_vs_bruteforce(gpu, port):
    from shiro_gb300 import scenes

    scene = scenes.field_scene(instances=24, levels=4, materials=4, env_width=16, env_height=8, seed=21, plane=16.0)
    rng = np.random.default_rng(7)
    n = 40000
    o = rng.uniform(-8, 8, (n, 3)).astype(np.float32)
    o[:, 1] = rng.uniform(0.02, 3.0, n)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tmax = rng.uniform(0.2, 30.0, n).astype(np.float32)
    prim, t, occ = gpu.trace_rays(scene, o, d, tmax)
    bp, bt, bo = api.trace_rays(port, scene, o, d, tmax, bruteforce=True)
    assert np.array_equal(prim, bp)
    assert np.array_equal(t, bt)
    assert np.array_equal(occ, bo)


def test_sampler_kat_bit_exact(gpu):
    """The device sampler on the 64 000 reference tuples (pixels, sample
    indices up to 2^32 - 1, branches over every prime base): bit for bit."""
    g = golden("sampler_kat.npz")
    out = gpu.sample(g["px"], g["py"], g["index"], g["branch"])
    assert (out.view(np.uint32) == g["out"].view(np.uint32)).all()


# progressive_batch3: the third consecutive batch of one reference tracer,
# matched by a single render of that batch (the reference's path guide,
# CpuPathTracer.cpp:1953-1987, never becomes active: its weights start at zero
# and grow only through records pushed while it is active)
RENDERS = ["sphere", "rich", "features_gradient_env", "angular_env", "field_small", "sphere_1spp_start5", "emissive",
           "opacity", "transmission", "progressive_batch3", "degenerate"]


@pytest.mark.parametrize("name", RENDERS)
def test_render_vs_oracle_and_golden(gpu, port, name):
    g = golden(f"render_{name}.npz")
    scene = scene_from_arrays(g)
    cam = camera_from_array(g["cam"])
    st = settings_from_array(g["settings"])
    start, count = int(g["start"]), int(g["count"])
    fb = gpu.render(scene, cam, st, start, count, flags=1)  # CDF env sampling: reference texel mapping
    ref = api.render(port, scene, cam, st, start, count)
    frac, mean = frame_match(fb, ref)
    assert frac >= MIN_MATCH and mean <= MEAN_TOL, (frac, mean)
    # the golden frame itself (produced by the reference)
    close = np.isclose(fb.beauty, g["beauty"], rtol=PIX_RTOL, atol=PIX_ATOL).all(1).mean()
    assert close >= MIN_MATCH
    # first-hit AOVs
    hit = np.isfinite(ref.depth)
    assert np.array_equal(np.isfinite(fb.depth), hit)
    np.testing.assert_allclose(fb.depth[hit], ref.depth[hit], rtol=1e-5)
    np.testing.assert_allclose(fb.albedo, ref.albedo, rtol=1e-4, atol=1e-6)
    assert (np.isclose(fb.normal, ref.normal, rtol=1e-4, atol=1e-5).all(1)).mean() > 0.999


def test_alias_sampling_matches_cdf_statistically(gpu):
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(64, 64, 64, 6, env_width=128, env_height=64)
    a = gpu.render(w.scene, w.camera, w.settings, 0, 64, flags=0)
    b = gpu.render(w.scene, w.camera, w.settings, 0, 64, flags=1)
    ma, mb = a.beauty[:, :3].mean(), b.beauty[:, :3].mean()
    assert abs(ma - mb) < 0.03 * mb, (ma, mb)
    assert np.array_equal(a.depth, b.depth)


def test_deterministic(gpu):
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(40, 30, 8, 8, env_width=64, env_height=32)
    a = gpu.render(w.scene, w.camera, w.settings)
    b = gpu.render(w.scene, w.camera, w.settings)
    for k in ("beauty", "albedo", "normal", "depth"):
        assert np.array_equal(getattr(a, k), getattr(b, k))


def test_sample_count_zero_clears(gpu):
    from shiro_gb300 import scenes

    w = scenes.sphere_workload(16, 8, 4, 4, env_width=32, env_height=16)
    fb = gpu.render(w.scene, w.camera, w.settings, 0, 0)
    assert (fb.beauty == 0).all() and np.isinf(fb.depth).all()


def test_single_pixel_and_odd_sizes(gpu, port):
    from shiro_gb300 import scenes

    for wd, ht in ((1, 1), (7, 3), (33, 17)):
        w = scenes.sphere_workload(wd, ht, 3, 5, env_width=32, env_height=16)
        fb = gpu.render(w.scene, w.camera, w.settings, 2, 3, flags=1)
        ref = api.render(port, w.scene, w.camera, w.settings, 2, 3)
        frac, mean = frame_match(fb, ref)
        assert frac >= 0.9 and mean < 0.05


@pytest.mark.parametrize("depths", [(0, 0, 0), (1, 1, 1), (4, 0, 4), (4, 4, 0), (3, 1, 0)])
def test_depth_limits(gpu, port, depths):
    """max / diffuse / specular depth limits, zero included (TracePath then
    traces nothing and the frame is cleared): plain and wavefront forms (into
    device staging and into page-locked planes) match the port."""
    import dataclasses

    from shiro_gb300 import scenes
    from shiro_gb300.abi import FrameBuffer

    w = scenes.sphere_workload(24, 16, 4, 4, env_width=32, env_height=16)
    md, dd, sd = depths
    st = dataclasses.replace(w.settings, max_depth=md, diffuse_depth=dd, specular_depth=sd)
    ref = api.render(port, w.scene, w.camera, st, 0, 4)
    fb = gpu.render(w.scene, w.camera, st, 0, 4, flags=1)
    frac, mean = frame_match(fb, ref)
    assert frac >= MIN_MATCH and mean <= MEAN_TOL, (frac, mean)
    assert np.array_equal(np.isfinite(fb.depth), np.isfinite(ref.depth))
    for pinned in (False, True):
        outs = [FrameBuffer(24, 16, pinned=pinned)]
        for p in (outs[0].beauty, outs[0].albedo, outs[0].normal, outs[0].depth):
            p[...] = 7.0  # stale values the render must overwrite
        (wave,) = gpu.render_batch(w.scene, [(w.camera, st, 0, 4)], flags=1, outs_fb=outs)
        for k in ("beauty", "albedo", "normal", "depth"):
            assert np.array_equal(getattr(wave, k).view(np.uint32), getattr(fb, k).view(np.uint32)), (pinned, k)
    if md == 0:
        assert not fb.beauty.any() and not fb.albedo.any() and not fb.normal.any() and np.isinf(fb.depth).all()


def test_errors_are_reported(gpu):
    from shiro_gb300 import ShiroGpuError, scenes
    from shiro_gb300.abi import Mesh, Scene

    sc = scenes.sphere_scene(16, 8)
    sc.materials[0].transmission = 1.0  # every lobe of the reference is supported
    assert gpu.supports_scene(sc)
    bad = Scene(materials=[], meshes=[Mesh(np.zeros((3, 3), np.float32), np.array([0, 1, 5], np.uint32))])
    with pytest.raises(ShiroGpuError):
        gpu.upload_scene(bad, force=True)


@pytest.mark.parametrize("kind", ["no_meshes", "empty_meshes"])
def test_scene_without_triangles_renders_the_environment(gpu, port, kind):
    """A scene without triangles (no meshes, or meshes without indices) is
    rendered as the CPU tracer renders it: every ray misses, so the frame is
    the environment (and nothing occludes the lights); plain and wavefront
    forms alike, and the scene reports no triangles."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import Mesh, Scene

    w = scenes.sphere_workload(24, 16, 4, 4, env_width=32, env_height=16)
    meshes = [] if kind == "no_meshes" else [Mesh(np.zeros((3, 3), np.float32), np.zeros(0, np.uint32), None, 0)]
    sc = Scene(materials=w.scene.materials, meshes=meshes, dome_lights=w.scene.dome_lights,
               distant_lights=w.scene.distant_lights)
    ref = api.render(port, sc, w.camera, w.settings, 0, 4)
    for flags in (1, 0):
        fb = gpu.render(sc, w.camera, w.settings, 0, 4, flags=flags)
        assert gpu.last_stats()["triangles"] == 0
        (wave,) = gpu.render_batch(sc, [(w.camera, w.settings, 0, 4)], flags=flags)
        assert np.array_equal(wave.beauty.view(np.uint32), fb.beauty.view(np.uint32))
        frac, mean = frame_match(fb, ref)
        assert frac >= MIN_MATCH and mean <= MEAN_TOL, (flags, frac, mean)
        assert np.isinf(fb.depth).all() and not fb.albedo.any() and not fb.normal.any()
        assert not fb.beauty[:, 3].any()


def test_cancel(gpu):
    from shiro_gb300 import ShiroGpuError, scenes

    w = scenes.sphere_workload(32, 32, 4, 4, env_width=32, env_height=16)
    flag = C.c_int(1)
    with pytest.raises(ShiroGpuError) as ei:
        gpu.render(w.scene, w.camera, w.settings, cancel=flag)
    assert ei.value.code == -6


def test_bvh_widths_agree(gpu, port):
    """The binary BVH and the compressed wide BVH return identical hits,
    distances and occlusion (the default lets the wavefront form traverse
    the wide one and the plain form the binary one, so the wavefront tests'
    bit-identity covers whole frames across the two)."""
    from shiro_gb300 import scenes

    scene = scenes.field_scene(instances=40, levels=4, materials=4, env_width=16, env_height=8, seed=33, plane=20.0)
    rng = np.random.default_rng(8)
    n = 60000
    o = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    o[:, 1] = rng.uniform(0.02, 4.0, n)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tmax = rng.uniform(0.2, 40.0, n).astype(np.float32)
    binary = gpu.trace_rays(scene, o, d, tmax)
    gpu.set_bvh_width(8)
    try:
        wide = gpu.trace_rays(scene, o, d, tmax)
        # a frame through the wide BVH equals the binary one bit for bit
        w = scenes.sphere_workload(40, 32, 4, 8, env_width=64, env_height=32)
        fw = gpu.render(w.scene, w.camera, w.settings)
    finally:
        gpu.set_bvh_width(2)
    fb = gpu.render(w.scene, w.camera, w.settings)
    gpu.set_bvh_width(0)
    assert np.array_equal(fw.beauty, fb.beauty)
    brute = api.trace_rays(port, scene, o, d, tmax, bruteforce=True)
    for a, b, c in zip(wide, binary, brute):
        assert np.array_equal(a, b) and np.array_equal(a, c)


@pytest.mark.parametrize("cluster", [2, 8, 32, 256])
def test_binned_sah_top_keeps_hits_exact(gpu, port, cluster):
    """The builder's binned-SAH top (Morton clusters of at most `cluster`
    triangles, the tree above them rebuilt by binned SAH) changes the tree,
    never the hits: closest hits, distances and occlusion equal the reference
    brute force for both BVH widths, and a frame equals the Morton-only
    build's bit for bit."""
    from shiro_gb300 import scenes

    scene = scenes.field_scene(instances=40, levels=4, materials=4, env_width=16, env_height=8, seed=33, plane=20.0)
    rng = np.random.default_rng(9)
    n = 60000
    o = rng.uniform(-10, 10, (n, 3)).astype(np.float32)
    o[:, 1] = rng.uniform(0.02, 4.0, n)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    tmax = rng.uniform(0.2, 40.0, n).astype(np.float32)
    brute = api.trace_rays(port, scene, o, d, tmax, bruteforce=True)
    w = scenes.field_workload(64, 36, 4, 6, instances=40, levels=4, materials=4, env_width=64, env_height=32, seed=33,
                              plane=20.0)
    gpu.set_bvh_build(0)
    morton_frame = gpu.render(w.scene, w.camera, w.settings)
    morton_nodes = gpu.last_stats()["bvh_nodes"]
    try:
        gpu.set_bvh_build(cluster)
        for width in (2, 8):
            gpu.set_bvh_width(width)
            got = gpu.trace_rays(scene, o, d, tmax)
            for a, b in zip(got, brute):
                assert np.array_equal(a, b), (cluster, width)
        gpu.set_bvh_width(0)
        frame = gpu.render(w.scene, w.camera, w.settings)
        (wf,) = gpu.render_batch(w.scene, [(w.camera, w.settings)])
        assert gpu.last_stats()["bvh_nodes"] > 0
        print(f"cluster {cluster}: binary nodes {morton_nodes} (Morton) -> {gpu.last_stats()['bvh_nodes']}")
    finally:
        gpu.set_bvh_width(0)
        gpu.set_bvh_build(2)  # the default
    for k in ("beauty", "albedo", "normal", "depth"):
        assert np.array_equal(getattr(frame, k), getattr(morton_frame, k)), k
        assert np.array_equal(getattr(wf, k), getattr(morton_frame, k)), k
