"""Scene uploads that keep the geometry.

An upload whose meshes (positions, normals, indices, per-mesh material
indices), material count and BVH build setting equal the resident ones only
refreshes what derives from materials, lights and environments; the BVHs,
triangles and per-triangle records stay.  The frame after such an upload
must equal, bit for bit, the frame of a fresh context that uploads the
edited snapshot in full; a geometry edit must still rebuild.
"""
import copy
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def same(a, b):
    return all(np.array_equal(getattr(a, k).view(np.uint32), getattr(b, k).view(np.uint32))
               for k in ("beauty", "albedo", "normal", "depth"))


def _fresh(scene, cam, st):
    from shiro_gb300 import GpuBackend

    with GpuBackend(0) as g:
        return g.render(scene, cam, st), g.render_batch(scene, [(cam, st)])[0]


def test_shading_edits_keep_the_geometry():
    from shiro_gb300 import GpuBackend, scenes

    w = scenes.field_workload(64, 36, 4, 6, instances=40, levels=4, materials=4, env_width=64, env_height=32,
                              seed=33, plane=20.0)
    sc = copy.deepcopy(w.scene)
    with GpuBackend(0) as gpu:
        gpu.upload_scene(sc)
        before = gpu.render(sc, w.camera, w.settings)
        # a light, a material and the environment edited in the same snapshot
        sc.distant_lights[0].radiance = tuple(1.7 * c for c in sc.distant_lights[0].radiance)
        sc.materials[1].base_color = (0.9, 0.1, 0.2)
        sc.materials[2].roughness = 0.07
        sc.dome_lights[0].env = (sc.dome_lights[0].env * 1.5).astype(np.float32)
        plain = gpu.render(sc, w.camera, w.settings)
        (wave,) = gpu.render_batch(sc, [(w.camera, w.settings)])
        assert not same(plain, before)
        ref_plain, ref_wave = _fresh(sc, w.camera, w.settings)
        assert same(plain, ref_plain) and same(wave, ref_wave)
        # a geometry edit rebuilds
        m = sc.meshes[3]
        m.positions = m.positions.copy()
        m.positions[0] += np.float32(0.25)
        plain = gpu.render(sc, w.camera, w.settings)
        ref_plain, _ = _fresh(sc, w.camera, w.settings)
        assert same(plain, ref_plain)
        # a mesh assigned another material rebuilds (the per-triangle records hold it)
        sc.meshes[5].material_index = (sc.meshes[5].material_index + 1) % len(sc.materials)
        plain = gpu.render(sc, w.camera, w.settings)
        ref_plain, _ = _fresh(sc, w.camera, w.settings)
        assert same(plain, ref_plain)


def test_shading_only_upload_is_fast():
    """On the 1.31 M-triangle field scene (with a small environment, so that
    the geometry is nearly all of the upload) an upload after a light edit
    skips the flattening, both BVH builds and the triangle records."""
    import torch

    from shiro_gb300 import GpuBackend, scenes

    sc = scenes.field_scene(env_width=64, env_height=32)
    with GpuBackend(0) as gpu:
        gpu.upload_scene(sc)  # warm (context, modules)
        sc.distant_lights[0].radiance = tuple(0.9 * c for c in sc.distant_lights[0].radiance)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gpu.upload_scene(sc, force=True)
        light = time.perf_counter() - t0
        gpu.set_bvh_build(8)  # another build setting: a full upload
        t0 = time.perf_counter()
        gpu.upload_scene(sc)
        full = time.perf_counter() - t0
        gpu.set_bvh_build(2)
        t0 = time.perf_counter()
        gpu.upload_scene(sc)  # and the default one
        full = min(full, time.perf_counter() - t0)
    print(f"upload: full {full:.3f} s, light edit {light:.3f} s")
    assert light < 0.35 * full, (light, full)


def test_index_out_of_range_is_refused():
    """The device flattening checks every vertex index before using it: a
    mesh with an index past its vertices is refused with the mesh and
    triangle named, and the context renders the next valid scene."""
    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.backend import ShiroGpuError

    w = scenes.sphere_workload(32, 24, 2, 4, env_width=64, env_height=32)
    bad = copy.deepcopy(w.scene)
    m = bad.meshes[0]
    m.indices = m.indices.copy()
    m.indices[3 * 5 + 1] = np.uint32(m.positions.shape[0] + 7)  # triangle 5 of mesh 0
    with GpuBackend(0) as gpu:
        with pytest.raises(ShiroGpuError) as ei:
            gpu.upload_scene(bad)
        assert ei.value.code == -1 and "mesh 0: index out of range at triangle 5" in str(ei.value), ei.value
        good = gpu.render(w.scene, w.camera, w.settings)
        ref, _ = _fresh(w.scene, w.camera, w.settings)
        assert same(good, ref)
