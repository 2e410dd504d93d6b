"""Generates the golden vectors in tests/golden from the reference itself.

Run in a tree where the reference sources exist (they are compiled by
oracle/Makefile into oracle/_ref/libshiro_ref.so together with
oracle/ref/ref_harness.cpp):

    python tests/golden/gen_golden.py            # everything
    python tests/golden/gen_golden.py emissive   # just the named render cases

Every output comes from the reference's own code (CpuPathTracer.cpp,
EnvironmentMap.cpp, OpenQmcSampler.cpp built with SHIRO_HAVE_EMBREE=0,
SHIRO_WITH_OPENQMC=0, SHIRO_HAVE_OIIO=0); the inputs are seeded and stored
next to the outputs so that the fixtures are self-contained.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from oracle import api  # noqa: E402
from scene_io import camera_to_array, scene_to_arrays, settings_to_array  # noqa: E402
from shiro_gb300 import scenes  # noqa: E402
from shiro_gb300.abi import (ENV_ANGULAR, ENV_LATLONG, DistantLight, DomeLight, Material, Mesh,  # noqa: E402
                             RenderSettings, Scene, lambert, standard_surface)


def random_unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def feature_materials():
    """Materials that exercise every reflective lobe of EvaluateBsdf."""
    return {
        "preview": scenes.usd_preview_surface((0.8, 0.8, 0.8), 0.3),
        "lambert": lambert((0.5, 0.5, 0.5)),
        "metal": standard_surface((0.9, 0.6, 0.3), 0.25, 1.0, 1.5),
        "rough_dielectric": standard_surface((0.2, 0.5, 0.8), 0.9, 0.0, 1.8),
        "coated": standard_surface((0.7, 0.1, 0.1), 0.4, 0.2, 1.5, coat_weight=0.8, coat_roughness=0.1,
                                   coat_color=(0.9, 0.95, 1.0), coat_affect_color=0.5, coat_affect_roughness=0.5),
        "sheen_oren": standard_surface((0.3, 0.6, 0.3), 0.6, 0.0, 1.5, sheen=0.7, sheen_roughness=0.4,
                                       sheen_color=(1.0, 0.9, 0.8), diffuse_roughness=0.7),
        "aniso_film": standard_surface((0.5, 0.5, 0.9), 0.35, 0.6, 1.5, specular_anisotropy=0.6,
                                       specular_rotation=0.15, thin_film_thickness=420.0, thin_film_ior=1.4,
                                       coat_weight=0.3, coat_anisotropy=-0.4, coat_rotation=0.3),
        "subsurface_wrap": standard_surface((0.9, 0.7, 0.6), 0.5, 0.0, 1.4, subsurface=0.6, subsurface_scale=0.8,
                                            subsurface_color=(1.0, 0.4, 0.3), subsurface_radius=(2.0, 1.0, 0.5),
                                            subsurface_anisotropy=0.3, base_weight=0.8),
        "overrides": standard_surface((0.6, 0.6, 0.6), 0.45, 0.1, 1.5, coat_weight=0.5,
                                      has_normal_override=True, normal_override=(0.2, 1.0, 0.1),
                                      has_coat_normal_override=True, coat_normal_override=(0.0, 1.0, 0.3),
                                      has_tangent_override=True, tangent_override=(1.0, 0.0, 0.2),
                                      specular_anisotropy=0.4),
        "spec_tint": standard_surface((0.4, 0.4, 0.4), 0.15, 0.0, 2.2, specular_color=(0.8, 1.0, 0.6),
                                      specular_weight=0.7),
    }


def gen_sampler(rng):
    n = 64_000
    px = rng.integers(0, 4096, n).astype(np.uint32)
    py = rng.integers(0, 4096, n).astype(np.uint32)
    idx = np.concatenate([rng.integers(0, 70000, n // 2), rng.integers(0, 2**32 - 2, n - n // 2)]).astype(np.uint32)
    br = np.concatenate([rng.integers(0, 8, n // 4), rng.integers(0, 12 * 12 + 8, n // 4),
                         rng.integers(128, 128 + 13 * 256 + 64 * 4, n - n // 2)]).astype(np.uint32)
    return dict(px=px, py=py, index=idx, branch=br, out=api.sampler(REF, px, py, idx, br))


def gen_camera():
    out = {}
    cams = [(scenes.sphere_camera(1.0), RenderSettings(width=64, height=64)),
            (scenes.field_camera(16 / 9), RenderSettings(width=96, height=54)),
            (scenes.look_at((3.0, 2.0, -4.0), (0.0, 0.5, 0.0), 70.0, 2.0), RenderSettings(width=80, height=40))]
    for k, (c, s) in enumerate(cams):
        o, d = api.camera_rays(REF, c, s, sample_start=7 * k)
        out[f"cam{k}"] = camera_to_array(c)
        out[f"settings{k}"] = settings_to_array(s)
        out[f"start{k}"] = np.array(7 * k)
        out[f"origins{k}"] = o
        out[f"dirs{k}"] = d
    out["count"] = np.array(len(cams))
    return out


def sphere_scene_small():
    return scenes.sphere_scene(env_width=128, env_height=64, seed=0)


def gen_hits(rng):
    scene = sphere_scene_small()
    out = scene_to_arrays(scene)
    st = RenderSettings(width=160, height=160)
    cam = scenes.sphere_camera(1.0)
    for k, start in enumerate((0, 1, 13)):
        prim, t = api.primary_hits(REF, scene, cam, st, start)
        out[f"prim{k}"], out[f"t{k}"], out[f"start{k}"] = prim, t, np.array(start)
    out["cam"], out["settings"] = camera_to_array(cam), settings_to_array(st)
    # random rays: uniform origins around the scene, plus rays aimed at
    # vertices and edge midpoints (tie / edge cases)
    n = 30_000
    o = rng.uniform(-4, 4, size=(n, 3)).astype(np.float32)
    o[:, 1] = np.abs(o[:, 1]) + 0.01
    pos = np.concatenate([m.positions for m in scene.meshes])
    tgt = pos[rng.integers(0, pos.shape[0], n)]
    sph = scene.meshes[0]
    tri = sph.indices.reshape(-1, 3)
    pick = tri[rng.integers(0, tri.shape[0], n // 3)]
    tgt[: n // 3] = 0.5 * (sph.positions[pick[:, 0]] + sph.positions[pick[:, 1]])
    tgt[n // 3: n // 2] += rng.normal(0, 0.05, size=(n // 2 - n // 3, 3)).astype(np.float32)
    d = tgt - o
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    d[-3000:] = random_unit(rng, 3000)
    tmax = np.where(rng.random(n) < 0.5, np.float32(np.finfo(np.float32).max),
                    rng.uniform(0.1, 8.0, n).astype(np.float32)).astype(np.float32)
    prim, t, occ = api.trace_rays(REF, scene, o, d, tmax)
    out.update(ray_o=o, ray_d=d, ray_tmax=tmax, ray_prim=prim, ray_t=t, ray_occ=occ)
    return out


def gen_bsdf(rng):
    out = {}
    mats = feature_materials()
    names = sorted(mats)
    n = 2000
    for name in names:
        nn = random_unit(rng, n)
        v = random_unit(rng, n)
        v = np.where((v * nn).sum(1, keepdims=True) < 0, -v, v)
        lt = random_unit(rng, n)
        lt[: n // 4] = np.where((lt[: n // 4] * nn[: n // 4]).sum(1, keepdims=True) < 0, -lt[: n // 4], lt[: n // 4])
        # near-mirror directions: reflect v about n (specular peak)
        r = (2 * (v * nn).sum(1, keepdims=True) * nn - v)[n // 4: n // 2]
        lt[n // 4: n // 2] = (r + rng.normal(0, 0.02, r.shape)).astype(np.float32)
        lt = (lt / np.linalg.norm(lt, axis=1, keepdims=True)).astype(np.float32)
        f, pdf, w = api.bsdf(REF, mats[name], nn, v, lt)
        out.update({f"{name}_n": nn, f"{name}_v": v, f"{name}_l": lt, f"{name}_f": f, f"{name}_pdf": pdf,
                    f"{name}_w": w})
    sc = Scene(materials=[mats[k] for k in names])
    out.update(scene_to_arrays(sc))
    out["names"] = np.array(names)
    return out


def gen_env(rng):
    env = scenes.procedural_hdri(96, 48, seed=11)
    env[5] = 0.0  # a black row (uniform conditional CDF, weight 1)
    env[20:23, 10:40] = 0.0
    row, cond = api.env_tables(REF, env)
    n = 8_000
    u2 = rng.random((n, 2), np.float32)
    u2[:50] = 0.0
    u2[50:100] = np.float32(0.99999994)
    dirs = random_unit(rng, n)
    dirs[:20] = [[0, 1, 0]] * 10 + [[0, -1, 0]] * 10
    q = api.env_query(REF, env, u2, dirs, ENV_LATLONG)
    qa = api.env_query(REF, env, u2, dirs, ENV_ANGULAR)
    out = dict(env=env, row_cdf=row, cond_cdf=cond, u2=u2, dirs=dirs)
    out.update({f"ll_{k}": v for k, v in q.items()})
    out.update({f"ang_{k}": v for k, v in qa.items()})
    return out


# frames rendered as the n-th consecutive batch of one reference tracer
PROGRESSIVE = {"progressive_batch3": 3}


def render_cases():
    """Small frames covering the integrator's branches."""
    cases = {}
    base = sphere_scene_small()
    cam = scenes.sphere_camera(1.0)

    st = RenderSettings(width=64, height=64, samples_per_pixel=8, max_depth=8, diffuse_depth=8, specular_depth=8,
                        dome_light_samples=1, backend=1)
    cases["sphere"] = (base, cam, st, 0, 8, 0)

    mats = feature_materials()
    rich = Scene(materials=[mats["coated"], mats["metal"], mats["sheen_oren"]],
                 meshes=[Mesh(m.positions, m.indices, m.normals, i) for i, m in enumerate(base.meshes)],
                 distant_lights=[DistantLight((-0.4, -1.0, 0.3), (3.0, 2.8, 2.5))],
                 dome_lights=[DomeLight((0.8, 0.9, 1.0), base.dome_lights[0].env, ENV_LATLONG,
                                        (0.0, 0.0, -1.0), (0.0, 1.0, 0.0), (1.0, 0.0, 0.0)),
                              DomeLight((0.2, 0.25, 0.3))])
    st2 = RenderSettings(width=48, height=48, samples_per_pixel=4, max_depth=6, diffuse_depth=3, specular_depth=2,
                         dome_light_samples=2, background_visible=False, backend=1)
    cases["rich"] = (rich, scenes.look_at((2.5, 1.8, 3.5), (0.0, 0.8, 0.0), 50.0, 1.0), st2, 3, 4, 0)

    feat = Scene(materials=[mats["aniso_film"], mats["subsurface_wrap"], mats["overrides"], mats["spec_tint"]],
                 meshes=[Mesh(base.meshes[0].positions, base.meshes[0].indices, base.meshes[0].normals, 0),
                         Mesh(base.meshes[1].positions, base.meshes[1].indices, None, 2),
                         Mesh(base.meshes[0].positions * np.float32(0.4) + np.float32([1.6, 0.0, 0.6]),
                              base.meshes[0].indices, base.meshes[0].normals, 1),
                         Mesh(base.meshes[0].positions * np.float32(0.3) + np.float32([-1.5, 0.2, 0.8]),
                              base.meshes[0].indices, None, 3)],
                 distant_lights=[DistantLight((0.3, -1.0, -0.5), (2.0, 2.0, 2.0))],
                 environment_top=(0.6, 0.7, 1.0), environment_bottom=(0.1, 0.08, 0.05))
    st3 = RenderSettings(width=48, height=48, samples_per_pixel=4, max_depth=5, diffuse_depth=2, specular_depth=3,
                         dome_light_samples=1, backend=1)
    cases["features_gradient_env"] = (feat, scenes.look_at((0.5, 2.2, 4.5), (0.0, 0.6, 0.0), 55.0, 1.0), st3, 0, 4, 0)

    ang = Scene(materials=[mats["rough_dielectric"], mats["lambert"]], meshes=base.meshes,
                dome_lights=[DomeLight((1.0, 1.0, 1.0), scenes.procedural_hdri(64, 64, seed=5), ENV_ANGULAR)])
    st4 = RenderSettings(width=40, height=40, samples_per_pixel=4, max_depth=4, diffuse_depth=4, specular_depth=4,
                         backend=1)
    cases["angular_env"] = (ang, cam, st4, 0, 4, 0)

    # a few noise-displaced icospheres with standard_surface materials
    field = scenes.field_scene(instances=6, levels=3, materials=6, env_width=128, env_height=64, seed=9, plane=8.0)
    st5 = RenderSettings(width=64, height=36, samples_per_pixel=4, max_depth=12, diffuse_depth=12,
                         specular_depth=12, backend=1)
    cases["field_small"] = (field, scenes.look_at((0.0, 3.5, 7.5), (0.0, 0.3, 0.0), 45.0, 16 / 9), st5, 0, 4, 0)

    # emissive triangles: a lamp quad and a small glowing sphere (emission
    # with MIS at hits, the emissive-triangle light sample), plus the dome
    spos, snrm, sidx = scenes.uv_sphere(center=(0.0, 1.0, 0.0), radius=1.0, segments=24, rings=12)
    lpos, lnrm, lidx = scenes.uv_sphere(center=(1.4, 0.5, 0.9), radius=0.35, segments=12, rings=6)
    gpos, gnrm, gidx = scenes.ground_quad(10.0)
    quad = np.array([[-0.8, 2.6, -0.6], [0.8, 2.6, -0.6], [0.8, 2.6, 0.6], [-0.8, 2.6, 0.6]], np.float32)
    qidx = np.array([0, 2, 1, 0, 3, 2], np.uint32)  # facing down
    lamp = Material(emission_color=(1.0, 0.85, 0.6), emission_strength=6.0, base_color=(0.1, 0.1, 0.1))
    glow = Material(emission_color=(0.3, 0.6, 1.0), emission_strength=3.0, base_color=(0.2, 0.2, 0.2))
    emi = Scene(materials=[mats["preview"], lambert((0.6, 0.6, 0.6)), lamp, glow],
                meshes=[Mesh(spos, sidx, snrm, 0), Mesh(gpos, gidx, gnrm, 1), Mesh(quad, qidx, None, 2),
                        Mesh(lpos, lidx, lnrm, 3)],
                dome_lights=[DomeLight((0.3, 0.3, 0.3), scenes.procedural_hdri(64, 32, seed=3))])
    st7 = RenderSettings(width=40, height=40, samples_per_pixel=4, max_depth=6, diffuse_depth=6, specular_depth=6,
                         backend=1)
    cases["emissive"] = (emi, scenes.look_at((2.5, 2.0, 4.0), (0.0, 1.0, 0.0), 50.0, 1.0), st7, 0, 4, 0)

    # opacity cut-outs (UsdPreviewSurface opacity < 1 is thin-walled)
    cut = Scene(materials=[scenes.usd_preview_surface((0.7, 0.3, 0.2), 0.4, opacity=0.45),
                           standard_surface((0.3, 0.5, 0.8), 0.3, 0.0, 1.5, opacity=0.8), lambert((0.5, 0.5, 0.5))],
                meshes=[Mesh(spos, sidx, snrm, 0), Mesh(lpos, lidx, lnrm, 1), Mesh(gpos, gidx, gnrm, 2)],
                distant_lights=[DistantLight((-0.3, -1.0, -0.2), (2.0, 2.0, 2.0))],
                dome_lights=[DomeLight((0.5, 0.5, 0.5), scenes.procedural_hdri(64, 32, seed=4))])
    cases["opacity"] = (cut, scenes.look_at((2.5, 2.0, 4.0), (0.0, 1.0, 0.0), 50.0, 1.0), st7, 0, 4, 0)

    # transmission: smooth and rough solid glass, a tinted absorbing medium,
    # a scattering medium and a thin-walled pane
    g1pos, g1nrm, g1idx = scenes.uv_sphere(center=(-1.2, 0.7, 0.0), radius=0.7, segments=24, rings=12)
    g2pos, g2nrm, g2idx = scenes.uv_sphere(center=(0.4, 0.6, 0.6), radius=0.6, segments=24, rings=12)
    g3pos, g3nrm, g3idx = scenes.uv_sphere(center=(1.5, 0.5, -0.4), radius=0.5, segments=24, rings=12)
    pane = np.array([[-1.8, 0.0, -1.4], [1.8, 0.0, -1.4], [1.8, 2.2, -1.4], [-1.8, 2.2, -1.4]], np.float32)
    pidx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    glass = standard_surface((1.0, 1.0, 1.0), 0.0, 0.0, 1.5, transmission=1.0)
    rough = standard_surface((1.0, 1.0, 1.0), 0.25, 0.0, 1.45, transmission=0.9, transmission_extra_roughness=0.1,
                             coat_weight=0.3, coat_roughness=0.05)
    tinted = standard_surface((1.0, 1.0, 1.0), 0.0, 0.0, 1.33, transmission=1.0,
                              transmission_color=(0.5, 0.8, 0.9), transmission_depth=0.8,
                              transmission_scatter=(0.3, 0.1, 0.05))
    thin = standard_surface((1.0, 1.0, 1.0), 0.1, 0.0, 1.5, transmission=0.8, thin_walled=True,
                            transmission_color=(0.9, 0.95, 1.0))
    tra = Scene(materials=[glass, rough, tinted, thin, lambert((0.55, 0.5, 0.45))],
                meshes=[Mesh(g1pos, g1idx, g1nrm, 0), Mesh(g2pos, g2idx, g2nrm, 1), Mesh(g3pos, g3idx, g3nrm, 2),
                        Mesh(pane, pidx, None, 3), Mesh(gpos, gidx, gnrm, 4)],
                distant_lights=[DistantLight((-0.2, -1.0, 0.5), (2.5, 2.4, 2.2))],
                dome_lights=[DomeLight((1.0, 1.0, 1.0), scenes.procedural_hdri(64, 32, seed=6))])
    st8 = RenderSettings(width=48, height=40, samples_per_pixel=4, max_depth=10, diffuse_depth=4, specular_depth=10,
                         backend=1)
    cases["transmission"] = (tra, scenes.look_at((0.5, 1.6, 4.5), (0.0, 0.7, 0.0), 50.0, 48 / 40), st8, 0, 4, 0)

    # degenerate geometry: an exact duplicate of the sphere under another
    # material (every hit ties in t: the first mesh must win), zero-area and
    # repeated-vertex triangles, vertex normals of zero length (the geometric
    # normal stands in), a material index out of range (default material),
    # an empty mesh, and a distant light from below the ground
    dup = Mesh(spos, sidx, snrm, 1)
    zpos = np.array([[-1.5, 0.3, 1.0], [-1.0, 0.8, 1.0], [-0.5, 1.3, 1.0],   # collinear
                     [0.6, 0.2, 1.2], [0.6, 0.2, 1.2], [1.0, 0.9, 1.2],     # repeated vertex
                     [-0.3, 1.9, 1.5], [0.3, 1.9, 1.5], [0.0, 2.4, 1.5]], np.float32)
    zidx = np.arange(9, dtype=np.uint32)
    znrm = np.zeros((9, 3), np.float32)
    znrm[6:] = [[0.0, 0.0, 1.0], [0.0, 0.0, 0.0], [0.0, 0.0, 1.0]]
    qpos = np.array([[1.2, 0.0, -0.5], [2.2, 0.0, -0.5], [2.2, 1.0, -0.5], [1.2, 1.0, -0.5]], np.float32)
    qidx = np.array([0, 1, 2, 0, 2, 3], np.uint32)
    empty = Mesh(np.zeros((0, 3), np.float32), np.zeros(0, np.uint32), None, 0)
    deg = Scene(materials=[lambert((0.7, 0.6, 0.5)), lambert((0.1, 0.9, 0.1)), mats["metal"]],
                meshes=[Mesh(spos, sidx, snrm, 0), dup, Mesh(zpos, zidx, znrm, 2), Mesh(qpos, qidx, None, 99), empty,
                        Mesh(gpos, gidx, gnrm, 0)],
                distant_lights=[DistantLight((-0.3, -1.0, -0.2), (2.0, 2.0, 2.0)),
                                DistantLight((0.0, 1.0, 0.0), (5.0, 5.0, 5.0))],
                dome_lights=[DomeLight((0.5, 0.5, 0.5), scenes.procedural_hdri(64, 32, seed=8))])
    cases["degenerate"] = (deg, scenes.look_at((0.5, 1.6, 4.5), (0.0, 0.9, 0.0), 50.0, 1.0), st7, 0, 4, 0)

    # third batch of a progressive render: batches of 4 samples at indices
    # 0, 4, 8 on one reference tracer, which keeps its path-guide weights
    # between batches of a scene; the frame is stored as the batch it is
    # (start 8, 4 samples), to be matched by a single render of that batch
    st9 = RenderSettings(width=48, height=48, samples_per_pixel=4, max_depth=8, diffuse_depth=8, specular_depth=8,
                         backend=1)
    cases["progressive_batch3"] = (base, cam, st9, 8, 4, 0)

    # single path per pixel at a non-zero sample index (per-path golden)
    st6 = RenderSettings(width=64, height=64, samples_per_pixel=1, max_depth=8, diffuse_depth=8, specular_depth=8,
                         backend=1)
    cases["sphere_1spp_start5"] = (base, cam, st6, 5, 1, 0)
    return cases


def gen_renders(only=None):
    out = {}
    cases = render_cases()
    for name, (scene, cam, st, start, count, flags) in cases.items():
        if only and name not in only:
            continue
        batches = PROGRESSIVE.get(name, 1)
        if batches > 1:
            fb = api.render_batches(REF, scene, cam, st, start - (batches - 1) * count, count, batches)
        else:
            fb = api.render(REF, scene, cam, st, start, count)
        out[name] = dict(scene_to_arrays(scene), cam=camera_to_array(cam), settings=settings_to_array(st),
                         start=np.array(start), count=np.array(count), flags=np.array(flags),
                         batches=np.array(batches),
                         beauty=fb.beauty, albedo=fb.albedo, normal=fb.normal, depth=fb.depth)
        print(f"  render {name}: {st.width}x{st.height} {count} spp, mean {fb.beauty[:, :3].mean():.4f}")
    return out


def main():
    global REF
    REF = oracle.ref_checker()
    if REF is None:
        sys.exit("reference tree not found; golden vectors can only be generated where it exists")
    only = sys.argv[1:]  # render case names: regenerate just those frames
    if only:
        for name, arrays in gen_renders(only).items():
            np.savez_compressed(os.path.join(HERE, f"render_{name}.npz"), **arrays)
        return
    rng = np.random.default_rng(20261203)
    np.savez_compressed(os.path.join(HERE, "sampler_kat.npz"), **gen_sampler(rng))
    np.savez_compressed(os.path.join(HERE, "camera_rays.npz"), **gen_camera())
    np.savez_compressed(os.path.join(HERE, "hits_sphere.npz"), **gen_hits(rng))
    np.savez_compressed(os.path.join(HERE, "bsdf_kat.npz"), **gen_bsdf(rng))
    np.savez_compressed(os.path.join(HERE, "env_kat.npz"), **gen_env(rng))
    for name, arrays in gen_renders().items():
        np.savez_compressed(os.path.join(HERE, f"render_{name}.npz"), **arrays)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
