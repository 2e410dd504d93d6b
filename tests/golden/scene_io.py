"""Store / load scene snapshots in .npz fixtures (flat numpy arrays)."""
from __future__ import annotations

from dataclasses import fields

import numpy as np

from shiro_gb300.abi import Camera, DistantLight, DomeLight, Material, Mesh, RenderSettings, Scene


def scene_to_arrays(scene: Scene, prefix: str = "scene_") -> dict:
    out = {}
    for f in fields(Material):
        out[f"{prefix}mat_{f.name}"] = np.array([getattr(m, f.name) for m in scene.materials],
                                                np.float32 if f.type != "bool" else np.uint8)
    out[f"{prefix}mesh_count"] = np.array(len(scene.meshes))
    for i, m in enumerate(scene.meshes):
        out[f"{prefix}mesh{i}_pos"] = np.asarray(m.positions, np.float32)
        out[f"{prefix}mesh{i}_idx"] = np.asarray(m.indices, np.uint32)
        out[f"{prefix}mesh{i}_mat"] = np.array(m.material_index)
        if m.normals is not None:
            out[f"{prefix}mesh{i}_nrm"] = np.asarray(m.normals, np.float32)
    out[f"{prefix}distant"] = np.array([list(l.direction) + list(l.radiance) for l in scene.distant_lights],
                                       np.float32).reshape(-1, 6)
    out[f"{prefix}dome_count"] = np.array(len(scene.dome_lights))
    for i, d in enumerate(scene.dome_lights):
        out[f"{prefix}dome{i}_frame"] = np.array([d.radiance, d.right, d.up, d.forward], np.float32)
        out[f"{prefix}dome{i}_layout"] = np.array(d.layout)
        if d.env is not None:
            out[f"{prefix}dome{i}_env"] = np.asarray(d.env, np.float32)
    out[f"{prefix}envgrad"] = np.array([scene.environment_top, scene.environment_bottom], np.float32)
    return out


def scene_from_arrays(a, prefix: str = "scene_") -> Scene:
    nmat = len(a[f"{prefix}mat_base_weight"])
    mats = []
    for k in range(nmat):
        kw = {}
        for f in fields(Material):
            v = a[f"{prefix}mat_{f.name}"][k]
            if f.type == "bool":
                kw[f.name] = bool(v)
            elif np.ndim(v) == 1:
                kw[f.name] = tuple(float(x) for x in v)
            else:
                kw[f.name] = float(v)
        mats.append(Material(**kw))
    meshes = []
    for i in range(int(a[f"{prefix}mesh_count"])):
        nk = f"{prefix}mesh{i}_nrm"
        meshes.append(Mesh(a[f"{prefix}mesh{i}_pos"], a[f"{prefix}mesh{i}_idx"],
                           a[nk] if nk in a else None, int(a[f"{prefix}mesh{i}_mat"])))
    distant = [DistantLight(tuple(map(float, r[:3])), tuple(map(float, r[3:]))) for r in a[f"{prefix}distant"]]
    domes = []
    for i in range(int(a[f"{prefix}dome_count"])):
        fr = a[f"{prefix}dome{i}_frame"]
        ek = f"{prefix}dome{i}_env"
        domes.append(DomeLight(tuple(map(float, fr[0])), a[ek] if ek in a else None, int(a[f"{prefix}dome{i}_layout"]),
                               tuple(map(float, fr[1])), tuple(map(float, fr[2])), tuple(map(float, fr[3]))))
    g = a[f"{prefix}envgrad"]
    return Scene(mats, meshes, distant, domes, tuple(map(float, g[0])), tuple(map(float, g[1])))


def camera_to_array(c: Camera) -> np.ndarray:
    return np.array(list(c.position) + list(c.forward) + list(c.right) + list(c.up)
                    + [c.vertical_fov_degrees, c.aspect_ratio], np.float32)


def camera_from_array(v) -> Camera:
    v = [float(x) for x in v]
    return Camera(tuple(v[0:3]), tuple(v[3:6]), tuple(v[6:9]), tuple(v[9:12]), v[12], v[13])


def settings_to_array(s: RenderSettings) -> np.ndarray:
    return np.array([int(getattr(s, f.name)) for f in fields(RenderSettings)], np.int64)


def settings_from_array(v) -> RenderSettings:
    kw = {}
    for f, x in zip(fields(RenderSettings), v):
        kw[f.name] = bool(x) if f.type == "bool" else int(x)
    return RenderSettings(**kw)
