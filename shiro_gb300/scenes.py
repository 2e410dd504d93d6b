"""Seeded procedural workloads.

The reference ships no benchmark scenes (its testscenes/*.usda need USD,
which is absent), so every workload is synthesised here from a seed:

* ``sphere_scene``   - UV sphere (64x32 segments) on a 10x10 ground quad, one
  UsdPreviewSurface on the sphere, Lambert ground, procedural HDRI dome.
* ``field_scene``    - 256 noise-displaced icospheres (5 120 triangles each,
  1 310 720 in total) scattered over a 50x50 plane with 64 standard_surface
  materials, a 2048x1024 HDRI dome and one directional light.
* ``batch_requests`` - 48 render requests of uneven resolution / spp / depth.
* ``split_sphere_scene`` - the sphere scene cut into 256 meshes with one
  material each (parameters of the differentiable renderer).

Geometry is generated in float64 and stored as float32.  Scenes are built as
``shiro_gb300.abi.Scene`` snapshots, i.e. the data the Hydra delegate hands the
backend (world-space positions, smooth normals, one material per mesh;
SceneBridge.cpp:967-1032, RenderParam.cpp:614-659).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from .abi import (Camera, DistantLight, DomeLight, Material, Mesh, RenderSettings, Scene, lambert,
                  standard_surface, usd_preview_surface)


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------

def uv_sphere(center=(0.0, 1.0, 0.0), radius=1.0, segments=64, rings=32) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Shared-vertex UV sphere, outward winding, analytic smooth normals.

    64x32 segments gives 2 + 31*64 = 1 986 vertices and 64*(2*30 + 2) = 3 968
    triangles."""
    c = np.asarray(center, np.float64)
    verts = [np.array([0.0, 1.0, 0.0])]
    for i in range(1, rings):
        th = math.pi * i / rings
        for j in range(segments):
            ph = 2.0 * math.pi * j / segments
            verts.append(np.array([math.sin(th) * math.sin(ph), math.cos(th), math.sin(th) * math.cos(ph)]))
    verts.append(np.array([0.0, -1.0, 0.0]))
    unit = np.stack(verts)
    south = unit.shape[0] - 1

    def ring(i, j):  # i in 1..rings-1
        return 1 + (i - 1) * segments + (j % segments)

    tris = []
    for j in range(segments):
        tris.append((0, ring(1, j), ring(1, j + 1)))
    for i in range(1, rings - 1):
        for j in range(segments):
            a, b = ring(i, j), ring(i, j + 1)
            cc, d = ring(i + 1, j), ring(i + 1, j + 1)
            tris.append((a, cc, b))
            tris.append((b, cc, d))
    for j in range(segments):
        tris.append((ring(rings - 1, j), south, ring(rings - 1, j + 1)))
    pos = (unit * radius + c).astype(np.float32)
    nrm = unit.astype(np.float32)
    idx = np.asarray(tris, np.uint32).reshape(-1)
    return pos, nrm, idx


def ground_quad(size=10.0, y=0.0):
    h = size * 0.5
    pos = np.array([[-h, y, -h], [h, y, -h], [h, y, h], [-h, y, h]], np.float32)
    nrm = np.tile(np.array([[0.0, 1.0, 0.0]], np.float32), (4, 1))
    idx = np.array([0, 2, 1, 0, 3, 2], np.uint32)
    return pos, nrm, idx


def icosphere(levels: int) -> Tuple[np.ndarray, np.ndarray]:
    """Unit icosphere; `levels` counts the base icosahedron as level 1, so
    level 5 has 20 * 4**4 = 5 120 triangles and 2 562 vertices."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
         (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(x, np.float64) / np.linalg.norm(x) for x in v]
    faces = f
    for _ in range(levels - 1):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.stack(verts), np.asarray(faces, np.int64)


def smooth_normals(pos: np.ndarray, faces: np.ndarray) -> np.ndarray:
    """Area-weighted vertex normals (what SceneBridge computes when a mesh has
    none, SceneBridge.cpp:147-180)."""
    p0, p1, p2 = pos[faces[:, 0]], pos[faces[:, 1]], pos[faces[:, 2]]
    fn = np.cross(p1 - p0, p2 - p0)
    acc = np.zeros_like(pos)
    for k in range(3):
        np.add.at(acc, faces[:, k], fn)
    n = np.linalg.norm(acc, axis=1, keepdims=True)
    return acc / np.maximum(n, 1e-20)


# ---------------------------------------------------------------------------
# environment
# ---------------------------------------------------------------------------

def latlong_directions(width: int, height: int) -> np.ndarray:
    """Texel-centre directions of a lat-long map with the reference's
    convention: u -> phi = 2 pi u, v -> theta = pi v, dir = (sin phi sin theta,
    cos theta, cos phi sin theta) (EnvironmentMap.cpp:132-141)."""
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    ph = 2.0 * np.pi * u[None, :]
    th = np.pi * v[:, None]
    return np.stack([np.sin(ph) * np.sin(th), np.cos(th) * np.ones_like(ph), np.cos(ph) * np.sin(th)], -1)


def procedural_hdri(width: int, height: int, seed: int, sun_dir=(0.45, 0.64, 0.62), sun_peak=1.0e3,
                    sun_sigma_deg=2.0, mu=0.0, sigma=1.0) -> np.ndarray:
    """Seeded HDRI: per-texel log-normal(mu, sigma) grey radiance plus one
    Gaussian sun lobe of the given peak.  Returns (H, W, 3) float32."""
    rng = np.random.default_rng(seed)
    base = np.exp(rng.normal(mu, sigma, size=(height, width)))
    d = latlong_directions(width, height)
    s = np.asarray(sun_dir, np.float64)
    s = s / np.linalg.norm(s)
    cosang = np.clip(d @ s, -1.0, 1.0)
    ang = np.arccos(cosang)
    sig = math.radians(sun_sigma_deg)
    sun = sun_peak * np.exp(-0.5 * (ang / sig) ** 2)
    img = (base + sun)[..., None] * np.array([1.0, 1.0, 1.0])
    return img.astype(np.float32)


# ---------------------------------------------------------------------------
# cameras
# ---------------------------------------------------------------------------

def look_at(position, target, fov=45.0, aspect=1.0, world_up=(0.0, 1.0, 0.0)) -> Camera:
    p = np.asarray(position, np.float64)
    f = np.asarray(target, np.float64) - p
    f /= np.linalg.norm(f)
    r = np.cross(f, np.asarray(world_up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    return Camera(tuple(float(x) for x in p.astype(np.float32)), tuple(float(x) for x in f.astype(np.float32)),
                  tuple(float(x) for x in r.astype(np.float32)), tuple(float(x) for x in u.astype(np.float32)),
                  float(fov), float(aspect))


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

@dataclass
class Workload:
    name: str
    scene: Scene
    camera: Camera
    settings: RenderSettings

    @property
    def paths(self) -> int:
        s = self.settings
        return int(s.width) * int(s.height) * int(s.samples_per_pixel)


def sphere_scene(env_width=512, env_height=256, seed=0, segments=64, rings=32) -> Scene:
    """UV sphere + ground quad under a procedural HDRI dome."""
    spos, snrm, sidx = uv_sphere(segments=segments, rings=rings)
    gpos, gnrm, gidx = ground_quad()
    mats = [usd_preview_surface(diffuse_color=(0.8, 0.8, 0.8), roughness=0.3), lambert((0.5, 0.5, 0.5))]
    env = procedural_hdri(env_width, env_height, seed)
    return Scene(materials=mats,
                 meshes=[Mesh(spos, sidx, snrm, 0), Mesh(gpos, gidx, gnrm, 1)],
                 dome_lights=[DomeLight(env=env)])


def sphere_camera(aspect=1.0) -> Camera:
    return look_at((0.0, 1.6, 4.5), (0.0, 0.9, 0.0), 45.0, aspect)


def sphere_workload(width=256, height=256, spp=16, depth=8, env_width=512, env_height=256, seed=0) -> Workload:
    st = RenderSettings(width=width, height=height, samples_per_pixel=spp, max_depth=depth,
                        diffuse_depth=depth, specular_depth=depth, dome_light_samples=1,
                        background_visible=True, backend=1)
    return Workload(f"sphere {width}x{height} {spp}spp depth {depth}", sphere_scene(env_width, env_height, seed),
                    sphere_camera(width / height), st)


def field_scene(instances=256, levels=5, materials=64, env_width=2048, env_height=1024, seed=1,
                plane=50.0) -> Scene:
    """Noise-displaced icospheres scattered over a plane (1 310 720 + 2
    triangles at the defaults)."""
    rng = np.random.default_rng(seed)
    unit, faces = icosphere(levels)
    idx = faces.astype(np.uint32).reshape(-1)
    mats: List[Material] = []
    for _ in range(materials):
        base = tuple(float(x) for x in rng.uniform(0.05, 0.95, 3))
        rough = float(rng.uniform(0.05, 1.0))
        metal = 1.0 if rng.random() < 0.3 else 0.0
        mats.append(standard_surface(base, rough, metal, 1.5))
    mats.append(lambert((0.5, 0.5, 0.5)))  # ground plane
    meshes = []
    h = plane * 0.5 - 1.5
    for _ in range(instances):
        radius = float(rng.uniform(0.4, 1.2))
        cx, cz = rng.uniform(-h, h, 2)
        freqs = rng.normal(0.0, 3.0, size=(3, 3))
        phases = rng.uniform(0, 2 * np.pi, 3)
        amps = rng.uniform(0.03, 0.08, 3)
        disp = 1.0 + (amps[None, :] * np.sin(unit @ freqs.T + phases[None, :])).sum(1)
        local = unit * disp[:, None] * radius
        center = np.array([cx, radius * 0.85, cz])
        pos = local + center
        nrm = smooth_normals(pos, faces)
        meshes.append(Mesh(pos.astype(np.float32), idx, nrm.astype(np.float32), int(rng.integers(0, materials))))
    gpos, gnrm, gidx = ground_quad(plane)
    meshes.append(Mesh(gpos, gidx, gnrm, materials))
    env = procedural_hdri(env_width, env_height, seed + 100, sun_dir=(-0.35, 0.55, 0.76))
    return Scene(materials=mats, meshes=meshes, dome_lights=[DomeLight(env=env)],
                 distant_lights=[DistantLight(direction=(-0.3, -1.0, -0.4), radiance=(2.5, 2.4, 2.2))])


def field_camera(aspect=16.0 / 9.0) -> Camera:
    return look_at((0.0, 14.0, 36.0), (0.0, 0.0, -2.0), 45.0, aspect)


def field_workload(width=1920, height=1080, spp=64, depth=12, **kw) -> Workload:
    st = RenderSettings(width=width, height=height, samples_per_pixel=spp, max_depth=depth,
                        diffuse_depth=depth, specular_depth=depth, dome_light_samples=1,
                        background_visible=True, backend=1)
    return Workload(f"field 1310720 tris {width}x{height} {spp}spp depth {depth}", field_scene(**kw),
                    field_camera(width / height), st)


@dataclass
class Request:
    camera: Camera
    settings: RenderSettings


def batch_requests(count=48, seed=3, lo=128, hi=1024) -> List[Request]:
    """Requests of log-uniform square resolution in [lo, hi], spp from
    {4, 16, 64} and depth from {4, 8, 12}, each with its own orbit camera."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        s = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        spp = int(rng.choice([4, 16, 64]))
        depth = int(rng.choice([4, 8, 12]))
        az = rng.uniform(0, 2 * np.pi)
        el = rng.uniform(0.05, 0.6)
        dist = rng.uniform(3.5, 6.0)
        pos = (dist * math.cos(el) * math.sin(az), 1.0 + dist * math.sin(el), dist * math.cos(el) * math.cos(az))
        cam = look_at(pos, (0.0, 0.9, 0.0), 45.0, 1.0)
        st = RenderSettings(width=s, height=s, samples_per_pixel=spp, max_depth=depth, diffuse_depth=depth,
                            specular_depth=depth, dome_light_samples=1, backend=1)
        out.append(Request(cam, st))
    return out


def split_sphere_scene(parts=256, env_width=512, env_height=256, seed=4) -> Scene:
    """The sphere scene cut into `parts` meshes (parts-1 sphere chunks + the
    ground), each with its own seeded material (base colour U(0.05, 0.95)^3,
    roughness U(0.05, 1), metalness U(0, 1))."""
    rng = np.random.default_rng(seed)
    spos, snrm, sidx = uv_sphere()
    tris = sidx.reshape(-1, 3)
    chunks = np.array_split(np.arange(tris.shape[0]), parts - 1)
    meshes, mats = [], []
    for k, ch in enumerate(chunks):
        t = tris[ch]
        used, inv = np.unique(t.reshape(-1), return_inverse=True)
        meshes.append(Mesh(spos[used], inv.astype(np.uint32), snrm[used], k))
        mats.append(standard_surface(tuple(float(x) for x in rng.uniform(0.05, 0.95, 3)),
                                     float(rng.uniform(0.05, 1.0)), float(rng.uniform(0.0, 1.0)), 1.5))
    gpos, gnrm, gidx = ground_quad()
    meshes.append(Mesh(gpos, gidx, gnrm, parts - 1))
    mats.append(standard_surface(tuple(float(x) for x in rng.uniform(0.05, 0.95, 3)),
                                 float(rng.uniform(0.05, 1.0)), float(rng.uniform(0.0, 1.0)), 1.5))
    env = procedural_hdri(env_width, env_height, seed + 100)
    return Scene(materials=mats, meshes=meshes, dome_lights=[DomeLight(env=env)])
