"""ctypes mirror of include/shiro_gpu.h plus the scene marshaller.

The same structs drive three libraries: the CUDA backend
(shiro_gb300/libshiro_gpu.so), the CPU restatement used as the oracle
(oracle/libshiro_oracle.so) and, in the development container only, the
reference integrator compiled from its own sources (oracle/_ref).

Field order follows shiro/render/Renderer.h:29-133 of ichin0se/Shiro.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, fields
from typing import List, Optional

import numpy as np

SHIRO_OK = 0
SHIRO_ERR_INVALID_ARGUMENT = -1
SHIRO_ERR_NO_DEVICE = -2
SHIRO_ERR_CUDA = -3
SHIRO_ERR_OUT_OF_MEMORY = -4
SHIRO_ERR_UNSUPPORTED_SCENE = -5
SHIRO_ERR_CANCELLED = -6
SHIRO_ERR_NO_SCENE = -7
SHIRO_ERR_TIMEOUT = -8
SHIRO_ERR_DEVICE_CHECK = -9

BACKEND_CPU, BACKEND_GPU, BACKEND_HYBRID = 0, 1, 2
ENV_AUTOMATIC, ENV_LATLONG, ENV_ANGULAR = 0, 1, 2
RENDER_ENV_CDF = 0x1
RENDER_NO_CLAMP = 0x2
RENDER_KEEP_PATHS = 0x4

# ShiroPixelsReady(user, request, first_pixel, pixel_count)
PixelsReady = C.CFUNCTYPE(None, C.c_void_p, C.c_uint32, C.c_uint64, C.c_uint64)

F3 = C.c_float * 3


class MaterialDesc(C.Structure):
    _fields_ = [
        ("base_color", F3), ("emission_color", F3), ("specular_color", F3),
        ("transmission_color", F3), ("transmission_scatter", F3), ("coat_color", F3),
        ("subsurface_color", F3), ("subsurface_radius", F3), ("sheen_color", F3),
        ("normal_override", F3), ("coat_normal_override", F3), ("tangent_override", F3),
        ("base_weight", C.c_float), ("emission_strength", C.c_float),
        ("specular_weight", C.c_float), ("metallic", C.c_float), ("roughness", C.c_float),
        ("diffuse_roughness", C.c_float), ("opacity", C.c_float),
        ("specular_anisotropy", C.c_float), ("specular_rotation", C.c_float),
        ("coat_weight", C.c_float), ("coat_roughness", C.c_float), ("coat_ior", C.c_float),
        ("coat_anisotropy", C.c_float), ("coat_rotation", C.c_float), ("sheen", C.c_float),
        ("sheen_roughness", C.c_float), ("subsurface", C.c_float),
        ("subsurface_scale", C.c_float), ("subsurface_anisotropy", C.c_float),
        ("transmission", C.c_float), ("transmission_depth", C.c_float),
        ("transmission_scatter_anisotropy", C.c_float), ("transmission_dispersion", C.c_float),
        ("transmission_extra_roughness", C.c_float), ("ior", C.c_float),
        ("coat_affect_color", C.c_float), ("coat_affect_roughness", C.c_float),
        ("thin_film_thickness", C.c_float), ("thin_film_ior", C.c_float),
        ("thin_walled", C.c_uint32), ("has_normal_override", C.c_uint32),
        ("has_coat_normal_override", C.c_uint32), ("has_tangent_override", C.c_uint32),
    ]


class MeshDesc(C.Structure):
    _fields_ = [
        ("positions", C.POINTER(C.c_float)), ("vertex_count", C.c_uint32),
        ("normals", C.POINTER(C.c_float)), ("normal_count", C.c_uint32),
        ("indices", C.POINTER(C.c_uint32)), ("index_count", C.c_uint32),
        ("material_index", C.c_uint32),
    ]


class DistantLightDesc(C.Structure):
    _fields_ = [("direction", F3), ("radiance", F3)]


class DomeLightDesc(C.Structure):
    _fields_ = [
        ("radiance", F3), ("right", F3), ("up", F3), ("forward", F3),
        ("layout", C.c_uint32), ("env_width", C.c_uint32), ("env_height", C.c_uint32),
        ("env_pixels", C.POINTER(C.c_float)),
    ]


class SceneDesc(C.Structure):
    _fields_ = [
        ("materials", C.POINTER(MaterialDesc)), ("material_count", C.c_uint32),
        ("meshes", C.POINTER(MeshDesc)), ("mesh_count", C.c_uint32),
        ("distant_lights", C.POINTER(DistantLightDesc)), ("distant_light_count", C.c_uint32),
        ("dome_lights", C.POINTER(DomeLightDesc)), ("dome_light_count", C.c_uint32),
        ("environment_top", F3), ("environment_bottom", F3),
    ]


class CameraDesc(C.Structure):
    _fields_ = [
        ("position", F3), ("forward", F3), ("right", F3), ("up", F3),
        ("vertical_fov_degrees", C.c_float), ("aspect_ratio", C.c_float),
    ]


class SettingsDesc(C.Structure):
    _fields_ = [
        ("width", C.c_uint32), ("height", C.c_uint32), ("samples_per_pixel", C.c_uint32),
        ("samples_per_update", C.c_uint32), ("dome_light_samples", C.c_uint32),
        ("max_depth", C.c_uint32), ("diffuse_depth", C.c_uint32),
        ("specular_depth", C.c_uint32), ("thread_limit", C.c_uint32),
        ("max_subdiv_level", C.c_uint32), ("backend", C.c_uint32),
        ("background_visible", C.c_uint32), ("enable_headlight", C.c_uint32),
        ("enable_caustics", C.c_uint32), ("enable_sss", C.c_uint32),
    ]


class RenderDesc(C.Structure):
    _fields_ = [
        ("camera", CameraDesc), ("settings", SettingsDesc),
        ("sample_start", C.c_uint32), ("sample_count", C.c_uint32),
        ("flags", C.c_uint32), ("reserved", C.c_uint32),
    ]


class Aovs(C.Structure):
    _fields_ = [
        ("beauty", C.POINTER(C.c_float)), ("albedo", C.POINTER(C.c_float)),
        ("normal", C.POINTER(C.c_float)), ("depth", C.POINTER(C.c_float)),
        ("on_device", C.c_uint32), ("reserved", C.c_uint32),
    ]


class BackendStatus(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32), ("available", C.c_uint32), ("uses_gpu", C.c_uint32),
        ("device_count", C.c_uint32), ("name", C.c_char * 32), ("device_name", C.c_char * 96),
        ("compute_major", C.c_int32), ("compute_minor", C.c_int32),
    ]


class WavefrontConfig(C.Structure):
    _fields_ = [
        ("paths_in_flight", C.c_uint32), ("extend_block", C.c_uint32),
        ("shade_block", C.c_uint32), ("shadow_block", C.c_uint32),
        ("use_graph", C.c_uint32), ("shade_regs", C.c_uint32), ("extend_steps", C.c_uint32),
        ("refill_idle", C.c_uint32), ("concurrent_waves", C.c_uint32), ("bin_rays", C.c_uint32),
        ("bin_shadow", C.c_uint32), ("coop_extend", C.c_uint32), ("coop_occlude", C.c_uint32),
        ("extend_regs", C.c_uint32), ("occlude_regs", C.c_uint32), ("occlude_refill", C.c_uint32),
    ]


class RenderStats(C.Structure):
    _fields_ = [
        ("kernel_ms", C.c_double), ("path_kernel_ms", C.c_double), ("path_kernel_launches", C.c_uint64),
        ("paths", C.c_uint64), ("kernel_launches", C.c_uint64),
        ("bvh_nodes", C.c_uint64), ("triangles", C.c_uint64), ("bvh_depth", C.c_uint32),
        ("bvh_max_leaf", C.c_uint32), ("device_bytes", C.c_uint64),
        ("stage_ms", C.c_double * 6), ("stage_launches", C.c_uint64 * 6), ("waves", C.c_uint64),
    ]


class WorkCounts(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("paths", "closest_rays", "occlusion_rays", "node_visits", "tri_tests", "hits",
                                          "env_evals", "env_samples", "bsdf_evals", "bsdf_pdfs",
                                          "occlusion_node_visits", "occlusion_tri_tests")]


# ---------------------------------------------------------------------------
# Python-side scene snapshot (mirrors shiro::render::Scene and friends).
# ---------------------------------------------------------------------------


@dataclass
class Material:
    """shiro::render::PbrMaterial (Renderer.h:56-102) with its defaults."""

    base_color: tuple = (0.8, 0.8, 0.8)
    emission_color: tuple = (0.0, 0.0, 0.0)
    specular_color: tuple = (1.0, 1.0, 1.0)
    transmission_color: tuple = (1.0, 1.0, 1.0)
    transmission_scatter: tuple = (0.0, 0.0, 0.0)
    coat_color: tuple = (1.0, 1.0, 1.0)
    subsurface_color: tuple = (1.0, 1.0, 1.0)
    subsurface_radius: tuple = (1.0, 1.0, 1.0)
    sheen_color: tuple = (1.0, 1.0, 1.0)
    normal_override: tuple = (0.0, 0.0, 0.0)
    coat_normal_override: tuple = (0.0, 0.0, 0.0)
    tangent_override: tuple = (0.0, 0.0, 0.0)
    base_weight: float = 1.0
    emission_strength: float = 0.0
    specular_weight: float = 1.0
    metallic: float = 0.0
    roughness: float = 0.5
    diffuse_roughness: float = 0.0
    opacity: float = 1.0
    specular_anisotropy: float = 0.0
    specular_rotation: float = 0.0
    coat_weight: float = 0.0
    coat_roughness: float = 0.03
    coat_ior: float = 1.5
    coat_anisotropy: float = 0.0
    coat_rotation: float = 0.0
    sheen: float = 0.0
    sheen_roughness: float = 0.3
    subsurface: float = 0.0
    subsurface_scale: float = 1.0
    subsurface_anisotropy: float = 0.0
    transmission: float = 0.0
    transmission_depth: float = 0.0
    transmission_scatter_anisotropy: float = 0.0
    transmission_dispersion: float = 0.0
    transmission_extra_roughness: float = 0.0
    ior: float = 1.5
    coat_affect_color: float = 0.0
    coat_affect_roughness: float = 0.0
    thin_film_thickness: float = 0.0
    thin_film_ior: float = 1.5
    thin_walled: bool = False
    has_normal_override: bool = False
    has_coat_normal_override: bool = False
    has_tangent_override: bool = False

    def to_desc(self) -> MaterialDesc:
        d = MaterialDesc()
        for f in fields(self):
            v = getattr(self, f.name)
            if isinstance(v, tuple):
                setattr(d, f.name, F3(*[float(x) for x in v]))
            elif isinstance(v, bool):
                setattr(d, f.name, 1 if v else 0)
            else:
                setattr(d, f.name, float(v))
        return d


def usd_preview_surface(diffuse_color=(0.18, 0.18, 0.18), roughness=0.5, metallic=0.0, ior=1.5,
                        opacity=1.0) -> Material:
    """Material produced by ParseUsdPreviewSurface (SceneBridge.cpp:648-662)."""
    return Material(base_color=tuple(diffuse_color), roughness=roughness, metallic=metallic, ior=ior,
                    opacity=opacity, thin_walled=opacity < 1.0, specular_weight=1.0,
                    specular_color=(1.0, 1.0, 1.0))


def standard_surface(base_color=(0.8, 0.8, 0.8), specular_roughness=0.2, metalness=0.0,
                     specular_ior=1.5, **extra) -> Material:
    """Material produced by ParseStandardSurface (SceneBridge.cpp:664-772)."""
    return Material(base_color=tuple(base_color), roughness=specular_roughness, metallic=metalness,
                    ior=specular_ior, **extra)


def lambert(color=(0.5, 0.5, 0.5)) -> Material:
    """Pure Lambert: specular weight 0, metallic 0, diffuse roughness 0."""
    return Material(base_color=tuple(color), specular_weight=0.0, metallic=0.0, diffuse_roughness=0.0,
                    roughness=1.0)


@dataclass
class Mesh:
    positions: np.ndarray  # (V, 3) float32
    indices: np.ndarray  # (T*3,) uint32
    normals: Optional[np.ndarray] = None  # (V, 3) float32 or None
    material_index: int = 0


@dataclass
class DistantLight:
    direction: tuple = (0.0, -1.0, -1.0)
    radiance: tuple = (2.0, 2.0, 2.0)


@dataclass
class DomeLight:
    radiance: tuple = (1.0, 1.0, 1.0)
    env: Optional[np.ndarray] = None  # (H, W, 3) float32
    layout: int = ENV_AUTOMATIC
    right: tuple = (1.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    forward: tuple = (0.0, 0.0, 1.0)


@dataclass
class Scene:
    materials: List[Material] = field(default_factory=list)
    meshes: List[Mesh] = field(default_factory=list)
    distant_lights: List[DistantLight] = field(default_factory=list)
    dome_lights: List[DomeLight] = field(default_factory=list)
    environment_top: tuple = (0.0, 0.0, 0.0)
    environment_bottom: tuple = (0.0, 0.0, 0.0)

    @property
    def triangle_count(self) -> int:
        return sum(int(m.indices.size) // 3 for m in self.meshes)


@dataclass
class Camera:
    position: tuple = (0.0, 0.0, 5.0)
    forward: tuple = (0.0, 0.0, -1.0)
    right: tuple = (1.0, 0.0, 0.0)
    up: tuple = (0.0, 1.0, 0.0)
    vertical_fov_degrees: float = 45.0
    aspect_ratio: float = 16.0 / 9.0

    def to_desc(self) -> CameraDesc:
        return CameraDesc(F3(*self.position), F3(*self.forward), F3(*self.right), F3(*self.up),
                          float(self.vertical_fov_degrees), float(self.aspect_ratio))


@dataclass
class RenderSettings:
    """shiro::render::RenderSettings (Renderer.h:29-45) with its defaults."""

    width: int = 1280
    height: int = 720
    samples_per_pixel: int = 32
    samples_per_update: int = 1
    dome_light_samples: int = 1
    max_depth: int = 3
    diffuse_depth: int = 2
    specular_depth: int = 2
    thread_limit: int = 0
    max_subdiv_level: int = 2
    backend: int = BACKEND_CPU
    background_visible: bool = True
    enable_headlight: bool = True
    enable_caustics: bool = True
    enable_sss: bool = True

    def to_desc(self) -> SettingsDesc:
        return SettingsDesc(*[int(getattr(self, f.name)) for f in fields(self)])


def render_desc(camera: Camera, settings: RenderSettings, sample_start: int = 0,
                sample_count: int = 1, flags: int = 0) -> RenderDesc:
    return RenderDesc(camera.to_desc(), settings.to_desc(), int(sample_start), int(sample_count),
                      int(flags), 0)


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _uptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def _same_memory(src, arr: np.ndarray) -> bool:
    return isinstance(src, np.ndarray) and src.size > 0 and src.ctypes.data == arr.ctypes.data


def scene_structure_key(scene: Scene) -> tuple:
    """Every small field of a scene by value and every large array by object
    identity: equal keys mean a MarshalledScene built earlier still describes
    the scene, provided it aliases the arrays (edits inside them are then seen
    through its pointers)."""
    return (tuple(tuple(vars(m).values()) for m in scene.materials),
            tuple((id(m.positions), id(m.indices), id(m.normals), int(m.material_index)) for m in scene.meshes),
            tuple((tuple(l.direction), tuple(l.radiance)) for l in scene.distant_lights),
            tuple((id(d.env), tuple(d.radiance), tuple(d.right), tuple(d.up), tuple(d.forward), int(d.layout))
                  for d in scene.dome_lights),
            tuple(scene.environment_top), tuple(scene.environment_bottom))


class MarshalledScene:
    """Holds a SceneDesc and every array it points into (keeps them alive).
    ``aliased`` is True when every array of the descriptor is the caller's own
    memory (float32 / uint32 and contiguous already), not a converted copy."""

    def __init__(self, scene: Scene):
        self._keep = []
        self.aliased = True
        mats = (MaterialDesc * max(1, len(scene.materials)))()
        for i, m in enumerate(scene.materials):
            mats[i] = m.to_desc()
        meshes = (MeshDesc * max(1, len(scene.meshes)))()
        for i, m in enumerate(scene.meshes):
            pos = np.ascontiguousarray(m.positions, dtype=np.float32).reshape(-1, 3)
            idx = np.ascontiguousarray(m.indices, dtype=np.uint32).reshape(-1)
            self._keep += [pos, idx]
            self.aliased &= (pos.size == 0 or _same_memory(m.positions, pos)) and (idx.size == 0 or _same_memory(m.indices, idx))
            nrm_ptr, ncount = None, 0
            if m.normals is not None:
                nrm = np.ascontiguousarray(m.normals, dtype=np.float32).reshape(-1, 3)
                self.aliased &= nrm.size == 0 or _same_memory(m.normals, nrm)
                self._keep.append(nrm)
                nrm_ptr, ncount = _fptr(nrm), nrm.shape[0]
            meshes[i] = MeshDesc(_fptr(pos), pos.shape[0], nrm_ptr, ncount, _uptr(idx), idx.size,
                                 int(m.material_index))
        dl = (DistantLightDesc * max(1, len(scene.distant_lights)))()
        for i, l in enumerate(scene.distant_lights):
            dl[i] = DistantLightDesc(F3(*l.direction), F3(*l.radiance))
        domes = (DomeLightDesc * max(1, len(scene.dome_lights)))()
        for i, d in enumerate(scene.dome_lights):
            ptr, w, h = None, 0, 0
            if d.env is not None:
                env = np.ascontiguousarray(d.env, dtype=np.float32)
                self.aliased &= env.size == 0 or _same_memory(d.env, env)
                self._keep.append(env)
                h, w = env.shape[0], env.shape[1]
                ptr = _fptr(env)
            domes[i] = DomeLightDesc(F3(*d.radiance), F3(*d.right), F3(*d.up), F3(*d.forward),
                                     int(d.layout), w, h, ptr)
        self._keep += [mats, meshes, dl, domes]
        self.desc = SceneDesc(
            C.cast(mats, C.POINTER(MaterialDesc)), len(scene.materials),
            C.cast(meshes, C.POINTER(MeshDesc)), len(scene.meshes),
            C.cast(dl, C.POINTER(DistantLightDesc)), len(scene.distant_lights),
            C.cast(domes, C.POINTER(DomeLightDesc)), len(scene.dome_lights),
            F3(*scene.environment_top), F3(*scene.environment_bottom))

    def ref(self):
        return C.byref(self.desc)


class FrameBuffer:
    """shiro::render::FrameBuffer (FrameBuffer.h:10-37) as numpy planes.

    pinned=True places the planes in page-locked host memory (allocated
    through torch), so a render's device-to-host copy of the AOVs runs at
    full link speed instead of through the driver's pageable staging."""

    def __init__(self, width: int, height: int, pinned: bool = False):
        self.width, self.height = int(width), int(height)
        n = self.width * self.height
        if pinned:
            import torch

            self._pinned = torch.empty(11 * n, dtype=torch.float32, pin_memory=True)
            flat = self._pinned.numpy()
            self.beauty = flat[:4 * n].reshape(n, 4)
            self.albedo = flat[4 * n:7 * n].reshape(n, 3)
            self.normal = flat[7 * n:10 * n].reshape(n, 3)
            self.depth = flat[10 * n:]
            self.beauty[:] = 0.0
            self.albedo[:] = 0.0
            self.normal[:] = 0.0
            self.depth[:] = np.inf
        else:
            self.beauty = np.zeros((n, 4), np.float32)
            self.albedo = np.zeros((n, 3), np.float32)
            self.normal = np.zeros((n, 3), np.float32)
            self.depth = np.full((n,), np.inf, np.float32)

    def aovs(self) -> Aovs:
        return Aovs(_fptr(self.beauty), _fptr(self.albedo), _fptr(self.normal), _fptr(self.depth), 0, 0)

    def image(self, name="beauty"):
        a = getattr(self, name)
        return a.reshape(self.height, self.width, -1) if a.ndim == 2 else a.reshape(self.height, self.width)
