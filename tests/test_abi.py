"""CPU-side checks of the C ABI: the native library loads and exports every
function include/*.h declares; struct layouts of the ctypes mirror match the
header; host-side behaviour without a device (no compute call is made)."""
import ctypes as C
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from shiro_gb300 import build

    build.build()
    from shiro_gb300.backend import load_library

    return load_library()


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:int|void|const char\*)\s+(shiro_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "shiro_gb300", "libshiro_gpu.so")],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (shiro_\w+)", out))
    assert set(names) <= exported


def test_constants_match_header():
    """Every SHIRO_ERR_* and SHIRO_RENDER_* value of the header has the same
    value in the ctypes mirror."""
    from shiro_gb300 import abi

    text = open(os.path.join(ROOT, "include", "shiro_gpu.h")).read()
    found = re.findall(r"^#define SHIRO_(ERR_\w+|RENDER_\w+)\s+\(?(-?(?:0x)?[0-9a-fA-F]+)u?\)?", text, flags=re.M)
    assert len(found) >= 12
    for name, value in found:
        mirror = ("SHIRO_" + name) if name.startswith("ERR_") else name
        assert getattr(abi, mirror) == int(value, 0), name


def test_struct_sizes_match_header():
    from shiro_gb300 import abi

    src = r"""
#include <stdio.h>
#include "shiro_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(ShiroMaterialDesc), sizeof(ShiroMeshDesc),
         sizeof(ShiroDistantLightDesc), sizeof(ShiroDomeLightDesc), sizeof(ShiroSceneDesc), sizeof(ShiroCameraDesc),
         sizeof(ShiroSettingsDesc), sizeof(ShiroRenderDesc), sizeof(ShiroAovs), sizeof(ShiroBackendStatus),
         sizeof(ShiroRenderStats));
  return 0;
}
"""
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "s")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    mirror = [C.sizeof(t) for t in (abi.MaterialDesc, abi.MeshDesc, abi.DistantLightDesc, abi.DomeLightDesc,
                                    abi.SceneDesc, abi.CameraDesc, abi.SettingsDesc, abi.RenderDesc, abi.Aovs,
                                    abi.BackendStatus, abi.RenderStats)]
    assert sizes == mirror


def test_status_without_device_is_unavailable(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    from shiro_gb300 import GpuBackend, ShiroGpuError

    st = GpuBackend.get_status()
    assert st["available"] is False and st["device_count"] == 0
    with pytest.raises(ShiroGpuError):
        GpuBackend(0)  # no silent CPU fallback


def test_scene_support_on_host(lib):
    """Every lobe of the reference's TracePath is implemented: opacity,
    transmission and emitters are accepted; only a malformed snapshot is not."""
    from shiro_gb300 import scenes
    from shiro_gb300.abi import MarshalledScene

    sc = scenes.sphere_scene(8, 4)
    buf = C.create_string_buffer(128)
    assert lib.shiro_gpu_supports_scene(MarshalledScene(sc).ref(), buf, 128) == 1
    sc.materials[0].opacity = 0.5
    sc.materials[0].transmission = 1.0
    sc.materials[1].emission_strength = 3.0
    sc.materials[1].emission_color = (1.0, 1.0, 1.0)
    assert lib.shiro_gpu_supports_scene(MarshalledScene(sc).ref(), buf, 128) == 1
    assert lib.shiro_gpu_supports_scene(None, buf, 128) == 0
    assert b"null" in buf.value


def test_scene_signature_tracks_every_uploaded_field(lib):
    """shiro_gpu_scene_signature (host code, no device): equal for equal
    content, different after an in-place edit of any field the upload reads."""
    import numpy as np

    from shiro_gb300 import scenes
    from shiro_gb300.abi import DistantLight, MarshalledScene

    def sig(sc):
        out = C.c_uint64(0)
        assert lib.shiro_gpu_scene_signature(MarshalledScene(sc).ref(), C.byref(out)) == 0
        return out.value

    sc = scenes.sphere_scene(env_width=64, env_height=32)
    sc.distant_lights = [DistantLight(direction=(-0.3, -1.0, -0.4), radiance=(2.5, 2.4, 2.2))]
    base = sig(sc)
    assert sig(sc) == base
    seen = {base}

    def changed(mutate, undo):
        mutate()
        s = sig(sc)
        undo()
        assert sig(sc) == base
        assert s not in seen
        seen.add(s)

    m0 = sc.meshes[0]
    pos, nrm, idx = m0.positions.copy(), m0.normals.copy(), m0.indices.copy()
    env = sc.dome_lights[0].env.copy()
    changed(lambda: sc.distant_lights[0].__setattr__("radiance", (7.0, 3.0, 1.0)),
            lambda: sc.distant_lights[0].__setattr__("radiance", (2.5, 2.4, 2.2)))
    changed(lambda: m0.positions.__setitem__((5, 1), m0.positions[5, 1] + 1e-3),
            lambda: m0.positions.__setitem__(slice(None), pos))
    changed(lambda: m0.normals.__setitem__((7, 0), 0.5), lambda: m0.normals.__setitem__(slice(None), nrm))
    changed(lambda: m0.indices.__setitem__(3, m0.indices[4]), lambda: m0.indices.__setitem__(slice(None), idx))
    changed(lambda: setattr(m0, "material_index", 1), lambda: setattr(m0, "material_index", 0))
    changed(lambda: setattr(sc.materials[1], "roughness", 0.77), lambda: setattr(sc.materials[1], "roughness", 1.0))
    changed(lambda: sc.dome_lights[0].env.__setitem__((3, 4, 2), 9.0),
            lambda: sc.dome_lights[0].env.__setitem__(slice(None), env))
    changed(lambda: setattr(sc.dome_lights[0], "up", (0.0, 0.0, 1.0)),
            lambda: setattr(sc.dome_lights[0], "up", (0.0, 1.0, 0.0)))
    changed(lambda: setattr(sc, "environment_top", (0.1, 0.2, 0.3)),
            lambda: setattr(sc, "environment_top", (0.0, 0.0, 0.0)))
    # a scene large enough for the multi-threaded pieces: stable across calls
    big = scenes.field_scene(instances=48, env_width=1024, env_height=512)
    a, b = sig(big), sig(big)
    assert a == b
    big.meshes[-2].positions[-1, 2] += 1e-3
    assert sig(big) != a
