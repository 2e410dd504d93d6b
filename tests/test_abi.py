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
