"""The backend inside the reference's own Renderer (src/render/Renderer.cpp).

Shiro holds its GPU backend in Renderer::Impl and falls back to the CPU
tracer when the backend is unavailable or declines the scene
(Renderer.cpp:12-31).  This test compiles the reference's Renderer.cpp with
the two-line change that swaps the OptiX backend for the GB300 adapter
(GpuBackend), the reference's EnvironmentMap.cpp with its no-OpenImageIO
branch calling the native image reader (shiro_hdri_load), and the reference
CPU tracer, all from the reference sources where they lie; the patched copies
are written to a temporary directory, never into this repository.  Then:

* linked against a stand-in device library that renders with the CPU oracle
  (tests/cpp/fake_device.cpp): Renderer::RenderSampleBatch with backend Gpu
  reaches GpuBackend (the stand-in counts its renders) and its frames, single
  and over a progressive render folded by Renderer::FrameAccumulator, equal
  the reference CPU tracer's bit for bit; a backend reported unavailable, or
  a scene the backend declines, falls back to the CPU tracer; settings asking
  for the CPU never reach the GPU backend; a set cancel flag gives a cleared
  frame;
* linked against the real device library on a machine without a usable GPU:
  GpuBackend reports itself unavailable and the Renderer renders on the CPU;
* an environment image written to disk loads through the patched
  EnvironmentMap::Load.

Runs where the reference tree and a host C++ compiler exist (not on a GPU
box, which has neither the reference nor needs it for the other tests).
"""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference"
CPP = os.path.join(ROOT, "tests", "cpp")

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src", "render")) or not shutil.which("g++"),
                                reason="needs the reference sources and g++")

# Renderer.cpp: hold the GB300 adapter where the OptiX backend was (the member
# keeps its name, so ResolveBackend - the reference's fallback rule - is
# compiled unchanged)
RENDERER_PATCH = [
    ('#include "shiro/backend/optix/OptixBackend.h"', '#include "GpuBackend.h"'),
    ("backend::optix::OptixBackend optixBackend;", "backend::gb300::GpuBackend optixBackend;"),
]
# EnvironmentMap.cpp: without OpenImageIO, read .hdr / .exr with the native reader
ENV_PATCH = [
    ('#include "shiro/core/Config.h"', '#include "shiro/core/Config.h"\n#include "shiro_gpu.h"'),
    ("""#else
    (void)filePath;
    (void)layout;
    return nullptr;
#endif""", """#else
    uint32_t width = 0, height = 0;
    float* texels = nullptr;
    if (shiro_hdri_load(filePath.c_str(), &width, &height, &texels, nullptr, 0) != 0) {
        return nullptr;
    }
    auto environment = std::shared_ptr<EnvironmentMap>(new EnvironmentMap());
    environment->width_ = width;
    environment->height_ = height;
    environment->layout_ = ResolveLayout(layout);
    environment->pixels_.resize(static_cast<size_t>(width) * static_cast<size_t>(height));
    for (size_t i = 0; i < environment->pixels_.size(); ++i) {
        environment->pixels_[i] = {texels[3 * i], texels[3 * i + 1], texels[3 * i + 2]};
    }
    shiro_hdri_free(texels);
    environment->BuildImportanceTable();
    return environment;
#endif"""),
]


def _patched(src, patches, out):
    text = open(src).read()
    for old, new in patches:
        assert text.count(old) == 1, f"patch anchor not found once in {src}: {old[:40]}"
        text = text.replace(old, new)
    with open(out, "w") as f:
        f.write(text)
    return out


@pytest.fixture(scope="module")
def binaries(tmp_path_factory):
    from shiro_gb300 import build

    lib = build.build()
    tmp = tmp_path_factory.mktemp("renderer")
    renderer = _patched(os.path.join(REF, "src", "render", "Renderer.cpp"), RENDERER_PATCH, str(tmp / "Renderer.cpp"))
    envmap = _patched(os.path.join(REF, "src", "render", "EnvironmentMap.cpp"), ENV_PATCH,
                      str(tmp / "EnvironmentMap.cpp"))
    common = [renderer, envmap,
              os.path.join(REF, "src", "backend", "cpu", "CpuPathTracer.cpp"),
              os.path.join(REF, "src", "render", "OpenQmcSampler.cpp"),
              os.path.join(REF, "src", "render", "FrameBuffer.cpp"),
              os.path.join(REF, "src", "backend", "RenderBackend.cpp"),
              os.path.join(ROOT, "shiro_gb300", "backend", "GpuBackend.cpp"),
              os.path.join(CPP, "renderer_integration.cpp")]
    flags = ["-O2", "-std=c++17", "-pthread", "-ffp-contract=off", "-w",
             "-DSHIRO_HAVE_EMBREE=0", "-DSHIRO_WITH_OPENQMC=0", "-DSHIRO_HAVE_OIIO=0", "-DSHIRO_HAVE_CUDA=0",
             "-DSHIRO_HAVE_OPTIX=0", "-I", os.path.join(REF, "include"), "-I", REF,
             "-I", os.path.join(ROOT, "shiro_gb300", "backend"), "-I", os.path.join(ROOT, "include")]
    objs = []
    for src in common:
        obj = str(tmp / (os.path.basename(src) + ".o"))
        subprocess.run(["g++"] + flags + ["-c", src, "-o", obj], check=True)
        objs.append(obj)
    fake_srcs = [os.path.join(CPP, "fake_device.cpp"), os.path.join(ROOT, "oracle", "port", "shiro_oracle.cpp"),
                 os.path.join(ROOT, "shiro_gb300", "csrc", "hdri_io.cpp")]
    fake = str(tmp / "renderer_fake")
    subprocess.run(["g++"] + flags + ["-o", fake] + objs + fake_srcs, check=True)
    real = str(tmp / "renderer_real")
    pkg = os.path.dirname(lib)
    subprocess.run(["g++"] + flags + ["-o", real] + objs + ["-L", pkg, "-lshiro_gpu", f"-Wl,-rpath,{pkg}"], check=True)
    # an environment image on disk (Radiance RGBE)
    from shiro_gb300 import scenes
    from test_hdri import float_to_rgbe, hdr_bytes

    hdr = tmp / "dome.hdr"
    hdr.write_bytes(hdr_bytes(float_to_rgbe(scenes.procedural_hdri(64, 32, 3)), "new"))
    return fake, real, str(hdr)


def _run(exe, env_path, **env):
    e = dict(os.environ)
    e.update({k: str(v) for k, v in env.items()})
    out = subprocess.run([exe, env_path], capture_output=True, text=True, env=e, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = [l for l in out.stdout.splitlines() if l.startswith("{")][-1]
    return json.loads(line)


def test_renderer_routes_to_the_gb300_backend(binaries):
    fake, _, hdr = binaries
    r = _run(fake, hdr)
    assert r["available"] and r["env_loaded"] and (r["env_width"], r["env_height"]) == (64, 32)
    assert r["gpu_calls_single"] == 1 and r["gpu_calls_progressive"] == 3  # routed through GpuBackend
    assert r["single_bit_exact"], r
    assert r["progressive_bit_exact"], r
    assert r["cpu_settings_bit_exact"] and r["gpu_calls_cpu_settings"] == 0
    assert r["cancelled_cleared"] and r["gpu_calls_cancelled"] == 0


@pytest.mark.parametrize("switch", ["SHIRO_FAKE_UNAVAILABLE", "SHIRO_FAKE_UNSUPPORTED"])
def test_renderer_falls_back_to_the_cpu_tracer(binaries, switch):
    fake, _, hdr = binaries
    r = _run(fake, hdr, **{switch: 1})
    assert r["gpu_calls_single"] == 0 and r["gpu_calls_progressive"] == 0
    assert r["single_bit_exact"] and r["progressive_bit_exact"], r


def test_real_device_library_without_a_gpu_falls_back(binaries):
    _, real, hdr = binaries
    import ctypes as C

    from shiro_gb300.backend import load_library
    from shiro_gb300.abi import BackendStatus

    st = BackendStatus()
    load_library().shiro_gpu_status(C.byref(st))
    if st.available:
        pytest.skip("a usable GPU is present: the Renderer would route to it (covered by the GPU tests)")
    r = _run(real, hdr)
    assert not r["available"] and r["env_loaded"]
    assert r["single_bit_exact"] and r["progressive_bit_exact"] and r["cpu_settings_bit_exact"], r
