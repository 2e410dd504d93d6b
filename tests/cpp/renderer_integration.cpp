// renderer_integration.cpp - TEST HARNESS: drives the reference's own
// shiro::render::Renderer (src/render/Renderer.cpp, compiled with the
// two-line patch that holds the GB300 backend instead of the OptiX one) and
// its CPU tracer, and prints one JSON line of checks.  Built by
// tests/test_renderer_integration.py from the reference sources where they
// lie (patched copies go to a temporary directory), either against the real
// device library or against tests/cpp/fake_device.cpp.
//
// Usage: renderer_integration [environment-image-path]
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#include "GpuBackend.h"
#include "shiro/backend/cpu/CpuPathTracer.h"
#include "shiro/render/EnvironmentMap.h"
#include "shiro/render/Renderer.h"

extern "C" int shiro_fake_render_calls __attribute__((weak));

using namespace shiro::render;

namespace {

int FakeCalls() { return &shiro_fake_render_calls ? shiro_fake_render_calls : -1; }

Scene MakeScene(const char* envPath, bool* envLoaded, uint32_t* envW, uint32_t* envH) {
    Scene s;
    PbrMaterial sphere;
    sphere.baseColor = {0.8f, 0.55f, 0.35f};
    sphere.roughness = 0.35f;
    sphere.metallic = 0.2f;
    PbrMaterial ground;
    ground.baseColor = {0.5f, 0.5f, 0.5f};
    ground.specularWeight = 0.0f;
    s.materials = {sphere, ground};
    TriangleMesh ball;
    const int segs = 24, rings = 12;
    const float pi = 3.14159265358979323846f;
    for (int r = 0; r <= rings; ++r)
        for (int k = 0; k <= segs; ++k) {
            const float th = pi * r / rings, ph = 2.0f * pi * k / segs;
            const Vec3f n{std::sin(th) * std::cos(ph), std::cos(th), std::sin(th) * std::sin(ph)};
            ball.positions.push_back({n.x, n.y + 1.0f, n.z});
            ball.normals.push_back(n);
        }
    for (int r = 0; r < rings; ++r)
        for (int k = 0; k < segs; ++k) {
            const uint32_t a = r * (segs + 1) + k, b = a + segs + 1;
            ball.indices.insert(ball.indices.end(), {a, b, a + 1, a + 1, b, b + 1});
        }
    ball.materialIndex = 0;
    TriangleMesh plane;
    plane.positions = {{-5.0f, 0.0f, -5.0f}, {5.0f, 0.0f, -5.0f}, {5.0f, 0.0f, 5.0f}, {-5.0f, 0.0f, 5.0f}};
    plane.normals = {{0, 1, 0}, {0, 1, 0}, {0, 1, 0}, {0, 1, 0}};
    plane.indices = {0, 2, 1, 0, 3, 2};
    plane.materialIndex = 1;
    s.meshes = {ball, plane};
    s.distantLights.push_back(DirectionalLight{{-0.3f, -1.0f, -0.4f}, {2.5f, 2.4f, 2.2f}});
    DomeLight dome;
    dome.radiance = {0.6f, 0.7f, 0.9f};
    *envLoaded = false;
    if (envPath) {
        dome.environment = EnvironmentMap::Load(envPath, EnvironmentMapLayout::LatLong);
        *envLoaded = dome.environment != nullptr;
        if (dome.environment) {
            *envW = dome.environment->Width();
            *envH = dome.environment->Height();
        }
    }
    s.domeLights.push_back(dome);
    return s;
}

float MaxDiff(const FrameBuffer& a, const FrameBuffer& b, bool* same) {
    *same = a.Width() == b.Width() && a.Height() == b.Height();
    if (!*same) return std::numeric_limits<float>::infinity();
    float m = 0.0f;
    auto cmp = [&](float x, float y) {
        uint32_t bx, by;
        std::memcpy(&bx, &x, 4);
        std::memcpy(&by, &y, 4);
        if (bx != by) *same = false;
        if (std::isfinite(x) && std::isfinite(y)) m = std::max(m, std::fabs(x - y));
    };
    for (size_t i = 0; i < a.Beauty().size(); ++i) {
        cmp(a.Beauty()[i].x, b.Beauty()[i].x);
        cmp(a.Beauty()[i].y, b.Beauty()[i].y);
        cmp(a.Beauty()[i].z, b.Beauty()[i].z);
        cmp(a.Beauty()[i].w, b.Beauty()[i].w);
        cmp(a.Albedo()[i].x, b.Albedo()[i].x);
        cmp(a.Normal()[i].y, b.Normal()[i].y);
        cmp(a.Depth()[i], b.Depth()[i]);
    }
    return m;
}

bool Cleared(const FrameBuffer& f) {
    for (size_t i = 0; i < f.Beauty().size(); ++i)
        if (f.Beauty()[i].x != 0.0f || f.Beauty()[i].w != 0.0f || !(f.Depth()[i] == std::numeric_limits<float>::infinity()))
            return false;
    return true;
}

}  // namespace

int main(int argc, char** argv) {
    bool envLoaded = false;
    uint32_t envW = 0, envH = 0;
    const Scene scene = MakeScene(argc > 1 ? argv[1] : nullptr, &envLoaded, &envW, &envH);
    Camera cam{{0.0f, 1.6f, 4.5f}, {0.0f, -0.15f, -0.99f}, {1.0f, 0.0f, 0.0f}, {0.0f, 0.99f, -0.15f}, 45.0f, 32.0f / 24.0f};
    RenderSettings st;
    st.width = 32;
    st.height = 24;
    st.samplesPerPixel = 6;
    st.maxDepth = 4;
    st.diffuseDepth = 4;
    st.specularDepth = 4;
    st.domeLightSamples = 1;
    st.backend = BackendKind::Gpu;

    shiro::backend::gb300::GpuBackend probe;
    const bool available = probe.GetStatus().available;
    Renderer renderer;
    renderer.SetSettings(st);
    shiro::backend::cpu::CpuPathTracer cpu;
    auto cpuBatch = [&](uint32_t start, uint32_t count, const RenderSettings& s) {
        shiro::backend::RenderRequest rq{scene, cam, s, start, count, nullptr};
        return cpu.RenderSampleBatch(rq);
    };

    // 1. one batch through Renderer::RenderSampleBatch (Renderer.cpp:119-128)
    const int calls0 = FakeCalls();
    const FrameBuffer viaRenderer = renderer.RenderSampleBatch(scene, cam, 0, 6);
    const int calls1 = FakeCalls();
    bool singleSame = false;
    const float singleDiff = MaxDiff(viaRenderer, cpuBatch(0, 6, st), &singleSame);

    // 2. a progressive render: batches at sample 0, 2, 3 through the
    // Renderer, folded by its FrameAccumulator (Renderer.cpp:47-110)
    Renderer::FrameAccumulator accR, accC;
    const uint32_t batches[3][2] = {{0, 2}, {2, 1}, {3, 3}};
    for (const auto& b : batches) {
        accR.Accumulate(renderer.RenderSampleBatch(scene, cam, b[0], b[1]), b[1]);
        accC.Accumulate(cpuBatch(b[0], b[1], st), b[1]);
    }
    bool progSame = false;
    const float progDiff = MaxDiff(accR.Resolve(), accC.Resolve(), &progSame);
    const int calls2 = FakeCalls();

    // 3. settings that ask for the CPU backend never reach the GPU one
    RenderSettings cpuSt = st;
    cpuSt.backend = BackendKind::Cpu;
    Renderer cpuRenderer;
    cpuRenderer.SetSettings(cpuSt);
    bool cpuSame = false;
    MaxDiff(cpuRenderer.RenderSampleBatch(scene, cam, 0, 2), cpuBatch(0, 2, cpuSt), &cpuSame);
    const int calls3 = FakeCalls();

    // 4. a cancel flag already set: the GPU route returns a cleared frame
    std::atomic<bool> cancel{true};
    const FrameBuffer cancelled = renderer.RenderSampleBatch(scene, cam, 0, 2, &cancel);
    const int calls4 = FakeCalls();

    std::printf("{\"available\": %s, \"env_loaded\": %s, \"env_width\": %u, \"env_height\": %u, "
                "\"single_bit_exact\": %s, \"single_max_diff\": %g, \"progressive_bit_exact\": %s, "
                "\"progressive_max_diff\": %g, \"cpu_settings_bit_exact\": %s, \"cancelled_cleared\": %s, "
                "\"gpu_calls_single\": %d, \"gpu_calls_progressive\": %d, \"gpu_calls_cpu_settings\": %d, "
                "\"gpu_calls_cancelled\": %d}\n",
                available ? "true" : "false", envLoaded ? "true" : "false", envW, envH, singleSame ? "true" : "false",
                singleDiff, progSame ? "true" : "false", progDiff, cpuSame ? "true" : "false",
                Cleared(cancelled) ? "true" : "false", calls0 < 0 ? -1 : calls1 - calls0,
                calls0 < 0 ? -1 : calls2 - calls1, calls0 < 0 ? -1 : calls3 - calls2, calls0 < 0 ? -1 : calls4 - calls3);
    return 0;
}
