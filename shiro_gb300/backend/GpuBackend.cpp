// GpuBackend.cpp - RenderBackend adapter over the GB300 C ABI.
#include "GpuBackend.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <limits>
#include <exception>
#include <functional>
#include <thread>
#include <vector>

#include "shiro/render/EnvironmentMap.h"
#include "shiro_gpu.h"

namespace shiro::backend::gb300 {

namespace {

using namespace shiro::render;

void Put3(float* d, const Vec3f& v) {
    d[0] = v.x;
    d[1] = v.y;
    d[2] = v.z;
}

ShiroMaterialDesc ToDesc(const PbrMaterial& m) {
    ShiroMaterialDesc d;
    std::memset(&d, 0, sizeof(d));
    Put3(d.base_color, m.baseColor);
    Put3(d.emission_color, m.emissionColor);
    Put3(d.specular_color, m.specularColor);
    Put3(d.transmission_color, m.transmissionColor);
    Put3(d.transmission_scatter, m.transmissionScatter);
    Put3(d.coat_color, m.coatColor);
    Put3(d.subsurface_color, m.subsurfaceColor);
    Put3(d.subsurface_radius, m.subsurfaceRadius);
    Put3(d.sheen_color, m.sheenColor);
    Put3(d.normal_override, m.normalOverride);
    Put3(d.coat_normal_override, m.coatNormalOverride);
    Put3(d.tangent_override, m.tangentOverride);
    d.base_weight = m.baseWeight;
    d.emission_strength = m.emissionStrength;
    d.specular_weight = m.specularWeight;
    d.metallic = m.metallic;
    d.roughness = m.roughness;
    d.diffuse_roughness = m.diffuseRoughness;
    d.opacity = m.opacity;
    d.specular_anisotropy = m.specularAnisotropy;
    d.specular_rotation = m.specularRotation;
    d.coat_weight = m.coatWeight;
    d.coat_roughness = m.coatRoughness;
    d.coat_ior = m.coatIor;
    d.coat_anisotropy = m.coatAnisotropy;
    d.coat_rotation = m.coatRotation;
    d.sheen = m.sheen;
    d.sheen_roughness = m.sheenRoughness;
    d.subsurface = m.subsurface;
    d.subsurface_scale = m.subsurfaceScale;
    d.subsurface_anisotropy = m.subsurfaceAnisotropy;
    d.transmission = m.transmission;
    d.transmission_depth = m.transmissionDepth;
    d.transmission_scatter_anisotropy = m.transmissionScatterAnisotropy;
    d.transmission_dispersion = m.transmissionDispersion;
    d.transmission_extra_roughness = m.transmissionExtraRoughness;
    d.ior = m.ior;
    d.coat_affect_color = m.coatAffectColor;
    d.coat_affect_roughness = m.coatAffectRoughness;
    d.thin_film_thickness = m.thinFilmThickness;
    d.thin_film_ior = m.thinFilmIor;
    d.thin_walled = m.thinWalled ? 1u : 0u;
    d.has_normal_override = m.hasNormalOverride ? 1u : 0u;
    d.has_coat_normal_override = m.hasCoatNormalOverride ? 1u : 0u;
    d.has_tangent_override = m.hasTangentOverride ? 1u : 0u;
    return d;
}

static_assert(sizeof(Vec3f) == 3 * sizeof(float), "Vec3f must be three packed floats");

// Flat ABI view of a Scene; points into the Scene's own vectors.
struct SceneView {
    std::vector<ShiroMaterialDesc> materials;
    std::vector<ShiroMeshDesc> meshes;
    std::vector<ShiroDistantLightDesc> distant;
    std::vector<ShiroDomeLightDesc> domes;
    ShiroSceneDesc desc{};

    explicit SceneView(const Scene& s) {
        for (const PbrMaterial& m : s.materials) materials.push_back(ToDesc(m));
        for (const TriangleMesh& m : s.meshes) {
            ShiroMeshDesc d{};
            d.positions = reinterpret_cast<const float*>(m.positions.data());
            d.vertex_count = static_cast<uint32_t>(m.positions.size());
            d.normals = m.normals.empty() ? nullptr : reinterpret_cast<const float*>(m.normals.data());
            d.normal_count = static_cast<uint32_t>(m.normals.size());
            d.indices = m.indices.data();
            d.index_count = static_cast<uint32_t>(m.indices.size());
            d.material_index = m.materialIndex;
            meshes.push_back(d);
        }
        for (const DirectionalLight& l : s.distantLights) {
            ShiroDistantLightDesc d{};
            Put3(d.direction, l.direction);
            Put3(d.radiance, l.radiance);
            distant.push_back(d);
        }
        for (const DomeLight& l : s.domeLights) {
            ShiroDomeLightDesc d{};
            Put3(d.radiance, l.radiance);
            Put3(d.right, l.right);
            Put3(d.up, l.up);
            Put3(d.forward, l.forward);
            d.layout = SHIRO_ENV_LAYOUT_LATLONG;
            if (l.environment && !l.environment->Pixels().empty()) {
                d.layout = l.environment->Layout() == EnvironmentMapLayout::Angular ? SHIRO_ENV_LAYOUT_ANGULAR
                                                                                      : SHIRO_ENV_LAYOUT_LATLONG;
                d.env_width = l.environment->Width();
                d.env_height = l.environment->Height();
                d.env_pixels = reinterpret_cast<const float*>(l.environment->Pixels().data());
            }
            domes.push_back(d);
        }
        desc.materials = materials.data();
        desc.material_count = static_cast<uint32_t>(materials.size());
        desc.meshes = meshes.data();
        desc.mesh_count = static_cast<uint32_t>(meshes.size());
        desc.distant_lights = distant.data();
        desc.distant_light_count = static_cast<uint32_t>(distant.size());
        desc.dome_lights = domes.data();
        desc.dome_light_count = static_cast<uint32_t>(domes.size());
        Put3(desc.environment_top, s.environmentTop);
        Put3(desc.environment_bottom, s.environmentBottom);
    }
};

// Forwards a RenderRequest's std::atomic<bool> cancel flag to the int the C
// ABI polls between launches: a watcher thread copies it every 200 us while
// the render runs (Hydra sets the flag from another thread,
// RenderParam.cpp:790-806; RenderBackend.h:18).
class CancelForward {
public:
    explicit CancelForward(const std::atomic<bool>* source) : source_(source) {
        if (source_) watcher_ = std::thread([this] { Watch(); });
    }
    ~CancelForward() {
        done_.store(true, std::memory_order_release);
        if (watcher_.joinable()) watcher_.join();
    }
    CancelForward(const CancelForward&) = delete;
    CancelForward& operator=(const CancelForward&) = delete;
    const volatile int* Flag() const { return source_ ? &flag_ : nullptr; }

private:
    void Watch() {
        while (!done_.load(std::memory_order_acquire)) {
            if (source_->load(std::memory_order_relaxed)) {
                flag_ = 1;
                return;
            }
            std::this_thread::sleep_for(std::chrono::microseconds(200));
        }
    }
    const std::atomic<bool>* source_;
    volatile int flag_ = 0;
    std::atomic<bool> done_{false};
    std::thread watcher_;
};

ShiroRenderDesc ToRequest(const RenderRequest& r) {
    ShiroRenderDesc d{};
    Put3(d.camera.position, r.camera.position);
    Put3(d.camera.forward, r.camera.forward);
    Put3(d.camera.right, r.camera.right);
    Put3(d.camera.up, r.camera.up);
    d.camera.vertical_fov_degrees = r.camera.verticalFovDegrees;
    d.camera.aspect_ratio = r.camera.aspectRatio;
    const RenderSettings& s = r.settings;
    d.settings = ShiroSettingsDesc{s.width, s.height, s.samplesPerPixel, s.samplesPerUpdate, s.domeLightSamples,
                                   s.maxDepth, s.diffuseDepth, s.specularDepth, s.threadLimit, s.maxSubdivLevel,
                                   static_cast<uint32_t>(s.backend), s.backgroundVisible ? 1u : 0u,
                                   s.enableHeadlight ? 1u : 0u, s.enableCaustics ? 1u : 0u, s.enableSss ? 1u : 0u};
    d.sample_start = r.sampleStart;
    d.sample_count = r.sampleCount;
    return d;
}

static_assert(sizeof(Vec4f) == 4 * sizeof(float), "Vec4f must be four packed floats");

// The FrameBuffer's own planes as the C ABI's host AOVs: the render writes
// straight into the vectors Resize sized (FrameBuffer.h exposes them const;
// the FrameBuffer itself is ours and not const, so writing is well defined).
ShiroAovs FrameAovs(FrameBuffer& fb) {
    return ShiroAovs{const_cast<float*>(&fb.Beauty().data()->x), const_cast<float*>(&fb.Albedo().data()->x),
                     const_cast<float*>(&fb.Normal().data()->x), const_cast<float*>(fb.Depth().data()), 0, 0};
}

bool Cancelled(const std::atomic<bool>* c) { return c && c->load(std::memory_order_relaxed); }

// Copies pixels [first, first + count) of the staged planes (beauty 4,
// albedo 3, normal 3, depth 1 floats per pixel, plane after plane, px pixels
// each) into the frame's own, on several host threads for a large range.
void CopyOut(const float* stage, FrameBuffer& fb, size_t px, size_t first, size_t count) {
    const ShiroAovs dst = FrameAovs(fb);
    struct Plane {
        const float* src;
        float* dst;
        size_t n;
    };
    const Plane planes[4] = {{stage + 4 * first, dst.beauty + 4 * first, 4 * count},
                             {stage + 4 * px + 3 * first, dst.albedo + 3 * first, 3 * count},
                             {stage + 7 * px + 3 * first, dst.normal + 3 * first, 3 * count},
                             {stage + 10 * px + first, dst.depth + first, count}};
    const unsigned threads = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    auto part = [&](unsigned t, unsigned of) {
        for (const Plane& p : planes) {
            const size_t a = p.n * t / of, b = p.n * (t + 1) / of;
            if (b > a) std::memcpy(p.dst + a, p.src + a, (b - a) * sizeof(float));
        }
    };
    if (threads == 1 || 11 * count < (size_t{1} << 20)) {
        part(0, 1);
        return;
    }
    // (also called from the render's progress callback: nothing may throw
    // through the library, so a part whose thread cannot start runs here)
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t) {
        try {
            pool.emplace_back(part, t, threads);
        } catch (...) {
            part(t, threads);
        }
    }
    part(0, threads);
    for (std::thread& th : pool) th.join();
}

// shiro_gpu_render_batch_ready's callback of RenderSampleBatch: each finished
// range goes from the staging into the frame while later waves render.
struct StagedFrame {
    const float* stage;
    FrameBuffer* frame;
    size_t px;
    std::function<bool()> ready;  // the frame is sized and cleared (false: that failed)
};

void CopyFinished(void* user, uint32_t, uint64_t first, uint64_t count) {
    StagedFrame& f = *static_cast<StagedFrame*>(user);
    if (f.ready()) CopyOut(f.stage, *f.frame, f.px, first, count);
}

}  // namespace

GpuBackend::GpuBackend(int device) : device_(device) {}

GpuBackend::~GpuBackend() {
    if (accum_) shiro_gpu_accum_destroy(accum_);
    if (ctx_) shiro_gpu_destroy(ctx_);
    shiro_gpu_host_free(staging_);
}

float* GpuBackend::Staging(size_t bytes) const {
    if (stagingBytes_ < bytes) {
        shiro_gpu_host_free(staging_);
        staging_ = nullptr;
        stagingBytes_ = 0;
        if (shiro_gpu_host_alloc(bytes, &staging_) != SHIRO_OK || !staging_) return nullptr;
        stagingBytes_ = bytes;
    }
    return static_cast<float*>(staging_);
}

BackendStatus GpuBackend::GetStatus() const {
    BackendStatus status;
    status.kind = render::BackendKind::Gpu;
    status.name = "gb300";
    status.usesGpu = true;
    ShiroBackendStatus s;
    status.available = shiro_gpu_status(&s) == SHIRO_OK && s.available != 0;
    std::scoped_lock lock(mutex_);
    if (runtimeAttempted_ && runtimeFailed_) status.available = false;
    return status;
}

bool GpuBackend::SupportsScene(const render::Scene& scene) const {
    SceneView view(scene);
    return shiro_gpu_supports_scene(&view.desc, nullptr, 0) != 0;
}

bool GpuBackend::EnsureRuntime(const render::Scene& scene) const {
    runtimeAttempted_ = true;
    if (!ctx_) {
        if (shiro_gpu_create(device_, &ctx_) != SHIRO_OK) {
            std::fprintf(stderr, "[shiro gb300] context creation failed: %s\n", shiro_gpu_last_error(nullptr));
            runtimeFailed_ = true;
            ctx_ = nullptr;
            return false;
        }
    }
    // The device copy is reused while the snapshot's content is unchanged: the
    // signature hashes every field the upload reads (what the OptiX backend's
    // ComputeSceneSignature hashes, OptixBackend.cpp:150-232).  Hydra builds an
    // edited snapshot as a new Scene that may land at the address just freed
    // (RenderParam.cpp:614-659), so the address alone cannot identify it.
    SceneView view(scene);
    uint64_t sig = 0;
    shiro_gpu_scene_signature(&view.desc, &sig);
    if (cachedScene_ != &scene || cachedSignature_ != sig) {
        if (shiro_gpu_upload_scene(ctx_, &view.desc) != SHIRO_OK) {
            std::fprintf(stderr, "[shiro gb300] scene upload failed: %s\n", shiro_gpu_last_error(ctx_));
            cachedScene_ = nullptr;
            return false;
        }
        cachedScene_ = &scene;
        cachedSignature_ = sig;
        ++uploads_;
    }
    return true;
}

render::FrameBuffer GpuBackend::RenderSampleBatch(const RenderRequest& request) const {
    render::FrameBuffer frame;
    const uint32_t w = request.settings.width, h = request.settings.height;
    if (request.sampleCount == 0 || Cancelled(request.cancel)) {
        frame.Resize(w, h);
        frame.Clear();
        return frame;
    }
    std::scoped_lock lock(mutex_);
    // The returned frame is sized and cleared (a 1080p one is 91 MB of fresh
    // pages) on a helper thread while the device renders into page-locked
    // staging, which the render writes in place; each wave's pixels are
    // copied over (on several threads) as soon as the wave has finished,
    // while the next ones render.
    std::exception_ptr failure;  // an allocation failure reaches the caller as before
    std::thread prepare([&frame, &failure, w, h] {
        try {
            frame.Resize(w, h);
            frame.Clear();
        } catch (...) {
            failure = std::current_exception();
        }
    });
    auto joined = [&] {
        if (prepare.joinable()) prepare.join();
        return !failure;
    };
    auto prepared = [&] {
        if (!joined()) std::rethrow_exception(failure);
    };
    if (!EnsureRuntime(request.scene)) {
        prepared();
        return frame;
    }
    const ShiroRenderDesc desc = ToRequest(request);
    const size_t px = static_cast<size_t>(w) * h;
    float* stage = Staging(11 * px * sizeof(float));
    ShiroAovs aovs;
    if (stage) {
        aovs = ShiroAovs{stage, stage + 4 * px, stage + 7 * px, stage + 10 * px, 0, 0};
    } else {  // no page-locked memory: render into the frame's own planes
        prepared();
        aovs = FrameAovs(frame);
    }
    // the wavefront form: the faster one, with frames bit-identical to the
    // one-thread-per-path form's
    int rc;
    {
        CancelForward cancel(request.cancel);
        StagedFrame staged{stage, &frame, px, joined};
        rc = stage ? shiro_gpu_render_batch_ready(ctx_, &desc, 1, cancel.Flag(), &aovs, CopyFinished, &staged)
                   : shiro_gpu_render_batch(ctx_, &desc, 1, cancel.Flag(), &aovs);
    }
    lastStatus_ = rc;
    prepared();
    if (rc != SHIRO_OK) {
        if (rc != SHIRO_ERR_CANCELLED)
            std::fprintf(stderr, "[shiro gb300] render failed (%d): %s\n", rc, shiro_gpu_last_error(ctx_));
        frame.Clear();
        return frame;
    }
    if (Cancelled(request.cancel)) {  // RenderParam.cpp:791-798 discards it anyway
        frame.Clear();
        return frame;
    }
    return frame;
}

std::vector<render::FrameBuffer> GpuBackend::RenderSampleBatches(const std::vector<RenderRequest>& requests) const {
    std::vector<render::FrameBuffer> frames(requests.size());
    for (size_t i = 0; i < requests.size(); ++i) {
        frames[i].Resize(requests[i].settings.width, requests[i].settings.height);
        frames[i].Clear();
    }
    if (requests.empty()) return frames;
    for (const RenderRequest& r : requests)
        if (&r.scene != &requests.front().scene) {
            std::fprintf(stderr, "[shiro gb300] batched requests must share one scene\n");
            return frames;
        }
    std::scoped_lock lock(mutex_);
    if (!EnsureRuntime(requests.front().scene)) return frames;
    std::vector<ShiroRenderDesc> descs;
    std::vector<ShiroAovs> aovs;
    for (size_t i = 0; i < requests.size(); ++i) {
        descs.push_back(ToRequest(requests[i]));
        aovs.push_back(FrameAovs(frames[i]));
    }
    int rc;
    {  // one flag for the batch: the first request's (they are one call)
        CancelForward cancel(requests.front().cancel);
        rc = shiro_gpu_render_batch(ctx_, descs.data(), static_cast<uint32_t>(descs.size()), cancel.Flag(), aovs.data());
    }
    lastStatus_ = rc;
    if (rc != SHIRO_OK) {
        if (rc != SHIRO_ERR_CANCELLED)
            std::fprintf(stderr, "[shiro gb300] batched render failed (%d): %s\n", rc, shiro_gpu_last_error(ctx_));
        for (render::FrameBuffer& f : frames) f.Clear();
    }
    return frames;
}

bool GpuBackend::RenderAndAccumulate(const RenderRequest& request, bool wavefront) const {
    if (request.sampleCount == 0 || Cancelled(request.cancel)) return false;
    std::scoped_lock lock(mutex_);
    if (!EnsureRuntime(request.scene)) return false;
    if (!accum_ && shiro_gpu_accum_create(ctx_, &accum_) != SHIRO_OK) {
        accum_ = nullptr;
        return false;
    }
    const ShiroRenderDesc desc = ToRequest(request);
    int rc;
    {
        CancelForward cancel(request.cancel);
        rc = shiro_gpu_accum_stage(accum_, &desc, cancel.Flag(), wavefront ? 1u : 0u);
    }
    lastStatus_ = rc;
    if (rc != SHIRO_OK) {
        if (rc != SHIRO_ERR_CANCELLED)
            std::fprintf(stderr, "[shiro gb300] render failed (%d): %s\n", rc, shiro_gpu_last_error(ctx_));
        return false;
    }
    if (Cancelled(request.cancel)) return false;  // RenderParam.cpp:791-798: a cancelled batch is discarded
    if (shiro_gpu_accum_commit(accum_) != SHIRO_OK) {
        std::fprintf(stderr, "[shiro gb300] accumulation failed: %s\n", shiro_gpu_last_error(ctx_));
        return false;
    }
    return true;
}

render::FrameBuffer GpuBackend::ResolveAccumulation() const {
    std::scoped_lock lock(mutex_);
    render::FrameBuffer frame;
    uint32_t samples = 0, w = 0, h = 0;
    if (!accum_ || shiro_gpu_accum_info(accum_, &samples, &w, &h) != SHIRO_OK) return frame;
    frame.Resize(w, h);
    ShiroAovs aovs = FrameAovs(frame);
    if (shiro_gpu_accum_resolve(accum_, &aovs) != SHIRO_OK) {
        std::fprintf(stderr, "[shiro gb300] resolve failed: %s\n", shiro_gpu_last_error(ctx_));
        frame.Clear();
    }
    return frame;
}

int GpuBackend::LastStatus() const {
    std::scoped_lock lock(mutex_);
    return lastStatus_;
}

uint64_t GpuBackend::SceneUploads() const {
    std::scoped_lock lock(mutex_);
    return uploads_;
}

uint32_t GpuBackend::AccumulatedSampleCount() const {
    std::scoped_lock lock(mutex_);
    uint32_t samples = 0;
    if (accum_) shiro_gpu_accum_info(accum_, &samples, nullptr, nullptr);
    return samples;
}

}  // namespace shiro::backend::gb300
