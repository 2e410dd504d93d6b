// backend_harness.cpp - TEST AND MEASUREMENT HARNESS, not part of the
// product library: C entry points that drive the C++ adapter
// shiro::backend::gb300::GpuBackend the way Renderer::RenderSampleBatch does
// (Renderer.cpp:119-128).  The scene descriptor is first turned into a
// renderer-owned Scene snapshot, then the RenderBackend methods are called.
// Built by tests/cpp/harness.py into its own library; used by the adapter
// tests and by bench.py's end-to-end timing through the adapter.
#include <atomic>
#include <chrono>
#include <cstring>
#include <memory>
#include <thread>

#include "GpuBackend.h"
#include "shiro/render/EnvironmentMap.h"
#include "shiro_gpu.h"

using namespace shiro::render;

namespace {

Vec3f V(const float* p) { return {p[0], p[1], p[2]}; }

Scene ToScene(const ShiroSceneDesc& d) {
    Scene s;
    for (uint32_t i = 0; i < d.material_count; ++i) {
        const ShiroMaterialDesc& m = d.materials[i];
        PbrMaterial p;
        p.baseColor = V(m.base_color);
        p.emissionColor = V(m.emission_color);
        p.specularColor = V(m.specular_color);
        p.transmissionColor = V(m.transmission_color);
        p.transmissionScatter = V(m.transmission_scatter);
        p.coatColor = V(m.coat_color);
        p.subsurfaceColor = V(m.subsurface_color);
        p.subsurfaceRadius = V(m.subsurface_radius);
        p.sheenColor = V(m.sheen_color);
        p.normalOverride = V(m.normal_override);
        p.coatNormalOverride = V(m.coat_normal_override);
        p.tangentOverride = V(m.tangent_override);
        p.baseWeight = m.base_weight;
        p.emissionStrength = m.emission_strength;
        p.specularWeight = m.specular_weight;
        p.metallic = m.metallic;
        p.roughness = m.roughness;
        p.diffuseRoughness = m.diffuse_roughness;
        p.opacity = m.opacity;
        p.specularAnisotropy = m.specular_anisotropy;
        p.specularRotation = m.specular_rotation;
        p.coatWeight = m.coat_weight;
        p.coatRoughness = m.coat_roughness;
        p.coatIor = m.coat_ior;
        p.coatAnisotropy = m.coat_anisotropy;
        p.coatRotation = m.coat_rotation;
        p.sheen = m.sheen;
        p.sheenRoughness = m.sheen_roughness;
        p.subsurface = m.subsurface;
        p.subsurfaceScale = m.subsurface_scale;
        p.subsurfaceAnisotropy = m.subsurface_anisotropy;
        p.transmission = m.transmission;
        p.transmissionDepth = m.transmission_depth;
        p.transmissionScatterAnisotropy = m.transmission_scatter_anisotropy;
        p.transmissionDispersion = m.transmission_dispersion;
        p.transmissionExtraRoughness = m.transmission_extra_roughness;
        p.ior = m.ior;
        p.coatAffectColor = m.coat_affect_color;
        p.coatAffectRoughness = m.coat_affect_roughness;
        p.thinFilmThickness = m.thin_film_thickness;
        p.thinFilmIor = m.thin_film_ior;
        p.thinWalled = m.thin_walled != 0;
        p.hasNormalOverride = m.has_normal_override != 0;
        p.hasCoatNormalOverride = m.has_coat_normal_override != 0;
        p.hasTangentOverride = m.has_tangent_override != 0;
        s.materials.push_back(p);
    }
    for (uint32_t i = 0; i < d.mesh_count; ++i) {
        const ShiroMeshDesc& m = d.meshes[i];
        TriangleMesh t;
        for (uint32_t v = 0; v < m.vertex_count; ++v) t.positions.push_back(V(m.positions + 3 * v));
        if (m.normals)
            for (uint32_t v = 0; v < m.normal_count; ++v) t.normals.push_back(V(m.normals + 3 * v));
        t.indices.assign(m.indices, m.indices + m.index_count);
        t.materialIndex = m.material_index;
        s.meshes.push_back(std::move(t));
    }
    for (uint32_t i = 0; i < d.distant_light_count; ++i)
        s.distantLights.push_back({V(d.distant_lights[i].direction), V(d.distant_lights[i].radiance)});
    for (uint32_t i = 0; i < d.dome_light_count; ++i) {
        const ShiroDomeLightDesc& l = d.dome_lights[i];
        DomeLight dl;
        dl.radiance = V(l.radiance);
        dl.right = V(l.right);
        dl.up = V(l.up);
        dl.forward = V(l.forward);
        if (l.env_pixels && l.env_width && l.env_height) {
            std::vector<Vec3f> px(static_cast<size_t>(l.env_width) * l.env_height);
            for (size_t k = 0; k < px.size(); ++k) px[k] = V(l.env_pixels + 3 * k);
            dl.environment = EnvironmentMap::FromPixels(
                l.env_width, l.env_height, std::move(px),
                l.layout == SHIRO_ENV_LAYOUT_ANGULAR ? EnvironmentMapLayout::Angular : EnvironmentMapLayout::LatLong);
        }
        s.domeLights.push_back(dl);
    }
    s.environmentTop = V(d.environment_top);
    s.environmentBottom = V(d.environment_bottom);
    return s;
}

void Copy(const FrameBuffer& fb, ShiroAovs* out) {
    const size_t n = static_cast<size_t>(fb.Width()) * fb.Height();
    for (size_t i = 0; i < n; ++i) {
        const Vec4f b = fb.Beauty()[i];
        out->beauty[4 * i] = b.x;
        out->beauty[4 * i + 1] = b.y;
        out->beauty[4 * i + 2] = b.z;
        out->beauty[4 * i + 3] = b.w;
        const Vec3f a = fb.Albedo()[i], nn = fb.Normal()[i];
        out->albedo[3 * i] = a.x;
        out->albedo[3 * i + 1] = a.y;
        out->albedo[3 * i + 2] = a.z;
        out->normal[3 * i] = nn.x;
        out->normal[3 * i + 1] = nn.y;
        out->normal[3 * i + 2] = nn.z;
        out->depth[i] = fb.Depth()[i];
    }
}

std::vector<shiro::backend::RenderRequest> Requests(const Scene& scene, const ShiroRenderDesc* reqs, uint32_t count,
                                                    std::vector<Camera>& cams, std::vector<RenderSettings>& settings,
                                                    const std::atomic<bool>* cancel) {
    cams.resize(count);
    settings.resize(count);
    std::vector<shiro::backend::RenderRequest> rq;
    for (uint32_t i = 0; i < count; ++i) {
        const ShiroRenderDesc& r = reqs[i];
        cams[i] = Camera{V(r.camera.position), V(r.camera.forward), V(r.camera.right), V(r.camera.up),
                         r.camera.vertical_fov_degrees, r.camera.aspect_ratio};
        const ShiroSettingsDesc& s = r.settings;
        RenderSettings& st = settings[i];
        st.width = s.width;
        st.height = s.height;
        st.samplesPerPixel = s.samples_per_pixel;
        st.samplesPerUpdate = s.samples_per_update;
        st.domeLightSamples = s.dome_light_samples;
        st.maxDepth = s.max_depth;
        st.diffuseDepth = s.diffuse_depth;
        st.specularDepth = s.specular_depth;
        st.backgroundVisible = s.background_visible != 0;
        st.backend = BackendKind::Gpu;
    }
    for (uint32_t i = 0; i < count; ++i)
        rq.push_back(shiro::backend::RenderRequest{scene, cams[i], settings[i], reqs[i].sample_start,
                                                   reqs[i].sample_count, cancel});
    return rq;
}

shiro::backend::gb300::GpuBackend& Backend() {
    static shiro::backend::gb300::GpuBackend backend(0);
    return backend;
}

}  // namespace

extern "C" {

// Renders `count` requests of one scene through GpuBackend.  mode 0:
// count == 1 uses RenderSampleBatch, count > 1 RenderSampleBatches.  mode 1:
// the requests are consecutive steps of a progressive render
// (RenderAndAccumulate, plain or wavefront form) and outs[0] receives
// ResolveAccumulation().  Returns 1 when the backend reported itself available
// and supported the scene, 0 otherwise, -1 when a step was not accumulated.
int shiro_backend_selftest(const ShiroSceneDesc* sd, const ShiroRenderDesc* reqs, uint32_t count, ShiroAovs* outs,
                           uint32_t mode, uint32_t wavefront) {
    shiro::backend::gb300::GpuBackend& backend = Backend();
    if (!backend.GetStatus().available) return 0;
    const Scene scene = ToScene(*sd);
    if (!backend.SupportsScene(scene)) return 0;
    std::vector<Camera> cams;
    std::vector<RenderSettings> settings;
    const std::vector<shiro::backend::RenderRequest> rq = Requests(scene, reqs, count, cams, settings, nullptr);
    if (mode == 1) {  // progressive: every request is one step, then one resolve
        for (uint32_t i = 0; i < count; ++i)
            if (!backend.RenderAndAccumulate(rq[i], wavefront != 0)) return -1;
        Copy(backend.ResolveAccumulation(), &outs[0]);
        return 1;
    }
    if (count == 1) {
        Copy(backend.RenderSampleBatch(rq[0]), &outs[0]);
    } else {
        const std::vector<FrameBuffer> fbs = backend.RenderSampleBatches(rq);
        for (uint32_t i = 0; i < count; ++i) Copy(fbs[i], &outs[i]);
    }
    return 1;
}

// End-to-end timing through the adapter: `warmup` untimed and `steps` timed
// RenderSampleBatch calls of one request (host FrameBuffer out, as Shiro
// receives it), each timed on the host clock around the call.  ms_out[k]
// receives step k's milliseconds; `last` (may be NULL) the last frame.
// Returns 1, or 0 when the backend is unavailable, -1 when a call failed.
int shiro_harness_time_render(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, uint32_t warmup, uint32_t steps,
                              double* ms_out, ShiroAovs* last) {
    shiro::backend::gb300::GpuBackend& backend = Backend();
    if (!backend.GetStatus().available) return 0;
    const Scene scene = ToScene(*sd);
    std::vector<Camera> cams;
    std::vector<RenderSettings> settings;
    const std::vector<shiro::backend::RenderRequest> rq = Requests(scene, req, 1, cams, settings, nullptr);
    FrameBuffer fb;
    for (uint32_t k = 0; k < warmup + steps; ++k) {
        const auto t0 = std::chrono::steady_clock::now();
        fb = backend.RenderSampleBatch(rq[0]);
        const auto t1 = std::chrono::steady_clock::now();
        if (backend.LastStatus() != 0) return -1;
        if (k >= warmup) ms_out[k - warmup] = std::chrono::duration<double, std::milli>(t1 - t0).count();
    }
    if (last) Copy(fb, last);
    return 1;
}

// Mid-frame cancel: another host thread sets the request's std::atomic<bool>
// cancel flag `delay_ms` after RenderSampleBatch starts.  out receives the
// returned frame, *status the backend's status of the call, *elapsed_ms the
// call's duration.  mode 0: RenderSampleBatch, 1: RenderAndAccumulate
// (wavefront) and *status is 1 when the batch was accumulated.
int shiro_harness_cancel_midframe(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, double delay_ms, uint32_t mode,
                                  ShiroAovs* out, int* status, double* elapsed_ms) {
    shiro::backend::gb300::GpuBackend& backend = Backend();
    if (!backend.GetStatus().available) return 0;
    const Scene scene = ToScene(*sd);
    std::atomic<bool> cancel{false};
    std::vector<Camera> cams;
    std::vector<RenderSettings> settings;
    const std::vector<shiro::backend::RenderRequest> rq = Requests(scene, req, 1, cams, settings, &cancel);
    // the scene upload is not part of the frame: do it first, uncancelled
    {
        ShiroRenderDesc tiny = *req;
        tiny.settings.width = tiny.settings.height = 1;
        tiny.sample_count = 1;
        std::vector<Camera> c2;
        std::vector<RenderSettings> s2;
        backend.RenderSampleBatch(Requests(scene, &tiny, 1, c2, s2, nullptr)[0]);
    }
    const auto t0 = std::chrono::steady_clock::now();
    std::thread setter([&] {
        std::this_thread::sleep_for(std::chrono::microseconds(static_cast<int64_t>(delay_ms * 1000.0)));
        cancel.store(true);
    });
    if (mode == 1) {
        const bool accumulated = backend.RenderAndAccumulate(rq[0], true);
        *status = accumulated ? 1 : backend.LastStatus();
    } else {
        const FrameBuffer fb = backend.RenderSampleBatch(rq[0]);
        *status = backend.LastStatus();
        Copy(fb, out);
    }
    const auto t1 = std::chrono::steady_clock::now();
    setter.join();
    *elapsed_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    return 1;
}

// Edits in place: renders `req` three times through one Scene object - as
// given, after setting distant light 0's radiance to `radiance`, and after
// moving vertex 0 of mesh 0 by `offset` - into outs[0..2]; uploads[k] is the
// adapter's scene-upload count after render k.
int shiro_harness_edit_in_place(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, const float* radiance,
                                const float* offset, ShiroAovs* outs, uint64_t* uploads) {
    shiro::backend::gb300::GpuBackend& backend = Backend();
    if (!backend.GetStatus().available) return 0;
    Scene scene = ToScene(*sd);
    if (scene.distantLights.empty() || scene.meshes.empty() || scene.meshes[0].positions.empty()) return -1;
    std::vector<Camera> cams;
    std::vector<RenderSettings> settings;
    const std::vector<shiro::backend::RenderRequest> rq = Requests(scene, req, 1, cams, settings, nullptr);
    Copy(backend.RenderSampleBatch(rq[0]), &outs[0]);
    uploads[0] = backend.SceneUploads();
    scene.distantLights[0].radiance = V(radiance);
    Copy(backend.RenderSampleBatch(rq[0]), &outs[1]);
    uploads[1] = backend.SceneUploads();
    Vec3f& p = scene.meshes[0].positions[0];
    p = Vec3f{p.x + offset[0], p.y + offset[1], p.z + offset[2]};
    Copy(backend.RenderSampleBatch(rq[0]), &outs[2]);
    uploads[2] = backend.SceneUploads();
    return 1;
}

}  // extern "C"
