// backend_selftest.cpp - C entry points that drive GpuBackend the way
// Renderer::RenderSampleBatch does (Renderer.cpp:119-128): the scene
// descriptor is first turned into a renderer-owned Scene snapshot, then the
// RenderBackend methods are called.  Used by the tests only.
#include <cstring>
#include <memory>

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
    static shiro::backend::gb300::GpuBackend backend(0);
    if (!backend.GetStatus().available) return 0;
    const Scene scene = ToScene(*sd);
    if (!backend.SupportsScene(scene)) return 0;
    std::vector<Camera> cams(count);
    std::vector<RenderSettings> settings(count);
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
        rq.push_back(shiro::backend::RenderRequest{scene, cams[i], settings[i], reqs[i].sample_start, reqs[i].sample_count,
                                                   nullptr});
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

}  // extern "C"
