// ref_harness.cpp - C entry points over the reference's own CPU integrator.
//
// TEST INFRASTRUCTURE ONLY.  This translation unit is compiled together with
// the unmodified reference sources where they lie (see oracle/Makefile):
//   src/backend/cpu/CpuPathTracer.cpp (included below so that its
//   anonymous-namespace functions - EvaluateBsdf, GenerateCameraRay,
//   IntersectScene, ... - are reachable), src/render/EnvironmentMap.cpp,
//   src/render/OpenQmcSampler.cpp, src/render/FrameBuffer.cpp,
//   src/backend/RenderBackend.cpp,
// with SHIRO_HAVE_EMBREE=0, SHIRO_WITH_OPENQMC=0, SHIRO_HAVE_OIIO=0 (none of
// Embree, OpenQMC or OpenImageIO is installed), i.e. the reference's
// brute-force intersector (CpuPathTracer.cpp:431-475) and its fallback QMC
// sampler (OpenQmcSampler.cpp:56-71).  It produces the golden vectors under
// tests/golden; nothing in the product links it.
//
// EnvironmentMap has a private constructor and loads only through OIIO
// (EnvironmentMap.h:28-48), so its private members are opened for this TU to
// inject decoded pixels and call BuildImportanceTable().

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

#define private public
#include "shiro/render/EnvironmentMap.h"
#undef private

#include "../../include/shiro_gpu.h"

// The reference integrator itself (anonymous-namespace helpers become visible
// to this TU).
#include "src/backend/cpu/CpuPathTracer.cpp"

using namespace shiro::render;
namespace cpu = shiro::backend::cpu;

namespace {

Vec3f V3(const float* p) { return {p[0], p[1], p[2]}; }

PbrMaterial ToMaterial(const ShiroMaterialDesc& d) {
    PbrMaterial m;
    m.baseColor = V3(d.base_color);
    m.emissionColor = V3(d.emission_color);
    m.specularColor = V3(d.specular_color);
    m.transmissionColor = V3(d.transmission_color);
    m.transmissionScatter = V3(d.transmission_scatter);
    m.coatColor = V3(d.coat_color);
    m.subsurfaceColor = V3(d.subsurface_color);
    m.subsurfaceRadius = V3(d.subsurface_radius);
    m.sheenColor = V3(d.sheen_color);
    m.normalOverride = V3(d.normal_override);
    m.coatNormalOverride = V3(d.coat_normal_override);
    m.tangentOverride = V3(d.tangent_override);
    m.baseWeight = d.base_weight;
    m.emissionStrength = d.emission_strength;
    m.specularWeight = d.specular_weight;
    m.metallic = d.metallic;
    m.roughness = d.roughness;
    m.diffuseRoughness = d.diffuse_roughness;
    m.opacity = d.opacity;
    m.specularAnisotropy = d.specular_anisotropy;
    m.specularRotation = d.specular_rotation;
    m.coatWeight = d.coat_weight;
    m.coatRoughness = d.coat_roughness;
    m.coatIor = d.coat_ior;
    m.coatAnisotropy = d.coat_anisotropy;
    m.coatRotation = d.coat_rotation;
    m.sheen = d.sheen;
    m.sheenRoughness = d.sheen_roughness;
    m.subsurface = d.subsurface;
    m.subsurfaceScale = d.subsurface_scale;
    m.subsurfaceAnisotropy = d.subsurface_anisotropy;
    m.transmission = d.transmission;
    m.transmissionDepth = d.transmission_depth;
    m.transmissionScatterAnisotropy = d.transmission_scatter_anisotropy;
    m.transmissionDispersion = d.transmission_dispersion;
    m.transmissionExtraRoughness = d.transmission_extra_roughness;
    m.ior = d.ior;
    m.coatAffectColor = d.coat_affect_color;
    m.coatAffectRoughness = d.coat_affect_roughness;
    m.thinFilmThickness = d.thin_film_thickness;
    m.thinFilmIor = d.thin_film_ior;
    m.thinWalled = d.thin_walled != 0;
    m.hasNormalOverride = d.has_normal_override != 0;
    m.hasCoatNormalOverride = d.has_coat_normal_override != 0;
    m.hasTangentOverride = d.has_tangent_override != 0;
    return m;
}

std::shared_ptr<EnvironmentMap> MakeEnvironment(uint32_t w, uint32_t h, const float* rgb, uint32_t layout) {
    auto env = std::shared_ptr<EnvironmentMap>(new EnvironmentMap());
    env->width_ = w;
    env->height_ = h;
    // EnvironmentMap.cpp:43-45: Automatic resolves to LatLong.
    env->layout_ = layout == SHIRO_ENV_LAYOUT_ANGULAR ? EnvironmentMapLayout::Angular : EnvironmentMapLayout::LatLong;
    env->pixels_.resize(static_cast<size_t>(w) * h);
    for (size_t i = 0; i < env->pixels_.size(); ++i) {
        env->pixels_[i] = {rgb[3 * i + 0], rgb[3 * i + 1], rgb[3 * i + 2]};
    }
    env->BuildImportanceTable();
    return env;
}

Scene ToScene(const ShiroSceneDesc& d) {
    Scene s;
    for (uint32_t i = 0; i < d.material_count; ++i) s.materials.push_back(ToMaterial(d.materials[i]));
    for (uint32_t i = 0; i < d.mesh_count; ++i) {
        const ShiroMeshDesc& m = d.meshes[i];
        TriangleMesh tm;
        tm.positions.resize(m.vertex_count);
        for (uint32_t v = 0; v < m.vertex_count; ++v) tm.positions[v] = V3(m.positions + 3 * v);
        if (m.normals) {
            tm.normals.resize(m.normal_count);
            for (uint32_t v = 0; v < m.normal_count; ++v) tm.normals[v] = V3(m.normals + 3 * v);
        }
        tm.indices.assign(m.indices, m.indices + m.index_count);
        tm.materialIndex = m.material_index;
        s.meshes.push_back(std::move(tm));
    }
    for (uint32_t i = 0; i < d.distant_light_count; ++i) {
        DirectionalLight l;
        l.direction = V3(d.distant_lights[i].direction);
        l.radiance = V3(d.distant_lights[i].radiance);
        s.distantLights.push_back(l);
    }
    for (uint32_t i = 0; i < d.dome_light_count; ++i) {
        const ShiroDomeLightDesc& dl = d.dome_lights[i];
        DomeLight l;
        l.radiance = V3(dl.radiance);
        l.right = V3(dl.right);
        l.up = V3(dl.up);
        l.forward = V3(dl.forward);
        if (dl.env_pixels && dl.env_width && dl.env_height) {
            l.environment = MakeEnvironment(dl.env_width, dl.env_height, dl.env_pixels, dl.layout);
        }
        s.domeLights.push_back(l);
    }
    s.environmentTop = V3(d.environment_top);
    s.environmentBottom = V3(d.environment_bottom);
    return s;
}

Camera ToCamera(const ShiroCameraDesc& c) {
    Camera cam;
    cam.position = V3(c.position);
    cam.forward = V3(c.forward);
    cam.right = V3(c.right);
    cam.up = V3(c.up);
    cam.verticalFovDegrees = c.vertical_fov_degrees;
    cam.aspectRatio = c.aspect_ratio;
    return cam;
}

RenderSettings ToSettings(const ShiroSettingsDesc& s) {
    RenderSettings r;
    r.width = s.width;
    r.height = s.height;
    r.samplesPerPixel = s.samples_per_pixel;
    r.samplesPerUpdate = s.samples_per_update;
    r.domeLightSamples = s.dome_light_samples;
    r.maxDepth = s.max_depth;
    r.diffuseDepth = s.diffuse_depth;
    r.specularDepth = s.specular_depth;
    r.threadLimit = s.thread_limit;
    r.maxSubdivLevel = s.max_subdiv_level;
    r.backend = static_cast<BackendKind>(s.backend);
    r.backgroundVisible = s.background_visible != 0;
    r.enableHeadlight = s.enable_headlight != 0;
    r.enableCaustics = s.enable_caustics != 0;
    r.enableSss = s.enable_sss != 0;
    return r;
}

uint32_t GlobalPrim(const Scene& scene, size_t mesh, uint32_t prim) {
    uint32_t base = 0;
    for (size_t m = 0; m < mesh; ++m) base += static_cast<uint32_t>(scene.meshes[m].indices.size() / 3);
    return base + prim;
}

}  // namespace

// Host copy of a reference frame into flat AOV planes.
namespace {
void CopyFrame(const FrameBuffer& fb, ShiroAovs* out) {
    const size_t n = static_cast<size_t>(fb.Width()) * fb.Height();
    for (size_t i = 0; i < n; ++i) {
        out->beauty[4 * i + 0] = fb.Beauty()[i].x;
        out->beauty[4 * i + 1] = fb.Beauty()[i].y;
        out->beauty[4 * i + 2] = fb.Beauty()[i].z;
        out->beauty[4 * i + 3] = fb.Beauty()[i].w;
        out->albedo[3 * i + 0] = fb.Albedo()[i].x;
        out->albedo[3 * i + 1] = fb.Albedo()[i].y;
        out->albedo[3 * i + 2] = fb.Albedo()[i].z;
        out->normal[3 * i + 0] = fb.Normal()[i].x;
        out->normal[3 * i + 1] = fb.Normal()[i].y;
        out->normal[3 * i + 2] = fb.Normal()[i].z;
        out->depth[i] = fb.Depth()[i];
    }
}
}  // namespace

extern "C" {

int ref_sampler(uint32_t n, const uint32_t* px, const uint32_t* py, const uint32_t* index,
                const uint32_t* branch, float* out2) {
    for (uint32_t i = 0; i < n; ++i) {
        OpenQmcSampler s({px[i], py[i], index[i]});
        const Vec2f v = s.Next2D(branch[i]);
        out2[2 * i + 0] = v.x;
        out2[2 * i + 1] = v.y;
    }
    return 0;
}

int ref_camera_rays(const ShiroRenderDesc* req, float* origins, float* dirs) {
    const Camera cam = ToCamera(req->camera);
    const RenderSettings st = ToSettings(req->settings);
    const uint32_t w = st.width, h = st.height;
    for (uint32_t y = 0; y < h; ++y) {
        for (uint32_t x = 0; x < w; ++x) {
            OpenQmcSampler sampler({x, y, req->sample_start});
            const cpu::Ray r = cpu::GenerateCameraRay(cam, st, x, y, sampler.Next2D(0));
            const size_t i = static_cast<size_t>(y) * w + x;
            origins[3 * i + 0] = r.origin.x;
            origins[3 * i + 1] = r.origin.y;
            origins[3 * i + 2] = r.origin.z;
            dirs[3 * i + 0] = r.direction.x;
            dirs[3 * i + 1] = r.direction.y;
            dirs[3 * i + 2] = r.direction.z;
        }
    }
    return 0;
}

int ref_trace_rays(const ShiroSceneDesc* sd, const float* origins, const float* dirs, const float* tmax,
                   uint32_t n, uint32_t* prim, float* t, uint32_t* occluded) {
    const Scene scene = ToScene(*sd);
    std::vector<std::thread> workers;
    const uint32_t threads = std::max(1u, std::thread::hardware_concurrency());
    for (uint32_t w = 0; w < threads; ++w) {
        workers.emplace_back([&, w]() {
            for (uint32_t i = w; i < n; i += threads) {
                cpu::Ray r;
                r.origin = V3(origins + 3 * i);
                r.direction = V3(dirs + 3 * i);
                cpu::Hit hit;
                if (cpu::IntersectScene(scene, nullptr, r, &hit)) {
                    prim[i] = GlobalPrim(scene, hit.meshIndex, hit.primitiveIndex);
                    t[i] = hit.distance;
                } else {
                    prim[i] = 0xffffffffu;
                    t[i] = FLT_MAX;
                }
                occluded[i] = cpu::Occluded(scene, nullptr, r.origin, r.direction, tmax[i]) ? 1u : 0u;
            }
        });
    }
    for (auto& th : workers) th.join();
    return 0;
}

// Closest hits of the camera rays of sample `sample_start` (one per pixel).
int ref_primary_hits(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, uint32_t* prim, float* t) {
    const Scene scene = ToScene(*sd);
    const Camera cam = ToCamera(req->camera);
    const RenderSettings st = ToSettings(req->settings);
    const uint32_t threads = std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> workers;
    for (uint32_t w = 0; w < threads; ++w) {
        workers.emplace_back([&, w]() {
            for (uint32_t y = w; y < st.height; y += threads) {
                for (uint32_t x = 0; x < st.width; ++x) {
                    OpenQmcSampler sampler({x, y, req->sample_start});
                    const cpu::Ray r = cpu::GenerateCameraRay(cam, st, x, y, sampler.Next2D(0));
                    cpu::Hit hit;
                    const size_t i = static_cast<size_t>(y) * st.width + x;
                    if (cpu::IntersectScene(scene, nullptr, r, &hit)) {
                        prim[i] = GlobalPrim(scene, hit.meshIndex, hit.primitiveIndex);
                        t[i] = hit.distance;
                    } else {
                        prim[i] = 0xffffffffu;
                        t[i] = FLT_MAX;
                    }
                }
            }
        });
    }
    for (auto& th : workers) th.join();
    return 0;
}

// EvaluateBsdf / EvaluateBsdfPdf (CpuPathTracer.cpp:1232-1354) and the lobe
// sample weights (:1376-1389) for n (normal, view, light) triples.
int ref_bsdf(const ShiroMaterialDesc* md, uint32_t n, const float* normals, const float* views,
             const float* lights, float* f_out, float* pdf_out, float* weights_out) {
    const PbrMaterial m = ToMaterial(*md);
    for (uint32_t i = 0; i < n; ++i) {
        const Vec3f nn = V3(normals + 3 * i);
        const Vec3f shading = cpu::ResolveShadingNormal(m, nn, false);
        const Vec3f coat = cpu::ResolveShadingNormal(m, shading, true);
        const Vec3f f = cpu::EvaluateBsdf(m, shading, coat, V3(views + 3 * i), V3(lights + 3 * i));
        f_out[3 * i + 0] = f.x;
        f_out[3 * i + 1] = f.y;
        f_out[3 * i + 2] = f.z;
        pdf_out[i] = cpu::EvaluateBsdfPdf(m, shading, coat, V3(views + 3 * i), V3(lights + 3 * i));
    }
    weights_out[0] = cpu::DiffuseSampleWeight(m);
    weights_out[1] = cpu::BaseSpecularSampleWeight(m);
    weights_out[2] = cpu::CoatSampleWeight(m);
    weights_out[3] = cpu::TransmissionSampleWeight(m);
    const Vec3f dc = cpu::DiffuseColor(m);
    weights_out[4] = dc.x;
    weights_out[5] = dc.y;
    weights_out[6] = dc.z;
    return 0;
}

// Importance table of a lat-long map (EnvironmentMap.cpp:185-236).
int ref_env_tables(uint32_t w, uint32_t h, const float* rgb, float* row_cdf, float* cond_cdf) {
    auto env = MakeEnvironment(w, h, rgb, SHIRO_ENV_LAYOUT_LATLONG);
    std::copy(env->rowCdf_.begin(), env->rowCdf_.end(), row_cdf);
    std::copy(env->conditionalCdf_.begin(), env->conditionalCdf_.end(), cond_cdf);
    return 0;
}

// EnvironmentMap::Sample / Pdf / Evaluate (EnvironmentMap.cpp:94-183).
int ref_env_query(uint32_t w, uint32_t h, const float* rgb, uint32_t layout, uint32_t n, const float* u2,
                  const float* dirs, float* sample_dir, float* sample_pdf, float* sample_rgb, float* pdf,
                  float* rgb_out) {
    auto env = MakeEnvironment(w, h, rgb, layout);
    for (uint32_t i = 0; i < n; ++i) {
        Vec3f d;
        float p = 0.0f;
        const Vec3f c = env->Sample({u2[2 * i], u2[2 * i + 1]}, &d, &p);
        sample_dir[3 * i + 0] = d.x;
        sample_dir[3 * i + 1] = d.y;
        sample_dir[3 * i + 2] = d.z;
        sample_pdf[i] = p;
        sample_rgb[3 * i + 0] = c.x;
        sample_rgb[3 * i + 1] = c.y;
        sample_rgb[3 * i + 2] = c.z;
        const Vec3f q = V3(dirs + 3 * i);
        pdf[i] = env->Pdf(q);
        const Vec3f e = env->Evaluate(q);
        rgb_out[3 * i + 0] = e.x;
        rgb_out[3 * i + 1] = e.y;
        rgb_out[3 * i + 2] = e.z;
    }
    return 0;
}

// CpuPathTracer::RenderSampleBatch (CpuPathTracer.cpp:2043-2170) on a fresh
// tracer instance (so the path guide starts empty).
int ref_render(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, ShiroAovs* out) {
    const Scene scene = ToScene(*sd);
    const Camera cam = ToCamera(req->camera);
    const RenderSettings st = ToSettings(req->settings);
    cpu::CpuPathTracer tracer;
    shiro::backend::RenderRequest request{scene, cam, st, req->sample_start, req->sample_count, nullptr};
    CopyFrame(tracer.RenderSampleBatch(request), out);
    return 0;
}

// `batches` consecutive batches of req->sample_count samples, starting at
// req->sample_start, on ONE tracer instance and the same Scene object, as a
// progressive render issues them (RenderParam.cpp:790): the tracer keeps its
// path-guide weights between batches of the same scene
// (CpuPathTracer.cpp:2054-2062, 2158-2167).  Writes the last batch's frame.
int ref_render_batches(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, uint32_t batches, ShiroAovs* out) {
    if (batches == 0) return -1;
    const Scene scene = ToScene(*sd);
    const Camera cam = ToCamera(req->camera);
    const RenderSettings st = ToSettings(req->settings);
    cpu::CpuPathTracer tracer;
    FrameBuffer fb;
    for (uint32_t b = 0; b < batches; ++b) {
        shiro::backend::RenderRequest request{scene, cam, st, req->sample_start + b * req->sample_count,
                                              req->sample_count, nullptr};
        fb = tracer.RenderSampleBatch(request);
    }
    CopyFrame(fb, out);
    return 0;
}

}  // extern "C"
