// integrator.cuh - the reference's Monte-Carlo estimator, split into the
// pieces shared by the plain megakernel and the wavefront stages.
//
// Restates TracePath (src/backend/cpu/CpuPathTracer.cpp:1650-2017) with
// DirectLighting (:1511-1576) and GenerateCameraRay (:1633-1648) for the
// scenes the backend accepts (shiro_gpu_supports_scene: no transmission, no
// opacity cut-outs, no emissive triangles).  Sample dimensions, lobe choice,
// clamps, Russian roulette and MIS are those of the reference, so a path is a
// deterministic function of (pixel, sample index) shared with the CPU tracer.
// The path guide of the reference is empty in the first batch of a scene
// (:2054-2062) and is not used here.
//
// Both GPU forms call the same functions for every float they produce: the
// per-light contribution (light_distant / light_dome), the in-order sum of the
// unoccluded contributions, the miss term and the continuation, so the
// wavefront form reproduces the plain form bit for bit.
#pragma once

#include "bsdf.cuh"
#include "common.cuh"
#include "env.cuh"
#include "sampler.cuh"
#include "scene.cuh"
#include "traverse.cuh"

namespace shiro_gpu {

// Light samples per shading point handled by the wavefront shadow stage
// (distant lights + dome lights x dome samples).
constexpr uint32_t kMaxLightSamples = 8;

struct PathResult {
    V3 radiance, albedo, normal;
    float depth;
};

struct Surface {
    V3 position, ng, ns;
    uint32_t material;
};

// Per-path state carried between bounces.
struct PathState {
    V3 ro, rd, T, radiance;
    uint32_t diffDepth, specDepth;
    bool prevDelta;
    float prevPdf;
};

// Shading context of one hit.
struct Vertex {
    Surface hit;
    V3 n, cn, view;
    LobeWeights w;
};

// Hit record of the brute-force intersector (:448-456) and
// TriangleShadingNormal (:142-168).
__device__ __forceinline__ Surface make_surface(const DevScene& s, const V3& o, const V3& d, const HitRec& h) {
    Surface sf;
    sf.position = o + d * h.t;
    const float4* tp = s.tris + 3 * static_cast<size_t>(h.slot);
    const V3 e1 = f4xyz(__ldg(tp + 1)), e2 = f4xyz(__ldg(tp + 2));
    const V3 ng = normalize(cross(e1, e2));
    sf.ng = ng;
    const uint4 tv = __ldg(&s.triVerts[h.gid]);
    V3 ns = ng;
    if (__ldg(&s.meshHasNormals[tv.w])) {
        const float b0 = 1.0f - h.u - h.v, b1 = h.u, b2 = h.v;
        const V3 n0 = f4xyz(__ldg(&s.normals[tv.x])), n1 = f4xyz(__ldg(&s.normals[tv.y])),
                 n2 = f4xyz(__ldg(&s.normals[tv.z]));
        const V3 interp = n0 * b0 + n1 * b1 + n2 * b2;
        if (length(interp) > 0.0f) ns = normalize(interp);
    }
    sf.ns = ns;
    sf.material = __ldg(&s.meshMaterial[tv.w]);
    return sf;
}

// GenerateCameraRay (:1633-1648); tanHalfFov comes from the host's std::tan.
__device__ __forceinline__ void camera_ray(const DevRequest& q, uint32_t x, uint32_t y, const V2& s, V3* o, V3* d) {
    const float fx = ((static_cast<float>(x) + s.x) / static_cast<float>(q.width)) * 2.0f - 1.0f;
    const float fy = ((static_cast<float>(y) + s.y) / static_cast<float>(q.height)) * 2.0f - 1.0f;
    const V3 dir = q.camForward + q.camRight * (fx * q.aspect * q.tanHalfFov) + q.camUp * (fy * q.tanHalfFov);
    *o = q.camPos;
    *d = normalize(dir);
}

__device__ __forceinline__ V3 clamp24(const DevRequest& q, const V3& v) {
    return (q.flags & SHIRO_RENDER_NO_CLAMP) ? v : clamp_max(v, kDirectSampleClamp);
}
__device__ __forceinline__ V3 clamp12(const DevRequest& q, const V3& v) {
    return (q.flags & SHIRO_RENDER_NO_CLAMP) ? v : clamp_max(v, kThroughputClamp);
}

// Shading frame of a hit (:1699-1712).
__device__ __forceinline__ void shading_frame(const Mat& m, const Surface& hit, const V3& rd, V3* n, V3* cn) {
    const bool front = dot(hit.ng, rd) < 0.0f;
    const V3 ng = front ? hit.ng : hit.ng * -1.0f;
    V3 sb = front ? hit.ns : hit.ns * -1.0f;
    if (dot(sb, ng) < 0.0f) sb = sb * -1.0f;
    V3 nn = resolve_normal(m, sb, false);
    if (dot(nn, ng) < 0.0f) nn = nn * -1.0f;
    *n = nn;
    *cn = resolve_normal(m, nn, true);
}

__device__ __forceinline__ Vertex make_vertex(const DevScene& s, const V3& ro, const V3& rd, const HitRec& h) {
    Vertex v;
    v.hit = make_surface(s, ro, rd, h);
    const Mat& m = s.materials[v.hit.material];
    shading_frame(m, v.hit, rd, &v.n, &v.cn);
    v.view = rd * -1.0f;
    v.w = lobe_weights(m);
    return v;
}

__device__ __forceinline__ uint32_t light_sample_count(const DevScene& s, const DevRequest& q) {
    return s.distantCount + s.domeCount * q.domeSamples;
}

// Origin of the shadow rays of a vertex (:1527).
__device__ __forceinline__ V3 shadow_origin(const Vertex& v) { return v.hit.position + v.n * kRayEpsilon; }

// Distant light i (:1529-1540): false when the light is below the horizon;
// otherwise the direction and the clamped contribution if unoccluded.
template <typename Ctr>
__device__ __forceinline__ bool light_distant(const DevScene& s, const DevRequest& q, const Vertex& v, uint32_t i, V3* dir,
                                              V3* c, Ctr& ctr) {
    const DevDistant l = s.distant[i];
    const V3 ld = normalize(l.direction * -1.0f);
    const float nl = sclamp(dot(v.n, ld), 0.0f, 1.0f);
    if (nl <= 0.0f) return false;
    const Mat& m = s.materials[v.hit.material];
    ctr.bsdf_eval();
    *dir = ld;
    *c = clamp24(q, bsdf_eval(m, v.n, v.cn, v.view, ld) * l.radiance * nl);
    return true;
}

// Sample k of dome light li (:1542-1573).
template <typename Ctr>
__device__ __forceinline__ bool light_dome(const DevScene& s, const DevRequest& q, const Vertex& v, const Sampler& smp,
                                           uint32_t depth, uint32_t li, uint32_t k, V3* dir, V3* c, Ctr& ctr) {
    const uint32_t dim = kDirectDimBase + depth * kDirectDepthStride + li * kDirectLightStride + k * kDirectSampleStride;
    V3 ld, lr;
    float lp = 0.0f;
    if (s.domes[li].env >= 0) {
        ctr.env_sample();
        ctr.env_eval();
    }
    const bool useCdf = (q.flags & SHIRO_RENDER_ENV_CDF) != 0u;
    if (!sample_dome(s, s.domes[li], smp.next2d(dim), useCdf, &ld, &lr, &lp) || lp <= 0.0f) return false;
    const float nl = sclamp(dot(v.n, ld), 0.0f, 1.0f);
    if (nl <= 0.0f) return false;
    const Mat& m = s.materials[v.hit.material];
    ctr.bsdf_pdf();
    ctr.bsdf_eval();
    const float bp = bsdf_pdf(m, v.w, v.n, v.cn, v.view, ld);
    const float mis = power_heuristic(lp, bp);
    *dir = ld;
    *c = clamp24(q, bsdf_eval(m, v.n, v.cn, v.view, ld) * lr * (nl * mis / lp));
    return true;
}

// Adds the unoccluded contributions in the reference's order: distant lights,
// then per dome the average of its samples.  `visible(k, dir, c)` returns
// whether light sample k (in that order) is present and unoccluded.
template <typename Visible>
__device__ __forceinline__ V3 sum_direct(const DevScene& s, const DevRequest& q, Visible&& visible) {
    V3 out{0.0f, 0.0f, 0.0f};
    uint32_t k = 0;
    for (uint32_t i = 0; i < s.distantCount; ++i, ++k) {
        V3 c;
        if (visible(k, &c)) out = out + c;
    }
    for (uint32_t li = 0; li < s.domeCount; ++li) {
        V3 acc{0.0f, 0.0f, 0.0f};
        for (uint32_t j = 0; j < q.domeSamples; ++j, ++k) {
            V3 c;
            if (visible(k, &c)) acc = acc + c;
        }
        out = out + acc / static_cast<float>(q.domeSamples);
    }
    return out;
}

// Light sample k of a vertex, in sum_direct's order.
template <typename Ctr>
__device__ __forceinline__ bool light_sample(const DevScene& s, const DevRequest& q, const Vertex& v, const Sampler& smp,
                                             uint32_t depth, uint32_t k, V3* dir, V3* c, Ctr& ctr) {
    if (k < s.distantCount) return light_distant(s, q, v, k, dir, c, ctr);
    const uint32_t r = k - s.distantCount;
    const uint32_t li = r / q.domeSamples, j = r - li * q.domeSamples;
    return light_dome(s, q, v, smp, depth, li, j, dir, c, ctr);
}

// MIS weight of an environment hit after a non-delta bounce (:1679-1688).
__device__ __forceinline__ float env_miss_mis(const DevScene& s, float prevPdf, const V3& dir) {
    float sum = 0.0f;
    for (uint32_t i = 0; i < s.domeCount; ++i) {
        const float p = dome_pdf(s, s.domes[i], dir);
        sum += p * p;
    }
    const float b2 = prevPdf * prevPdf;
    return b2 / smax(b2 + sum, 1.0e-6f);
}

// Ray leaving the scene at `depth` (:1675-1693).
template <typename Ctr>
__device__ __forceinline__ void add_miss(const DevScene& s, const DevRequest& q, PathState& ps, uint32_t depth, Ctr& ctr) {
    if (depth > 0 || q.backgroundVisible) {
        const V3 env = environment_radiance(s, ps.rd);
        ctr.env_eval(s.domeCount);
        if (s.domeCount == 0 || depth == 0 || ps.prevDelta) {
            ps.radiance = ps.radiance + ps.T * env;
        } else {
            ctr.env_sample(s.domeCount);
            ps.radiance = ps.radiance + ps.T * env * env_miss_mis(s, ps.prevPdf, ps.rd);
        }
    }
}

// Lobe choice, direction sampling, throughput update and Russian roulette
// (:1765-2013).  Returns false when the path ends at this vertex.
template <typename Ctr>
__device__ __forceinline__ bool continue_path(const DevScene& s, const DevRequest& q, const Vertex& v, const Sampler& smp,
                                              uint32_t depth, PathState& ps, Ctr& ctr) {
    const uint32_t base = depth * kPathDimStride;
    const Mat& m = s.materials[v.hit.material];
    const float rw = v.w.diffuse + v.w.spec + v.w.coat;
    const float tw = rw + 0.0f;
    if (tw <= 0.0f) return false;
    const float sel = smp.next1d(base + 1u) * tw;
    const V2 ds = smp.next2d(base + 2u);
    V3 next;
    float pdf;
    bool delta = false;
    const float rs = sel - 0.0f;
    if (rs < v.w.diffuse) {
        if (ps.diffDepth >= q.diffuseDepth) return false;
        ++ps.diffDepth;
        next = cosine_hemisphere(v.n, ds);
        const float cpdf = sclamp(dot(v.n, next), 0.0f, 1.0f) * kInvPi;
        pdf = smax((rw / tw) * (1.0f * cpdf + 0.0f * 0.0f), 1.0e-6f);
    } else {
        const bool coat = !(rs < v.w.diffuse + v.w.spec);
        if (ps.specDepth >= q.specularDepth) return false;
        ++ps.specDepth;
        const V3 sn = coat ? v.cn : v.n;
        const float sr = coat ? roughness_for(m.coat_roughness, m.coat_anisotropy, m.coat_rotation)
                              : roughness_for(base_roughness(m), m.specular_anisotropy, m.specular_rotation);
        const V3 hv = ggx_half(sn, ds, sr);
        next = normalize(reflect(ps.rd, hv));
        const float rc = sclamp(dot(sn, next), 0.0f, 1.0f);
        if (rc <= 0.0f) return false;
        ctr.bsdf_pdf();
        pdf = smax((rw / tw) * bsdf_pdf(m, v.w, v.n, v.cn, v.view, next), 1.0e-6f);
        delta = sr <= kDeltaRoughness;
    }
    // one evaluation site for both lobes, so a warp whose lanes chose
    // different lobes runs the BSDF once
    ctr.bsdf_eval();
    const V3 f = bsdf_eval(m, v.n, v.cn, v.view, next);
    const float cosT = sclamp(dot(v.n, next), 0.0f, 1.0f);
    if (cosT <= 0.0f) return false;
    ps.T = clamp12(q, ps.T * f * (cosT / pdf));
    const float off = dot(v.n, next) >= 0.0f ? 1.0f : -1.0f;
    ps.ro = v.hit.position + v.n * (kRayEpsilon * off);
    ps.rd = next;
    ps.prevDelta = delta;
    ps.prevPdf = pdf;
    if (depth >= 2) {
        const float cp = sclamp(maxc(ps.T), 0.05f, 0.95f);
        if (smp.next1d(base + 4u) > cp) return false;
        ps.T = ps.T / cp;
    }
    return true;
}

__device__ __forceinline__ void init_path(const DevRequest& q, const Sampler& smp, PathState& ps) {
    camera_ray(q, smp.px, smp.py, smp.next2d(0u), &ps.ro, &ps.rd);
    ps.T = V3{1.0f, 1.0f, 1.0f};
    ps.radiance = V3{0.0f, 0.0f, 0.0f};
    ps.diffDepth = 0;
    ps.specDepth = 0;
    ps.prevDelta = true;
    ps.prevPdf = 0.0f;
}

// The whole path in one thread (the plain form).
template <typename Ctr>
__device__ __forceinline__ PathResult trace_path(const DevScene& s, const DevRequest& q, uint32_t x, uint32_t y,
                                                 uint32_t sampleIndex, Ctr& ctr) {
    PathResult res;
    res.albedo = V3{0.0f, 0.0f, 0.0f};
    res.normal = V3{0.0f, 0.0f, 0.0f};
    res.depth = __int_as_float(0x7f800000);  // +inf
    const Sampler smp{x, y, sampleIndex};
    PathState ps;
    init_path(q, smp, ps);
    for (uint32_t depth = 0; depth < q.maxDepth; ++depth) {
        HitRec h;
        if (!trace_closest(s, ps.ro, ps.rd, &h, ctr)) {
            add_miss(s, q, ps, depth, ctr);
            break;
        }
        ctr.hit();
        const Vertex v = make_vertex(s, ps.ro, ps.rd, h);
        if (depth == 0) {
            res.albedo = diffuse_color(s.materials[v.hit.material]);
            res.normal = v.n * 0.5f + V3{0.5f, 0.5f, 0.5f};
            res.depth = h.t;
        }
        const V3 origin = shadow_origin(v);
        const V3 direct = sum_direct(s, q, [&](uint32_t k, V3* c) {
            V3 dir;
            if (!light_sample(s, q, v, smp, depth, k, &dir, c, ctr)) return false;
            return !trace_occluded(s, origin, dir, FLT_MAX, ctr);
        });
        ps.radiance = ps.radiance + ps.T * direct;
        if (!continue_path(s, q, v, smp, depth, ps, ctr)) break;
    }
    res.radiance = ps.radiance;
    return res;
}

}  // namespace shiro_gpu
