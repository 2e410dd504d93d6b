// integrator.cuh - one path of the reference's Monte-Carlo estimator.
//
// trace_path restates TracePath (src/backend/cpu/CpuPathTracer.cpp:1650-2017)
// with DirectLighting (:1511-1576) and GenerateCameraRay (:1633-1648) for the
// scenes the backend accepts (shiro_gpu_supports_scene: no transmission, no
// opacity cut-outs, no emissive triangles).  Sample dimensions, lobe choice,
// clamps, Russian roulette and MIS are those of the reference, so a path is
// a deterministic function of (pixel, sample index) shared with the CPU
// tracer.  The path guide of the reference is empty in the first batch of a
// scene (:2054-2062) and is not used here.
#pragma once

#include "bsdf.cuh"
#include "common.cuh"
#include "env.cuh"
#include "sampler.cuh"
#include "scene.cuh"
#include "traverse.cuh"

namespace shiro_gpu {

struct PathResult {
    V3 radiance, albedo, normal;
    float depth;
};

struct Surface {
    V3 position, ng, ns;
    uint32_t material;
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

// DirectLighting without the emissive-triangle term (:1511-1576).
template <typename Ctr>
__device__ __forceinline__ V3 direct_lighting(const DevScene& s, const DevRequest& q, const Surface& hit, const V3& n,
                                              const V3& cn, const Mat& m, const LobeWeights& w, const V3& view,
                                              const Sampler& smp, uint32_t depth, Ctr& ctr) {
    V3 out{0.0f, 0.0f, 0.0f};
    const V3 origin = hit.position + n * kRayEpsilon;
    for (uint32_t i = 0; i < s.distantCount; ++i) {
        const DevDistant l = s.distant[i];
        const V3 ld = normalize(l.direction * -1.0f);
        const float nl = sclamp(dot(n, ld), 0.0f, 1.0f);
        if (nl <= 0.0f || trace_occluded(s, origin, ld, FLT_MAX, ctr)) continue;
        ctr.bsdf_eval();
        out = out + clamp24(q, bsdf_eval(m, n, cn, view, ld) * l.radiance * nl);
    }
    const bool useCdf = (q.flags & SHIRO_RENDER_ENV_CDF) != 0u;
    for (uint32_t li = 0; li < s.domeCount; ++li) {
        V3 acc{0.0f, 0.0f, 0.0f};
        for (uint32_t k = 0; k < q.domeSamples; ++k) {
            const uint32_t dim = kDirectDimBase + depth * kDirectDepthStride + li * kDirectLightStride + k * kDirectSampleStride;
            V3 ld, lr;
            float lp = 0.0f;
            if (s.domes[li].env >= 0) {
                ctr.env_sample();
                ctr.env_eval();
            }
            if (!sample_dome(s, s.domes[li], smp.next2d(dim), useCdf, &ld, &lr, &lp) || lp <= 0.0f) continue;
            const float nl = sclamp(dot(n, ld), 0.0f, 1.0f);
            if (nl <= 0.0f || trace_occluded(s, origin, ld, FLT_MAX, ctr)) continue;
            ctr.bsdf_pdf();
            ctr.bsdf_eval();
            const float bp = bsdf_pdf(m, w, n, cn, view, ld);
            const float mis = power_heuristic(lp, bp);
            acc = acc + clamp24(q, bsdf_eval(m, n, cn, view, ld) * lr * (nl * mis / lp));
        }
        out = out + acc / static_cast<float>(q.domeSamples);
    }
    return out;
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

template <typename Ctr>
__device__ __forceinline__ PathResult trace_path(const DevScene& s, const DevRequest& q, uint32_t x, uint32_t y,
                                                 uint32_t sampleIndex, Ctr& ctr) {
    PathResult res;
    res.radiance = V3{0.0f, 0.0f, 0.0f};
    res.albedo = V3{0.0f, 0.0f, 0.0f};
    res.normal = V3{0.0f, 0.0f, 0.0f};
    res.depth = __int_as_float(0x7f800000);  // +inf
    const Sampler smp{x, y, sampleIndex};
    V3 ro, rd;
    camera_ray(q, x, y, smp.next2d(0u), &ro, &rd);
    V3 T{1.0f, 1.0f, 1.0f};
    uint32_t diffDepth = 0, specDepth = 0;
    bool prevDelta = true;
    float prevPdf = 0.0f;
    for (uint32_t depth = 0; depth < q.maxDepth; ++depth) {
        const uint32_t base = depth * kPathDimStride;
        HitRec h;
        if (!trace_closest(s, ro, rd, &h, ctr)) {
            if (depth > 0 || q.backgroundVisible) {
                const V3 env = environment_radiance(s, rd);
                ctr.env_eval(s.domeCount);
                if (s.domeCount == 0 || depth == 0 || prevDelta) {
                    res.radiance = res.radiance + T * env;
                } else {
                    ctr.env_sample(s.domeCount);
                    res.radiance = res.radiance + T * env * env_miss_mis(s, prevPdf, rd);
                }
            }
            break;
        }
        ctr.hit();
        const Surface hit = make_surface(s, ro, rd, h);
        const Mat& m = s.materials[hit.material];
        V3 n, cn;
        shading_frame(m, hit, rd, &n, &cn);
        const V3 view = rd * -1.0f;
        if (depth == 0) {
            res.albedo = diffuse_color(m);
            res.normal = n * 0.5f + V3{0.5f, 0.5f, 0.5f};
            res.depth = h.t;
        }
        const LobeWeights w = lobe_weights(m);
        res.radiance = res.radiance + T * direct_lighting(s, q, hit, n, cn, m, w, view, smp, depth, ctr);

        const float rw = w.diffuse + w.spec + w.coat;
        const float tw = rw + 0.0f;
        if (tw <= 0.0f) break;
        const float sel = smp.next1d(base + 1u) * tw;
        const V2 ds = smp.next2d(base + 2u);
        V3 next, f;
        float pdf;
        bool delta = false;
        const float rs = sel - 0.0f;
        if (rs < w.diffuse) {
            if (diffDepth >= q.diffuseDepth) break;
            ++diffDepth;
            next = cosine_hemisphere(n, ds);
            const float cpdf = sclamp(dot(n, next), 0.0f, 1.0f) * kInvPi;
            pdf = smax((rw / tw) * (1.0f * cpdf + 0.0f * 0.0f), 1.0e-6f);
            ctr.bsdf_eval();
            f = bsdf_eval(m, n, cn, view, next);
        } else {
            const bool coat = !(rs < w.diffuse + w.spec);
            if (specDepth >= q.specularDepth) break;
            ++specDepth;
            const V3 sn = coat ? cn : n;
            const float sr = coat ? roughness_for(m.coat_roughness, m.coat_anisotropy, m.coat_rotation)
                                  : roughness_for(base_roughness(m), m.specular_anisotropy, m.specular_rotation);
            const V3 hv = ggx_half(sn, ds, sr);
            next = normalize(reflect(rd, hv));
            const float rc = sclamp(dot(sn, next), 0.0f, 1.0f);
            if (rc <= 0.0f) break;
            ctr.bsdf_pdf();
            ctr.bsdf_eval();
            pdf = smax((rw / tw) * bsdf_pdf(m, w, n, cn, view, next), 1.0e-6f);
            f = bsdf_eval(m, n, cn, view, next);
            delta = sr <= kDeltaRoughness;
        }
        const float cosT = sclamp(dot(n, next), 0.0f, 1.0f);
        if (cosT <= 0.0f) break;
        T = clamp12(q, T * f * (cosT / pdf));
        const float off = dot(n, next) >= 0.0f ? 1.0f : -1.0f;
        ro = hit.position + n * (kRayEpsilon * off);
        rd = next;
        prevDelta = delta;
        prevPdf = pdf;
        if (depth >= 2) {
            const float cp = sclamp(maxc(T), 0.05f, 0.95f);
            if (smp.next1d(base + 4u) > cp) break;
            T = T / cp;
        }
    }
    return res;
}

}  // namespace shiro_gpu
