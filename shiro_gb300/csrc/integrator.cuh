// integrator.cuh - the reference's Monte-Carlo estimator, split into the
// pieces shared by the plain megakernel and the wavefront stages.
//
// Restates TracePath (src/backend/cpu/CpuPathTracer.cpp:1650-2017) with
// DirectLighting (:1511-1631) and GenerateCameraRay (:1633-1648): reflection
// lobes, transmission (thin-walled panes, smooth and rough dielectrics) with
// homogeneous media, opacity cut-outs, emitters with their MIS weight and the
// emissive-triangle light sample.  Sample dimensions, lobe choice,
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
// (distant lights + dome lights x dome samples + one emissive triangle).
constexpr uint32_t kMaxLightSamples = 8;

// BounceType of TracePath (CpuPathTracer.cpp:79-84).
constexpr uint32_t kBounceNone = 0, kBounceDiffuse = 1, kBounceReflective = 2, kBounceTransmission = 3;

struct PathResult {
    V3 radiance, albedo, normal;
    float depth;
};

struct Surface {
    V3 position, ng, ns;
    uint32_t material;
    uint32_t gid;  // global triangle index (mesh, primitive)
};

// Per-path state carried between bounces.
struct PathState {
    V3 ro, rd, T, radiance;
    uint32_t diffDepth, specDepth;
    bool prevDelta;
    float prevPdf;
    uint32_t prevType;     // kBounce*
    bool inside;           // inside a transmissive object (insideMedium)
    bool mediumActive;     // its medium attenuates
    V3 extinction;
};

// Shading context of one hit.
struct Vertex {
    Surface hit;
    V3 n, cn, view;
    V3 ngf;  // geometric normal facing the incoming ray
    LobeWeights w;
};

// Hit record of the brute-force intersector (:448-456) and
// TriangleShadingNormal (:142-168).
__device__ __forceinline__ Surface make_surface(const DevScene& s, const V3& o, const V3& d, const HitRec& h) {
    Surface sf;
    sf.position = o + d * h.t;
    const float4* r = s.shade + kShadeRec * static_cast<size_t>(h.gid);
    const float4 r0 = __ldg(r);
    const uint32_t bits = __float_as_uint(r0.w);
    const V3 ng = f4xyz(r0);  // normalize(cross(e1, e2)) of the triangle, formed at upload
    sf.ng = ng;
    V3 ns = ng;
    if (bits & kShadeNormals) {
        const float b0 = 1.0f - h.u - h.v, b1 = h.u, b2 = h.v;
        const V3 n0 = f4xyz(__ldg(r + 1)), n1 = f4xyz(__ldg(r + 2)), n2 = f4xyz(__ldg(r + 3));
        const V3 interp = n0 * b0 + n1 * b1 + n2 * b2;
        if (length(interp) > 0.0f) ns = normalize(interp);
    }
    sf.ns = ns;
    sf.material = bits & ~kShadeNormals;
    sf.gid = h.gid;
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
__device__ __forceinline__ void shading_frame(const Mat& m, const Surface& hit, const V3& rd, V3* n, V3* cn, V3* ngf) {
    const bool front = dot(hit.ng, rd) < 0.0f;
    const V3 ng = front ? hit.ng : hit.ng * -1.0f;
    *ngf = ng;
    V3 sb = front ? hit.ns : hit.ns * -1.0f;
    if (dot(sb, ng) < 0.0f) sb = sb * -1.0f;
    V3 nn = resolve_normal(m, sb, false);
    if (dot(nn, ng) < 0.0f) nn = nn * -1.0f;
    *n = nn;
    *cn = resolve_normal(m, nn, true);
}

__device__ __forceinline__ const float4* bsdf_rec(const DevScene& s, uint32_t material) {
    return s.bsdfRecs + kBsdfRec * static_cast<size_t>(material);
}

__device__ __forceinline__ Vertex make_vertex(const DevScene& s, const V3& ro, const V3& rd, const HitRec& h) {
    Vertex v;
    v.hit = make_surface(s, ro, rd, h);
    const Mat& m = s.materials[v.hit.material];
    shading_frame(m, v.hit, rd, &v.n, &v.cn, &v.ngf);
    v.view = rd * -1.0f;
    v.w = rec_weights(bsdf_rec(s, v.hit.material));
    return v;
}

__device__ __forceinline__ bool has_emitters(const DevScene& s) { return s.emissiveCount > 0u && s.emissiveSum > 0.0f; }

// kExt (here and below) compiles the lobes of transmission, media, opacity
// and emitters in; kernels for scenes without them are built with kExt =
// false, which drops branches that such scenes never take.
template <bool kExt>
__device__ __forceinline__ uint32_t light_sample_count(const DevScene& s, const DevRequest& q) {
    return s.distantCount + s.domeCount * q.domeSamples + (kExt && has_emitters(s) ? 1u : 0u);
}

// SampleEmissiveTriangleLight (:1443-1460): the first entry whose running
// sum is not below u * sum, else the last.
__device__ __forceinline__ uint32_t sample_emitter(const DevScene& s, float u) {
    const float target = sclamp(u, 0.0f, 0.99999994f) * s.emissiveSum;
    uint32_t lo = 0, hi = s.emissiveCount;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&s.emissiveCdf[mid]) < target) lo = mid + 1u; else hi = mid;
    }
    return lo == s.emissiveCount ? s.emissiveCount - 1u : lo;
}

// EmissiveTrianglePdf (:1475-1495) of global triangle `gid`.
__device__ __forceinline__ float emitter_pdf(const DevScene& s, uint32_t gid, const V3& origin, const V3& position) {
    if (s.emissiveCount == 0u) return 0.0f;
    const int32_t k = __ldg(&s.emissiveOf[gid]);
    if (k < 0) return 0.0f;
    const float4 e0 = __ldg(&s.emissive[3 * k]), e2 = __ldg(&s.emissive[3 * k + 2]);
    if (e0.x <= 0.0f || s.emissiveSum <= 0.0f) return 0.0f;
    const V3 to = position - origin;
    const float d2 = dot(to, to);
    if (d2 <= 1.0e-10f) return 0.0f;
    const V3 ld = normalize(to);
    const float cosL = smax(fabsf(dot(f4xyz(e2), ld * -1.0f)), 1.0e-6f);
    const float sel = e0.y / s.emissiveSum;
    const float areaPdf = sel / e0.x;
    return areaPdf * d2 / cosL;
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
    *c = clamp24(q, bsdf_eval_rec(bsdf_rec(s, v.hit.material), m, v.n, v.cn, v.view, ld) * l.radiance * nl);
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
    const float4* rec = bsdf_rec(s, v.hit.material);
    const float bp = bsdf_pdf_rec(rec, m, v.w, v.n, v.cn, v.view, ld);
    const float mis = power_heuristic(lp, bp);
    *dir = ld;
    *c = clamp24(q, bsdf_eval_rec(rec, m, v.n, v.cn, v.view, ld) * lr * (nl * mis / lp));
    return true;
}

// Adds the unoccluded contributions in the reference's order: distant lights,
// then per dome the average of its samples.  `visible(k, dir, c)` returns
// whether light sample k (in that order) is present and unoccluded.
template <bool kExt, typename Visible>
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
    if constexpr (kExt) {
        if (has_emitters(s)) {
            V3 c;
            if (visible(k, &c)) out = out + c;
        }
    }
    return out;
}

// The emissive-triangle sample's geometry (:1578-1616): the point picked on
// an emitter, its direction *ld from the vertex, the emitted radiance *le,
// the sample's solid-angle pdf *lp, the cosine *nl at the vertex and the
// reach of its shadow ray, which stops short of the light.
__device__ __forceinline__ bool emissive_geometry(const DevScene& s, const Vertex& v, const Sampler& smp, uint32_t depth,
                                                  V3* ld, V3* le, float* lp, float* nl, float* maxDist) {
    if (!has_emitters(s)) return false;
    const uint32_t db = kEmissiveDimBase + depth * kEmissiveDepthStride;
    const uint32_t k = sample_emitter(s, smp.next1d(db + 0u));
    const float4 e0 = __ldg(&s.emissive[3 * k]), e1 = __ldg(&s.emissive[3 * k + 1]), e2 = __ldg(&s.emissive[3 * k + 2]);
    const uint32_t gid = __float_as_uint(e0.w);
    if (gid == v.hit.gid) return false;
    const V2 u = smp.next2d(db + 1u);
    const float su = sqrtf(sclamp(u.x, 0.0f, 1.0f));  // UniformTriangleBarycentrics, :240-253
    const float b0 = 1.0f - su;
    const float b1 = sclamp(u.y, 0.0f, 1.0f) * su;
    const float b2 = 1.0f - b0 - b1;
    const uint4 tv = __ldg(&s.triVerts[gid]);
    const V3 p = f4xyz(__ldg(&s.positions[tv.x])) * b0 + f4xyz(__ldg(&s.positions[tv.y])) * b1 +
                 f4xyz(__ldg(&s.positions[tv.z])) * b2;  // TrianglePoint, :224-238
    const V3 to = p - v.hit.position;
    const float d2 = dot(to, to);
    if (d2 <= 1.0e-10f) return false;
    const float dist = sqrtf(d2);
    *ld = to / dist;
    *nl = sclamp(dot(v.n, *ld), 0.0f, 1.0f);
    const float cosL = fabsf(dot(f4xyz(e2), *ld * -1.0f));
    if (*nl <= 0.0f || cosL <= 0.0f) return false;
    const float sel = e0.y / s.emissiveSum;
    const float areaPdf = sel / smax(e0.x, 1.0e-6f);
    *lp = areaPdf * d2 / smax(cosL, 1.0e-6f);
    if (*lp <= 0.0f) return false;
    *le = f4xyz(e1);
    *maxDist = smax(dist - 2.0f * kRayEpsilon, kRayEpsilon);
    return true;
}

// The emissive-triangle sample (:1578-1628); its shadow ray stops short of
// the light (*maxDist).
template <typename Ctr>
__device__ __forceinline__ bool light_emissive(const DevScene& s, const DevRequest& q, const Vertex& v, const Sampler& smp,
                                               uint32_t depth, V3* dir, V3* c, float* maxDist, Ctr& ctr) {
    V3 ld, le;
    float lp, nl;
    if (!emissive_geometry(s, v, smp, depth, &ld, &le, &lp, &nl, maxDist)) return false;
    const Mat& m = s.materials[v.hit.material];
    ctr.bsdf_pdf();
    ctr.bsdf_eval();
    const float4* rec = bsdf_rec(s, v.hit.material);
    const float bp = bsdf_pdf_rec(rec, m, v.w, v.n, v.cn, v.view, ld);
    const float mis = power_heuristic(lp, bp);
    *dir = ld;
    *c = clamp24(q, bsdf_eval_rec(rec, m, v.n, v.cn, v.view, ld) * le * (nl * mis / lp));
    return true;
}

// Light sample k of a vertex, in sum_direct's order; *maxDist is the reach
// of its shadow ray.
template <bool kExt, typename Ctr>
__device__ __forceinline__ bool light_sample(const DevScene& s, const DevRequest& q, const Vertex& v, const Sampler& smp,
                                             uint32_t depth, uint32_t k, V3* dir, V3* c, float* maxDist, Ctr& ctr) {
    *maxDist = FLT_MAX;
    if (k < s.distantCount) return light_distant(s, q, v, k, dir, c, ctr);
    const uint32_t r = k - s.distantCount;
    if constexpr (kExt) {
        if (r >= s.domeCount * q.domeSamples) return light_emissive(s, q, v, smp, depth, dir, c, maxDist, ctr);
    }
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

// Ray leaving the scene at `depth` (:1675-1693): EnvironmentRadiance, and
// after a non-delta reflection its MIS weight against the dome lights'
// sampling (:1679-1688); each dome's direction angles are formed once for
// both.
template <typename Ctr>
__device__ __forceinline__ void add_miss(const DevScene& s, const DevRequest& q, PathState& ps, uint32_t depth, Ctr& ctr) {
    if (!(depth > 0 || q.backgroundVisible)) return;
    ctr.env_eval(s.domeCount);
    const bool weighted = !(s.domeCount == 0 || depth == 0 || ps.prevDelta || ps.prevType == kBounceTransmission);
    if (s.domeCount == 0) {
        const float t = sclamp(ps.rd.y * 0.5f + 0.5f, 0.0f, 1.0f);
        ps.radiance = ps.radiance + ps.T * lerp(s.envBottom, s.envTop, t);
        return;
    }
    V3 env{0.0f, 0.0f, 0.0f};
    float sum = 0.0f;
    for (uint32_t i = 0; i < s.domeCount; ++i) {
        const DevDome& d = s.domes[i];
        float p = kInvFourPi;
        if (d.env >= 0) {
            env = env + env_evaluate_pdf(s.envs[d.env], world_to_light(d, ps.rd), weighted, &p) * d.radiance;
        } else {
            env = env + d.radiance;
        }
        sum += p * p;
    }
    if (!weighted) {
        ps.radiance = ps.radiance + ps.T * env;
    } else {
        ctr.env_sample(s.domeCount);
        const float b2 = ps.prevPdf * ps.prevPdf;
        ps.radiance = ps.radiance + ps.T * env * (b2 / smax(b2 + sum, 1.0e-6f));
    }
}

// Medium attenuation and the opacity test at a hit (:1695-1720): false when
// the path passes through the surface (ps.ro moved past it, the hit is not
// shaded and the bounce counts toward the depth).
__device__ __forceinline__ bool enter_hit(const DevScene& s, const Sampler& smp, uint32_t depth, const Vertex& v, float t,
                                          PathState& ps) {
    if (ps.mediumActive) ps.T = ps.T * medium_attenuation(ps.extinction, t);
    const float op = sclamp(s.materials[v.hit.material].opacity, 0.0f, 1.0f);
    if (op < 0.999f) {
        if (smp.next1d(depth * kPathDimStride + 0u) > op) {
            ps.ro = v.hit.position + ps.rd * kRayEpsilon;
            return false;
        }
        ps.T = ps.T / smax(op, 1.0e-4f);
    }
    return true;
}

// Emitted radiance of a hit, MIS-weighted against the emissive-triangle
// light sample after a non-delta reflection (:1728-1744).
__device__ __forceinline__ void add_emission(const DevScene& s, const Vertex& v, uint32_t depth, PathState& ps) {
    const Mat& m = s.materials[v.hit.material];
    if (!(m.emission_strength > 0.0f)) return;
    const V3 le = emitted_radiance(m);
    if (depth == 0 || ps.prevDelta || ps.prevType == kBounceTransmission) {
        ps.radiance = ps.radiance + ps.T * le;
    } else {
        const float lp = emitter_pdf(s, v.hit.gid, ps.ro, v.hit.position);
        const float mis = lp > 0.0f ? power_heuristic(ps.prevPdf, lp) : 1.0f;
        ps.radiance = ps.radiance + ps.T * le * mis;
    }
}

__device__ __forceinline__ void toggle_medium(const Mat& m, PathState& ps) {
    ps.inside = !ps.inside;
    if (ps.inside) {
        ps.extinction = medium_extinction(m);
        ps.mediumActive = m.transmission_depth > 0.0f || maxc(ld3(m.transmission_scatter)) > 0.0f;
    } else {
        ps.mediumActive = false;
    }
}

// Lobe choice (transmission first, then diffuse / base specular / coat),
// direction sampling, throughput update and Russian roulette (:1746-2013).
// Returns false when the path ends at this vertex.
template <bool kExt, typename Ctr>
__device__ __forceinline__ bool continue_path(const DevScene& s, const DevRequest& q, const Vertex& v, const Sampler& smp,
                                              uint32_t depth, PathState& ps, Ctr& ctr) {
    const uint32_t base = depth * kPathDimStride;
    const Mat& m = s.materials[v.hit.material];
    const float4* rec = bsdf_rec(s, v.hit.material);
    const float dw = v.w.diffuse, cw = v.w.coat;
    float bw = v.w.spec;
    const float rawTw = kExt ? transmission_weight(m) : 0.0f;
    float tw = rawTw;
    if (kExt && rawTw > 0.0f) {
        const float etaI = ps.inside ? smax(m.ior, 1.0f) : 1.0f;
        const float etaT = ps.inside ? 1.0f : smax(m.ior, 1.0f);
        const float refl = fresnel_dielectric(fabsf(dot(v.ngf, v.view)), etaI, etaT);
        const float pass = m.thin_walled ? thin_pane_transmittance(refl) : (1.0f - refl);
        tw = rawTw * pass;
        bw += rawTw * (1.0f - pass);
    }
    const float rw = dw + bw + cw;
    const float total = rw + tw;
    if (total <= 0.0f) return false;
    const float sel = smp.next1d(base + 1u) * total;
    const V2 ds = smp.next2d(base + 2u);
    V3 next, f;
    float pdf = 1.0f;
    uint32_t type = kBounceDiffuse;
    bool delta = false;
    bool chooseT = false, chooseC = false;
    bool reflEval = true;  // f is the reflection BSDF at `next`
    if (kExt && sel < tw) {
        chooseT = true;
    } else {
        const float rs = sel - tw;
        chooseC = !(rs < dw) && !(rs < dw + bw);
        if (!(rs < dw)) type = kBounceReflective;
    }
    if (kExt && chooseT) {  // :1811-1925
        if (ps.specDepth >= q.specularDepth) return false;
        ++ps.specDepth;
        type = kBounceTransmission;
        const float tp = smax(tw / total, 1.0e-6f);
        const float tr =
            m.thin_walled ? 0.0f : roughness_for(transmission_roughness(m), m.specular_anisotropy, m.specular_rotation);
        const float mt = sclamp(m.transmission, 0.0f, 1.0f) * (1.0f - sclamp(m.metallic, 0.0f, 1.0f));
        if (m.thin_walled) {
            next = ps.rd;
            const float refl = fresnel_dielectric(fabsf(dot(v.ngf, v.view)), 1.0f, smax(m.ior, 1.0f));
            const float pane = thin_pane_transmittance(refl);
            const V3 scale = transmission_surface_tint(m) * coat_transmission_scale(m, v.cn, v.view, next) * mt;
            const float ac = smax(fabsf(dot(v.ngf, next)), 1.0e-4f);
            f = scale * pane / ac;
            pdf = tp;
            delta = true;
            reflEval = false;
        } else {
            const float etaI = ps.inside ? smax(m.ior, 1.0f) : 1.0f;
            const float etaT = ps.inside ? 1.0f : smax(m.ior, 1.0f);
            const float ratio = etaI / etaT;
            const float rel = etaT / smax(etaI, 1.0f);
            const float refl = fresnel_dielectric(fabsf(dot(v.ngf, v.view)), etaI, etaT);
            const V3 mn0 = tr <= kDeltaRoughness ? v.ngf : ggx_half(v.ngf, ds, tr);
            const V3 mn = dot(mn0, v.view) < 0.0f && tr > kDeltaRoughness ? mn0 * -1.0f : mn0;
            if (!refract_dir(ps.rd, mn, ratio, &next)) {
                // total internal reflection: the reflection lobes take the path
                next = normalize(reflect(ps.rd, mn));
                if (rw <= 0.0f) return false;
                ctr.bsdf_pdf();
                pdf = smax((rw / total) * bsdf_pdf_rec(rec, m, v.w, v.n, v.cn, v.view, next), 1.0e-6f);
                type = kBounceReflective;
                delta = tr <= kDeltaRoughness;
                chooseT = false;
            } else if (tr <= kDeltaRoughness) {
                const V3 scale = transmission_surface_tint(m) * coat_transmission_scale(m, v.cn, v.view, next) * mt;
                const float ac = smax(fabsf(dot(v.ngf, next)), 1.0e-4f);
                const float transport = 1.0f / smax(rel * rel, 1.0e-6f);
                f = scale * (1.0f - refl) * transport / ac;
                pdf = tp;
                toggle_medium(m, ps);
                delta = true;
                reflEval = false;
            } else {
                f = transmission_lobe(m, v.ngf, v.cn, v.view, next, etaI, etaT, tr);
                pdf = smax(tp * transmission_pdf(v.ngf, v.view, next, etaT / etaI, tr), 1.0e-6f);
                toggle_medium(m, ps);
                delta = tr <= kDeltaRoughness;
                reflEval = false;
            }
        }
    } else if (type == kBounceReflective) {  // base specular or coat
        if (ps.specDepth >= q.specularDepth) return false;
        ++ps.specDepth;
        const V3 sn = chooseC ? v.cn : v.n;
        const float sr = chooseC ? roughness_for(m.coat_roughness, m.coat_anisotropy, m.coat_rotation)
                                 : roughness_for(base_roughness(m), m.specular_anisotropy, m.specular_rotation);
        const V3 hv = ggx_half(sn, ds, sr);
        next = normalize(reflect(ps.rd, hv));
        const float rc = sclamp(dot(sn, next), 0.0f, 1.0f);
        if (rc <= 0.0f) return false;
        ctr.bsdf_pdf();
        pdf = smax((rw / total) * bsdf_pdf_rec(rec, m, v.w, v.n, v.cn, v.view, next), 1.0e-6f);
        delta = sr <= kDeltaRoughness;
    } else {  // diffuse
        if (ps.diffDepth >= q.diffuseDepth) return false;
        ++ps.diffDepth;
        next = cosine_hemisphere(v.n, ds);
        const float cpdf = sclamp(dot(v.n, next), 0.0f, 1.0f) * kInvPi;
        pdf = smax((rw / total) * (1.0f * cpdf + 0.0f * 0.0f), 1.0e-6f);
    }
    // one evaluation site for the reflection lobes, so a warp whose lanes
    // chose different lobes runs the BSDF once
    if (reflEval) {
        ctr.bsdf_eval();
        f = bsdf_eval_rec(rec, m, v.n, v.cn, v.view, next);
    }
    const float cosT = chooseT ? smax(fabsf(dot(v.ngf, next)), 1.0e-4f) : sclamp(dot(v.n, next), 0.0f, 1.0f);
    if (cosT <= 0.0f) return false;
    ps.T = clamp12(q, ps.T * f * (cosT / pdf));
    const V3 rn = chooseT ? v.ngf : v.n;
    const float off = dot(rn, next) >= 0.0f ? 1.0f : -1.0f;
    ps.ro = v.hit.position + rn * (kRayEpsilon * off);
    ps.rd = next;
    ps.prevType = type;
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
    ps.prevType = kBounceNone;
    ps.inside = false;
    ps.mediumActive = false;
    ps.extinction = V3{0.0f, 0.0f, 0.0f};
}

// The whole path in one thread (the plain form).
template <bool kExt, typename Ctr>
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
        if constexpr (kExt) {
            if (!enter_hit(s, smp, depth, v, h.t, ps)) continue;
        }
        if (depth == 0) {
            const float4 dc = __ldg(bsdf_rec(s, v.hit.material) + 3);  // DiffuseColor
            res.albedo = V3{dc.x, dc.y, dc.z};
            res.normal = v.n * 0.5f + V3{0.5f, 0.5f, 0.5f};
            res.depth = h.t;
        }
        if constexpr (kExt) add_emission(s, v, depth, ps);
        const V3 origin = shadow_origin(v);
        const V3 direct = sum_direct<kExt>(s, q, [&](uint32_t k, V3* c) {
            V3 dir;
            float reach;
            if (!light_sample<kExt>(s, q, v, smp, depth, k, &dir, c, &reach, ctr)) return false;
            return !trace_occluded(s, origin, dir, reach, ctr);
        });
        ps.radiance = ps.radiance + ps.T * direct;
        if (!continue_path<kExt>(s, q, v, smp, depth, ps, ctr)) break;
    }
    res.radiance = ps.radiance;
    return res;
}

}  // namespace shiro_gpu
