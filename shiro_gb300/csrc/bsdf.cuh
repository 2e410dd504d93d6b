// bsdf.cuh - layered BSDF of the reference CPU tracer.
//
// Restates src/backend/cpu/CpuPathTracer.cpp: SafeNormalized :836-839,
// AdjustedRoughness :845-893, ProjectedTangent :852-860, DielectricF0Scalar
// :895-899, DiffuseColor :901-909, BaseLayerRoughness :911-916, SpecularF0
// :918-928, ThinFilmColor / ApplyThinFilm :934-968, ResolveShadingNormal
// :970-986, GgxDistribution / GgxSmithVisibility / FresnelSchlick :988-1009,
// layer transmittances :1035-1082, EvaluateSpecularLobe / Pdf :1096-1132,
// PowerHeuristic :1218-1222, ClampMaxComponentValue :1224-1230,
// EvaluateBsdfPdf :1232-1273, EvaluateBsdf :1275-1354, sample weights
// :1376-1403, CosineSampleHemisphere :276-286, GgxSampleHalfVector :288-302.
// Materials are the PbrMaterial fields verbatim (ShiroMaterialDesc); derived
// quantities are recomputed per evaluation exactly as the reference does.
#pragma once

#include "common.cuh"
#include "scene.cuh"

namespace shiro_gpu {

using Mat = ShiroMaterialDesc;

__device__ __forceinline__ float sq(float v) { return v * v; }
__device__ __forceinline__ V3 safe_normalized(const V3& v, const V3& fb) {
    const float l = length(v);
    return l > 0.0f ? v / l : fb;
}
__device__ __forceinline__ V3 ortho_x(const V3& n) {  // BuildOrthonormalX
    const V3 axis = fabsf(n.z) < 0.999f ? V3{0.0f, 0.0f, 1.0f} : V3{0.0f, 1.0f, 0.0f};
    return normalize(cross(axis, n));
}
__device__ __forceinline__ float f0_dielectric(float ior) {
    const float s = smax(ior, 1.0f);
    return sq((s - 1.0f) / (s + 1.0f));
}
__device__ __forceinline__ V3 diffuse_color(const Mat& m) {
    const float metal = sclamp(m.metallic, 0.0f, 1.0f);
    const float trans = sclamp(m.transmission, 0.0f, 1.0f);
    const float sss = sclamp(m.subsurface, 0.0f, 1.0f);
    const float blend = sclamp(maxc(ld3(m.subsurface_radius)) / 3.0f, 0.0f, 1.0f);
    const V3 tint = lerp(ld3(m.base_color), ld3(m.subsurface_color), blend);
    const V3 base = lerp(ld3(m.base_color), tint, sss);
    return base * (sclamp(m.base_weight, 0.0f, 1.0f) * (1.0f - metal) * (1.0f - trans));
}
__device__ __forceinline__ float base_roughness(const Mat& m) {
    return sclamp(m.roughness + m.coat_affect_roughness * m.coat_weight * m.coat_roughness, 0.0f, 1.0f);
}
__device__ __forceinline__ V3 spec_f0(const Mat& m) {
    const float metal = sclamp(m.metallic, 0.0f, 1.0f);
    const V3 d = ld3(m.specular_color) * (sclamp(m.specular_weight, 0.0f, 1.0f) * f0_dielectric(m.ior));
    return lerp(d, ld3(m.base_color), metal);
}
__device__ __forceinline__ V3 coat_f0(const Mat& m) {
    return ld3(m.coat_color) * (sclamp(m.coat_weight, 0.0f, 1.0f) * f0_dielectric(m.coat_ior));
}
__device__ __forceinline__ V3 one_minus_clamped(const V3& v) {
    return {sclamp(1.0f - v.x, 0.0f, 1.0f), sclamp(1.0f - v.y, 0.0f, 1.0f), sclamp(1.0f - v.z, 0.0f, 1.0f)};
}
__device__ __forceinline__ V3 schlick(const V3& f0, float vDotH) {
    const float c = sclamp(1.0f - vDotH, 0.0f, 1.0f);
    const float f = c * c * c * c * c;
    return f0 + (V3{1.0f, 1.0f, 1.0f} - f0) * f;
}
__device__ __forceinline__ V3 coat_tint(const Mat& m) {
    const float a = sclamp(m.coat_affect_color * m.coat_weight, 0.0f, 1.0f);
    return lerp(V3{1.0f, 1.0f, 1.0f}, sclamp3(ld3(m.coat_color), 0.0f, 1.0f), a);
}
__device__ __forceinline__ V3 layer_transmittance(const V3& f0, float nDotV, float nDotL) {
    const V3 fv = schlick(f0, sclamp(nDotV, 0.0f, 1.0f));
    const V3 fl = schlick(f0, sclamp(nDotL, 0.0f, 1.0f));
    return one_minus_clamped((fv + fl) * 0.5f);
}
__device__ __forceinline__ float ggx_d(float nDotH, float r) {
    const float a = smax(0.02f, r * r);
    const float a2 = a * a;
    const float den = smax(1.0e-6f, sq(nDotH * nDotH * (a2 - 1.0f) + 1.0f));
    return a2 / (kPi * den);
}
__device__ __forceinline__ float ggx_lambda(float x, float a2) {
    const float c = smax(x, 1.0e-6f);
    return (-1.0f + sqrtf(1.0f + a2 * (1.0f - c * c) / (c * c))) * 0.5f;
}
__device__ __forceinline__ float ggx_vis(float nDotV, float nDotL, float r) {
    const float a = smax(0.02f, r * r);
    const float a2 = a * a;
    return 1.0f / (1.0f + ggx_lambda(nDotV, a2) + ggx_lambda(nDotL, a2));
}
__device__ __forceinline__ V3 spec_lobe(const V3& n, const V3& v, const V3& l, const V3& f0, float r) {
    const float nv = sclamp(dot(n, v), 0.0f, 1.0f);
    const float nl = sclamp(dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return {0.0f, 0.0f, 0.0f};
    const V3 h = safe_normalized(v + l, n);
    const float nh = sclamp(dot(n, h), 0.0f, 1.0f);
    const float vh = sclamp(dot(v, h), 0.0f, 1.0f);
    const float d = ggx_d(nh, r);
    const float g = ggx_vis(nv, nl, r);
    return schlick(f0, vh) * (d * g / smax(4.0f * nv * nl, 1.0e-6f));
}
__device__ __forceinline__ float spec_pdf(const V3& n, const V3& v, const V3& l, float r) {
    const float nv = sclamp(dot(n, v), 0.0f, 1.0f);
    const float nl = sclamp(dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return 0.0f;
    const V3 h = safe_normalized(v + l, n);
    const float nh = sclamp(dot(n, h), 0.0f, 1.0f);
    const float vh = sclamp(dot(v, h), 1.0e-6f, 1.0f);
    return ggx_d(nh, r) * nh / smax(4.0f * vh, 1.0e-6f);
}
__device__ __forceinline__ V3 proj_tangent(const Mat& m, const V3& n) {
    if (m.has_tangent_override) {
        const V3 to = ld3(m.tangent_override);
        const V3 t = to - n * dot(to, n);
        if (length(t) > 0.0f) return normalize(t);
    }
    return ortho_x(n);
}
// AdjustedRoughness with the half-vector anisotropy phase; with zero
// anisotropy the phase is multiplied by zero, so neither it nor the tangent
// (ProjectedTangent) is computed.
__device__ __forceinline__ float roughness_for(float r, float aniso, float rot, const Mat& m, const V3& n, const V3& v,
                                               const V3& l) {
    const float ca = sclamp(aniso, -0.95f, 0.95f);
    float phase = 0.0f;
    if (ca != 0.0f) {
        const V3 tangent = proj_tangent(m, n);
        const V3 td = safe_normalized(tangent - n * dot(tangent, n), ortho_x(n));
        const V3 bt = normalize(cross(n, td));
        const V3 h = safe_normalized(v + l, n);
        const V3 hp = h - n * dot(n, h);
        if (length(hp) <= 1.0e-6f) {
            phase = cosf(rot * 2.0f * kPi);
        } else {
            const V3 hd = normalize(hp);
            phase = cosf(atan2f(dot(hd, bt), dot(hd, td)) - rot * 2.0f * kPi);
        }
    }
    return sclamp(r * (1.0f - 0.35f * ca * phase), 0.02f, 1.0f);
}
__device__ __forceinline__ float roughness_for(float r, float aniso, float rot) {
    const float ca = sclamp(aniso, -0.95f, 0.95f);
    const float phase = cosf(rot * 2.0f * kPi);
    return sclamp(r * (1.0f - 0.35f * ca * phase), 0.02f, 1.0f);
}
__device__ __forceinline__ V3 film_color(float thickness, float ior, float vDotH) {
    if (thickness <= 0.0f) return {1.0f, 1.0f, 1.0f};
    const float si = smax(ior, 1.0f);
    const float op = 2.0f * si * thickness * sclamp(vDotH, 0.05f, 1.0f);
    const float p0 = 4.0f * kPi * op / smax(650.0f, 1.0f);
    const float p1 = 4.0f * kPi * op / smax(510.0f, 1.0f);
    const float p2 = 4.0f * kPi * op / smax(475.0f, 1.0f);
    const V3 iri{0.5f + 0.5f * cosf(p0), 0.5f + 0.5f * cosf(p1), 0.5f + 0.5f * cosf(p2)};
    const float strength = sclamp(thickness / 1200.0f, 0.0f, 1.0f);
    return lerp(V3{1.0f, 1.0f, 1.0f}, (V3{1.0f, 1.0f, 1.0f} + iri) * 0.5f, strength);
}
__device__ __forceinline__ V3 thin_film(const V3& lobe, const Mat& m, const V3& n, const V3& v, const V3& l) {
    if (m.thin_film_thickness <= 0.0f) return lobe;
    const V3 h = safe_normalized(v + l, n);
    const float vh = sclamp(dot(v, h), 0.0f, 1.0f);
    return lobe * film_color(m.thin_film_thickness, m.thin_film_ior, vh);
}
__device__ __forceinline__ V3 resolve_normal(const Mat& m, const V3& fb, bool coat) {
    const bool has = coat ? m.has_coat_normal_override != 0u : m.has_normal_override != 0u;
    if (!has) return fb;
    const V3 c = coat ? ld3(m.coat_normal_override) : ld3(m.normal_override);
    if (length(c) <= 0.0f) return fb;
    V3 n = normalize(c);
    if (dot(n, fb) < 0.0f) n = n * -1.0f;
    return n;
}

struct LobeWeights {
    float diffuse, spec, coat;
};
__device__ __forceinline__ LobeWeights lobe_weights(const Mat& m) {
    const V3 uc = coat_tint(m) * one_minus_clamped(coat_f0(m));
    const V3 sf0 = spec_f0(m);
    const V3 ub = one_minus_clamped(sf0);
    LobeWeights w;
    w.diffuse = smax(0.0f, maxc(diffuse_color(m) * uc * ub));
    w.spec = smax(0.0f, maxc(uc * sf0));
    w.coat = smax(0.0f, maxc(coat_f0(m)));
    return w;
}
__device__ __forceinline__ float transmission_weight(const Mat& m) {
    const float tr = sclamp(m.transmission, 0.0f, 1.0f);
    const float metal = sclamp(m.metallic, 0.0f, 1.0f);
    if (tr <= 0.0f || metal >= 0.999f) return 0.0f;
    const V3 uc = coat_tint(m) * one_minus_clamped(coat_f0(m));
    const V3 ub = one_minus_clamped(spec_f0(m));
    return smax(0.0f, maxc(sclamp3(ld3(m.transmission_color), 0.0f, 1.0f) * uc * ub)) * tr * (1.0f - metal);
}

// Per-material record of the quantities EvaluateBsdf / EvaluateBsdfPdf
// derive from the material alone (6 x float4), evaluated once per material
// with the same expressions as above, so every float is unchanged:
//   [0] SpecularF0, diffuse roughness sigma     [1] CoatF0, subsurface wrap
//   [2] coat underlayer tint, base GGX roughness (clamped; valid without anisotropy)
//   [3] DiffuseColor, coat GGX roughness (clamped; valid without anisotropy)
//   [4] sheen colour x sheen weight, 1 - 0.5 sheen roughness
//   [5] lobe sample weights (diffuse, base specular, coat), flag bits
constexpr uint32_t kRecAnisoSpec = 1u, kRecAnisoCoat = 2u, kRecSheen = 4u;
constexpr int kBsdfRec = 6;

__device__ __forceinline__ void make_bsdf_rec(const Mat& m, float4 r[kBsdfRec]) {
    const V3 f0 = spec_f0(m), cf0 = coat_f0(m), ct = coat_tint(m), dc = diffuse_color(m);
    const float sigma = sclamp(m.diffuse_roughness, 0.0f, 1.0f);
    const float wrap = sclamp(m.subsurface * m.subsurface_scale *
                                  (0.35f + 0.15f * sclamp(m.subsurface_anisotropy, -1.0f, 1.0f) +
                                   0.1f * sclamp(maxc(ld3(m.subsurface_radius)) / 3.0f, 0.0f, 1.0f)),
                              0.0f, 0.9f);
    const float sw = sclamp(m.sheen, 0.0f, 1.0f);
    const V3 scw = ld3(m.sheen_color) * sw;
    const LobeWeights w = lobe_weights(m);
    uint32_t flags = 0;
    if (sclamp(m.specular_anisotropy, -0.95f, 0.95f) != 0.0f) flags |= kRecAnisoSpec;
    if (sclamp(m.coat_anisotropy, -0.95f, 0.95f) != 0.0f) flags |= kRecAnisoCoat;
    if (sw != 0.0f) flags |= kRecSheen;
    r[0] = make_float4(f0.x, f0.y, f0.z, sigma);
    r[1] = make_float4(cf0.x, cf0.y, cf0.z, wrap);
    r[2] = make_float4(ct.x, ct.y, ct.z, sclamp(base_roughness(m), 0.02f, 1.0f));
    r[3] = make_float4(dc.x, dc.y, dc.z, sclamp(m.coat_roughness, 0.02f, 1.0f));
    r[4] = make_float4(scw.x, scw.y, scw.z, 1.0f - 0.5f * sclamp(m.sheen_roughness, 0.0f, 1.0f));
    r[5] = make_float4(w.diffuse, w.spec, w.coat, __uint_as_float(flags));
}
__device__ __forceinline__ LobeWeights rec_weights(const float4* r) {
    const float4 x = r[5];
    return {x.x, x.y, x.z};
}
// AdjustedRoughness of the base / coat lobe: the record's clamped value
// unless the lobe is anisotropic (then the half-vector phase is needed).
__device__ __forceinline__ float rec_spec_roughness(const float4* r, uint32_t flags, const Mat& m, const V3& n, const V3& v,
                                                    const V3& l) {
    return (flags & kRecAnisoSpec) ? roughness_for(base_roughness(m), m.specular_anisotropy, m.specular_rotation, m, n, v, l)
                                   : r[2].w;
}
__device__ __forceinline__ float rec_coat_roughness(const float4* r, uint32_t flags, const Mat& m, const V3& cn, const V3& v,
                                                    const V3& l) {
    return (flags & kRecAnisoCoat) ? roughness_for(m.coat_roughness, m.coat_anisotropy, m.coat_rotation, m, cn, v, l)
                                   : r[3].w;
}

// The out-of-line functions take their vectors by value: a reference
// argument of a call that is not inlined makes the caller store the vector
// to its stack and the callee load it back.
static __device__ __noinline__ float bsdf_pdf_rec(const float4* r, const Mat& m, const LobeWeights w, const V3 n,
                                                  const V3 cn, const V3 v, const V3 l) {
    const float nl = sclamp(dot(n, l), 0.0f, 1.0f);
    if (nl <= 0.0f) return 0.0f;
    const float rw = w.diffuse + w.spec + w.coat;
    if (rw <= 0.0f) return 0.0f;
    const float dp = w.diffuse / rw, bp = w.spec / rw, cp = w.coat / rw;
    const uint32_t flags = __float_as_uint(r[5].w);
    const float sr = rec_spec_roughness(r, flags, m, n, v, l);
    float coatTerm = 0.0f;
    if (cp != 0.0f) {
        const float cr = rec_coat_roughness(r, flags, m, cn, v, l);
        coatTerm = cp * spec_pdf(cn, v, l, cr);
    }
    return dp * nl * kInvPi + bp * spec_pdf(n, v, l, sr) + coatTerm;
}

static __device__ __noinline__ V3 bsdf_eval_rec(const float4* r, const Mat& m, const V3 n, const V3 cn, const V3 v,
                                               const V3 l) {
    const float nv = sclamp(dot(n, v), 0.0f, 1.0f);
    const float nl = sclamp(dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return {0.0f, 0.0f, 0.0f};
    const float4 r0 = r[0], r1 = r[1], r2 = r[2];
    const V3 baseF0{r0.x, r0.y, r0.z};
    const V3 cF0{r1.x, r1.y, r1.z};
    const V3 underCoat = V3{r2.x, r2.y, r2.z} * layer_transmittance(cF0, dot(cn, v), dot(cn, l));
    const V3 underBase = layer_transmittance(baseF0, nv, nl);
    const float sigma = r0.w;
    const float wrap = r1.w;
    const float wrapped = sclamp((nl + wrap) / (1.0f + wrap), 0.0f, 1.0f);
    float term;
    if (sigma == 0.0f) {
        // Lambert: orenA = 1 and orenB = 0 exactly, so the Oren-Nayar factor
        // (finite) multiplies zero and the sum is 1.
        term = 1.0f * (wrapped / smax(nl, 1.0e-6f));
    } else {
        const V3 vp = normalize(v - n * nv);
        const V3 lp = normalize(l - n * nl);
        const float cosPhi = length(vp) > 0.0f && length(lp) > 0.0f ? sclamp(dot(vp, lp), -1.0f, 1.0f) : 0.0f;
        const float s2 = sigma * sigma;
        const float orenA = 1.0f - (s2 / (2.0f * (s2 + 0.33f)));
        const float orenB = 0.45f * s2 / (s2 + 0.09f);
        const float sinV = sqrtf(smax(0.0f, 1.0f - nv * nv));
        const float sinL = sqrtf(smax(0.0f, 1.0f - nl * nl));
        const float sinAlpha = smax(sinV, sinL);
        const float tanBeta = smin(sinV / smax(nv, 1.0e-6f), sinL / smax(nl, 1.0e-6f));
        term = (orenA + orenB * smax(0.0f, cosPhi) * sinAlpha * tanBeta) * (wrapped / smax(nl, 1.0e-6f));
    }
    const float4 r3 = r[3];
    const V3 diffuse = V3{r3.x, r3.y, r3.z} * underCoat * underBase * (kInvPi * term);
    const uint32_t flags = __float_as_uint(r[5].w);
    const float sr = rec_spec_roughness(r, flags, m, n, v, l);
    const V3 spec = underCoat * thin_film(spec_lobe(n, v, l, baseF0, sr), m, n, v, l);
    const float cr = rec_coat_roughness(r, flags, m, cn, v, l);
    const V3 coat = thin_film(spec_lobe(cn, v, l, cF0, cr), m, cn, v, l);
    // With zero sheen weight the factor sf (finite, >= 0) only multiplies a
    // signed zero; 1 gives the same signed zero without the powf.
    float sf = 1.0f;
    const float4 r4 = r[4];
    if (flags & kRecSheen) {
        const V3 h = safe_normalized(v + l, n);
        const float lh = sclamp(dot(l, h), 0.0f, 1.0f);
        sf = powf(1.0f - lh, 5.0f) * r4.w;
    }
    const V3 sheen = V3{r4.x, r4.y, r4.z} * sf * underCoat * underBase;
    return diffuse + spec + coat + sheen;
}

// The BSDF value from the material alone (record formed per call): for
// materials that have no stored record, i.e. the second parameter set of a
// frozen render of the differentiable form.  Out of line, so the record code
// exists once.
static __device__ __noinline__ V3 bsdf_eval(const Mat& m, const V3 n, const V3 cn, const V3 v, const V3 l) {
    float4 r[kBsdfRec];
    make_bsdf_rec(m, r);
    return bsdf_eval_rec(r, m, n, cn, v, l);
}

// ---- transmission, media, emitters (CpuPathTracer.cpp:930-932, 1011-1033,
// 1059-1063, 1084-1094, 1136-1212, 1355-1373, 1405-1441) ------------------
__device__ __forceinline__ float transmission_roughness(const Mat& m) {
    return sclamp(m.roughness + m.transmission_extra_roughness, 0.0f, 1.0f);
}
__device__ __forceinline__ float fresnel_dielectric(float cosThetaI, float etaI, float etaT) {
    float c = sclamp(cosThetaI, -1.0f, 1.0f);
    float ei = smax(etaI, 1.0e-6f);
    float et = smax(etaT, 1.0e-6f);
    if (c <= 0.0f) {
        const float t = ei;
        ei = et;
        et = t;
        c = fabsf(c);
    }
    const float sinI = sqrtf(smax(0.0f, 1.0f - c * c));
    const float sinT = ei / et * sinI;
    if (sinT >= 1.0f) return 1.0f;
    const float cosT = sqrtf(smax(0.0f, 1.0f - sinT * sinT));
    const float rPar = ((et * c) - (ei * cosT)) / smax((et * c) + (ei * cosT), 1.0e-6f);
    const float rPer = ((ei * c) - (et * cosT)) / smax((ei * c) + (et * cosT), 1.0e-6f);
    return 0.5f * (rPar * rPar + rPer * rPer);
}
__device__ __forceinline__ V3 interface_transmittance(const V3& f0, float a, float b) {
    const V3 fa = schlick(f0, sclamp(fabsf(a), 0.0f, 1.0f));
    const V3 fb = schlick(f0, sclamp(fabsf(b), 0.0f, 1.0f));
    return one_minus_clamped((fa + fb) * 0.5f);
}
__device__ __forceinline__ V3 coat_transmission_scale(const Mat& m, const V3& cn, const V3& v, const V3& l) {
    return coat_tint(m) * interface_transmittance(coat_f0(m), dot(cn, v), dot(cn, l));
}
__device__ __forceinline__ V3 transmission_surface_tint(const Mat& m) {
    if (!m.thin_walled && m.transmission_depth > 0.0f) return {1.0f, 1.0f, 1.0f};
    return sclamp3(ld3(m.transmission_color), 0.0f, 1.0f);
}
__device__ __forceinline__ float thin_pane_transmittance(float r) {
    const float c = sclamp(r, 0.0f, 1.0f);
    return sclamp((1.0f - c) / smax(1.0f + c, 1.0e-6f), 0.0f, 1.0f);
}
__device__ __forceinline__ V3 medium_extinction(const Mat& m) {
    V3 e{smax(m.transmission_scatter[0], 0.0f), smax(m.transmission_scatter[1], 0.0f),
         smax(m.transmission_scatter[2], 0.0f)};
    if (m.thin_walled || m.transmission_depth <= 0.0f) return e;
    const float depth = smax(m.transmission_depth, 1.0e-3f);
    const V3 tint = sclamp3(ld3(m.transmission_color), 1.0e-4f, 1.0f);
    e.x += -logf(tint.x) / depth;
    e.y += -logf(tint.y) / depth;
    e.z += -logf(tint.z) / depth;
    return e;
}
__device__ __forceinline__ V3 medium_attenuation(const V3& e, float d) {
    return {expf(-e.x * d), expf(-e.y * d), expf(-e.z * d)};
}
__device__ __forceinline__ bool refract_dir(const V3& i, const V3& n, float eta, V3* out) {
    const float c = sclamp(-dot(i, n), -1.0f, 1.0f);
    const float sin2 = smax(0.0f, 1.0f - c * c);
    const float k = 1.0f - eta * eta * sin2;
    if (k <= 0.0f) return false;
    *out = normalize(i * eta + n * (eta * c - sqrtf(k)));
    return true;
}
static __device__ __noinline__ V3 transmission_lobe(const Mat& m, const V3 n, const V3 cn, const V3 v, const V3 l,
                                                    float etaI, float etaT, float r) {
    const float cosWo = dot(n, v), cosWi = dot(n, l);
    const float aWo = fabsf(cosWo), aWi = fabsf(cosWi);
    if (aWo <= 0.0f || aWi <= 0.0f || cosWo * cosWi >= 0.0f) return {0.0f, 0.0f, 0.0f};
    const float rel = etaT / smax(etaI, 1.0e-6f);
    V3 h = safe_normalized(v + l * rel, n);
    if (dot(n, h) < 0.0f) h = h * -1.0f;
    const float woH = dot(v, h), wiH = dot(l, h);
    if (woH * wiH >= 0.0f) return {0.0f, 0.0f, 0.0f};
    const float nh = sclamp(dot(n, h), 0.0f, 1.0f);
    const float sd = woH + rel * wiH;
    if (nh <= 0.0f || fabsf(sd) <= 1.0e-6f) return {0.0f, 0.0f, 0.0f};
    const float dist = ggx_d(nh, r);
    const float vis = ggx_vis(aWo, aWi, r);
    const float fres = 1.0f - fresnel_dielectric(fabsf(woH), etaI, etaT);
    const V3 scale = transmission_surface_tint(m) * coat_transmission_scale(m, cn, v, l) *
                     (sclamp(m.transmission, 0.0f, 1.0f) * (1.0f - sclamp(m.metallic, 0.0f, 1.0f)));
    const float factor = fabsf(dist * vis * fabsf(wiH) * fabsf(woH) / smax(aWo * aWi * sq(sd), 1.0e-6f));
    const float transport = 1.0f / smax(rel * rel, 1.0e-6f);
    return scale * fres * (factor * transport);
}
static __device__ __noinline__ float transmission_pdf(const V3 n, const V3 v, const V3 l, float eta, float r) {
    const float cosWo = dot(n, v), cosWi = dot(n, l);
    if (fabsf(cosWo) <= 0.0f || fabsf(cosWi) <= 0.0f || cosWo * cosWi >= 0.0f) return 0.0f;
    V3 h = safe_normalized(v + l * eta, n);
    if (dot(n, h) < 0.0f) h = h * -1.0f;
    const float woH = dot(v, h), wiH = dot(l, h);
    const float sd = woH + eta * wiH;
    if (woH * wiH >= 0.0f || fabsf(sd) <= 1.0e-6f) return 0.0f;
    const float nh = sclamp(dot(n, h), 0.0f, 1.0f);
    const float pdfWh = ggx_d(nh, r) * nh;
    const float dwh = fabsf((eta * eta * wiH) / sq(sd));
    return pdfWh * dwh;
}
__device__ __forceinline__ V3 emitted_radiance(const Mat& m) {  // :1722-1727
    return {smax(m.emission_color[0] * m.emission_strength, 0.0f), smax(m.emission_color[1] * m.emission_strength, 0.0f),
            smax(m.emission_color[2] * m.emission_strength, 0.0f)};
}

__device__ __forceinline__ V3 cosine_hemisphere(const V3& n, const V2& s) {
    const float phi = 2.0f * kPi * s.x;
    const float r = sqrtf(s.y);
    const float x = r * cosf(phi);
    const float y = r * sinf(phi);
    const float z = sqrtf(smax(0.0f, 1.0f - s.y));
    const V3 t = ortho_x(n);
    const V3 b = cross(n, t);
    return normalize(t * x + b * y + n * z);
}
__device__ __forceinline__ V3 ggx_half(const V3& n, const V2& s, float rough) {
    const float a = smax(0.02f, rough * rough);
    const float a2 = a * a;
    const float phi = 2.0f * kPi * s.x;
    const float ct = sqrtf(smax(0.0f, (1.0f - s.y) / smax(1.0e-6f, 1.0f + (a2 - 1.0f) * s.y)));
    const float st = sqrtf(smax(0.0f, 1.0f - ct * ct));
    const float x = st * cosf(phi);
    const float y = st * sinf(phi);
    const V3 t = ortho_x(n);
    const V3 b = cross(n, t);
    return normalize(t * x + b * y + n * ct);
}
__device__ __forceinline__ V3 clamp_max(const V3& v, float mx) {
    const float c = maxc(v);
    if (c <= mx || c <= 0.0f) return v;
    return v * (mx / c);
}
__device__ __forceinline__ float power_heuristic(float a, float b) {
    const float a2 = a * a, b2 = b * b;
    return a2 / smax(a2 + b2, 1.0e-6f);
}

}  // namespace shiro_gpu
