// bsdf_diff.cuh - EvaluateBsdf with forward-mode derivatives.
//
// bsdf_eval_d restates EvaluateBsdf (src/backend/cpu/CpuPathTracer.cpp:
// 1275-1354) on dual numbers carrying the derivatives with respect to the
// differentiable material parameters: base colour (r, g, b), specular
// roughness and metalness.  The value part performs the same float
// operations in the same order as bsdf_eval (bsdf.cuh), so value(f) equals
// the forward BSDF bit for bit; clamps and max/min propagate the derivative
// of the branch they select (zero when a bound is selected).
#pragma once

#include "bsdf.cuh"

namespace shiro_gpu {

constexpr int kDualN = 5;  // d/d base_r, base_g, base_b, roughness, metallic
constexpr int kDRough = 3, kDMetal = 4;

struct Dual {
    float v;
    float d[kDualN];
};

__device__ __forceinline__ Dual dconst(float v) {
    Dual r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = 0.0f;
    return r;
}
__device__ __forceinline__ Dual dvar(float v, int i) {
    Dual r = dconst(v);
    r.d[i] = 1.0f;
    return r;
}
__device__ __forceinline__ Dual operator+(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = a.d[i] + b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator+(const Dual& a, float b) {
    Dual r = a;
    r.v = a.v + b;
    return r;
}
__device__ __forceinline__ Dual operator+(float a, const Dual& b) {
    Dual r = b;
    r.v = a + b.v;
    return r;
}
__device__ __forceinline__ Dual operator-(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = a.d[i] - b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator-(float a, const Dual& b) {
    Dual r;
    r.v = a - b.v;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = -b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator-(const Dual& a, float b) {
    Dual r = a;
    r.v = a.v - b;
    return r;
}
__device__ __forceinline__ Dual operator*(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator*(const Dual& a, float b) {
    Dual r;
    r.v = a.v * b;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = a.d[i] * b;
    return r;
}
__device__ __forceinline__ Dual operator*(float a, const Dual& b) {
    Dual r;
    r.v = a * b.v;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = a * b.d[i];
    return r;
}
__device__ __forceinline__ Dual operator/(const Dual& a, const Dual& b) {
    Dual r;
    r.v = a.v / b.v;
    const float inv2 = 1.0f / (b.v * b.v);
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) * inv2;
    return r;
}
__device__ __forceinline__ Dual operator/(const Dual& a, float b) {
    Dual r;
    r.v = a.v / b;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = a.d[i] / b;
    return r;
}
__device__ __forceinline__ Dual operator/(float a, const Dual& b) {
    Dual r;
    r.v = a / b.v;
    const float k = -a / (b.v * b.v);
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = k * b.d[i];
    return r;
}
__device__ __forceinline__ Dual dsqrt(const Dual& a) {
    Dual r;
    r.v = sqrtf(a.v);
    const float k = r.v > 0.0f ? 0.5f / r.v : 0.0f;
#pragma unroll
    for (int i = 0; i < kDualN; ++i) r.d[i] = k * a.d[i];
    return r;
}
// std::max / std::min / std::clamp: the derivative follows the selected value.
__device__ __forceinline__ Dual dmax(float a, const Dual& b) { return a < b.v ? b : dconst(a); }
__device__ __forceinline__ Dual dclamp(const Dual& x, float lo, float hi) {
    if (x.v < lo) return dconst(lo);
    if (hi < x.v) return dconst(hi);
    return x;
}

struct DV3 {
    Dual x, y, z;
};
__device__ __forceinline__ DV3 dv3(const V3& v) { return {dconst(v.x), dconst(v.y), dconst(v.z)}; }
__device__ __forceinline__ DV3 operator+(const DV3& a, const DV3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ DV3 operator*(const DV3& a, const DV3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ DV3 operator*(const DV3& a, const V3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ DV3 operator*(const V3& a, const DV3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ DV3 operator*(const DV3& a, const Dual& s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ DV3 operator*(const DV3& a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ DV3 operator*(const V3& a, const Dual& s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 dval(const DV3& a) { return {a.x.v, a.y.v, a.z.v}; }

// lerp(a, b, t) = a * (1 - t) + b * t with dual b and t (spec_f0's metal lerp).
__device__ __forceinline__ DV3 dlerp(const V3& a, const DV3& b, const Dual& t) {
    const Dual omt = 1.0f - t;
    return {a.x * omt + b.x * t, a.y * omt + b.y * t, a.z * omt + b.z * t};
}
__device__ __forceinline__ DV3 dlerp(const DV3& a, const V3& b, float t) {
    return {a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t, a.z * (1.0f - t) + b.z * t};
}
__device__ __forceinline__ DV3 dlerp(const DV3& a, const DV3& b, float t) {
    return {a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t, a.z * (1.0f - t) + b.z * t};
}

// Differentiable material parameters of one material.
struct MatParams {
    DV3 base;
    Dual rough;  // m.roughness
    Dual metal;  // sclamp(m.metallic, 0, 1)
};

__device__ __forceinline__ MatParams mat_params(const Mat& m) {
    MatParams p;
    p.base = DV3{dvar(m.base_color[0], 0), dvar(m.base_color[1], 1), dvar(m.base_color[2], 2)};
    p.rough = dvar(m.roughness, kDRough);
    p.metal = dclamp(dvar(m.metallic, kDMetal), 0.0f, 1.0f);
    return p;
}

__device__ __forceinline__ DV3 diffuse_color_d(const Mat& m, const MatParams& p) {
    const float trans = sclamp(m.transmission, 0.0f, 1.0f);
    const float sss = sclamp(m.subsurface, 0.0f, 1.0f);
    const float blend = sclamp(maxc(ld3(m.subsurface_radius)) / 3.0f, 0.0f, 1.0f);
    const DV3 tint = dlerp(p.base, ld3(m.subsurface_color), blend);
    const DV3 base = dlerp(p.base, tint, sss);
    return base * (sclamp(m.base_weight, 0.0f, 1.0f) * (1.0f - p.metal) * (1.0f - trans));
}
__device__ __forceinline__ DV3 spec_f0_d(const Mat& m, const MatParams& p) {
    const V3 d = ld3(m.specular_color) * (sclamp(m.specular_weight, 0.0f, 1.0f) * f0_dielectric(m.ior));
    return dlerp(d, p.base, p.metal);
}
__device__ __forceinline__ Dual one_minus_clamped1(const Dual& v) { return dclamp(1.0f - v, 0.0f, 1.0f); }
__device__ __forceinline__ DV3 schlick_d(const DV3& f0, float vDotH) {
    const float c = sclamp(1.0f - vDotH, 0.0f, 1.0f);
    const float f = c * c * c * c * c;
    return {f0.x + (1.0f - f0.x) * f, f0.y + (1.0f - f0.y) * f, f0.z + (1.0f - f0.z) * f};
}
__device__ __forceinline__ DV3 layer_transmittance_d(const DV3& f0, float nDotV, float nDotL) {
    const DV3 fv = schlick_d(f0, sclamp(nDotV, 0.0f, 1.0f));
    const DV3 fl = schlick_d(f0, sclamp(nDotL, 0.0f, 1.0f));
    const DV3 s = (fv + fl) * 0.5f;
    return {one_minus_clamped1(s.x), one_minus_clamped1(s.y), one_minus_clamped1(s.z)};
}
__device__ __forceinline__ Dual ggx_d_d(float nDotH, const Dual& r) {
    const Dual a = dmax(0.02f, r * r);
    const Dual a2 = a * a;
    const Dual t = nDotH * nDotH * (a2 - 1.0f) + 1.0f;
    const Dual den = dmax(1.0e-6f, t * t);
    return a2 / (kPi * den);
}
__device__ __forceinline__ Dual ggx_lambda_d(float x, const Dual& a2) {
    const float c = smax(x, 1.0e-6f);
    return (-1.0f + dsqrt(1.0f + a2 * (1.0f - c * c) / (c * c))) * 0.5f;
}
__device__ __forceinline__ Dual ggx_vis_d(float nDotV, float nDotL, const Dual& r) {
    const Dual a = dmax(0.02f, r * r);
    const Dual a2 = a * a;
    return 1.0f / (1.0f + ggx_lambda_d(nDotV, a2) + ggx_lambda_d(nDotL, a2));
}
__device__ __forceinline__ DV3 spec_lobe_d(const V3& n, const V3& v, const V3& l, const DV3& f0, const Dual& r) {
    const float nv = sclamp(dot(n, v), 0.0f, 1.0f);
    const float nl = sclamp(dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return dv3(V3{0.0f, 0.0f, 0.0f});
    const V3 h = safe_normalized(v + l, n);
    const float nh = sclamp(dot(n, h), 0.0f, 1.0f);
    const float vh = sclamp(dot(v, h), 0.0f, 1.0f);
    const Dual d = ggx_d_d(nh, r);
    const Dual g = ggx_vis_d(nv, nl, r);
    return schlick_d(f0, vh) * (d * g / smax(4.0f * nv * nl, 1.0e-6f));
}
// AdjustedRoughness on a dual base roughness (the phase factor is geometry).
__device__ __forceinline__ Dual roughness_for_d(const Dual& r, float aniso, float rot, const Mat& m, const V3& n,
                                                const V3& v, const V3& l) {
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
    return dclamp(r * (1.0f - 0.35f * ca * phase), 0.02f, 1.0f);
}

// EvaluateBsdf with derivatives (value identical to bsdf_eval).
static __device__ __noinline__ DV3 bsdf_eval_d(const Mat& m, const V3& n, const V3& cn, const V3& v, const V3& l) {
    const float nv = sclamp(dot(n, v), 0.0f, 1.0f);
    const float nl = sclamp(dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return dv3(V3{0.0f, 0.0f, 0.0f});
    const MatParams p = mat_params(m);
    const DV3 baseF0 = spec_f0_d(m, p);
    const V3 cF0 = coat_f0(m);
    const V3 underCoat = coat_tint(m) * layer_transmittance(cF0, dot(cn, v), dot(cn, l));
    const DV3 underBase = layer_transmittance_d(baseF0, nv, nl);
    const float sigma = sclamp(m.diffuse_roughness, 0.0f, 1.0f);
    const float wrap = sclamp(m.subsurface * m.subsurface_scale *
                                  (0.35f + 0.15f * sclamp(m.subsurface_anisotropy, -1.0f, 1.0f) +
                                   0.1f * sclamp(maxc(ld3(m.subsurface_radius)) / 3.0f, 0.0f, 1.0f)),
                              0.0f, 0.9f);
    const float wrapped = sclamp((nl + wrap) / (1.0f + wrap), 0.0f, 1.0f);
    float term;
    if (sigma == 0.0f) {
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
    const DV3 diffuse = diffuse_color_d(m, p) * underCoat * underBase * (kInvPi * term);
    const Dual baseRough = dclamp(p.rough + m.coat_affect_roughness * m.coat_weight * m.coat_roughness, 0.0f, 1.0f);
    const Dual sr = roughness_for_d(baseRough, m.specular_anisotropy, m.specular_rotation, m, n, v, l);
    DV3 spec = underCoat * spec_lobe_d(n, v, l, baseF0, sr);
    if (m.thin_film_thickness > 0.0f) {
        const V3 h = safe_normalized(v + l, n);
        spec = underCoat * (spec_lobe_d(n, v, l, baseF0, sr) * film_color(m.thin_film_thickness, m.thin_film_ior,
                                                                          sclamp(dot(v, h), 0.0f, 1.0f)));
    }
    const float cr = roughness_for(m.coat_roughness, m.coat_anisotropy, m.coat_rotation, m, cn, v, l);
    const V3 coat = thin_film(spec_lobe(cn, v, l, cF0, cr), m, cn, v, l);
    const float sw = sclamp(m.sheen, 0.0f, 1.0f);
    float sf = 1.0f;
    if (sw != 0.0f) {
        const V3 h = safe_normalized(v + l, n);
        const float lh = sclamp(dot(l, h), 0.0f, 1.0f);
        sf = powf(1.0f - lh, 5.0f) * (1.0f - 0.5f * sclamp(m.sheen_roughness, 0.0f, 1.0f));
    }
    const DV3 sheen = (ld3(m.sheen_color) * sw * sf * underCoat) * underBase;
    return diffuse + spec + dv3(coat) + sheen;
}

}  // namespace shiro_gpu
