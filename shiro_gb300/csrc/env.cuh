// env.cuh - dome light: environment evaluation, pdf and importance sampling.
//
// Follows src/render/EnvironmentMap.cpp (Evaluate :94-107, Sample :109-163,
// Pdf :165-183, EvaluateLatLong :238-245, EvaluateAngular :247-264,
// BilinearSample :266-300, LatLongPdf :302-313, SampleCdf :315-330) and the
// dome-light helpers of src/backend/cpu/CpuPathTracer.cpp:315-384.
//
// Two samplers pick the same texel distribution (probability rowMass *
// columnMass per texel, the reference's discrete pdf):
//   * CDF mode: binary search over the row and conditional CDFs exactly as
//     SampleCdf does, so a given 2-D sample selects the reference's texel;
//   * alias mode (default): one O(1) lookup in a Walker/Vose alias table
//     built from the same texel masses.
// Both map the texel to its centre direction and report the reference's pdf.
#pragma once

#include "common.cuh"
#include "scene.cuh"

namespace shiro_gpu {

__device__ __forceinline__ float env_wrap(float v) {  // WrapUnit, :23-26
    v = fmodf(v, 1.0f);
    return v < 0.0f ? v + 1.0f : v;
}

__device__ __forceinline__ V3 env_texel(const DevEnv& e, int x, int y) {
    int xx = x % static_cast<int>(e.w);
    if (xx < 0) xx += static_cast<int>(e.w);
    const int yy = y < 0 ? 0 : (y > static_cast<int>(e.h) - 1 ? static_cast<int>(e.h) - 1 : y);
    const float4 t = __ldg(&e.texels[static_cast<size_t>(yy) * e.w + static_cast<size_t>(xx)]);
    return {t.x, t.y, t.z};
}

__device__ __forceinline__ V3 env_bilinear(const DevEnv& e, float u, float v) {  // :266-300
    if (e.w == 0 || e.h == 0) return {0.0f, 0.0f, 0.0f};
    u = env_wrap(u) * static_cast<float>(e.w) - 0.5f;
    v = sclamp(v, 0.0f, 1.0f) * static_cast<float>(e.h) - 0.5f;
    const int x0 = static_cast<int>(floorf(u));
    const int y0 = static_cast<int>(floorf(v));
    const int x1 = x0 + 1;
    const int y1 = min(y0 + 1, static_cast<int>(e.h) - 1);
    const float tx = u - static_cast<float>(x0);
    const float ty = v - static_cast<float>(y0);
    const V3 c0 = lerp(env_texel(e, x0, y0), env_texel(e, x1, y0), tx);
    const V3 c1 = lerp(env_texel(e, x0, y1), env_texel(e, x1, y1), tx);
    return lerp(c0, c1, ty);
}

__device__ __forceinline__ V3 env_evaluate(const DevEnv& e, const V3& local) {  // :94-107, 238-264
    if (e.w == 0 || e.h == 0) return {0.0f, 0.0f, 0.0f};
    const V3 d = normalize(local);
    if (!e.latlong) {
        const float rl = sqrtf(d.x * d.x + d.y * d.y);
        if (rl <= 1.0e-6f) return env_bilinear(e, 0.5f, 0.5f);
        const float angle = acosf(sclamp(d.z, -1.0f, 1.0f));
        const float radius = angle / kPi;
        const float nx = d.x / rl;
        const float ny = d.y / rl;
        const float u = 0.5f + 0.5f * radius * nx;
        const float v = 0.5f + 0.5f * radius * ny;
        if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f) return {0.0f, 0.0f, 0.0f};
        return env_bilinear(e, u, v);
    }
    const float phi = atan2f(d.x, d.z);
    const float theta = acosf(sclamp(d.y, -1.0f, 1.0f));
    return env_bilinear(e, env_wrap(phi / kTwoPi), sclamp(theta / kPi, 0.0f, 1.0f));
}

// Lat-long angles of a local direction (EvaluateLatLong :238-245 and
// LatLongPdf :302-313 form them the same way).
struct EnvAngles {
    float phi, theta;
};
__device__ __forceinline__ EnvAngles env_angles(const V3& local) {
    const V3 d = normalize(local);
    return {atan2f(d.x, d.z), acosf(sclamp(d.y, -1.0f, 1.0f))};
}

// LatLongPdf (:302-313) from the angles.
__device__ __forceinline__ float env_latlong_pdf(const DevEnv& e, const EnvAngles& a) {
    const float u = env_wrap(a.phi / kTwoPi);
    const float v = sclamp(a.theta / kPi, 0.0f, 1.0f);
    const uint32_t x = ::min(static_cast<uint32_t>(u * static_cast<float>(e.w)), e.w - 1u);
    const uint32_t y = ::min(static_cast<uint32_t>(v * static_cast<float>(e.h)), e.h - 1u);
    const float sinT = sinf(a.theta);
    if (sinT <= 1.0e-6f) return 0.0f;
    const float mass = __ldg(&e.texels[static_cast<size_t>(y) * e.w + x]).w;
    return mass * static_cast<float>(e.w * e.h) / (2.0f * kPi * kPi * sinT);
}

__device__ __forceinline__ float env_pdf(const DevEnv& e, const V3& local) {  // :165-183, 302-313
    if (e.w == 0 || e.h == 0) return 0.0f;
    if (!e.latlong || !e.hasTable) return kInvFourPi;
    return env_latlong_pdf(e, env_angles(local));
}

// Radiance and (when wantPdf) pdf of one direction with the angles formed
// once: the miss of a path needs both.
__device__ __forceinline__ V3 env_evaluate_pdf(const DevEnv& e, const V3& local, bool wantPdf, float* pdf) {
    if (e.w == 0 || e.h == 0) {
        *pdf = 0.0f;
        return {0.0f, 0.0f, 0.0f};
    }
    if (!e.latlong) {
        *pdf = kInvFourPi;
        return env_evaluate(e, local);
    }
    const EnvAngles a = env_angles(local);
    *pdf = !wantPdf ? 0.0f : (e.hasTable ? env_latlong_pdf(e, a) : kInvFourPi);
    return env_bilinear(e, env_wrap(a.phi / kTwoPi), sclamp(a.theta / kPi, 0.0f, 1.0f));
}

// Sampling texel (row, col) of a lat-long map (EnvironmentMap::Sample
// :137-162): its centre direction, the reference's pdf, the radiance there.
// Evaluated once per texel when the tables are built (k_env_samples).
__device__ __forceinline__ V3 env_centre_sample(const DevEnv& e, uint32_t row, uint32_t col, float mass, V3* dir,
                                                float* pdf) {
    const float uu = (static_cast<float>(col) + 0.5f) / static_cast<float>(e.w);
    const float vv = (static_cast<float>(row) + 0.5f) / static_cast<float>(e.h);
    const float theta = vv * kPi;
    const float phi = uu * kTwoPi;
    const float sinT = sinf(theta);
    const V3 d{sinf(phi) * sinT, cosf(theta), cosf(phi) * sinT};
    *dir = d;
    *pdf = sinT > 1.0e-6f ? mass * static_cast<float>(e.w * e.h) / (2.0f * kPi * kPi * sinT) : 0.0f;
    return env_evaluate(e, d);
}

// lower_bound over cdf[begin+1 .. end] (SampleCdf, :315-330); returns the
// absolute index `idx` with cdf[idx] < key <= cdf[idx + 1].
__device__ __forceinline__ uint32_t env_cdf_search(const float* cdf, uint32_t begin, uint32_t end, float s) {
    const float key = sclamp(s, 0.0f, 0.99999994f);
    uint32_t lo = begin + 1u, count = end - begin;
    while (count > 0u) {
        const uint32_t step = count >> 1;
        const uint32_t it = lo + step;
        if (__ldg(&cdf[it]) < key) {
            lo = it + 1u;
            count -= step + 1u;
        } else {
            count = step;
        }
    }
    return lo - 1u;
}

// The texel a 2-D sample picks in a lat-long map with an importance table:
// the CDF search of SampleCdf (row on u.y, column on u.x), or the alias
// lookup (bucket floor(u.y * n) - exact for a power-of-two n, as u.y * n then
// only shifts the exponent - accepted when u.x is below its threshold, else
// its alias).
__device__ __forceinline__ size_t env_pick(const DevEnv& e, const V2& u, bool useCdf) {
    if (useCdf) {
        const uint32_t r = env_cdf_search(e.rowCdf, 0u, e.h, u.y);
        const uint32_t off = r * (e.w + 1u);
        const uint32_t c = env_cdf_search(e.condCdf, off, off + e.w, u.x);
        return static_cast<size_t>(r) * e.w + (c - off);
    }
    const uint32_t n = e.w * e.h;
    uint32_t i = static_cast<uint32_t>(u.y * static_cast<float>(n));
    i = i >= n ? n - 1u : i;
    const uint2 a = __ldg(&e.alias[i]);
    return u.x < __uint_as_float(a.x) ? i : a.y;
}

// EnvironmentMap::Sample (:109-163).  Returns the radiance; *pdf = 0 marks
// a failed sample.
__device__ __forceinline__ V3 env_sample(const DevEnv& e, const V2& u, bool useCdf, V3* dir, float* pdf) {
    if (e.w == 0 || e.h == 0) {
        *dir = {0.0f, 1.0f, 0.0f};
        *pdf = 0.0f;
        return {0.0f, 0.0f, 0.0f};
    }
    if (e.latlong && e.hasTable) {
        // the texel; its centre direction, pdf (mass rowMass * columnMass)
        // and radiance come from the per-texel sample records
        const size_t t = env_pick(e, u, useCdf);
        const float4 a = __ldg(&e.samples[2 * t]), b = __ldg(&e.samples[2 * t + 1]);
        *dir = V3{a.x, a.y, a.z};
        *pdf = a.w;
        return {b.x, b.y, b.z};
    }
    const float y = 1.0f - 2.0f * u.y;
    const float r = sqrtf(smax(0.0f, 1.0f - y * y));
    const float phi = kTwoPi * u.x;
    const V3 d{sinf(phi) * r, y, cosf(phi) * r};
    *dir = d;
    *pdf = kInvFourPi;
    return env_evaluate(e, d);
}

// ---- dome light helpers (CpuPathTracer.cpp:315-384) -----------------------
__device__ __forceinline__ V3 world_to_light(const DevDome& d, const V3& v) {
    return normalize(V3{dot(v, d.right), dot(v, d.up), dot(v, d.forward)});
}
__device__ __forceinline__ V3 light_to_world(const DevDome& d, const V3& v) {
    return normalize(d.right * v.x + d.up * v.y + d.forward * v.z);
}

__device__ __forceinline__ V3 dome_radiance(const DevScene& s, const DevDome& d, const V3& dir) {
    if (d.env >= 0) return env_evaluate(s.envs[d.env], world_to_light(d, dir)) * d.radiance;
    return d.radiance;
}

// EnvironmentRadiance (:334-345)
__device__ __forceinline__ V3 environment_radiance(const DevScene& s, const V3& dir) {
    if (s.domeCount > 0) {
        V3 r{0.0f, 0.0f, 0.0f};
        for (uint32_t i = 0; i < s.domeCount; ++i) r = r + dome_radiance(s, s.domes[i], dir);
        return r;
    }
    const float t = sclamp(dir.y * 0.5f + 0.5f, 0.0f, 1.0f);
    return lerp(s.envBottom, s.envTop, t);
}

__device__ __forceinline__ float dome_pdf(const DevScene& s, const DevDome& d, const V3& dir) {  // :347-352
    if (d.env >= 0) return env_pdf(s.envs[d.env], world_to_light(d, dir));
    return kInvFourPi;
}

// SampleDomeLight (:354-384)
__device__ __forceinline__ bool sample_dome(const DevScene& s, const DevDome& d, const V2& u, bool useCdf, V3* dir,
                                            V3* rad, float* pdf) {
    V3 ld;
    float lp;
    V3 lr;
    if (d.env >= 0) {
        lr = env_sample(s.envs[d.env], u, useCdf, &ld, &lp);
    } else {
        const float y = 1.0f - 2.0f * u.y;
        const float r = sqrtf(smax(0.0f, 1.0f - y * y));
        const float phi = 2.0f * kPi * u.x;
        ld = V3{sinf(phi) * r, y, cosf(phi) * r};
        lp = kInvFourPi;
        lr = V3{1.0f, 1.0f, 1.0f};
    }
    if (lp <= 0.0f) return false;
    *dir = light_to_world(d, ld);
    *rad = lr * d.radiance;
    *pdf = lp;
    return true;
}

}  // namespace shiro_gpu
