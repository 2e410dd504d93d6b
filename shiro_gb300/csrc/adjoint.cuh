// adjoint.cuh - pieces of the differentiable form shared by the
// one-thread-per-path replay (adjoint.cu) and the wavefront replay stages
// (wavefront.cu): the parameter view, the gradient accumulation into
// materials and environment texels, and the clamp scale held constant.
#pragma once

#include "bsdf_diff.cuh"
#include "integrator.cuh"

namespace shiro_gpu {

struct AdjView {
    const Mat* evalMats;  // BSDF values (= scene materials except for frozen renders)
    DevEnv evalEnv;       // dome 0's environment for radiance values
    int32_t env0;         // env index of dome 0, -1 if it has none
    uint32_t materialCount;
    const float* dBeauty;  // 4 per pixel
    float* dBase;          // 3 per material
    float* dRough;
    float* dMetal;
    float4* dEnv4;  // per texel of env0: gradient (rgb, unused), summed into the caller's 3-per-texel array after
    uint32_t distinctEval;  // evalMats differ from the scene's: track the sampling throughput too
    uint32_t targetReq;     // wavefront replay: the wave's request whose paths are replayed
};

__device__ __forceinline__ const DevEnv& env_for_eval(const DevScene& s, const AdjView& a, int32_t env) {
    return env == a.env0 ? a.evalEnv : s.envs[env];
}

// Texels and weights of the bilinear lookup env_evaluate makes for `local`
// (EvaluateLatLong / EvaluateAngular + BilinearSample).
__device__ __forceinline__ int env_footprint(const DevEnv& e, const V3& local, uint32_t idx[4], float wgt[4]) {
    if (e.w == 0 || e.h == 0) return 0;
    const V3 d = normalize(local);
    float u, v;
    if (!e.latlong) {
        const float rl = sqrtf(d.x * d.x + d.y * d.y);
        if (rl <= 1.0e-6f) {
            u = 0.5f;
            v = 0.5f;
        } else {
            const float angle = acosf(sclamp(d.z, -1.0f, 1.0f));
            const float radius = angle / kPi;
            u = 0.5f + 0.5f * radius * (d.x / rl);
            v = 0.5f + 0.5f * radius * (d.y / rl);
            if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f) return 0;
        }
    } else {
        const float phi = atan2f(d.x, d.z);
        const float theta = acosf(sclamp(d.y, -1.0f, 1.0f));
        u = env_wrap(phi / kTwoPi);
        v = sclamp(theta / kPi, 0.0f, 1.0f);
    }
    u = env_wrap(u) * static_cast<float>(e.w) - 0.5f;
    v = sclamp(v, 0.0f, 1.0f) * static_cast<float>(e.h) - 0.5f;
    const int x0 = static_cast<int>(floorf(u));
    const int y0 = static_cast<int>(floorf(v));
    const int x1 = x0 + 1;
    const int y1 = min(y0 + 1, static_cast<int>(e.h) - 1);
    const float tx = u - static_cast<float>(x0);
    const float ty = v - static_cast<float>(y0);
    const int xs[4] = {x0, x1, x0, x1}, ys[4] = {y0, y0, y1, y1};
    const float ws[4] = {(1.0f - tx) * (1.0f - ty), tx * (1.0f - ty), (1.0f - tx) * ty, tx * ty};
    for (int k = 0; k < 4; ++k) {
        int xx = xs[k] % static_cast<int>(e.w);
        if (xx < 0) xx += static_cast<int>(e.w);
        const int yy = ys[k] < 0 ? 0 : (ys[k] > static_cast<int>(e.h) - 1 ? static_cast<int>(e.h) - 1 : ys[k]);
        idx[k] = static_cast<uint32_t>(yy) * e.w + static_cast<uint32_t>(xx);
        wgt[k] = ws[k];
    }
    return 4;
}

// Sums v over the lanes of `active` that hold the same key; the group's
// lowest lane ends with the sum and is the one that returns true.  Each round
// a lane adds the partial sum of the next remaining peer above it, then the
// lanes of odd rank drop out: log2(group size) rounds of shuffles (the peer
// reduction of E. Westphal, "Voting and Shuffling to Optimize Atomic
// Operations", NVIDIA developer blog, 2015).  Every lane of `active` must call
// it with the same N.
template <int N>
__device__ __forceinline__ bool group_sum(uint32_t active, uint32_t key, float (&v)[N]) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t peers = __match_any_sync(active, key);
    const bool leader = static_cast<uint32_t>(__ffs(peers) - 1) == lane;
    uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    peers &= ~((2u << lane) - 1u);  // peers above this lane (none above lane 31)
    while (__any_sync(active, peers != 0u)) {
        const int next = __ffs(peers);
        const int src = next ? next - 1 : static_cast<int>(lane);
#pragma unroll
        for (int p = 0; p < N; ++p) {
            const float t = __shfl_sync(active, v[p], src);
            if (next) v[p] += t;
        }
        peers &= __ballot_sync(active, (rank & 1u) == 0u);
        rank >>= 1;
    }
    return leader;
}

// One vector atomic per texel of the bilinear footprint (16-byte aligned
// float4 accumulators instead of three scalar atomics on the caller's rgb),
// after the lanes that add to the same texel have summed: importance-sampled
// dome samples crowd onto the few brightest texels, and lanes adding to one
// address one after another stalled the whole replay.
__device__ __forceinline__ void add_env_grad(const AdjView& a, const DevEnv& e, const V3& local, const V3& coef) {
    if (!a.dEnv4) return;
    uint32_t idx[4] = {0u, 0u, 0u, 0u};
    float w[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    const int n = (coef.x == 0.0f && coef.y == 0.0f && coef.z == 0.0f) ? 0 : env_footprint(e, local, idx, w);
    const uint32_t active = __activemask();
    for (int k = 0; k < 4; ++k) {
        const uint32_t key = (k < n && w[k] != 0.0f) ? idx[k] : 0xffffffffu;
        float g[3] = {coef.x * w[k], coef.y * w[k], coef.z * w[k]};
        if (group_sum(active, key, g) && key != 0xffffffffu) atomicAdd(&a.dEnv4[key], make_float4(g[0], g[1], g[2], 0.0f));
    }
}

// dL/dparams of material `mat` += sum_c coef_c * df_c (df from the duals).
// The lanes on one material sum first and add once.
__device__ __forceinline__ void add_mat_grad(const AdjView& a, uint32_t mat, const DV3& f, const V3& coef) {
    float g[kDualN];
#pragma unroll
    for (int p = 0; p < kDualN; ++p) g[p] = coef.x * f.x.d[p] + coef.y * f.y.d[p] + coef.z * f.z.d[p];
    const uint32_t key = mat < a.materialCount ? mat : 0xffffffffu;
    if (!group_sum(__activemask(), key, g) || key == 0xffffffffu) return;
    if (a.dBase) {
        for (int c = 0; c < 3; ++c)
            if (g[c] != 0.0f) atomicAdd(&a.dBase[3 * mat + c], g[c]);
    }
    if (a.dRough && g[kDRough] != 0.0f) atomicAdd(&a.dRough[mat], g[kDRough]);
    if (a.dMetal && g[kDMetal] != 0.0f) atomicAdd(&a.dMetal[mat], g[kDMetal]);
}

__device__ __forceinline__ float clamp_scale(const DevRequest& q, const V3& v, float mx) {
    if (q.flags & SHIRO_RENDER_NO_CLAMP) return 1.0f;
    const float c = maxc(v);
    if (c <= mx || c <= 0.0f) return 1.0f;
    return mx / c;
}

// Environment radiance of a miss with dome 0 evaluated from the eval texels.
__device__ __forceinline__ V3 env_radiance_eval(const DevScene& s, const AdjView& a, const V3& dir) {
    if (s.domeCount > 0) {
        V3 r{0.0f, 0.0f, 0.0f};
        for (uint32_t i = 0; i < s.domeCount; ++i) {
            const DevDome& d = s.domes[i];
            r = r + (d.env >= 0 ? env_evaluate(env_for_eval(s, a, d.env), world_to_light(d, dir)) * d.radiance : d.radiance);
        }
        return r;
    }
    const float t = sclamp(dir.y * 0.5f + 0.5f, 0.0f, 1.0f);
    return lerp(s.envBottom, s.envTop, t);
}

}  // namespace shiro_gpu
