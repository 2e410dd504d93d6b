// sampler.cuh - QMC sample generation, bit-exact with the reference.
//
// Shiro's OpenQmcSampler (src/render/OpenQmcSampler.cpp) draws from OpenQMC's
// pmj-bn sampler when built with it and otherwise from its own deterministic
// fallback (:56-71): dimensions 0/1 are the R2 sequence frac(0.5 + a_d * i)
// without per-pixel scrambling; dimension d >= 2 is the radical inverse of
// i + 1 in base prime[d mod 24], rotated (Cranley-Patterson) by a hash of
// (pixel x, pixel y, d).  OpenQMC is not vendored in the reference checkout
// (empty submodule), so the fallback is the bit-exact target here.  Every
// operation below is an integer op or a single IEEE float op in the same order
// as the reference, hence identical results.
#pragma once

#include "common.cuh"

namespace shiro_gpu {

__device__ __forceinline__ uint32_t qmc_scramble(uint32_t s) {  // MixBits, :30-37
    s ^= s >> 16;
    s *= 0x7feb352du;
    s ^= s >> 15;
    s *= 0x846ca68bu;
    s ^= s >> 16;
    return s;
}

// Radical inverse with a compile-time base (division by a constant).
template <uint32_t B>
__device__ __forceinline__ float qmc_radical(uint32_t i) {  // RadicalInverse, :43-54
    const float invBase = 1.0f / static_cast<float>(B);
    float scale = invBase;
    float acc = 0.0f;
    while (i > 0u) {
        const uint32_t q = i / B;
        acc += static_cast<float>(i - q * B) * scale;
        i = q;
        scale *= invBase;
    }
    return acc;
}

static __device__ __noinline__ float qmc_radical_dim(uint32_t dim, uint32_t i) {
    switch (dim % 24u) {
        case 0: return qmc_radical<2>(i);
        case 1: return qmc_radical<3>(i);
        case 2: return qmc_radical<5>(i);
        case 3: return qmc_radical<7>(i);
        case 4: return qmc_radical<11>(i);
        case 5: return qmc_radical<13>(i);
        case 6: return qmc_radical<17>(i);
        case 7: return qmc_radical<19>(i);
        case 8: return qmc_radical<23>(i);
        case 9: return qmc_radical<29>(i);
        case 10: return qmc_radical<31>(i);
        case 11: return qmc_radical<37>(i);
        case 12: return qmc_radical<41>(i);
        case 13: return qmc_radical<43>(i);
        case 14: return qmc_radical<47>(i);
        case 15: return qmc_radical<53>(i);
        case 16: return qmc_radical<59>(i);
        case 17: return qmc_radical<61>(i);
        case 18: return qmc_radical<67>(i);
        case 19: return qmc_radical<71>(i);
        case 20: return qmc_radical<73>(i);
        case 21: return qmc_radical<79>(i);
        case 22: return qmc_radical<83>(i);
        default: return qmc_radical<89>(i);
    }
}

__device__ __forceinline__ float qmc_dim(uint32_t px, uint32_t py, uint32_t index, uint32_t dim) {  // :56-71
    if (dim < 2u) {
        const float step = dim == 0u ? 0.7548776662466927f : 0.5698402909980532f;
        const float v = 0.5f + step * static_cast<float>(index);
        return v - floorf(v);
    }
    const float seq = qmc_radical_dim(dim, index + 1u);
    const uint32_t key = px * 0x8da6b343u ^ py * 0xd8163841u ^ dim * 0xcb1ab31fu ^ 0x9e3779b9u;
    const float rot = static_cast<float>(qmc_scramble(key) & 0x00ffffffu) / 16777216.0f;
    const float v = seq + rot;
    return v - floorf(v);
}

struct Sampler {
    uint32_t px, py, index;
    // OpenQmcSampler::Next2D / Next1D (OpenQmcSampler.cpp:110-135)
    __device__ __forceinline__ V2 next2d(uint32_t branch) const {
        return {qmc_dim(px, py, index, branch * 2u), qmc_dim(px, py, index, branch * 2u + 1u)};
    }
    __device__ __forceinline__ float next1d(uint32_t branch) const { return qmc_dim(px, py, index, branch * 2u); }
};

}  // namespace shiro_gpu
