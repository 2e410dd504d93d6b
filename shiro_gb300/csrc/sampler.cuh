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

// RadicalInverse (:43-54) in base prime[dim mod 24]: digits d = i mod B
// summed as acc += float(d) * scale, scale *= 1 / B, in the reference's
// order.  One loop for every base: the quotient i / B comes from a
// multiply-high by a per-base constant (Granlund & Montgomery 1994, unsigned
// division by invariant integers, Fig. 4.1: m = floor(2^32 (2^l - B) / B) + 1,
// l = ceil(log2 B); q = (t + ((i - t) >> 1)) >> (l - 1), t = mulhi(m, i)),
// exact for every 32-bit i; 1 / B is the IEEE float quotient the reference
// forms.  (One small body instead of 24 specialised loops behind a jump
// table keeps the samplers' code compact in the instruction cache.)
static __constant__ uint32_t kQmcPrime[24] = {
    2u, 3u, 5u, 7u, 11u, 13u, 17u, 19u, 23u, 29u, 31u, 37u,
    41u, 43u, 47u, 53u, 59u, 61u, 67u, 71u, 73u, 79u, 83u, 89u,
};
static __constant__ uint32_t kQmcMagic[24] = {
    0x00000001u, 0x55555556u, 0x9999999au, 0x24924925u, 0x745d1746u, 0x3b13b13cu,
    0xe1e1e1e2u, 0xaf286bcbu, 0x642c8591u, 0x1a7b9612u, 0x08421085u, 0xbacf914du,
    0x8f9c18fau, 0x7d05f418u, 0x5c9882bau, 0x3521cfb3u, 0x15b1e5f8u, 0x0c9714fcu,
    0xe9131ac0u, 0xcd856891u, 0xc0e07039u, 0x9ec8e952u, 0x8acb90f7u, 0x702e05c1u,
};
static __constant__ uint32_t kQmcShift[24] = {
    0u, 1u, 2u, 2u, 3u, 3u, 4u, 4u, 4u, 4u, 4u, 5u,
    5u, 5u, 5u, 5u, 5u, 5u, 6u, 6u, 6u, 6u, 6u, 6u,
};
static __constant__ uint32_t kQmcInvBase[24] = {  // float bits of 1.0f / prime
    0x3f000000u, 0x3eaaaaabu, 0x3e4ccccdu, 0x3e124925u, 0x3dba2e8cu, 0x3d9d89d9u,
    0x3d70f0f1u, 0x3d579436u, 0x3d321643u, 0x3d0d3dcbu, 0x3d042108u, 0x3cdd67c9u,
    0x3cc7ce0cu, 0x3cbe82fau, 0x3cae4c41u, 0x3c9a90e8u, 0x3c8ad8f3u, 0x3c864b8au,
    0x3c74898du, 0x3c66c2b4u, 0x3c607038u, 0x3c4f6475u, 0x3c4565c8u, 0x3c381703u,
};

static __device__ __noinline__ float qmc_radical_dim(uint32_t dim, uint32_t i) {
    const uint32_t k = dim % 24u;
    const uint32_t base = kQmcPrime[k], magic = kQmcMagic[k], shift = kQmcShift[k];
    const float invBase = __uint_as_float(kQmcInvBase[k]);
    float scale = invBase;
    float acc = 0.0f;
    while (i > 0u) {
        const uint32_t t = __umulhi(magic, i);
        const uint32_t q = (t + ((i - t) >> 1)) >> shift;
        acc += static_cast<float>(i - q * base) * scale;
        i = q;
        scale *= invBase;
    }
    return acc;
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
