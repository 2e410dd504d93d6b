// render_plain.cu - the plain GPU form: one thread per path.
//
// CpuPathTracer::RenderSampleBatch (src/backend/cpu/CpuPathTracer.cpp:
// 2043-2170) loops pixels on host threads and samples inside each pixel; here
// every (pixel, sample) path is one CUDA thread running the whole estimator
// (camera ray, traversal, shading, next-event estimation, Russian roulette)
// to completion, and writes a 48-byte record.  A second kernel sums each
// pixel's records in sample order, so the batch average is formed with the
// same additions, in the same order, as the reference.
#include "integrator.cuh"
#include "kernels.h"

namespace shiro_gpu {

namespace {

// Four blocks of 128 per SM (a 128-register cap, a few bytes of spills):
// measured 11 % faster than the 165 registers the compiler otherwise takes.
template <bool kExt>
__global__ void __launch_bounds__(128, 4) k_plain_paths(const DevScene s, const DevRequest q, uint64_t pathBase,
                                                     uint32_t count, float4* __restrict__ records) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint64_t path = pathBase + i;
    const uint64_t pixel = path / q.sampleCount;
    const uint32_t smp = static_cast<uint32_t>(path - pixel * q.sampleCount);
    const uint32_t y = static_cast<uint32_t>(pixel / q.width);
    const uint32_t x = static_cast<uint32_t>(pixel - static_cast<uint64_t>(y) * q.width);
    NullCounter ctr;
    const PathResult r = trace_path<kExt>(s, q, x, y, q.sampleStart + smp, ctr);
    float4* o = records + 3 * static_cast<size_t>(i);
    o[0] = make_float4(r.radiance.x, r.radiance.y, r.radiance.z, r.depth);
    o[1] = make_float4(r.albedo.x, r.albedo.y, r.albedo.z, 0.0f);
    o[2] = make_float4(r.normal.x, r.normal.y, r.normal.z, 0.0f);
}

__global__ void k_resolve(const DevRequest q, uint64_t pixelBase, uint32_t count, const float4* __restrict__ records,
                          AovPtrs aov) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint32_t n = q.sampleCount;
    float b0 = 0.0f, b1 = 0.0f, b2 = 0.0f, b3 = 0.0f;
    V3 alb{0.0f, 0.0f, 0.0f}, nrm{0.0f, 0.0f, 0.0f};
    float depth = __int_as_float(0x7f800000);
    const float4* r = records + 3 * static_cast<size_t>(i) * n;
    for (uint32_t k = 0; k < n; ++k) {
        const float4 a = r[3 * k], b = r[3 * k + 1], c = r[3 * k + 2];
        b0 = b0 + a.x;
        b1 = b1 + a.y;
        b2 = b2 + a.z;
        b3 = b3 + (a.w < __int_as_float(0x7f800000) ? 1.0f : 0.0f);
        alb = alb + V3{b.x, b.y, b.z};
        nrm = nrm + V3{c.x, c.y, c.z};
        if (a.w < depth) depth = a.w;
    }
    const float cnt = static_cast<float>(n);
    const float inv = 1.0f / cnt;
    const size_t p = static_cast<size_t>(pixelBase + i);
    aov.beauty[4 * p + 0] = b0 / cnt;
    aov.beauty[4 * p + 1] = b1 / cnt;
    aov.beauty[4 * p + 2] = b2 / cnt;
    aov.beauty[4 * p + 3] = b3 / cnt;
    const V3 a = alb * inv, nn = nrm * inv;
    aov.albedo[3 * p + 0] = a.x;
    aov.albedo[3 * p + 1] = a.y;
    aov.albedo[3 * p + 2] = a.z;
    aov.normal[3 * p + 0] = nn.x;
    aov.normal[3 * p + 1] = nn.y;
    aov.normal[3 * p + 2] = nn.z;
    aov.depth[p] = depth;
}

__global__ void k_primary_hits(const DevScene s, const DevRequest q, uint32_t* __restrict__ prim, float* __restrict__ tout) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= q.width * q.height) return;
    const uint32_t y = i / q.width, x = i - y * q.width;
    const Sampler smp{x, y, q.sampleStart};
    V3 o, d;
    camera_ray(q, x, y, smp.next2d(0u), &o, &d);
    HitRec h;
    NullCounter ctr;
    const bool hit = trace_closest(s, o, d, &h, ctr);
    prim[i] = hit ? h.gid : 0xffffffffu;
    tout[i] = hit ? h.t : FLT_MAX;
}

__global__ void k_trace_rays(const DevScene s, const float* __restrict__ o, const float* __restrict__ d,
                             const float* __restrict__ tmax, uint32_t n, uint32_t* __restrict__ prim,
                             float* __restrict__ tout, uint32_t* __restrict__ occ) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V3 ro{o[3 * i], o[3 * i + 1], o[3 * i + 2]};
    const V3 rd{d[3 * i], d[3 * i + 1], d[3 * i + 2]};
    HitRec h;
    NullCounter ctr;
    const bool hit = trace_closest(s, ro, rd, &h, ctr);
    prim[i] = hit ? h.gid : 0xffffffffu;
    tout[i] = hit ? h.t : FLT_MAX;
    occ[i] = trace_occluded(s, ro, rd, tmax[i], ctr) ? 1u : 0u;
}

// Work-counting variant: every `stride`-th path of the request, same
// decisions as k_plain_paths; totals accumulated with one atomic per field
// per warp.
__global__ void __launch_bounds__(128) k_count_paths(const DevScene s, const DevRequest q, uint64_t totalPaths,
                                                     uint32_t stride, unsigned long long* __restrict__ totals) {
    const uint64_t i = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint64_t path = i * stride;
    LocalCounter c;
    uint32_t traced = 0;
    if (path < totalPaths) {
        const uint64_t pixel = path / q.sampleCount;
        const uint32_t smp = static_cast<uint32_t>(path - pixel * q.sampleCount);
        const uint32_t y = static_cast<uint32_t>(pixel / q.width);
        const uint32_t x = static_cast<uint32_t>(pixel - static_cast<uint64_t>(y) * q.width);
        trace_path<true>(s, q, x, y, q.sampleStart + smp, c);
        traced = 1;
    }
    const uint32_t v[12] = {traced,  c.closestRays, c.occlusionRays, c.nodes + c.onodes, c.tris + c.otris, c.hits,
                            c.envEvals, c.envSamples, c.bsdfEvals, c.bsdfPdfs, c.onodes, c.otris};
    for (int k = 0; k < 12; ++k) {
        unsigned long long x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(&totals[k], x);
    }
}

// The sampler of the kernels on explicit tuples (diagnostic).
__global__ void k_sample_probe(const uint4* __restrict__ tuples, uint32_t n, float* __restrict__ out) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint4 t = tuples[k];
    const V2 v = Sampler{t.x, t.y, t.z}.next2d(t.w);
    out[2 * static_cast<size_t>(k)] = v.x;
    out[2 * static_cast<size_t>(k) + 1] = v.y;
}

// Listed paths of the plain form (diagnostic): out[10 i ..] = radiance,
// albedo, normal, depth of path (pixels[i], sample index sampleIdx[i]).
template <bool kExt>
__global__ void __launch_bounds__(128) k_render_paths(const DevScene s, const DevRequest q, const uint32_t* __restrict__ pixels,
                                                      const uint32_t* __restrict__ sampleIdx, uint32_t n,
                                                      float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t y = pixels[i] / q.width, x = pixels[i] - y * q.width;
    NullCounter ctr;
    const PathResult r = trace_path<kExt>(s, q, x, y, sampleIdx[i], ctr);
    float* o = out + 10 * static_cast<size_t>(i);
    o[0] = r.radiance.x;
    o[1] = r.radiance.y;
    o[2] = r.radiance.z;
    o[3] = r.albedo.x;
    o[4] = r.albedo.y;
    o[5] = r.albedo.z;
    o[6] = r.normal.x;
    o[7] = r.normal.y;
    o[8] = r.normal.z;
    o[9] = r.depth;
}

// Texel picks of a dome texture for explicit 2-D points (diagnostic).
__global__ void k_env_pick(const DevEnv e, const float2* __restrict__ u, uint32_t n, uint32_t useCdf,
                           uint32_t* __restrict__ texel, float* __restrict__ pdf) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 v = u[i];
    const size_t t = env_pick(e, V2{v.x, v.y}, useCdf != 0u);
    texel[i] = static_cast<uint32_t>(t);
    pdf[i] = e.samples[2 * t].w;
}

inline unsigned grid(uint64_t n, unsigned b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace

void launch_sample_probe(const uint4* tuples, uint32_t n, float* out, cudaStream_t stream) {
    if (n == 0) return;
    k_sample_probe<<<grid(n, 256), 256, 0, stream>>>(tuples, n, out);
}

void launch_plain_paths(const DevScene& s, const DevRequest& q, uint64_t pathBase, uint32_t count, float4* records,
                        cudaStream_t stream) {
    if (count == 0) return;
    if (s.extended)
        k_plain_paths<true><<<grid(count, 128), 128, 0, stream>>>(s, q, pathBase, count, records);
    else
        k_plain_paths<false><<<grid(count, 128), 128, 0, stream>>>(s, q, pathBase, count, records);
}

void launch_render_paths(const DevScene& s, const DevRequest& q, const uint32_t* pixels, const uint32_t* sampleIdx,
                         uint32_t n, float* out, cudaStream_t stream) {
    if (n == 0) return;
    if (s.extended)
        k_render_paths<true><<<grid(n, 128), 128, 0, stream>>>(s, q, pixels, sampleIdx, n, out);
    else
        k_render_paths<false><<<grid(n, 128), 128, 0, stream>>>(s, q, pixels, sampleIdx, n, out);
}

void launch_env_pick(const DevEnv& e, const float2* u, uint32_t n, bool useCdf, uint32_t* texel, float* pdf,
                     cudaStream_t stream) {
    if (n == 0) return;
    k_env_pick<<<grid(n, 256), 256, 0, stream>>>(e, u, n, useCdf ? 1u : 0u, texel, pdf);
}

cudaError_t preload_plain_kernels() {
    cudaFuncAttributes a;
    cudaError_t e = cudaFuncGetAttributes(&a, k_plain_paths<false>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_plain_paths<true>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_resolve);
    return e;
}

void launch_resolve_pixels(const DevRequest& q, uint64_t pixelBase, uint32_t count, const float4* records, AovPtrs aov,
                           cudaStream_t stream) {
    if (count == 0) return;
    k_resolve<<<grid(count, 128), 128, 0, stream>>>(q, pixelBase, count, records, aov);
}

void launch_primary_hits(const DevScene& s, const DevRequest& q, uint32_t* prim, float* t, cudaStream_t stream) {
    const uint64_t n = static_cast<uint64_t>(q.width) * q.height;
    if (n == 0) return;
    k_primary_hits<<<grid(n, 128), 128, 0, stream>>>(s, q, prim, t);
}

void launch_count_paths(const DevScene& s, const DevRequest& q, uint32_t stride, unsigned long long* totals,
                        cudaStream_t stream) {
    const uint64_t total = static_cast<uint64_t>(q.width) * q.height * q.sampleCount;
    const uint64_t n = (total + stride - 1) / stride;
    if (n == 0) return;
    k_count_paths<<<grid(n, 128), 128, 0, stream>>>(s, q, total, stride, totals);
}

void launch_trace_rays(const DevScene& s, const float* o, const float* d, const float* tmax, uint32_t n, uint32_t* prim,
                       float* t, uint32_t* occ, cudaStream_t stream) {
    if (n == 0) return;
    k_trace_rays<<<grid(n, 128), 128, 0, stream>>>(s, o, d, tmax, n, prim, t, occ);
}

}  // namespace shiro_gpu
