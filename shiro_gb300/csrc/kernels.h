// kernels.h - host-side launchers of the render kernels.
#pragma once

#include <cuda_runtime.h>

#include "scene.cuh"

namespace shiro_gpu {

// Per-path result in the scratch buffer: 3 x float4 =
// (radiance rgb, depth), (albedo rgb, 0), (normal rgb, 0).
constexpr size_t kPathRecordBytes = 3 * sizeof(float4);

struct AovPtrs {
    float* beauty;  // 4 floats per pixel
    float* albedo;  // 3
    float* normal;  // 3
    float* depth;   // 1
};

// One thread per path: paths [pathBase, pathBase + count) of the request,
// path p = pixel * sampleCount + s (sample index sampleStart + s).
void launch_plain_paths(const DevScene& s, const DevRequest& q, uint64_t pathBase, uint32_t count, float4* records,
                        cudaStream_t stream);
// One thread per pixel of [pixelBase, pixelBase + count): averages the
// pixel's sampleCount records in sample order into the AOV planes
// (CpuPathTracer.cpp:2093-2137).
void launch_resolve_pixels(const DevRequest& q, uint64_t pixelBase, uint32_t count, const float4* records, AovPtrs aov,
                           cudaStream_t stream);
// Diagnostics: listed paths of the plain form (10 floats each: radiance,
// albedo, normal, depth), and the texel a dome texture's sampler picks for
// explicit 2-D points (with its pdf).
void launch_render_paths(const DevScene& s, const DevRequest& q, const uint32_t* pixels, const uint32_t* sampleIdx,
                         uint32_t n, float* out, cudaStream_t stream);
void launch_env_pick(const DevEnv& e, const float2* u, uint32_t n, bool useCdf, uint32_t* texel, float* pdf,
                     cudaStream_t stream);
// Loads the plain-form kernels (both k_plain_paths variants and k_resolve)
// into the current device's context now: under CUDA's lazy module loading a
// kernel's code is otherwise placed in device memory at its first launch.
cudaError_t preload_plain_kernels();
// out[2k], out[2k+1] = Sampler{px, py, index}.next2d(branch) of tuple k
// (tuples packed as uint4 px, py, index, branch).
void launch_sample_probe(const uint4* tuples, uint32_t n, float* out, cudaStream_t stream);
void launch_primary_hits(const DevScene& s, const DevRequest& q, uint32_t* prim, float* t, cudaStream_t stream);
// Work counts of every stride-th path (12 totals, see ShiroWorkCounts).
void launch_count_paths(const DevScene& s, const DevRequest& q, uint32_t stride, unsigned long long* totals,
                        cudaStream_t stream);
void launch_trace_rays(const DevScene& s, const float* o, const float* d, const float* tmax, uint32_t n, uint32_t* prim,
                       float* t, uint32_t* occ, cudaStream_t stream);

}  // namespace shiro_gpu
