// accumulate.cu - device-resident progressive accumulation: the running sums
// of Renderer::FrameAccumulator (src/render/Renderer.cpp:47-110) kept in
// device memory, so that a progressive render folds every batch in where it
// was rendered and copies a resolved frame out only on request.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <limits>

#include "context.h"

struct ShiroAccumulator {
    ShiroGpuContext* ctx = nullptr;
    int device = 0;                     // the context's device (destroy needs nothing of the context)
    uint32_t width = 0, height = 0;
    uint32_t samples = 0;               // FrameAccumulator::sampleCount_
    shiro_gpu::DeviceBlock sums;        // beauty 4n, albedo 3n, normal 3n, depth sum n (float), depth samples n (u32)
    shiro_gpu::DeviceBlock frame;       // 11n floats: a batch rendered on the device, or a staged host frame
    bool pending = false;               // frame holds a rendered batch not yet folded in
    uint32_t pendingWidth = 0, pendingHeight = 0, pendingStart = 0, pendingCount = 0;
};

namespace shiro_gpu {
namespace {

constexpr uint32_t kAccumBlock = 256;

struct SumPlanes {
    float* beauty;
    float* albedo;
    float* normal;
    float* depthSum;
    uint32_t* depthSamples;
};

SumPlanes sum_planes(ShiroAccumulator* a) {
    const size_t n = static_cast<size_t>(a->width) * a->height;
    float* f = static_cast<float*>(a->sums.ptr);
    return SumPlanes{f, f + 4 * n, f + 7 * n, f + 10 * n, reinterpret_cast<uint32_t*>(f + 11 * n)};
}

AovPtrs frame_planes(ShiroAccumulator* a, size_t n) {
    float* f = static_cast<float*>(a->frame.ptr);
    return AovPtrs{f, f + 4 * n, f + 7 * n, f + 10 * n};
}

int grid_of(size_t n) {
    return static_cast<int>(std::min<size_t>((n + kAccumBlock - 1) / kAccumBlock, 152 * 16));
}

// Accumulate (Renderer.cpp:72-81): sum + frame * weight per component; the
// depth of a pixel that saw a hit adds depth * weight and its sample count.
__global__ void __launch_bounds__(kAccumBlock) k_accum_add(size_t n, const float* __restrict__ beauty,
                                                           const float* __restrict__ albedo,
                                                           const float* __restrict__ normal,
                                                           const float* __restrict__ depth, float weight,
                                                           uint32_t count, SumPlanes s) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        for (int c = 0; c < 4; ++c) s.beauty[4 * i + c] = s.beauty[4 * i + c] + beauty[4 * i + c] * weight;
        for (int c = 0; c < 3; ++c) {
            s.albedo[3 * i + c] = s.albedo[3 * i + c] + albedo[3 * i + c] * weight;
            s.normal[3 * i + c] = s.normal[3 * i + c] + normal[3 * i + c] * weight;
        }
        const float d = depth[i];
        if (d < __int_as_float(0x7f800000)) {
            s.depthSum[i] += d * weight;
            s.depthSamples[i] += count;
        }
    }
}

// Resolve (Renderer.cpp:94-107): sums times 1 / total samples; depth averaged
// over the samples that hit, +inf where none did.
__global__ void __launch_bounds__(kAccumBlock) k_accum_resolve(size_t n, float inv, SumPlanes s, AovPtrs o) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        for (int c = 0; c < 4; ++c) o.beauty[4 * i + c] = s.beauty[4 * i + c] * inv;
        for (int c = 0; c < 3; ++c) {
            o.albedo[3 * i + c] = s.albedo[3 * i + c] * inv;
            o.normal[3 * i + c] = s.normal[3 * i + c] * inv;
        }
        const uint32_t k = s.depthSamples[i];
        o.depth[i] = k > 0u ? s.depthSum[i] / static_cast<float>(k) : __int_as_float(0x7f800000);
    }
}

// FrameBuffer::Resize (FrameBuffer.cpp:8-17): zeros, depth +inf.
__global__ void __launch_bounds__(kAccumBlock) k_accum_clear(size_t n, AovPtrs o) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        for (int c = 0; c < 4; ++c) o.beauty[4 * i + c] = 0.0f;
        for (int c = 0; c < 3; ++c) o.albedo[3 * i + c] = o.normal[3 * i + c] = 0.0f;
        o.depth[i] = __int_as_float(0x7f800000);
    }
}

int accum_reset(ShiroAccumulator* a, uint32_t width, uint32_t height) {
    ContextImpl* ctx = &a->ctx->impl;
    const size_t n = static_cast<size_t>(width) * height;
    a->width = width;
    a->height = height;
    a->samples = 0;
    if (n == 0) return SHIRO_OK;
    if (!ensure_block(ctx, &a->sums, n * 12 * sizeof(float), "accumulator sums")) return SHIRO_ERR_OUT_OF_MEMORY;
    const cudaError_t e = cudaMemsetAsync(a->sums.ptr, 0, n * 12 * sizeof(float), ctx->stream);
    return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "accumulator reset");
}

// Folds device planes of a width x height frame into the sums.
int accum_add_device(ShiroAccumulator* a, const AovPtrs& f, uint32_t width, uint32_t height, uint32_t count) {
    ContextImpl* ctx = &a->ctx->impl;
    if (width == 0 || height == 0 || count == 0) return SHIRO_OK;
    if (width != a->width || height != a->height) {
        const int rc = accum_reset(a, width, height);
        if (rc != SHIRO_OK) return rc;
    }
    const size_t n = static_cast<size_t>(width) * height;
    k_accum_add<<<grid_of(n), kAccumBlock, 0, ctx->stream>>>(n, f.beauty, f.albedo, f.normal, f.depth,
                                                               static_cast<float>(count), count, sum_planes(a));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "accumulate");
    a->samples += count;
    return SHIRO_OK;
}

}  // namespace
}  // namespace shiro_gpu

using namespace shiro_gpu;

extern "C" {

int shiro_gpu_accum_create(ShiroGpuContext* ctx, ShiroAccumulator** out) {
    if (!ctx || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    *out = new ShiroAccumulator();
    (*out)->ctx = ctx;
    (*out)->device = ctx->impl.device;
    return SHIRO_OK;
}

void shiro_gpu_accum_destroy(ShiroAccumulator* a) {
    if (!a) return;
    cudaSetDevice(a->device);  // cudaFree waits for the work in flight on the blocks
    if (a->sums.ptr) cudaFree(a->sums.ptr);
    if (a->frame.ptr) cudaFree(a->frame.ptr);
    delete a;
}

int shiro_gpu_accum_reset(ShiroAccumulator* a, uint32_t width, uint32_t height) {
    if (!a) return SHIRO_ERR_INVALID_ARGUMENT;
    cudaSetDevice(a->ctx->impl.device);
    return accum_reset(a, width, height);
}

int shiro_gpu_accum_add(ShiroAccumulator* a, const ShiroAovs* frame, uint32_t width, uint32_t height,
                        uint32_t sample_count) {
    if (!a || !frame) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &a->ctx->impl;
    cudaSetDevice(ctx->device);
    if (width == 0 || height == 0 || sample_count == 0) return SHIRO_OK;
    if (!frame->beauty || !frame->albedo || !frame->normal || !frame->depth)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "null AOV pointer");
    const size_t n = static_cast<size_t>(width) * height;
    if (frame->on_device)
        return accum_add_device(a, AovPtrs{frame->beauty, frame->albedo, frame->normal, frame->depth}, width, height,
                                sample_count);
    a->pending = false;  // the staging planes are the pending frame's
    if (!ensure_block(ctx, &a->frame, n * 11 * sizeof(float), "accumulator frame")) return SHIRO_ERR_OUT_OF_MEMORY;
    const AovPtrs f = frame_planes(a, n);
    const float* src[4] = {frame->beauty, frame->albedo, frame->normal, frame->depth};
    float* dst[4] = {f.beauty, f.albedo, f.normal, f.depth};
    const size_t comps[4] = {4, 3, 3, 1};
    for (int k = 0; k < 4; ++k) {
        const cudaError_t e =
            cudaMemcpyAsync(dst[k], src[k], n * comps[k] * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "accumulator frame upload");
    }
    const int rc = accum_add_device(a, f, width, height, sample_count);
    if (rc != SHIRO_OK) return rc;
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);  // the host planes may be reused on return
    return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "accumulate");
}

int shiro_gpu_accum_stage(ShiroAccumulator* a, const ShiroRenderDesc* req, const volatile int* cancel,
                          uint32_t wavefront) {
    if (!a || !req) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &a->ctx->impl;
    cudaSetDevice(ctx->device);
    a->pending = false;
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    const uint32_t w = req->settings.width, h = req->settings.height;
    const size_t n = static_cast<size_t>(w) * h;
    if (!ensure_block(ctx, &a->frame, std::max<size_t>(n, 1) * 11 * sizeof(float), "accumulator frame"))
        return SHIRO_ERR_OUT_OF_MEMORY;
    if (req->sample_count > 0) {  // the worker renders nothing for an empty batch
        const AovPtrs f = frame_planes(a, n);
        ShiroAovs dev{f.beauty, f.albedo, f.normal, f.depth, 1u, 0u};
        rc = wavefront ? shiro_gpu_render_batch(a->ctx, req, 1, cancel, &dev)
                       : shiro_gpu_render(a->ctx, req, cancel, &dev);
        if (rc != SHIRO_OK) return rc;
    }
    a->pending = true;
    a->pendingWidth = w;
    a->pendingHeight = h;
    a->pendingStart = req->sample_start;
    a->pendingCount = req->sample_count;
    return SHIRO_OK;
}

int shiro_gpu_accum_commit(ShiroAccumulator* a) {
    if (!a) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &a->ctx->impl;
    cudaSetDevice(ctx->device);
    if (!a->pending) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "no pending batch to commit");
    a->pending = false;
    if (a->pendingCount == 0) return SHIRO_OK;
    // RenderParam.cpp:800-805: a batch at sample 0 (or onto empty sums)
    // starts a new accumulation
    if (a->pendingStart == 0 || a->samples == 0) {
        const int rc = accum_reset(a, a->pendingWidth, a->pendingHeight);
        if (rc != SHIRO_OK) return rc;
    }
    const size_t n = static_cast<size_t>(a->pendingWidth) * a->pendingHeight;
    return accum_add_device(a, frame_planes(a, n), a->pendingWidth, a->pendingHeight, a->pendingCount);
}

int shiro_gpu_accum_render(ShiroAccumulator* a, const ShiroRenderDesc* req, const volatile int* cancel,
                           uint32_t wavefront) {
    const int rc = shiro_gpu_accum_stage(a, req, cancel, wavefront);
    return rc != SHIRO_OK ? rc : shiro_gpu_accum_commit(a);
}

int shiro_gpu_accum_resolve(ShiroAccumulator* a, ShiroAovs* out) {
    if (!a || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &a->ctx->impl;
    cudaSetDevice(ctx->device);
    const size_t n = static_cast<size_t>(a->width) * a->height;
    if (n == 0) return SHIRO_OK;
    if (!out->beauty || !out->albedo || !out->normal || !out->depth)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "null AOV pointer");
    AovPtrs o{out->beauty, out->albedo, out->normal, out->depth};
    if (!out->on_device) {
        a->pending = false;  // the staging planes are the pending frame's
        if (!ensure_block(ctx, &a->frame, n * 11 * sizeof(float), "accumulator frame")) return SHIRO_ERR_OUT_OF_MEMORY;
        o = frame_planes(a, n);
    }
    if (a->samples == 0) {
        k_accum_clear<<<grid_of(n), kAccumBlock, 0, ctx->stream>>>(n, o);
    } else {
        const float inv = 1.0f / static_cast<float>(a->samples);
        k_accum_resolve<<<grid_of(n), kAccumBlock, 0, ctx->stream>>>(n, inv, sum_planes(a), o);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "resolve");
    if (!out->on_device) {
        float* dst[4] = {out->beauty, out->albedo, out->normal, out->depth};
        const float* src[4] = {o.beauty, o.albedo, o.normal, o.depth};
        const size_t comps[4] = {4, 3, 3, 1};
        for (int k = 0; k < 4 && e == cudaSuccess; ++k)
            e = cudaMemcpyAsync(dst[k], src[k], n * comps[k] * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "resolve download");
        e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "resolve");
    }
    return SHIRO_OK;
}

int shiro_gpu_accum_info(const ShiroAccumulator* a, uint32_t* sample_count, uint32_t* width, uint32_t* height) {
    if (!a) return SHIRO_ERR_INVALID_ARGUMENT;
    if (sample_count) *sample_count = a->samples;
    if (width) *width = a->width;
    if (height) *height = a->height;
    return SHIRO_OK;
}

}  // extern "C"
