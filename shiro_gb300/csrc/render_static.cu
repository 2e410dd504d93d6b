// render_static.cu - plain render with statically reserved path-record scratch.
//
// shiro_gpu_render grows a cudaMalloc'ed block for the per-path records it
// averages per pixel.  Some callers must not allocate device memory while
// they render: a process that gave all device memory to its own allocator at
// start-up, or a render loop that must not stall on the allocator's implicit
// device-wide synchronisation while other streams of the process keep running.
// shiro_gpu_render_static serves them: it renders exactly like
// shiro_gpu_render (same kernels, same results) but takes its scratch from
// the file-scope device array below and calls no allocating routine.
//
// Limits and rules (also stated in include/shiro_gpu.h):
//  * the array holds kStaticPaths path records (1 048 576 x 48 B = 48 MiB);
//    every device that loads this library holds it until the process exits;
//  * a frame is rendered in launches of whole pixels of at most kStaticPaths
//    paths, so a request whose sample_count exceeds kStaticPaths is refused;
//  * all calls share the one array: calls that overlap on the GPU (other
//    threads, other contexts, other streams) race on it and must be serialised
//    by the caller.  Every record a launch reads was written by the same call,
//    so nothing needs clearing between calls;
//  * shiro_gpu_create sets the array up for its device (static_scratch_setup
//    below): it looks the array's device address up and loads this module and
//    the plain-form kernels, so the device memory they take is taken then,
//    not at the first shiro_gpu_render_static call.  A context made after a
//    cudaDeviceReset looks the address up again.
#include <cuda_runtime.h>

#include <string>

#include "context.h"
#include "kernels.h"

namespace shiro_gpu {

namespace {

constexpr uint32_t kStaticPaths = 1u << 20;
static __device__ __align__(256) float4 gStaticRecords[3 * static_cast<size_t>(kStaticPaths)];

__global__ void k_fill(float* __restrict__ p, uint64_t n, float v) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        p[i] = v;
}

}  // namespace

// Called by shiro_gpu_create with the context's device current.  In host code
// gStaticRecords names a host-side stand-in, so the array's device address is
// looked up here (which also loads this module, allocating the array); the
// kernels the static path launches are loaded too, because CUDA's lazy
// loading would otherwise place their code in device memory at their first
// launch.  A failure leaves the context usable for every other entry point;
// shiro_gpu_render_static then reports it.
void static_scratch_setup(ContextImpl* ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, gStaticRecords);
    if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
    cudaFuncAttributes a;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, k_fill);
    if (e == cudaSuccess) e = preload_plain_kernels();
    if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->staticRecords = nullptr;
        ctx->staticError = std::string("static scratch set-up: ") + cudaGetErrorString(e);
        return;
    }
    ctx->staticRecords = static_cast<float4*>(p);
}

}  // namespace shiro_gpu

using namespace shiro_gpu;

extern "C" int shiro_gpu_render_static(ShiroGpuContext* handle, const ShiroRenderDesc* req, const volatile int* cancel,
                                       ShiroAovs* out) {
    if (!handle || !req || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    if (!out->on_device || !out->beauty || !out->albedo || !out->normal || !out->depth)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "shiro_gpu_render_static writes device AOV planes only (on_device = 1)");
    if (req->sample_count > kStaticPaths)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT,
                    "sample_count " + std::to_string(req->sample_count) + " exceeds the static scratch capacity of " +
                        std::to_string(kStaticPaths) + " paths per launch");
    float4* rec = ctx->staticRecords;
    if (!rec) return fail(ctx, SHIRO_ERR_CUDA, ctx->staticError);
    const DevRequest q = make_request(*req);
    const uint64_t pixels = static_cast<uint64_t>(q.width) * q.height;
    const AovPtrs aov{out->beauty, out->albedo, out->normal, out->depth};
    ctx->stats.paths = 0;
    ctx->stats.kernel_launches = 0;
    ctx->stats.kernel_ms = 0.0;  // not timed: this entry point records no events
    ctx->stats.path_kernel_ms = 0.0;
    ctx->stats.path_kernel_launches = 0;
    if (req->sample_count == 0 || pixels == 0) {
        // FrameBuffer::Clear semantics (FrameBuffer.cpp:19-24)
        if (pixels) {
            k_fill<<<256, 256, 0, ctx->stream>>>(out->beauty, 4 * pixels, 0.0f);
            k_fill<<<256, 256, 0, ctx->stream>>>(out->albedo, 3 * pixels, 0.0f);
            k_fill<<<256, 256, 0, ctx->stream>>>(out->normal, 3 * pixels, 0.0f);
            k_fill<<<256, 256, 0, ctx->stream>>>(out->depth, pixels, __builtin_inff());
        }
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "clear");
    }
    const uint64_t pixelsPerLaunch = kStaticPaths / q.sampleCount;
    LaunchThrottle throttle(cancel, 2);
    for (uint64_t p0 = 0; p0 < pixels; p0 += pixelsPerLaunch) {
        if (!throttle.before_launch()) {
            cudaStreamSynchronize(ctx->stream);
            k_fill<<<256, 256, 0, ctx->stream>>>(out->beauty, 4 * pixels, 0.0f);
            k_fill<<<256, 256, 0, ctx->stream>>>(out->albedo, 3 * pixels, 0.0f);
            k_fill<<<256, 256, 0, ctx->stream>>>(out->normal, 3 * pixels, 0.0f);
            k_fill<<<256, 256, 0, ctx->stream>>>(out->depth, pixels, __builtin_inff());
            cudaStreamSynchronize(ctx->stream);
            return fail(ctx, SHIRO_ERR_CANCELLED, "cancelled");
        }
        const uint32_t np = static_cast<uint32_t>(std::min(pixelsPerLaunch, pixels - p0));
        const uint32_t paths = np * q.sampleCount;
        launch_plain_paths(ctx->scene, q, p0 * q.sampleCount, paths, rec, ctx->stream);
        launch_resolve_pixels(q, p0, np, rec, aov, ctx->stream);
        throttle.after_launch(ctx->stream);
        ctx->stats.kernel_launches += 2;
        ctx->stats.path_kernel_launches += 1;
        ctx->stats.paths += paths;
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(ctx, e, "render launch");
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render");
    return check_device_error(ctx);
}
