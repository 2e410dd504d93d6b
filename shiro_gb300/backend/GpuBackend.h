// GpuBackend - the GB300 path tracer as a shiro::backend::RenderBackend.
//
// Drop-in replacement of backend::optix::OptixBackend
// (include/shiro/backend/optix/OptixBackend.h:10-27 of ichin0se/Shiro): same
// public methods (GetStatus, SupportsScene, RenderSampleBatch), same error
// convention (a failed batch logs to stderr and returns a cleared, sized
// FrameBuffer; a failed runtime reports available = false, which makes
// Renderer::Impl::ResolveBackend fall back to the CPU tracer,
// Renderer.cpp:16-31).  All device work goes through the C ABI of
// include/shiro_gpu.h.
#pragma once

#include <cstdint>
#include <memory>
#include <mutex>
#include <vector>

#include "shiro/backend/RenderBackend.h"

struct ShiroGpuContext;
struct ShiroAccumulator;

namespace shiro::backend::gb300 {

class GpuBackend final : public RenderBackend {
public:
    explicit GpuBackend(int device = 0);
    ~GpuBackend() override;

    GpuBackend(const GpuBackend&) = delete;
    GpuBackend& operator=(const GpuBackend&) = delete;

    BackendStatus GetStatus() const override;
    bool SupportsScene(const render::Scene& scene) const;
    render::FrameBuffer RenderSampleBatch(const RenderRequest& request) const override;

    // Batched wavefront form: several requests against the same scene in one
    // call (all requests must reference the same Scene object).
    std::vector<render::FrameBuffer> RenderSampleBatches(const std::vector<RenderRequest>& requests) const;

    // Progressive accumulation kept in device memory
    // (Renderer::FrameAccumulator, Renderer.cpp:47-110): one call per step of
    // HdShiroRenderParam's worker (RenderParam.cpp:790-806) renders the batch
    // and, unless request.cancel was set by the time it returned, folds it into
    // the device sums (restarting them for a batch at sample 0); nothing is
    // copied to the host.  Returns false when the batch was not accumulated.
    bool RenderAndAccumulate(const RenderRequest& request, bool wavefront = false) const;
    // FrameAccumulator::Resolve: the accumulated frame, copied out once.
    render::FrameBuffer ResolveAccumulation() const;
    // FrameAccumulator::SampleCount.
    uint32_t AccumulatedSampleCount() const;

    // Status code of the last render call (SHIRO_OK, SHIRO_ERR_CANCELLED, ...):
    // the reference reports failures on stderr only; this lets a caller tell a
    // cancelled batch from a failed one.
    int LastStatus() const;
    // Scene uploads so far (a changed snapshot is uploaded again).
    uint64_t SceneUploads() const;

private:
    bool EnsureRuntime(const render::Scene& scene) const;
    // The page-locked staging planes of RenderSampleBatch (grown on demand;
    // NULL when page-locked memory cannot be had).
    float* Staging(size_t bytes) const;

    int device_;
    mutable std::mutex mutex_;
    mutable ShiroGpuContext* ctx_ = nullptr;
    mutable ShiroAccumulator* accum_ = nullptr;
    mutable bool runtimeAttempted_ = false;
    mutable bool runtimeFailed_ = false;
    mutable const render::Scene* cachedScene_ = nullptr;
    mutable uint64_t cachedSignature_ = 0;
    mutable int lastStatus_ = 0;
    mutable uint64_t uploads_ = 0;
    mutable void* staging_ = nullptr;
    mutable size_t stagingBytes_ = 0;
};

}  // namespace shiro::backend::gb300
