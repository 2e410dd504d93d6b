// context.h - state behind a ShiroGpuContext handle.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/shiro_gpu.h"
#include "kernels.h"
#include "scene.cuh"

namespace shiro_gpu {

// Owns one cudaMalloc'ed block.
struct DeviceBlock {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct EnvHost {
    uint32_t w = 0, h = 0;
    bool latlong = true;
    const float* rgb = nullptr;  // w * h * 3: the caller's texels (read during the upload only)
};

// Default cluster size of the binned-SAH top (shiro_gpu_set_bvh_build):
// measured on the 1.31 M-triangle field frame, clusters of 2 gave the fewest
// node visits (wide 26.2 -> 25.0 per path against the Morton hierarchy; 8:
// 25.5, 16 and up fewer gains), at a longer build.
constexpr uint32_t kDefaultSahCluster = 2;

struct WavefrontState;
struct AdjointState;
struct AdjView;

struct ContextImpl {
    int device = 0;
    cudaStream_t ownStream = nullptr;
    cudaStream_t stream = nullptr;
    std::string lastError;

    // scene
    bool hasScene = false;
    DevScene scene{};
    std::vector<DeviceBlock> sceneBlocks;  // geometry blocks first, then shading ones
    size_t geomBlocks = 0;                 // sceneBlocks[0, geomBlocks): BVHs, triangles, shading records
    bool geomValid = false;                // geomSignature describes the resident geometry
    uint64_t geomSignature = 0;
    std::vector<DevEnv> envDev;        // host copy of the device env table
    std::vector<EnvHost> envHost;      // host copy of the textures (for parameter updates)
    std::vector<int32_t> domeEnv;      // dome -> env index
    std::vector<ShiroMaterialDesc> materialsHost;
    uint32_t materialCount = 0;        // user materials (the default one follows)
    bool extendedMaterials = false;    // transmission, opacity or emission present
    bool transmissiveMaterials = false;  // transmission present (the adjoint rejects it)
    bool noGeometry = false;           // the scene has no triangles (the BVHs hold two that nothing hits)
    uint32_t bvhDepth = 0, bvhMaxLeaf = 0;
    const float4* nodes8 = nullptr;   // wide BVH (kept even while the binary one is selected)
    const float4* tris8 = nullptr;    // triangles in the wide BVH's leaf order
    const float4* tris2 = nullptr;    // triangles in the binary BVH's leaf order
    uint32_t node8Count = 0, bvh8Depth = 0;
    // 2: traverse the binary BVH, 8: the compressed wide BVH, 0: the wide one
    // in the wavefront stages and the binary one in the one-thread-per-path
    // kernels (each measured faster there on GB300)
    uint32_t bvhWidth = 0;
    // triangles per cluster below the binned-SAH top of the binary BVHs built
    // at the next upload (0: the Morton hierarchy throughout)
    uint32_t sahClusterSize = kDefaultSahCluster;
    // 1: the adjoint replays paths with the wavefront stages (after each
    // wave's forward stages); 0: one thread per path (k_adjoint)
    uint32_t adjointWavefront = 1;
    // bumped by every call that changes what a render computes (scene,
    // parameters, BVH choice, wavefront configuration): a forward wave kept
    // for the adjoint is replayed only while it is unchanged
    uint64_t epoch = 0;

    // scratch (grown on demand, kept between calls)
    DeviceBlock pathRecords;
    DeviceBlock aovScratch;
    DeviceBlock probeScratch;
    uint32_t* errorWord = nullptr;
    // device address of the static path-record array of shiro_gpu_render_static
    // (render_static.cu), looked up when the context is created; staticError
    // says why it is NULL
    float4* staticRecords = nullptr;
    std::string staticError;

    // last call statistics
    ShiroRenderStats stats{};

    WavefrontState* wavefront = nullptr;
    AdjointState* adjoint = nullptr;

    ~ContextImpl();
    void freeScene();
    // frees what an upload derives from materials, lights and environments,
    // keeping the geometry (BVHs, triangles, per-triangle shading records)
    void freeShading();
    size_t deviceBytes() const;
};

// Allocation helpers; on failure they set ctx->lastError and return false.
bool ensure_block(ContextImpl* ctx, DeviceBlock* b, size_t bytes, const char* what);
int fail(ContextImpl* ctx, int code, const std::string& msg);
int cuda_fail(ContextImpl* ctx, cudaError_t e, const char* what);

// Request constants from the ABI descriptor (computes std::tan of the half
// field of view on the host, as GenerateCameraRay does).
DevRequest make_request(const ShiroRenderDesc& r);
int validate_request(ContextImpl* ctx, const ShiroRenderDesc& r);

// Uploads the dome textures of envHost and builds their tables on the device.
int upload_envs(ContextImpl* ctx);
// (Re)builds env k's importance tables, texel masses and sample records from
// its resident texels (after a scene upload or a parameter update).
int finish_env(ContextImpl* ctx, size_t k);
// env_tables.cu: the reference importance table, the texel masses (into
// texels.w) and the alias table of one lat-long texture, on the device.
int build_env_tables_device(ContextImpl* ctx, DevEnv& d);
// (Re)computes the per-material BSDF records (after the materials change).
int build_bsdf_recs(ContextImpl* ctx);

int check_device_error(ContextImpl* ctx);

// Launches are asynchronous, so a loop that enqueues a whole frame finishes
// before the GPU has run any of it and a cancel flag read there is read too
// early.  Loops that take a cancel flag therefore keep at most a few launches
// queued: before enqueueing launch k they wait for the event recorded after
// launch k - depth, polling the flag meanwhile.  Returns true (without
// waiting further) once the flag is set.
bool wait_or_cancel(cudaEvent_t ev, const volatile int* cancel);

// A ring of `depth` events for that throttling (created only when a cancel
// flag is given; every method is a no-op otherwise).
struct LaunchThrottle {
    std::vector<cudaEvent_t> ring;
    uint64_t issued = 0;
    const volatile int* cancel = nullptr;
    LaunchThrottle(const volatile int* c, uint32_t depth);
    ~LaunchThrottle();
    // Before launch number `issued`: false when the caller should stop (the
    // flag was set while an earlier launch ran).
    bool before_launch();
    // After a launch on `stream`.
    void after_launch(cudaStream_t stream);
};

// render_static.cu: sets up the static scratch of shiro_gpu_render_static for
// the current device (called once per context by shiro_gpu_create).
void static_scratch_setup(ContextImpl* ctx);

// wavefront.cu / adjoint.cu
// ready (may be null): told of each request's finished pixel ranges while
// later waves render (shiro_gpu_render_batch_ready).
int wavefront_render(ContextImpl* ctx, const ShiroRenderDesc* reqs, uint32_t count, const volatile int* cancel,
                     ShiroAovs* outs, ShiroPixelsReady ready = nullptr, void* user = nullptr);
void wavefront_free(ContextImpl* ctx);
// Every path of one request by the wavefront form, its record (radiance,
// first-hit depth) written to out[path] in request path order (pixel-major,
// sample-minor) instead of resolved pixels: the radiance a path replay needs.
int wavefront_path_records(ContextImpl* ctx, const ShiroRenderDesc& req, float4* out);
// The adjoint of one request by the wavefront form: each wave runs its
// forward stages, then replays its paths with the gradient stages into the
// buffers of `adj` (host copy; its device pointers are used as they are).
int wavefront_adjoint(ContextImpl* ctx, const ShiroRenderDesc& req, const AdjView& adj);
int wavefront_get_config(const ContextImpl* ctx, ShiroWavefrontConfig* out);
int wavefront_set_config(ContextImpl* ctx, const ShiroWavefrontConfig* cfg);
int wavefront_autotune(ContextImpl* ctx, const ShiroRenderDesc* req, ShiroWavefrontConfig* chosen);
int adjoint_run(ContextImpl* ctx, const ShiroRenderDesc* req, const float* dBeauty, float* dBase, float* dRough,
                float* dMetal, float* dEnv);
int adjoint_set_params(ContextImpl* ctx, const float* base, const float* rough, const float* metal, const float* env);
void adjoint_free(ContextImpl* ctx);
int adjoint_render_frozen(ContextImpl* ctx, const ShiroRenderDesc* req, const float* base, const float* rough,
                          const float* metal, const float* env, float* beauty);

}  // namespace shiro_gpu

struct ShiroGpuContext {
    shiro_gpu::ContextImpl impl;
};
