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
    std::vector<float> rgb;  // w * h * 3
    std::vector<float> rowCdf, condCdf;
    std::vector<float> mass;  // rowMass * columnMass per texel
};

struct WavefrontState;
struct AdjointState;

struct ContextImpl {
    int device = 0;
    cudaStream_t ownStream = nullptr;
    cudaStream_t stream = nullptr;
    std::string lastError;

    // scene
    bool hasScene = false;
    DevScene scene{};
    std::vector<DeviceBlock> sceneBlocks;
    std::vector<DevEnv> envDev;        // host copy of the device env table
    std::vector<EnvHost> envHost;      // host copy of the textures (for parameter updates)
    std::vector<int32_t> domeEnv;      // dome -> env index
    std::vector<ShiroMaterialDesc> materialsHost;
    uint32_t materialCount = 0;        // user materials (the default one follows)
    bool extendedMaterials = false;    // transmission, opacity or emission present (the adjoint rejects them)
    uint32_t bvhDepth = 0, bvhMaxLeaf = 0;
    const float4* nodes8 = nullptr;   // wide BVH (kept even while the binary one is selected)
    const float4* tris8 = nullptr;    // triangles in the wide BVH's leaf order
    const float4* tris2 = nullptr;    // triangles in the binary BVH's leaf order
    uint32_t node8Count = 0, bvh8Depth = 0;
    // 2: traverse the binary BVH, 8: the compressed wide BVH, 0: the wide one
    // in the wavefront stages and the binary one in the one-thread-per-path
    // kernels (each measured faster there on GB300)
    uint32_t bvhWidth = 0;

    // scratch (grown on demand, kept between calls)
    DeviceBlock pathRecords;
    DeviceBlock aovScratch;
    DeviceBlock probeScratch;
    uint32_t* errorWord = nullptr;

    // last call statistics
    ShiroRenderStats stats{};

    WavefrontState* wavefront = nullptr;
    AdjointState* adjoint = nullptr;

    ~ContextImpl();
    void freeScene();
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

// Uploads / refreshes the dome textures of envHost (texels + CDF + alias).
int upload_envs(ContextImpl* ctx);
// (Re)computes the per-material BSDF records (after the materials change).
int build_bsdf_recs(ContextImpl* ctx);
// Builds the reference importance table (EnvironmentMap.cpp:185-236).
void build_env_table(EnvHost& e);

int check_device_error(ContextImpl* ctx);

// wavefront.cu / adjoint.cu
int wavefront_render(ContextImpl* ctx, const ShiroRenderDesc* reqs, uint32_t count, const volatile int* cancel,
                     ShiroAovs* outs);
void wavefront_free(ContextImpl* ctx);
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
