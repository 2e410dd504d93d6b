// bvh_build.h - host interface of the device BVH builder (bvh_build.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/shiro_gpu.h"

namespace shiro_gpu {

// A triangle kept out of the Morton tree (its box spans much of the scene).
struct LargeTri {
    float4 tri[3];  // (p0, gid), (e1, 0), (e2, 0)
    float lo[3], hi[3];
};

struct BvhInput {
    const float4* triData;    // device, 3 per small triangle: (p0, gid), (e1, 0), (e2, 0)
    const float4* primBoxes;  // device, 2 per small triangle: inflated lo, hi
    const float4* centroids;  // device, 1 per small triangle
    uint32_t smallCount;
    std::vector<LargeTri> largeSlots;  // at most 8
};

struct BvhOutput {
    float4* nodes = nullptr;  // cudaMalloc'ed, owned by the caller afterwards
    uint32_t nodeCount = 0;
    float4* tris = nullptr;   // cudaMalloc'ed, leaf order
    uint32_t triCount = 0;
    uint32_t depth = 0;
    uint32_t maxLeaf = 0;
};

inline int leaf_link_host(int first, int count) { return ~((first << 3) | (count - 1)); }

int build_bvh(const BvhInput& in, cudaStream_t stream, BvhOutput* out, std::string& err);

}  // namespace shiro_gpu
