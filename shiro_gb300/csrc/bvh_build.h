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

// 8-wide BVH with quantised child boxes, collapsed from the binary BVH.
// Node layout (96 B = 6 x float4):
//   [0] origin.xyz, bits: ex | ey << 8 | ez << 16 (biased float exponents of
//       the per-axis power-of-two scales)
//   [1] child links 0-3, [2] child links 4-7: >= 0 wide node index, < 0 the
//       binary BVH's leaf link ~((first << 3) | (count - 1)), kEmptyChild empty
//   [3..5] 8 x (qlo.x, qlo.y, qlo.z, qhi.x, qhi.y, qhi.z) bytes, stored as
//       qlo.x[8] qlo.y[8] qlo.z[8] qhi.x[8] qhi.y[8] qhi.z[8]; a child box is
//       origin + q * scale, rounded outward at build time.
constexpr int kEmptyChild = 0x7fffffff;

struct Bvh8Output {
    float4* nodes = nullptr;  // cudaMalloc'ed, 6 float4 per node
    uint32_t nodeCount = 0;
    uint32_t depth = 0;
};

// Collapses the binary BVH (scene.cuh layout, root = node 0) into 8-wide
// nodes by repeatedly opening the largest-area internal child.
int collapse_bvh8(const float4* nodes2, uint32_t nodeCount2, cudaStream_t stream, Bvh8Output* out, std::string& err);

int build_bvh(const BvhInput& in, cudaStream_t stream, BvhOutput* out, std::string& err);

}  // namespace shiro_gpu
