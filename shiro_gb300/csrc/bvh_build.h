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
    uint32_t maxLeaf = 8;              // largest SAH leaf (1..8)
    // > 0: the Morton tree's subtrees of at most this many triangles are kept
    // as clusters and the tree above them is rebuilt by binned SAH; 0: the
    // Morton (LBVH) hierarchy throughout
    uint32_t sahClusterSize = 0;
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

// Compressed 8-wide BVH (after Ylitie, Karras and Laine, "Efficient
// incoherent ray traversal on GPUs through compressed wide BVHs", HPG 2017),
// collapsed from a binary BVH.  Node layout (80 B = 5 x float4):
//   [0] origin.xyz, bits: ex | ey << 8 | ez << 16 | imask << 24; ex..ez are
//       biased float exponents of the per-axis power-of-two scales, imask
//       bit i marks child slot i as an internal node
//   [1] childBase, triBase, meta[0..3], meta[4..7]: internal children are
//       wide nodes childBase + (number of internal children in lower slots);
//       a leaf child's meta byte is (count - 1) << 5 | offset, its triangles
//       are triBase + offset .. + count - 1 of the wide BVH's own triangle
//       array (offset + count <= 32); an empty slot has meta 0xff
//   [2..4] qlo.x[8] qlo.y[8] qlo.z[8] qhi.x[8] qhi.y[8] qhi.z[8] bytes; a
//       child box is origin + q * scale, rounded outward and widened by one
//       step per side at build time (origin = node box minus one step)
// Child slot s holds the child lying most in direction
// ((s & 1) ? -x : +x, (s & 2) ? -y : +y, (s & 4) ? -z : +z) from the node
// centre, so a ray visits slots in the order of s ^ (7 ^ octant) to go
// roughly front to back without sorting.
constexpr uint32_t kWideEmptyMeta = 0xffu;
constexpr uint32_t kWideMaxTris = 32;  // triangle bits of one node
constexpr uint32_t kWideLeaf = 1;      // leaf size of the binary tree the wide BVH is collapsed from

struct WideOutput {
    float4* nodes = nullptr;  // cudaMalloc'ed, 5 float4 per node
    uint32_t nodeCount = 0;
    float4* tris = nullptr;   // cudaMalloc'ed, 3 float4 per triangle, wide-leaf order
    uint32_t triCount = 0;
    uint32_t depth = 0;
};

// Collapses a binary BVH (scene.cuh layout, root = node 0, leaves of at most
// 8 triangles in `tris2`) into compressed wide nodes; which binary nodes
// become wide nodes minimises a surface-area cost (optimal collapse over
// at most 8 slots per node, evaluated bottom-up on the device).
int collapse_wide(const float4* nodes2, uint32_t nodeCount2, const float4* tris2, uint32_t triCount2, cudaStream_t stream,
                  WideOutput* out, std::string& err);

int build_bvh(const BvhInput& in, cudaStream_t stream, BvhOutput* out, std::string& err);

}  // namespace shiro_gpu
