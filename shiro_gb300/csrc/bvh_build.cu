// bvh_build.cu - device BVH construction.
//
// Counterpart of CpuPathTracer::BuildAccelerationScene's Embree build
// (src/backend/cpu/CpuPathTracer.cpp:524-592, RTC_BUILD_QUALITY_LOW) and of
// the OptiX GAS build (src/backend/optix/OptixBackend.cpp:974-1015).
//
// Pipeline (all on the device, one stream):
//   1. centroid bounds            (block reduction + ordered-int atomics)
//   2. 63-bit Morton codes        (21 bits per axis)
//   3. radix sort of (code, prim) (CUB DeviceRadixSort - a library sort)
//   4. Karras 2012 hierarchy      (one thread per internal node)
//   5. bottom-up boxes + SAH      (atomic arrival counters; a subtree of <= 8
//                                  triangles becomes a leaf when the SAH leaf
//                                  cost does not exceed the split cost)
//   6. compaction + emission      (surviving internal nodes renumbered by an
//                                  exclusive scan, written in the traversal
//                                  layout of scene.cuh)
// Triangles whose box spans a large part of the scene (ground planes) would
// inflate every Morton-neighbour box up to the root; up to 8 of them are kept
// out of the Morton tree and placed in a leaf beside it under the root.
#include <cub/cub.cuh>

#include "bvh_build.h"
#include "common.cuh"

namespace shiro_gpu {

namespace {

constexpr float kCostNode = 1.2f;
constexpr float kCostTri = 1.0f;
constexpr uint32_t kMaxLeafLimit = 8;

__device__ __forceinline__ uint32_t f2ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__global__ void k_centroid_bounds(const float4* __restrict__ cen, uint32_t n, uint32_t* __restrict__ out6) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 c = cen[i];
        lo[0] = fminf(lo[0], c.x);
        lo[1] = fminf(lo[1], c.y);
        lo[2] = fminf(lo[2], c.z);
        hi[0] = fmaxf(hi[0], c.x);
        hi[1] = fmaxf(hi[1], c.y);
        hi[2] = fmaxf(hi[2], c.z);
    }
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; ++k) {
            atomicMin(&out6[k], f2ord(lo[k]));
            atomicMax(&out6[3 + k], f2ord(hi[k]));
        }
    }
}

__device__ __forceinline__ uint64_t spread21(uint64_t v) {
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x1f00000000ffffull;
    v = (v | (v << 16)) & 0x1f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

__global__ void k_morton(const float4* __restrict__ cen, uint32_t n, const uint32_t* __restrict__ b6,
                         uint64_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float lo[3] = {ord2f(b6[0]), ord2f(b6[1]), ord2f(b6[2])};
    const float hi[3] = {ord2f(b6[3]), ord2f(b6[4]), ord2f(b6[5])};
    const float4 c = cen[i];
    const float cc[3] = {c.x, c.y, c.z};
    // one scale for all axes (the largest extent): a flat scene's short axis
    // then splits only once the long axes are refined to its size, instead
    // of cutting every object at the top of the tree
    const float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
    uint64_t q[3];
    for (int k = 0; k < 3; ++k) {
        float f = ext > 0.0f ? (cc[k] - lo[k]) / ext : 0.5f;
        f = fminf(fmaxf(f, 0.0f), 1.0f);
        q[k] = static_cast<uint64_t>(fminf(f * 2097152.0f, 2097151.0f));
    }
    keys[i] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
    vals[i] = i;
}

__device__ __forceinline__ int delta(const uint64_t* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint64_t a = keys[i], b = keys[j];
    if (a != b) return __clzll(static_cast<long long>(a ^ b));
    return 64 + __clz(i ^ j);
}

// Karras 2012, "Maximizing parallelism in the construction of BVHs, octrees
// and k-d trees", algorithm 2.  Child encoding: >= 0 internal node index,
// < 0 leaf ~(sorted position).
__global__ void k_karras(const uint64_t* __restrict__ keys, int n, int2* __restrict__ child, int2* __restrict__ range,
                         int* __restrict__ nodeParent, int* __restrict__ leafParent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(keys, n, i, j);
    int s = 0;
    int div = 2;
    int t;
    do {
        t = (l + div - 1) / div;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
        div <<= 1;
    } while (t > 1);
    const int g = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    const int left = (first == g) ? ~g : g;
    const int right = (last == g + 1) ? ~(g + 1) : g + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(first, last);
    if (left < 0) leafParent[~left] = i; else nodeParent[left] = i;
    if (right < 0) leafParent[~right] = i; else nodeParent[right] = i;
    if (i == 0) nodeParent[0] = -1;
}

struct Box {
    float lo[3], hi[3];
};

__device__ __forceinline__ float box_area(const Box& b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__device__ __forceinline__ Box load_prim_box(const float4* pb, uint32_t prim) {
    const float4 a = pb[2 * prim], b = pb[2 * prim + 1];
    Box r;
    r.lo[0] = a.x; r.lo[1] = a.y; r.lo[2] = a.z;
    r.hi[0] = b.x; r.hi[1] = b.y; r.hi[2] = b.z;
    return r;
}

// Bottom-up: the second thread to reach a node computes its box, triangle
// count and SAH cost.
__global__ void k_bottom_up(int n, const uint32_t* __restrict__ sortedPrim, const float4* __restrict__ primBox,
                            const int2* __restrict__ child, const int* __restrict__ nodeParent,
                            const int* __restrict__ leafParent, unsigned int* __restrict__ arrivals,
                            float4* __restrict__ nodeBox, float* __restrict__ nodeCost, int* __restrict__ nodeCount,
                            uint8_t* __restrict__ collapse, int maxLeaf, const uint8_t* __restrict__ noCollapse) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    int node = leafParent[j];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(&arrivals[node], 1u) == 0u) return;
        __threadfence();
        const int2 c = child[node];
        Box bb[2];
        float cost[2];
        int cnt[2];
        const int cs[2] = {c.x, c.y};
        for (int k = 0; k < 2; ++k) {
            if (cs[k] < 0) {
                bb[k] = load_prim_box(primBox, sortedPrim[~cs[k]]);
                cnt[k] = 1;
                cost[k] = kCostTri * box_area(bb[k]);
            } else {
                const float4 a = __ldcg(&nodeBox[2 * cs[k]]), b = __ldcg(&nodeBox[2 * cs[k] + 1]);
                bb[k].lo[0] = a.x; bb[k].lo[1] = a.y; bb[k].lo[2] = a.z;
                bb[k].hi[0] = b.x; bb[k].hi[1] = b.y; bb[k].hi[2] = b.z;
                cnt[k] = __ldcg(&nodeCount[cs[k]]);
                cost[k] = __ldcg(&nodeCost[cs[k]]);
            }
        }
        Box u;
        for (int k = 0; k < 3; ++k) {
            u.lo[k] = fminf(bb[0].lo[k], bb[1].lo[k]);
            u.hi[k] = fmaxf(bb[0].hi[k], bb[1].hi[k]);
        }
        const float area = box_area(u);
        const int count = cnt[0] + cnt[1];
        const float split = kCostNode * area + cost[0] + cost[1];
        const float leaf = kCostTri * area * static_cast<float>(count);
        // a node of the SAH top spans clusters that need not be adjacent in
        // the triangle array, so it never becomes a (contiguous) leaf
        const bool asLeaf = count <= maxLeaf && leaf <= split && !(noCollapse && noCollapse[node]);
        nodeBox[2 * node] = make_float4(u.lo[0], u.lo[1], u.lo[2], 0.0f);
        nodeBox[2 * node + 1] = make_float4(u.hi[0], u.hi[1], u.hi[2], 0.0f);
        nodeCount[node] = count;
        nodeCost[node] = asLeaf ? leaf : split;
        collapse[node] = asLeaf ? 1 : 0;
        node = nodeParent[node];
    }
}

// ---- binned-SAH top (HLBVH style) -------------------------------------------
// Subtrees of the Morton tree with at most `clusterSize` triangles are kept as
// they are ("clusters"); the tree above them is rebuilt top-down by binned
// SAH over the clusters' boxes (16 bins per axis, one block per node being
// split, level by level).  The rebuilt top reuses the Karras node slots of
// the old top (a binary tree over C clusters has C - 1 internal nodes either
// way), so boxes, SAH leaf collapse, emission and the wide collapse run
// unchanged afterwards.  Splits are chosen and partitions written in a fixed
// order, so the build is deterministic.
constexpr int kSahBins = 16;
constexpr int kSahBlock = 256;

// Top nodes (more than clusterSize triangles) and, at each cluster's first
// sorted position, the cluster's root (internal node or ~leaf position).
__global__ void k_mark_clusters(int nInternal, int m, const int2* __restrict__ range, const int* __restrict__ nodeParent,
                                const int* __restrict__ leafParent, int clusterSize, uint8_t* __restrict__ top,
                                uint32_t* __restrict__ topFlag, uint32_t* __restrict__ startFlag, int* __restrict__ rootAt) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    auto size = [&](int node) { return range[node].y - range[node].x + 1; };
    if (k < nInternal) {
        const int sz = size(k);
        top[k] = sz > clusterSize ? 1 : 0;
        topFlag[k] = sz > clusterSize ? 1u : 0u;
        const int p = nodeParent[k];
        if (sz <= clusterSize && (p < 0 || size(p) > clusterSize)) {
            startFlag[range[k].x] = 1u;
            rootAt[range[k].x] = k;
        }
    }
    if (k < m && size(leafParent[k]) > clusterSize) {  // a single triangle hanging off the top
        startFlag[k] = 1u;
        rootAt[k] = ~k;
    }
}

struct SahItem {
    float lo[3], hi[3];
    int ref;        // cluster root: internal node >= 0, ~leaf position < 0
    float weight;   // triangles
};

__global__ void k_gather_clusters(int m, const uint32_t* __restrict__ startFlag, const uint32_t* __restrict__ startPos,
                                  const int* __restrict__ rootAt, const float4* __restrict__ nodeBox,
                                  const int* __restrict__ nodeCount, const uint32_t* __restrict__ sortedPrim,
                                  const float4* __restrict__ primBox, SahItem* __restrict__ items,
                                  uint32_t* __restrict__ perm) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= m || !startFlag[p]) return;
    const uint32_t c = startPos[p];
    const int ref = rootAt[p];
    SahItem it;
    float4 a, b;
    if (ref >= 0) {
        a = nodeBox[2 * ref];
        b = nodeBox[2 * ref + 1];
        it.weight = static_cast<float>(nodeCount[ref]);
    } else {
        const uint32_t prim = sortedPrim[~ref];
        a = primBox[2 * prim];
        b = primBox[2 * prim + 1];
        it.weight = 1.0f;
    }
    it.lo[0] = a.x; it.lo[1] = a.y; it.lo[2] = a.z;
    it.hi[0] = b.x; it.hi[1] = b.y; it.hi[2] = b.z;
    it.ref = ref;
    items[c] = it;
    perm[c] = c;
}

__global__ void k_top_slots(int nInternal, const uint32_t* __restrict__ top, const uint32_t* __restrict__ topPos,
                            int* __restrict__ slots) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nInternal && top[k]) slots[topPos[k]] = k;
}

struct SahTask {
    uint32_t begin, end;  // range of perm
    uint32_t node;        // SAH node id (0 = root)
    uint32_t pad;
};

// What a split produced: per side either a cluster (one item) or a new task.
struct SahResult {
    uint32_t mid;         // first item of the right side
    uint32_t pad;
};

__device__ __forceinline__ float item_centroid(const SahItem& it, int a) { return 0.5f * (it.lo[a] + it.hi[a]); }

// The split plane of least SAH cost (area(left) * weight(left) + area(right)
// * weight(right)) from a node's bins in shared memory: choice[0] = axis (-1:
// no usable plane), choice[1] = plane.  Every thread of the block calls it;
// the first 3 * (kSahBins - 1) threads cost one plane each.
__device__ __forceinline__ void sah_choose(const unsigned int (&binLo)[3][kSahBins][3],
                                           const unsigned int (&binHi)[3][kSahBins][3],
                                           const unsigned int (&binW)[3][kSahBins], const unsigned int (&binN)[3][kSahBins],
                                           const float (&cext)[3], float* bestCost, int* choice) {
    const int tid = threadIdx.x;
    if (tid < 3 * (kSahBins - 1)) {
        const int a = tid / (kSahBins - 1), sp = tid % (kSahBins - 1);
        float l[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, h[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        float r[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, g[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        unsigned int nl = 0, nr = 0, wl = 0, wr = 0;
        for (int b = 0; b < kSahBins; ++b) {
            if (binN[a][b] == 0u) continue;
            float* bl = b <= sp ? l : r;
            float* bh = b <= sp ? h : g;
            for (int k = 0; k < 3; ++k) {
                bl[k] = fminf(bl[k], ord2f(binLo[a][b][k]));
                bh[k] = fmaxf(bh[k], ord2f(binHi[a][b][k]));
            }
            if (b <= sp) { wl += binW[a][b]; nl += binN[a][b]; } else { wr += binW[a][b]; nr += binN[a][b]; }
        }
        float cost = FLT_MAX;
        if (cext[a] > 0.0f && nl > 0u && nr > 0u) {
            const float al = 2.0f * ((h[0] - l[0]) * (h[1] - l[1]) + (h[1] - l[1]) * (h[2] - l[2]) + (h[2] - l[2]) * (h[0] - l[0]));
            const float ar = 2.0f * ((g[0] - r[0]) * (g[1] - r[1]) + (g[1] - r[1]) * (g[2] - r[2]) + (g[2] - r[2]) * (g[0] - r[0]));
            cost = al * static_cast<float>(wl) + ar * static_cast<float>(wr);
        }
        bestCost[tid] = cost;
    }
    __syncthreads();
    if (tid == 0) {
        int best = -1;
        float bc = FLT_MAX;
        for (int k = 0; k < 3 * (kSahBins - 1); ++k)
            if (bestCost[k] < bc) {  // first of equal costs: lowest axis, lowest plane
                bc = bestCost[k];
                best = k;
            }
        choice[0] = best < 0 ? -1 : best / (kSahBins - 1);
        choice[1] = best < 0 ? 0 : best % (kSahBins - 1);
    }
    __syncthreads();
}

// Block-wide exclusive scan of one value per thread (kSahBlock threads).
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* warpSums, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warpSums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kSahBlock / 32 ? warpSums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kSahBlock / 32) warpSums[lane] = w;  // inclusive
    }
    __syncthreads();
    const uint32_t before = (warp > 0 ? warpSums[warp - 1] : 0u) + x - v;
    *total = warpSums[kSahBlock / 32 - 1];
    __syncthreads();
    return before;
}

__global__ void __launch_bounds__(kSahBlock) k_sah_split(const SahTask* __restrict__ tasks, const SahItem* __restrict__ items,
                                                        const uint32_t* __restrict__ permIn, uint32_t* __restrict__ permOut,
                                                        SahResult* __restrict__ results, uint32_t* __restrict__ newTasks,
                                                        uint32_t bigMin) {
    __shared__ unsigned int cbo[6];
    __shared__ unsigned int binLo[3][kSahBins][3], binHi[3][kSahBins][3];
    __shared__ unsigned int binW[3][kSahBins], binN[3][kSahBins];
    __shared__ float bestCost[3 * (kSahBins - 1)];
    __shared__ int choice[2];
    __shared__ uint32_t warpSums[kSahBlock / 32];
    const SahTask t = tasks[blockIdx.x];
    const uint32_t n = t.end - t.begin;
    if (bigMin && n >= bigMin) return;  // split by the multi-block kernels below
    const int tid = threadIdx.x;
    if (tid < 6) cbo[tid] = tid < 3 ? 0xffffffffu : 0u;
    for (int e = tid; e < 3 * kSahBins * 3; e += kSahBlock) {
        (&binLo[0][0][0])[e] = 0xffffffffu;
        (&binHi[0][0][0])[e] = 0u;
    }
    for (int e = tid; e < 3 * kSahBins; e += kSahBlock) {
        (&binW[0][0])[e] = 0u;
        (&binN[0][0])[e] = 0u;
    }
    __syncthreads();
    // centroid bounds of the node's clusters (ordered-integer min / max)
    {
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = tid; i < n; i += kSahBlock) {
            const SahItem& it = items[permIn[t.begin + i]];
            for (int a = 0; a < 3; ++a) {
                const float c = item_centroid(it, a);
                lo[a] = fminf(lo[a], c);
                hi[a] = fmaxf(hi[a], c);
            }
        }
        for (int a = 0; a < 3; ++a) {
            for (int o = 16; o > 0; o >>= 1) {
                lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
                hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
            }
            if ((tid & 31) == 0) {
                atomicMin(&cbo[a], f2ord(lo[a]));
                atomicMax(&cbo[3 + a], f2ord(hi[a]));
            }
        }
    }
    __syncthreads();
    float clo[3], cext[3];
    for (int a = 0; a < 3; ++a) {
        clo[a] = ord2f(cbo[a]);
        cext[a] = ord2f(cbo[3 + a]) - clo[a];
    }
    // binning: item weight and box per bin and axis
    for (uint32_t i = tid; i < n; i += kSahBlock) {
        const SahItem& it = items[permIn[t.begin + i]];
        for (int a = 0; a < 3; ++a) {
            if (!(cext[a] > 0.0f)) continue;
            int b = static_cast<int>(kSahBins * ((item_centroid(it, a) - clo[a]) / cext[a]));
            b = b < 0 ? 0 : (b >= kSahBins ? kSahBins - 1 : b);
            atomicAdd(&binW[a][b], static_cast<unsigned int>(it.weight));
            atomicAdd(&binN[a][b], 1u);
            for (int k = 0; k < 3; ++k) {
                atomicMin(&binLo[a][b][k], f2ord(it.lo[k]));
                atomicMax(&binHi[a][b][k], f2ord(it.hi[k]));
            }
        }
    }
    __syncthreads();
    sah_choose(binLo, binHi, binW, binN, cext, bestCost, choice);
    const int axis = choice[0], plane = choice[1];
    // stable partition: left side first, each side in its input order; with
    // no usable plane (all centroids in one bin) the range splits in the
    // middle of its Morton order
    const uint32_t half = n / 2u;
    auto goesLeft = [&](uint32_t i, const SahItem& it) {
        if (axis < 0) return i < half;
        int b = static_cast<int>(kSahBins * ((item_centroid(it, axis) - clo[axis]) / cext[axis]));
        b = b < 0 ? 0 : (b >= kSahBins ? kSahBins - 1 : b);
        return b <= plane;
    };
    uint32_t leftBase = 0, rightBase = 0, nLeft = 0;
    {
        uint32_t cnt = 0;
        for (uint32_t i = tid; i < n; i += kSahBlock) cnt += goesLeft(i, items[permIn[t.begin + i]]) ? 1u : 0u;
        uint32_t tot;
        block_scan(cnt, warpSums, &tot);
        nLeft = tot;
    }
    for (uint32_t base = 0; base < n; base += kSahBlock) {
        const uint32_t i = base + tid;
        const bool valid = i < n;
        const uint32_t v = valid ? permIn[t.begin + i] : 0u;
        const bool left = valid && goesLeft(i, items[v]);
        uint32_t totL, totR;
        const uint32_t rl = block_scan(left ? 1u : 0u, warpSums, &totL);
        const uint32_t rr = block_scan((valid && !left) ? 1u : 0u, warpSums, &totR);
        if (valid) permOut[t.begin + (left ? leftBase + rl : nLeft + rightBase + rr)] = v;
        leftBase += totL;
        rightBase += totR;
    }
    if (tid == 0) {
        const uint32_t mid = t.begin + nLeft;
        results[blockIdx.x] = SahResult{mid, 0u};
        newTasks[blockIdx.x] = (nLeft > 1u ? 1u : 0u) + (n - nLeft > 1u ? 1u : 0u);
    }
}

// ---- big tasks: one task split by many blocks --------------------------------
// At the top levels a few tasks hold most clusters; k_sah_split gives each
// one block.  For tasks of at least bigMin items the same split is computed
// by chunks of kSahChunk items, one block each: centroid bounds and bins are
// merged into per-task global arrays with min / max / integer-add atomics
// (order-independent, so the bins and the chosen plane equal k_sah_split's),
// and the stable partition places each chunk's items after the earlier
// chunks' (a prefix over the chunks' left counts), so the tree is the same.
constexpr uint32_t kSahChunk = 4096;

struct SahChunk {
    uint32_t task;         // index of the task at this level
    uint32_t begin, end;   // item range in perm (within the task's)
    uint32_t first;        // 1 for the task's first chunk
};

struct SahBig {
    unsigned int cbo[6];
    unsigned int lo[3][kSahBins][3], hi[3][kSahBins][3];
    unsigned int w[3][kSahBins], n[3][kSahBins];
    int axis, plane;
    uint32_t nLeft, pad;
};

__global__ void k_big_init(SahBig* __restrict__ big, uint32_t count) {
    SahBig& b = big[blockIdx.x];
    for (int e = threadIdx.x; e < 3 * kSahBins * 3; e += blockDim.x) {
        (&b.lo[0][0][0])[e] = 0xffffffffu;
        (&b.hi[0][0][0])[e] = 0u;
    }
    for (int e = threadIdx.x; e < 3 * kSahBins; e += blockDim.x) {
        (&b.w[0][0])[e] = 0u;
        (&b.n[0][0])[e] = 0u;
    }
    if (threadIdx.x < 6) b.cbo[threadIdx.x] = threadIdx.x < 3 ? 0xffffffffu : 0u;
}

__global__ void __launch_bounds__(kSahBlock) k_big_bounds(const SahChunk* __restrict__ chunks, const SahItem* __restrict__ items,
                                                          const uint32_t* __restrict__ permIn, SahBig* __restrict__ big) {
    __shared__ unsigned int cbo[6];
    const SahChunk c = chunks[blockIdx.x];
    const int tid = threadIdx.x;
    if (tid < 6) cbo[tid] = tid < 3 ? 0xffffffffu : 0u;
    __syncthreads();
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = c.begin + tid; i < c.end; i += kSahBlock) {
        const SahItem& it = items[permIn[i]];
        for (int a = 0; a < 3; ++a) {
            const float x = item_centroid(it, a);
            lo[a] = fminf(lo[a], x);
            hi[a] = fmaxf(hi[a], x);
        }
    }
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
        if ((tid & 31) == 0) {
            atomicMin(&cbo[a], f2ord(lo[a]));
            atomicMax(&cbo[3 + a], f2ord(hi[a]));
        }
    }
    __syncthreads();
    if (tid < 3) atomicMin(&big[c.task].cbo[tid], cbo[tid]);
    else if (tid < 6) atomicMax(&big[c.task].cbo[tid], cbo[tid]);
}

__device__ __forceinline__ void big_extent(const SahBig& b, float (&clo)[3], float (&cext)[3]) {
    for (int a = 0; a < 3; ++a) {
        clo[a] = ord2f(b.cbo[a]);
        cext[a] = ord2f(b.cbo[3 + a]) - clo[a];
    }
}

__global__ void __launch_bounds__(kSahBlock) k_big_bins(const SahChunk* __restrict__ chunks, const SahItem* __restrict__ items,
                                                        const uint32_t* __restrict__ permIn, SahBig* __restrict__ big) {
    __shared__ unsigned int binLo[3][kSahBins][3], binHi[3][kSahBins][3];
    __shared__ unsigned int binW[3][kSahBins], binN[3][kSahBins];
    const SahChunk c = chunks[blockIdx.x];
    SahBig& b = big[c.task];
    const int tid = threadIdx.x;
    for (int e = tid; e < 3 * kSahBins * 3; e += kSahBlock) {
        (&binLo[0][0][0])[e] = 0xffffffffu;
        (&binHi[0][0][0])[e] = 0u;
    }
    for (int e = tid; e < 3 * kSahBins; e += kSahBlock) {
        (&binW[0][0])[e] = 0u;
        (&binN[0][0])[e] = 0u;
    }
    float clo[3], cext[3];
    big_extent(b, clo, cext);
    __syncthreads();
    for (uint32_t i = c.begin + tid; i < c.end; i += kSahBlock) {
        const SahItem& it = items[permIn[i]];
        for (int a = 0; a < 3; ++a) {
            if (!(cext[a] > 0.0f)) continue;
            int bi = static_cast<int>(kSahBins * ((item_centroid(it, a) - clo[a]) / cext[a]));
            bi = bi < 0 ? 0 : (bi >= kSahBins ? kSahBins - 1 : bi);
            atomicAdd(&binW[a][bi], static_cast<unsigned int>(it.weight));
            atomicAdd(&binN[a][bi], 1u);
            for (int k = 0; k < 3; ++k) {
                atomicMin(&binLo[a][bi][k], f2ord(it.lo[k]));
                atomicMax(&binHi[a][bi][k], f2ord(it.hi[k]));
            }
        }
    }
    __syncthreads();
    for (int e = tid; e < 3 * kSahBins; e += kSahBlock) {
        const int a = e / kSahBins, bi = e % kSahBins;
        if (binN[a][bi] == 0u) continue;
        atomicAdd(&b.w[a][bi], binW[a][bi]);
        atomicAdd(&b.n[a][bi], binN[a][bi]);
        for (int k = 0; k < 3; ++k) {
            atomicMin(&b.lo[a][bi][k], binLo[a][bi][k]);
            atomicMax(&b.hi[a][bi][k], binHi[a][bi][k]);
        }
    }
}

// One block per big task: its plane, with k_sah_split's choice code.
__global__ void __launch_bounds__(64) k_big_choose(SahBig* __restrict__ big) {
    __shared__ unsigned int binLo[3][kSahBins][3], binHi[3][kSahBins][3];
    __shared__ unsigned int binW[3][kSahBins], binN[3][kSahBins];
    __shared__ float bestCost[3 * (kSahBins - 1)];
    __shared__ int choice[2];
    SahBig& b = big[blockIdx.x];
    for (int e = threadIdx.x; e < 3 * kSahBins * 3; e += blockDim.x) {
        (&binLo[0][0][0])[e] = (&b.lo[0][0][0])[e];
        (&binHi[0][0][0])[e] = (&b.hi[0][0][0])[e];
    }
    for (int e = threadIdx.x; e < 3 * kSahBins; e += blockDim.x) {
        (&binW[0][0])[e] = (&b.w[0][0])[e];
        (&binN[0][0])[e] = (&b.n[0][0])[e];
    }
    float clo[3], cext[3];
    big_extent(b, clo, cext);
    __syncthreads();
    sah_choose(binLo, binHi, binW, binN, cext, bestCost, choice);
    if (threadIdx.x == 0) {
        b.axis = choice[0];
        b.plane = choice[1];
    }
}

__device__ __forceinline__ bool big_goes_left(const SahBig& b, const float (&clo)[3], const float (&cext)[3], uint32_t i,
                                              uint32_t half, const SahItem& it) {
    if (b.axis < 0) return i < half;
    int bi = static_cast<int>(kSahBins * ((item_centroid(it, b.axis) - clo[b.axis]) / cext[b.axis]));
    bi = bi < 0 ? 0 : (bi >= kSahBins ? kSahBins - 1 : bi);
    return bi <= b.plane;
}

__global__ void __launch_bounds__(kSahBlock) k_big_count(const SahChunk* __restrict__ chunks, const SahTask* __restrict__ tasks,
                                                         const SahItem* __restrict__ items,
                                                         const uint32_t* __restrict__ permIn, const SahBig* __restrict__ big,
                                                         uint32_t* __restrict__ chunkLeft) {
    __shared__ uint32_t warpSums[kSahBlock / 32];
    const SahChunk c = chunks[blockIdx.x];
    const SahTask t = tasks[c.task];
    const SahBig& b = big[c.task];
    float clo[3], cext[3];
    big_extent(b, clo, cext);
    const uint32_t half = (t.end - t.begin) / 2u;
    uint32_t cnt = 0;
    for (uint32_t i = c.begin + threadIdx.x; i < c.end; i += kSahBlock)
        cnt += big_goes_left(b, clo, cext, i - t.begin, half, items[permIn[i]]) ? 1u : 0u;
    uint32_t tot;
    block_scan(cnt, warpSums, &tot);
    if (threadIdx.x == 0) chunkLeft[blockIdx.x] = tot;
}

// Per big task (one thread each): exclusive prefix of its chunks' left
// counts (its chunks are consecutive), and its left total.
__global__ void k_big_offsets(const SahChunk* __restrict__ chunks, uint32_t nChunks, uint32_t* __restrict__ chunkLeft,
                              SahBig* __restrict__ big, uint32_t count) {
    const uint32_t task = blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= count) return;
    uint32_t acc = 0;
    bool any = false;
    for (uint32_t k = 0; k < nChunks; ++k) {
        if (chunks[k].task != task) continue;
        any = true;
        const uint32_t v = chunkLeft[k];
        chunkLeft[k] = acc;
        acc += v;
    }
    if (any) big[task].nLeft = acc;
}

__global__ void __launch_bounds__(kSahBlock) k_big_scatter(const SahChunk* __restrict__ chunks, const SahTask* __restrict__ tasks,
                                                           const SahItem* __restrict__ items,
                                                           const uint32_t* __restrict__ permIn, uint32_t* __restrict__ permOut,
                                                           const SahBig* __restrict__ big,
                                                           const uint32_t* __restrict__ chunkLeft,
                                                           SahResult* __restrict__ results, uint32_t* __restrict__ newTasks) {
    __shared__ uint32_t warpSums[kSahBlock / 32];
    const SahChunk c = chunks[blockIdx.x];
    const SahTask t = tasks[c.task];
    const SahBig& b = big[c.task];
    float clo[3], cext[3];
    big_extent(b, clo, cext);
    const uint32_t n = t.end - t.begin, half = n / 2u, nLeft = b.nLeft;
    const uint32_t leftBefore = chunkLeft[blockIdx.x];
    const uint32_t rightBefore = (c.begin - t.begin) - leftBefore;
    uint32_t leftBase = 0, rightBase = 0;
    for (uint32_t base = c.begin; base < c.end; base += kSahBlock) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < c.end;
        const uint32_t v = valid ? permIn[i] : 0u;
        const bool left = valid && big_goes_left(b, clo, cext, i - t.begin, half, items[v]);
        uint32_t totL, totR;
        const uint32_t rl = block_scan(left ? 1u : 0u, warpSums, &totL);
        const uint32_t rr = block_scan((valid && !left) ? 1u : 0u, warpSums, &totR);
        if (valid)
            permOut[left ? t.begin + leftBefore + leftBase + rl : t.begin + nLeft + rightBefore + rightBase + rr] = v;
        leftBase += totL;
        rightBase += totR;
    }
    if (c.first && threadIdx.x == 0) {
        results[c.task] = SahResult{t.begin + nLeft, 0u};
        newTasks[c.task] = (nLeft > 1u ? 1u : 0u) + (n - nLeft > 1u ? 1u : 0u);
    }
}

// Children of the level's tasks: a side of one item is a cluster, a larger
// side a new task whose SAH node id follows the ids handed out so far.
__global__ void k_sah_children(const SahTask* __restrict__ tasks, uint32_t count, const SahResult* __restrict__ results,
                               const uint32_t* __restrict__ taskPos, uint32_t nextId, const uint32_t* __restrict__ perm,
                               const SahItem* __restrict__ items, SahTask* __restrict__ next, int2* __restrict__ sahChild) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const SahTask t = tasks[k];
    const SahResult r = results[k];
    uint32_t pos = taskPos[k];
    int link[2];
    const uint32_t b[2] = {t.begin, r.mid}, e[2] = {r.mid, t.end};
    for (int q = 0; q < 2; ++q) {
        if (e[q] - b[q] == 1u) {
            link[q] = ~static_cast<int>(perm[b[q]]);  // cluster (item index)
        } else {
            const uint32_t id = nextId + pos;
            next[pos] = SahTask{b[q], e[q], id, 0u};
            link[q] = static_cast<int>(id);
            ++pos;
        }
    }
    sahChild[t.node] = make_int2(link[0], link[1]);
}

// The SAH top written into the Karras arrays: SAH node i lives in top slot
// slots[i]; a cluster child is the cluster's root node (or leaf).
__global__ void k_sah_link(uint32_t nSah, const int2* __restrict__ sahChild, const int* __restrict__ slots,
                           const SahItem* __restrict__ items, int2* __restrict__ child, int* __restrict__ nodeParent,
                           int* __restrict__ leafParent) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nSah) return;
    const int slot = slots[i];
    const int2 c = sahChild[i];
    const int cs[2] = {c.x, c.y};
    int out[2];
    for (int q = 0; q < 2; ++q) {
        const int ref = cs[q] >= 0 ? slots[cs[q]] : items[~cs[q]].ref;
        out[q] = ref;
        if (ref >= 0) nodeParent[ref] = slot;
        else leafParent[~ref] = slot;
    }
    child[slot] = make_int2(out[0], out[1]);
    if (i == 0) nodeParent[slot] = -1;
}

// A node is emitted when neither it nor any ancestor became a leaf.
__global__ void k_emit_flags(int nInternal, const int* __restrict__ nodeParent, const uint8_t* __restrict__ collapse,
                             uint32_t* __restrict__ flag, unsigned int* __restrict__ maxDepth) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nInternal) return;
    bool emitted = collapse[k] == 0;
    unsigned int depth = 0;
    for (int p = nodeParent[k]; p >= 0; p = nodeParent[p]) {
        if (collapse[p]) emitted = false;
        ++depth;
    }
    flag[k] = emitted ? 1u : 0u;
    if (emitted) atomicMax(maxDepth, depth + 1u);
}

__device__ __forceinline__ int leaf_link(int first, int count) { return ~((first << 3) | (count - 1)); }

__global__ void k_emit_nodes(int nInternal, const uint32_t* __restrict__ flag, const uint32_t* __restrict__ newIndex,
                             uint32_t offset, const int2* __restrict__ child, const int2* __restrict__ range,
                             const uint8_t* __restrict__ collapse, const float4* __restrict__ nodeBox,
                             const uint32_t* __restrict__ sortedPrim, const float4* __restrict__ primBox,
                             float4* __restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nInternal || !flag[k]) return;
    const int2 c = child[k];
    const int cs[2] = {c.x, c.y};
    Box bb[2];
    int link[2];
    for (int q = 0; q < 2; ++q) {
        const int ch = cs[q];
        if (ch < 0) {
            bb[q] = load_prim_box(primBox, sortedPrim[~ch]);
            link[q] = leaf_link(~ch, 1);
        } else {
            const float4 a = nodeBox[2 * ch], b = nodeBox[2 * ch + 1];
            bb[q].lo[0] = a.x; bb[q].lo[1] = a.y; bb[q].lo[2] = a.z;
            bb[q].hi[0] = b.x; bb[q].hi[1] = b.y; bb[q].hi[2] = b.z;
            if (collapse[ch]) {
                const int2 r = range[ch];
                link[q] = leaf_link(r.x, r.y - r.x + 1);
            } else {
                link[q] = static_cast<int>(newIndex[ch] + offset);
            }
        }
    }
    float4* o = out + 4 * static_cast<size_t>(newIndex[k] + offset);
    o[0] = make_float4(bb[0].lo[0], bb[0].hi[0], bb[0].lo[1], bb[0].hi[1]);
    o[1] = make_float4(bb[1].lo[0], bb[1].hi[0], bb[1].lo[1], bb[1].hi[1]);
    o[2] = make_float4(bb[0].lo[2], bb[0].hi[2], bb[1].lo[2], bb[1].hi[2]);
    o[3] = make_float4(__int_as_float(link[0]), __int_as_float(link[1]), 0.0f, 0.0f);
}

__global__ void k_write_tris(uint32_t n, const uint32_t* __restrict__ sortedPrim, const float4* __restrict__ triIn,
                             float4* __restrict__ triOut) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t p = sortedPrim[s];
    triOut[3 * static_cast<size_t>(s)] = triIn[3 * static_cast<size_t>(p)];
    triOut[3 * static_cast<size_t>(s) + 1] = triIn[3 * static_cast<size_t>(p) + 1];
    triOut[3 * static_cast<size_t>(s) + 2] = triIn[3 * static_cast<size_t>(p) + 2];
}

// Root node for trees with fewer than two emitted Morton nodes and for the
// top node that holds the large triangles: child 0 / child 1 given as
// (box, link); an absent child gets an empty (inverted) box.
__global__ void k_write_root(float4* out, float4 b0lo, float4 b0hi, int l0, float4 b1lo, float4 b1hi, int l1) {
    out[0] = make_float4(b0lo.x, b0hi.x, b0lo.y, b0hi.y);
    out[1] = make_float4(b1lo.x, b1hi.x, b1lo.y, b1hi.y);
    out[2] = make_float4(b0lo.z, b0hi.z, b1lo.z, b1hi.z);
    out[3] = make_float4(__int_as_float(l0), __int_as_float(l1), 0.0f, 0.0f);
}


#define BVH_CHECK(x)                                                       \
    do {                                                                   \
        cudaError_t e_ = (x);                                              \
        if (e_ != cudaSuccess) {                                           \
            err = std::string(#x) + ": " + cudaGetErrorString(e_);         \
            return e_ == cudaErrorMemoryAllocation ? SHIRO_ERR_OUT_OF_MEMORY \
                                                   : SHIRO_ERR_CUDA;       \
        }                                                                  \
    } while (0)

struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <typename T>
    cudaError_t alloc(T** p, size_t count) {
        void* v = nullptr;
        const cudaError_t e = cudaMalloc(&v, count * sizeof(T) + 16);
        if (e == cudaSuccess) ptrs.push_back(v);
        *p = static_cast<T*>(v);
        return e;
    }
};

inline unsigned blocks(size_t n, unsigned b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace

// Rebuilds the Morton tree's top above its clusters by binned SAH (kernels
// above).  *topOut marks the rebuilt nodes (never collapsed into leaves).
static int sah_top(Scratch& sc, int m, int nInternal, int clusterSize, const uint32_t* sortedPrim, const float4* primBox,
            int2* child, const int2* range, int* nodeParent, int* leafParent, const float4* nodeBox,
            const int* nodeCount, uint8_t** topOut, cudaStream_t stream, std::string& err) {
    uint8_t* top = nullptr;
    uint32_t *topFlag = nullptr, *topPos = nullptr, *startFlag = nullptr, *startPos = nullptr;
    int* rootAt = nullptr;
    BVH_CHECK(sc.alloc(&top, nInternal));
    BVH_CHECK(sc.alloc(&topFlag, nInternal));
    BVH_CHECK(sc.alloc(&topPos, nInternal));
    BVH_CHECK(sc.alloc(&startFlag, m));
    BVH_CHECK(sc.alloc(&startPos, m));
    BVH_CHECK(sc.alloc(&rootAt, m));
    BVH_CHECK(cudaMemsetAsync(startFlag, 0, sizeof(uint32_t) * m, stream));
    k_mark_clusters<<<blocks(std::max(nInternal, m), 256), 256, 0, stream>>>(nInternal, m, range, nodeParent, leafParent,
                                                                            clusterSize, top, topFlag, startFlag, rootAt);
    BVH_CHECK(cudaGetLastError());
    size_t need = 0, tmpBytes = 0;
    BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, need, startFlag, startPos, m, stream));
    tmpBytes = std::max(tmpBytes, need);
    BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, need, topFlag, topPos, nInternal, stream));
    tmpBytes = std::max(tmpBytes, need);
    uint8_t* tmp = nullptr;
    BVH_CHECK(sc.alloc(&tmp, tmpBytes));
    BVH_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, startFlag, startPos, m, stream));
    BVH_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, topFlag, topPos, nInternal, stream));
    uint32_t h4[4];
    BVH_CHECK(cudaMemcpyAsync(&h4[0], startPos + m - 1, 4, cudaMemcpyDeviceToHost, stream));
    BVH_CHECK(cudaMemcpyAsync(&h4[1], startFlag + m - 1, 4, cudaMemcpyDeviceToHost, stream));
    BVH_CHECK(cudaMemcpyAsync(&h4[2], topPos + nInternal - 1, 4, cudaMemcpyDeviceToHost, stream));
    BVH_CHECK(cudaMemcpyAsync(&h4[3], topFlag + nInternal - 1, 4, cudaMemcpyDeviceToHost, stream));
    BVH_CHECK(cudaStreamSynchronize(stream));
    const uint32_t clusters = h4[0] + h4[1], tops = h4[2] + h4[3];
    if (clusters < 2 || tops + 1u != clusters) {
        err = "binned-SAH top: inconsistent cluster cut";
        return SHIRO_ERR_DEVICE_CHECK;
    }
    SahItem* items = nullptr;
    uint32_t *perm[2] = {nullptr, nullptr}, *newTasks = nullptr, *taskPos = nullptr;
    int* slots = nullptr;
    SahTask* tasks[2] = {nullptr, nullptr};
    SahResult* results = nullptr;
    int2* sahChild = nullptr;
    BVH_CHECK(sc.alloc(&items, clusters));
    BVH_CHECK(sc.alloc(&perm[0], clusters));
    BVH_CHECK(sc.alloc(&perm[1], clusters));
    BVH_CHECK(sc.alloc(&slots, tops));
    BVH_CHECK(sc.alloc(&tasks[0], clusters));
    BVH_CHECK(sc.alloc(&tasks[1], clusters));
    BVH_CHECK(sc.alloc(&results, clusters));
    BVH_CHECK(sc.alloc(&newTasks, clusters));
    BVH_CHECK(sc.alloc(&taskPos, clusters));
    BVH_CHECK(sc.alloc(&sahChild, tops));
    k_gather_clusters<<<blocks(m, 256), 256, 0, stream>>>(m, startFlag, startPos, rootAt, nodeBox, nodeCount, sortedPrim,
                                                           primBox, items, perm[0]);
    k_top_slots<<<blocks(nInternal, 256), 256, 0, stream>>>(nInternal, topFlag, topPos, slots);
    BVH_CHECK(cudaGetLastError());
    const SahTask root{0u, clusters, 0u, 0u};
    BVH_CHECK(cudaMemcpyAsync(tasks[0], &root, sizeof(root), cudaMemcpyHostToDevice, stream));
    BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, need, newTasks, taskPos, static_cast<int>(clusters), stream));
    uint8_t* scanTmp = nullptr;
    BVH_CHECK(sc.alloc(&scanTmp, need));
    const size_t scanBytes = need;
    // levels of at most kBigLevelTasks tasks split their tasks of at least
    // kBigMin items with the multi-block kernels (the top of the tree)
    constexpr uint32_t kBigLevelTasks = 64, kBigMin = 2 * kSahChunk;
    SahBig* big = nullptr;
    SahChunk* dChunks = nullptr;
    uint32_t* chunkLeft = nullptr;
    const size_t maxChunks = clusters / kSahChunk + kBigLevelTasks + 1;
    BVH_CHECK(sc.alloc(&big, kBigLevelTasks));
    BVH_CHECK(sc.alloc(&dChunks, maxChunks));
    BVH_CHECK(sc.alloc(&chunkLeft, maxChunks));
    std::vector<SahTask> hTasks;
    std::vector<SahChunk> hChunks;
    uint32_t count = 1, nextId = 1;
    int cur = 0, pin = 0;
    for (int level = 0; count > 0; ++level) {
        if (level > 64) {
            err = "binned-SAH top deeper than 64 levels";
            return SHIRO_ERR_DEVICE_CHECK;
        }
        uint32_t bigMin = 0;
        hChunks.clear();
        if (count <= kBigLevelTasks) {
            hTasks.resize(count);
            BVH_CHECK(cudaMemcpyAsync(hTasks.data(), tasks[cur], count * sizeof(SahTask), cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaStreamSynchronize(stream));
            for (uint32_t t = 0; t < count; ++t) {
                if (hTasks[t].end - hTasks[t].begin < kBigMin) continue;
                for (uint32_t b = hTasks[t].begin; b < hTasks[t].end; b += kSahChunk)
                    hChunks.push_back(SahChunk{t, b, std::min(b + kSahChunk, hTasks[t].end), b == hTasks[t].begin ? 1u : 0u});
            }
            if (!hChunks.empty()) bigMin = kBigMin;
        }
        k_sah_split<<<count, kSahBlock, 0, stream>>>(tasks[cur], items, perm[pin], perm[pin ^ 1], results, newTasks,
                                                     bigMin);
        BVH_CHECK(cudaGetLastError());
        if (bigMin) {
            const unsigned nc = static_cast<unsigned>(hChunks.size());
            if (nc > maxChunks) {
                err = "binned-SAH top: chunk list overflow";
                return SHIRO_ERR_DEVICE_CHECK;
            }
            BVH_CHECK(cudaMemcpyAsync(dChunks, hChunks.data(), nc * sizeof(SahChunk), cudaMemcpyHostToDevice, stream));
            k_big_init<<<count, 128, 0, stream>>>(big, count);
            k_big_bounds<<<nc, kSahBlock, 0, stream>>>(dChunks, items, perm[pin], big);
            k_big_bins<<<nc, kSahBlock, 0, stream>>>(dChunks, items, perm[pin], big);
            k_big_choose<<<count, 64, 0, stream>>>(big);
            k_big_count<<<nc, kSahBlock, 0, stream>>>(dChunks, tasks[cur], items, perm[pin], big, chunkLeft);
            k_big_offsets<<<blocks(count, 64), 64, 0, stream>>>(dChunks, nc, chunkLeft, big, count);
            k_big_scatter<<<nc, kSahBlock, 0, stream>>>(dChunks, tasks[cur], items, perm[pin], perm[pin ^ 1], big, chunkLeft,
                                                        results, newTasks);
            BVH_CHECK(cudaGetLastError());
        }
        size_t sb = scanBytes;
        BVH_CHECK(cub::DeviceScan::ExclusiveSum(scanTmp, sb, newTasks, taskPos, static_cast<int>(count), stream));
        uint32_t lastPos = 0, lastNew = 0;
        BVH_CHECK(cudaMemcpyAsync(&lastPos, taskPos + count - 1, 4, cudaMemcpyDeviceToHost, stream));
        BVH_CHECK(cudaMemcpyAsync(&lastNew, newTasks + count - 1, 4, cudaMemcpyDeviceToHost, stream));
        BVH_CHECK(cudaStreamSynchronize(stream));
        const uint32_t made = lastPos + lastNew;
        k_sah_children<<<blocks(count, 128), 128, 0, stream>>>(tasks[cur], count, results, taskPos, nextId, perm[pin ^ 1],
                                                               items, tasks[cur ^ 1], sahChild);
        BVH_CHECK(cudaGetLastError());
        nextId += made;
        count = made;
        cur ^= 1;
        pin ^= 1;
    }
    if (nextId != tops) {
        err = "binned-SAH top: node count mismatch";
        return SHIRO_ERR_DEVICE_CHECK;
    }
    k_sah_link<<<blocks(tops, 128), 128, 0, stream>>>(tops, sahChild, slots, items, child, nodeParent, leafParent);
    BVH_CHECK(cudaGetLastError());
    *topOut = top;
    return SHIRO_OK;
}

int build_bvh(const BvhInput& in, cudaStream_t stream, BvhOutput* out, std::string& err) {
    const uint32_t m = in.smallCount;
    const uint32_t L = static_cast<uint32_t>(in.largeSlots.size());
    const uint32_t total = m + L;
    if (total == 0) {
        err = "scene has no triangles";
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    if (total >= (1u << 28)) {
        err = "too many triangles for the leaf encoding (2^28)";
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    if (in.maxLeaf < 1 || in.maxLeaf > kMaxLeafLimit) {
        err = "leaf size out of range [1, 8]";
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    Scratch sc;
    float4* triOut = nullptr;
    BVH_CHECK(cudaMalloc(&triOut, 3 * sizeof(float4) * static_cast<size_t>(total)));
    out->tris = triOut;
    out->triCount = total;

    // Morton tree over the small triangles -------------------------------
    uint32_t* sortedPrim = nullptr;  // sorted position -> small prim index
    int2 *child = nullptr, *range = nullptr;
    int *nodeParent = nullptr, *leafParent = nullptr;
    float4* nodeBox = nullptr;
    float* nodeCost = nullptr;
    int* nodeCount = nullptr;
    uint8_t* collapse = nullptr;
    uint32_t emittedMorton = 0;
    bool mortonRootIsNode = false;
    float4 mortonLo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0), mortonHi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0);
    unsigned int depthHost = 0;
    uint32_t* flag = nullptr;
    uint32_t* newIndex = nullptr;
    const int nInternal = m >= 2 ? static_cast<int>(m) - 1 : 0;

    if (m > 0) {
        uint32_t* b6 = nullptr;
        uint64_t *keys = nullptr, *keysOut = nullptr;
        uint32_t* vals = nullptr;
        BVH_CHECK(sc.alloc(&b6, 6));
        BVH_CHECK(sc.alloc(&keys, m));
        BVH_CHECK(sc.alloc(&keysOut, m));
        BVH_CHECK(sc.alloc(&vals, m));
        BVH_CHECK(sc.alloc(&sortedPrim, m));
        const uint32_t init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
        BVH_CHECK(cudaMemcpyAsync(b6, init, sizeof(init), cudaMemcpyHostToDevice, stream));
        k_centroid_bounds<<<std::min(blocks(m, 256), 1024u), 256, 0, stream>>>(in.centroids, m, b6);
        k_morton<<<blocks(m, 256), 256, 0, stream>>>(in.centroids, m, b6, keys, vals);
        BVH_CHECK(cudaGetLastError());
        size_t tmpBytes = 0;
        BVH_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, tmpBytes, keys, keysOut, vals, sortedPrim, static_cast<int>(m), 0,
                                                  63, stream));
        void* tmp = nullptr;
        BVH_CHECK(sc.alloc(reinterpret_cast<uint8_t**>(&tmp), tmpBytes));
        BVH_CHECK(cub::DeviceRadixSort::SortPairs(tmp, tmpBytes, keys, keysOut, vals, sortedPrim, static_cast<int>(m), 0,
                                                  63, stream));
        if (nInternal > 0) {
            BVH_CHECK(sc.alloc(&child, nInternal));
            BVH_CHECK(sc.alloc(&range, nInternal));
            BVH_CHECK(sc.alloc(&nodeParent, nInternal));
            BVH_CHECK(sc.alloc(&leafParent, m));
            BVH_CHECK(sc.alloc(&nodeBox, 2 * static_cast<size_t>(nInternal)));
            BVH_CHECK(sc.alloc(&nodeCost, nInternal));
            BVH_CHECK(sc.alloc(&nodeCount, nInternal));
            BVH_CHECK(sc.alloc(&collapse, nInternal));
            unsigned int* arrivals = nullptr;
            unsigned int* maxDepth = nullptr;
            BVH_CHECK(sc.alloc(&arrivals, nInternal));
            BVH_CHECK(sc.alloc(&maxDepth, 1));
            BVH_CHECK(sc.alloc(&flag, nInternal));
            BVH_CHECK(sc.alloc(&newIndex, nInternal));
            BVH_CHECK(cudaMemsetAsync(arrivals, 0, sizeof(unsigned int) * nInternal, stream));
            BVH_CHECK(cudaMemsetAsync(maxDepth, 0, sizeof(unsigned int), stream));
            k_karras<<<blocks(nInternal, 256), 256, 0, stream>>>(keysOut, static_cast<int>(m), child, range, nodeParent,
                                                                  leafParent);
            k_bottom_up<<<blocks(m, 256), 256, 0, stream>>>(static_cast<int>(m), sortedPrim, in.primBoxes, child, nodeParent,
                                                             leafParent, arrivals, nodeBox, nodeCost, nodeCount, collapse,
                                                             static_cast<int>(in.maxLeaf), nullptr);
            BVH_CHECK(cudaGetLastError());
            if (in.sahClusterSize > 0 && m > in.sahClusterSize) {
                uint8_t* top = nullptr;
                int rc = sah_top(sc, static_cast<int>(m), nInternal, static_cast<int>(in.sahClusterSize), sortedPrim,
                                 in.primBoxes, child, range, nodeParent, leafParent, nodeBox, nodeCount, &top, stream, err);
                if (rc != SHIRO_OK) return rc;
                // boxes, counts, SAH costs and leaf decisions again, over the new top
                BVH_CHECK(cudaMemsetAsync(arrivals, 0, sizeof(unsigned int) * nInternal, stream));
                k_bottom_up<<<blocks(m, 256), 256, 0, stream>>>(static_cast<int>(m), sortedPrim, in.primBoxes, child,
                                                                 nodeParent, leafParent, arrivals, nodeBox, nodeCost,
                                                                 nodeCount, collapse, static_cast<int>(in.maxLeaf), top);
            }
            k_emit_flags<<<blocks(nInternal, 256), 256, 0, stream>>>(nInternal, nodeParent, collapse, flag, maxDepth);
            BVH_CHECK(cudaGetLastError());
            size_t scanBytes = 0;
            BVH_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, flag, newIndex, nInternal, stream));
            void* scanTmp = nullptr;
            BVH_CHECK(sc.alloc(reinterpret_cast<uint8_t**>(&scanTmp), scanBytes));
            BVH_CHECK(cub::DeviceScan::ExclusiveSum(scanTmp, scanBytes, flag, newIndex, nInternal, stream));
            uint32_t lastIdx = 0, lastFlag = 0;
            uint8_t rootCollapsed = 0;
            BVH_CHECK(cudaMemcpyAsync(&lastIdx, newIndex + nInternal - 1, 4, cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaMemcpyAsync(&lastFlag, flag + nInternal - 1, 4, cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaMemcpyAsync(&rootCollapsed, collapse, 1, cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaMemcpyAsync(&depthHost, maxDepth, 4, cudaMemcpyDeviceToHost, stream));
            float4 rb[2];
            BVH_CHECK(cudaMemcpyAsync(rb, nodeBox, sizeof(rb), cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaStreamSynchronize(stream));
            emittedMorton = lastIdx + lastFlag;
            mortonRootIsNode = rootCollapsed == 0;
            mortonLo = rb[0];
            mortonHi = rb[1];
        } else {
            // a single small triangle
            float4 pb[2];
            uint32_t p0 = 0;
            BVH_CHECK(cudaMemcpyAsync(&p0, sortedPrim, 4, cudaMemcpyDeviceToHost, stream));
            BVH_CHECK(cudaStreamSynchronize(stream));
            BVH_CHECK(cudaMemcpy(pb, in.primBoxes + 2 * p0, sizeof(pb), cudaMemcpyDeviceToHost));
            mortonLo = pb[0];
            mortonHi = pb[1];
        }
        k_write_tris<<<blocks(m, 256), 256, 0, stream>>>(m, sortedPrim, in.triData, triOut);
        BVH_CHECK(cudaGetLastError());
    }
    // large triangles follow the Morton-ordered ones
    float4 largeLo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0), largeHi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0);
    for (uint32_t k = 0; k < L; ++k) {
        const LargeTri& lt = in.largeSlots[k];
        BVH_CHECK(cudaMemcpyAsync(triOut + 3 * static_cast<size_t>(m + k), lt.tri, 3 * sizeof(float4), cudaMemcpyHostToDevice,
                                  stream));
        largeLo.x = std::min(largeLo.x, lt.lo[0]);
        largeLo.y = std::min(largeLo.y, lt.lo[1]);
        largeLo.z = std::min(largeLo.z, lt.lo[2]);
        largeHi.x = std::max(largeHi.x, lt.hi[0]);
        largeHi.y = std::max(largeHi.y, lt.hi[1]);
        largeHi.z = std::max(largeHi.z, lt.hi[2]);
    }

    // Node array: [top root if needed] + emitted Morton nodes -------------
    const bool mortonTree = m >= 2 && mortonRootIsNode;
    const bool needTop = !mortonTree || L > 0;
    const uint32_t offset = needTop ? 1u : 0u;
    const uint32_t nodeCountOut = offset + (mortonTree ? emittedMorton : 0u);
    float4* nodes = nullptr;
    BVH_CHECK(cudaMalloc(&nodes, 4 * sizeof(float4) * static_cast<size_t>(nodeCountOut)));
    out->nodes = nodes;
    out->nodeCount = nodeCountOut;
    if (mortonTree) {
        k_emit_nodes<<<blocks(nInternal, 256), 256, 0, stream>>>(nInternal, flag, newIndex, offset, child, range, collapse,
                                                                  nodeBox, sortedPrim, in.primBoxes, nodes);
        BVH_CHECK(cudaGetLastError());
    }
    const float4 emptyLo = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0), emptyHi = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0);
    const int emptyLink = leaf_link_host(0, 1);
    if (needTop) {
        int l0 = emptyLink, l1 = emptyLink;
        float4 b0lo = emptyLo, b0hi = emptyHi, b1lo = emptyLo, b1hi = emptyHi;
        if (m > 0) {
            b0lo = mortonLo;
            b0hi = mortonHi;
            l0 = mortonTree ? 1 : leaf_link_host(0, static_cast<int>(m));
        }
        if (L > 0) {
            b1lo = largeLo;
            b1hi = largeHi;
            l1 = leaf_link_host(static_cast<int>(m), static_cast<int>(L));
        }
        k_write_root<<<1, 1, 0, stream>>>(nodes, b0lo, b0hi, l0, b1lo, b1hi, l1);
        BVH_CHECK(cudaGetLastError());
    }
    BVH_CHECK(cudaStreamSynchronize(stream));
    out->depth = depthHost + offset + 1u;
    out->maxLeaf = in.maxLeaf;
    return SHIRO_OK;
}

namespace {

struct Entry {
    int link;  // >= 0 binary node, < 0 binary leaf link
    float lo[3], hi[3];
};

__device__ __forceinline__ float entry_area(const Entry& e) {
    const float dx = e.hi[0] - e.lo[0], dy = e.hi[1] - e.lo[1], dz = e.hi[2] - e.lo[2];
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__device__ __forceinline__ int leaf_count(int link) { return static_cast<int>((~static_cast<uint32_t>(link)) & 7u) + 1; }

__device__ __forceinline__ void node2_children(const float4* nodes2, int n, Entry* a, Entry* b) {
    const float4 n0 = nodes2[4 * static_cast<size_t>(n)], n1 = nodes2[4 * static_cast<size_t>(n) + 1];
    const float4 n2 = nodes2[4 * static_cast<size_t>(n) + 2], n3 = nodes2[4 * static_cast<size_t>(n) + 3];
    a->link = __float_as_int(n3.x);
    a->lo[0] = n0.x; a->hi[0] = n0.y; a->lo[1] = n0.z; a->hi[1] = n0.w; a->lo[2] = n2.x; a->hi[2] = n2.y;
    b->link = __float_as_int(n3.y);
    b->lo[0] = n1.x; b->hi[0] = n1.y; b->lo[1] = n1.z; b->hi[1] = n1.w; b->lo[2] = n2.z; b->hi[2] = n2.w;
}

// ---- slot assignment by dynamic programming ----------------------------------
// Which binary nodes become wide nodes is chosen to minimise a surface-area
// cost (the optimal collapse of Ylitie, Karras and Laine 2017, restated):
// G(n, k) is the least cost of representing the subtree of binary node n with
// at most k child slots of a wide node,
//   G(n, 1)  = kWideNodeCost * area(n) + S(n, 8)       (n becomes a wide node)
//   G(n, k)  = min(G(n, k - 1), S(n, k))               (k >= 2: n is opened)
//   S(n, k)  = min over j of Gc(left, j) + Gc(right, k - j)
// where Gc of a binary leaf is kWideTriCost * area * triangles for any k.
// Costs are evaluated bottom-up (a node after both children), decisions are
// kept per (node, k) and replayed top-down by k_collapse_wide.
constexpr float kWideNodeCost = 1.0f;
constexpr float kWideTriCost = 0.3f;

struct WideDp {
    float* G;            // [node][8]: G(n, k + 1)
    uint8_t* split;      // [node][8]: best j of S(n, k + 1) (k >= 1)
    uint8_t* keep;       // [node]: bit k set when G(n, k + 1) = G(n, k)
    int* parent;         // binary parent (-1: root)
    unsigned int* ready; // children whose costs are known
    uint8_t* start;      // both children are leaves / absent
};

__global__ void k_wide_parents(const float4* __restrict__ nodes2, uint32_t n2, WideDp dp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    Entry a, b;
    node2_children(nodes2, static_cast<int>(i), &a, &b);
    unsigned int known = 0;
    for (const Entry* e : {&a, &b}) {
        if (e->lo[0] > e->hi[0] || e->link < 0) {
            ++known;
        } else {
            dp.parent[e->link] = static_cast<int>(i);
        }
    }
    dp.ready[i] = known;
    dp.start[i] = known == 2 ? 1 : 0;
}

// Gc(child, j) for j = 1..8 into g[0..7].
__device__ __forceinline__ void child_costs(const WideDp& dp, const Entry& e, float g[8]) {
    if (e.lo[0] > e.hi[0]) {
        for (int j = 0; j < 8; ++j) g[j] = 0.0f;
    } else if (e.link < 0) {
        const float c = kWideTriCost * entry_area(e) * static_cast<float>(leaf_count(e.link));
        for (int j = 0; j < 8; ++j) g[j] = c;
    } else {
        for (int j = 0; j < 8; ++j) g[j] = __ldcg(&dp.G[8 * static_cast<size_t>(e.link) + j]);
    }
}

__global__ void k_wide_costs(const float4* __restrict__ nodes2, uint32_t n2, WideDp dp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2 || !dp.start[i]) return;
    int n = static_cast<int>(i);
    for (;;) {
        Entry a, b;
        node2_children(nodes2, n, &a, &b);
        float ga[8], gb[8];
        child_costs(dp, a, ga);
        child_costs(dp, b, gb);
        float S[9];
        uint8_t js[9];
        for (int k = 2; k <= 8; ++k) {
            float best = FLT_MAX;
            uint8_t bj = 1;
            for (int j = 1; j < k; ++j) {
                const float c = ga[j - 1] + gb[k - j - 1];
                if (c < best) {
                    best = c;
                    bj = static_cast<uint8_t>(j);
                }
            }
            S[k] = best;
            js[k] = bj;
        }
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(a.lo[k] <= a.hi[k] ? a.lo[k] : FLT_MAX, b.lo[k] <= b.hi[k] ? b.lo[k] : FLT_MAX);
            hi[k] = fmaxf(a.lo[k] <= a.hi[k] ? a.hi[k] : -FLT_MAX, b.lo[k] <= b.hi[k] ? b.hi[k] : -FLT_MAX);
        }
        const float area = 2.0f * ((hi[0] - lo[0]) * (hi[1] - lo[1]) + (hi[1] - lo[1]) * (hi[2] - lo[2]) +
                                   (hi[2] - lo[2]) * (hi[0] - lo[0]));
        float* G = dp.G + 8 * static_cast<size_t>(n);
        uint8_t* sp = dp.split + 8 * static_cast<size_t>(n);
        float prev = kWideNodeCost * area + S[8];
        G[0] = prev;
        sp[0] = js[8];  // the split of n as a wide node
        uint8_t keep = 0;
        for (int k = 2; k <= 8; ++k) {
            if (S[k] < prev) {
                prev = S[k];
                sp[k - 1] = js[k];
            } else {
                keep |= static_cast<uint8_t>(1u << (k - 1));
                sp[k - 1] = 0;
            }
            G[k - 1] = prev;
        }
        dp.keep[n] = keep;
        __threadfence();
        const int p = dp.parent[n];
        if (p < 0) break;
        if (atomicAdd(&dp.ready[p], 1u) != 1u) break;
        __threadfence();
        n = p;
    }
}

// One thread per task (binary node -> wide node).  The wide node's internal
// children get consecutive wide-node indices from `nodeCounter` and become
// the next level's tasks; its leaf children's triangles get consecutive
// slots of the wide triangle array from `triCounter` and are copied there.
__global__ void k_collapse_wide(const float4* __restrict__ nodes2, const float4* __restrict__ tris2,
                                const int2* __restrict__ tasks, uint32_t taskCount, int2* __restrict__ nextTasks,
                                unsigned int* __restrict__ nextCount, unsigned int* __restrict__ nodeCounter,
                                unsigned int* __restrict__ triCounter, float4* __restrict__ out,
                                float4* __restrict__ trisOut, WideDp dp) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= taskCount) return;
    const int2 task = tasks[t];
    // the slots of this wide node: replay the cost table's decisions from
    // binary node task.x with 8 slots
    Entry e[8];
    int n = 0, tris = 0;
    {
        struct Pending {
            Entry e;
            int k;
        };
        Pending st[16];
        int sp = 0;
        Entry a, b;
        node2_children(nodes2, task.x, &a, &b);
        const int j0 = dp.split[8 * static_cast<size_t>(task.x)];
        st[sp++] = {a, j0};
        st[sp++] = {b, 8 - j0};
        while (sp > 0) {
            const Pending pe = st[--sp];
            if (pe.e.lo[0] > pe.e.hi[0]) continue;  // absent child
            if (pe.e.link < 0 || n + sp >= 8) {
                if (n < 8) e[n++] = pe.e;
                continue;
            }
            int k = pe.k;
            const uint8_t keep = dp.keep[pe.e.link];
            while (k > 1 && ((keep >> (k - 1)) & 1u)) --k;
            if (k <= 1) {
                if (n < 8) e[n++] = pe.e;  // its own wide node
                continue;
            }
            const int j = dp.split[8 * static_cast<size_t>(pe.e.link) + (k - 1)];
            Entry ca, cb;
            node2_children(nodes2, pe.e.link, &ca, &cb);
            st[sp++] = {ca, j};
            st[sp++] = {cb, k - j};
        }
        for (int i = 0; i < n; ++i)
            if (e[i].link < 0) tris += leaf_count(e[i].link);
    }
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], e[i].lo[k]);
            hi[k] = fmaxf(hi[k], e[i].hi[k]);
        }
    // slot s takes the child lying most in direction D(s) from the centre
    // (greedy assignment by decreasing projection)
    int slotOf[8];
    int childIn[8];
    for (int s = 0; s < 8; ++s) childIn[s] = -1;
    {
        float proj[8][8];
        for (int i = 0; i < n; ++i) {
            float c[3];
            for (int k = 0; k < 3; ++k) c[k] = 0.5f * (e[i].lo[k] + e[i].hi[k]) - 0.5f * (lo[k] + hi[k]);
            for (int s = 0; s < 8; ++s)
                proj[i][s] = ((s & 1) ? -c[0] : c[0]) + ((s & 2) ? -c[1] : c[1]) + ((s & 4) ? -c[2] : c[2]);
            slotOf[i] = -1;
        }
        for (int r = 0; r < n; ++r) {
            int bi = -1, bs = -1;
            float bv = -FLT_MAX;
            for (int i = 0; i < n; ++i) {
                if (slotOf[i] >= 0) continue;
                for (int s = 0; s < 8; ++s)
                    if (childIn[s] < 0 && (bi < 0 || proj[i][s] > bv)) {
                        bv = proj[i][s];
                        bi = i;
                        bs = s;
                    }
            }
            slotOf[bi] = bs;
            childIn[bs] = bi;
        }
    }
    // Per axis a power-of-two scale with extent / scale <= 252 and the
    // quantisation origin one step below the node box.  Every child box is
    // widened by one step on each side: the traversal folds the float
    // conversion of the 8-bit plane into its FMA (bias 2^23 * scale * inv),
    // which can err by half a step.
    uint32_t ex[3];
    float sc[3];
    for (int k = 0; k < 3; ++k) {
        const float ext = __fsub_ru(hi[k], lo[k]);
        int eb = 1;  // smallest normal exponent
        if (ext > 0.0f) {
            int e2;
            frexpf(ext / 252.0f, &e2);  // ext/252 < 2^e2
            eb = min(max(e2 + 127, 1), 254);
        }
        ex[k] = static_cast<uint32_t>(eb);
        sc[k] = __uint_as_float(static_cast<uint32_t>(eb) << 23);
        while (__fmul_ru(252.0f, sc[k]) < ext && ex[k] < 254) {  // guard the rounding of ext / 252
            ++ex[k];
            sc[k] = __uint_as_float(ex[k] << 23);
        }
        lo[k] = __fsub_rd(lo[k], sc[k]);
    }
    int inner = 0;
    for (int i = 0; i < n; ++i) inner += e[i].link >= 0 ? 1 : 0;
    const uint32_t childBase = inner ? atomicAdd(nodeCounter, static_cast<unsigned int>(inner)) : 0u;
    const uint32_t triBase = tris ? atomicAdd(triCounter, static_cast<unsigned int>(tris)) : 0u;
    uint8_t q[6][8];
    uint8_t meta[8];
    uint32_t imask = 0;
    int rank = 0, off = 0;
    for (int s = 0; s < 8; ++s) {
        const int i = childIn[s];
        if (i < 0) {
            meta[s] = static_cast<uint8_t>(kWideEmptyMeta);
            for (int k = 0; k < 3; ++k) {
                q[k][s] = 255;
                q[3 + k][s] = 0;
            }
            continue;
        }
        for (int k = 0; k < 3; ++k) {
            const float a = floorf(__fdiv_rd(__fsub_rd(e[i].lo[k], lo[k]), sc[k])) - 1.0f;
            const float b = ceilf(__fdiv_ru(__fsub_ru(e[i].hi[k], lo[k]), sc[k])) + 1.0f;
            q[k][s] = static_cast<uint8_t>(fminf(fmaxf(a, 0.0f), 255.0f));
            q[3 + k][s] = static_cast<uint8_t>(fminf(fmaxf(b, 0.0f), 255.0f));
        }
        if (e[i].link >= 0) {
            imask |= 1u << s;
            meta[s] = 0;
            const unsigned int slot = atomicAdd(nextCount, 1u);
            nextTasks[slot] = make_int2(e[i].link, static_cast<int>(childBase) + rank);
            ++rank;
        } else {
            const uint32_t enc = ~static_cast<uint32_t>(e[i].link);
            const uint32_t first = enc >> 3, cnt = (enc & 7u) + 1u;
            meta[s] = static_cast<uint8_t>(((cnt - 1u) << 5) | static_cast<uint32_t>(off));
            for (uint32_t k = 0; k < cnt; ++k) {
                const size_t src = 3 * static_cast<size_t>(first + k), dst = 3 * (static_cast<size_t>(triBase) + off + k);
                trisOut[dst] = tris2[src];
                trisOut[dst + 1] = tris2[src + 1];
                trisOut[dst + 2] = tris2[src + 2];
            }
            off += static_cast<int>(cnt);
        }
    }
    float4* o = out + 5 * static_cast<size_t>(task.y);
    o[0] = make_float4(lo[0], lo[1], lo[2], __uint_as_float(ex[0] | (ex[1] << 8) | (ex[2] << 16) | (imask << 24)));
    const uint32_t m0 = meta[0] | (meta[1] << 8) | (meta[2] << 16) | (static_cast<uint32_t>(meta[3]) << 24);
    const uint32_t m1 = meta[4] | (meta[5] << 8) | (meta[6] << 16) | (static_cast<uint32_t>(meta[7]) << 24);
    o[1] = make_float4(__uint_as_float(childBase), __uint_as_float(triBase), __uint_as_float(m0), __uint_as_float(m1));
    uint32_t w[12];
    for (int r = 0; r < 6; ++r) {
        w[2 * r] = q[r][0] | (q[r][1] << 8) | (q[r][2] << 16) | (static_cast<uint32_t>(q[r][3]) << 24);
        w[2 * r + 1] = q[r][4] | (q[r][5] << 8) | (q[r][6] << 16) | (static_cast<uint32_t>(q[r][7]) << 24);
    }
    o[2] = make_float4(__uint_as_float(w[0]), __uint_as_float(w[1]), __uint_as_float(w[2]), __uint_as_float(w[3]));
    o[3] = make_float4(__uint_as_float(w[4]), __uint_as_float(w[5]), __uint_as_float(w[6]), __uint_as_float(w[7]));
    o[4] = make_float4(__uint_as_float(w[8]), __uint_as_float(w[9]), __uint_as_float(w[10]), __uint_as_float(w[11]));
}

}  // namespace

int collapse_wide(const float4* nodes2, uint32_t nodeCount2, const float4* tris2, uint32_t triCount2, cudaStream_t stream,
                  WideOutput* out, std::string& err) {
    Scratch sc;
    int2 *ta = nullptr, *tb = nullptr;
    unsigned int* cnt = nullptr;  // [0] node counter, [1] next task count, [2] triangle counter
    const uint32_t cap = std::max<uint32_t>(nodeCount2, 1);
    BVH_CHECK(sc.alloc(&ta, cap));
    BVH_CHECK(sc.alloc(&tb, cap));
    BVH_CHECK(sc.alloc(&cnt, 3));
    float4* nodes = nullptr;
    BVH_CHECK(cudaMalloc(&nodes, 5 * sizeof(float4) * static_cast<size_t>(cap)));
    out->nodes = nodes;
    float4* tris = nullptr;
    BVH_CHECK(cudaMalloc(&tris, 3 * sizeof(float4) * static_cast<size_t>(std::max<uint32_t>(triCount2, 1))));
    out->tris = tris;
    // cost table of the slot assignment (bottom-up over the binary tree)
    WideDp dp;
    BVH_CHECK(sc.alloc(&dp.G, 8 * static_cast<size_t>(cap)));
    BVH_CHECK(sc.alloc(&dp.split, 8 * static_cast<size_t>(cap)));
    BVH_CHECK(sc.alloc(&dp.keep, cap));
    BVH_CHECK(sc.alloc(&dp.parent, cap));
    BVH_CHECK(sc.alloc(&dp.ready, cap));
    BVH_CHECK(sc.alloc(&dp.start, cap));
    BVH_CHECK(cudaMemsetAsync(dp.parent, 0xff, sizeof(int) * cap, stream));
    k_wide_parents<<<blocks(nodeCount2, 128), 128, 0, stream>>>(nodes2, nodeCount2, dp);
    k_wide_costs<<<blocks(nodeCount2, 128), 128, 0, stream>>>(nodes2, nodeCount2, dp);
    BVH_CHECK(cudaGetLastError());
    const int2 root = make_int2(0, 0);
    const unsigned int init[3] = {1u, 0u, 0u};
    BVH_CHECK(cudaMemcpyAsync(ta, &root, sizeof(root), cudaMemcpyHostToDevice, stream));
    BVH_CHECK(cudaMemcpyAsync(cnt, init, sizeof(init), cudaMemcpyHostToDevice, stream));
    uint32_t tasks = 1, depth = 0;
    unsigned int h[3] = {0, 0, 0};
    while (tasks > 0) {
        k_collapse_wide<<<blocks(tasks, 128), 128, 0, stream>>>(nodes2, tris2, ta, tasks, tb, cnt + 1, cnt, cnt + 2, nodes,
                                                                 tris, dp);
        BVH_CHECK(cudaGetLastError());
        BVH_CHECK(cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, stream));
        BVH_CHECK(cudaMemsetAsync(cnt + 1, 0, sizeof(unsigned int), stream));
        BVH_CHECK(cudaStreamSynchronize(stream));
        tasks = h[1];
        out->nodeCount = h[0];
        std::swap(ta, tb);
        ++depth;
        if (depth > 64) {
            err = "wide BVH collapse did not terminate";
            return SHIRO_ERR_INVALID_ARGUMENT;
        }
    }
    if (h[2] != triCount2) {
        err = "wide BVH collapse lost triangles";
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    out->triCount = h[2];
    out->depth = depth;
    return SHIRO_OK;
}

}  // namespace shiro_gpu
