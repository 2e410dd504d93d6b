// wavefront.cu - the batched wavefront form.
//
// The reference has no wavefront path (its README and docs list one only as
// planned).  This form renders many requests (views / frames of uneven
// resolution, spp and depth) in one call, against one resident scene, with
// the estimator of integrator.cuh split into stages over a pool of paths:
//
//   generate : camera rays of the wave's paths                -> ray queue
//   extend   : closest hit of every queued ray
//   shade    : miss / hit shading, light samples (+ their
//              contributions), continuation & Russian roulette -> next ray queue,
//                                                               shadow queue
//   shadow   : occlusion of each queued path's light samples,
//              in-order sum of the visible contributions
//   resolve  : per-pixel average of the wave's path records
//
// Paths are packed into waves of at most `paths_in_flight` paths (whole
// pixels; a wave may span several requests).  One wave is one CUDA graph -
// generate, max-depth x (extend, shade, shadow, bookkeeping), resolve - and
// the graph is replayed for every wave; the stage kernels are persistent
// (grid sized to the resident capacity) and read their queue lengths from
// device memory, so nothing returns to the host between bounces.  Queue
// slots are claimed with warp-aggregated atomics (one atomicAdd per warp).
//
// Every float of a path is produced by the same integrator.cuh functions as
// the plain form, in the same order, so results are bit-identical to
// shiro_gpu_render.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <functional>
#include <vector>

#include "adjoint.cuh"
#include "context.h"
#include "integrator.cuh"

namespace shiro_gpu {

namespace {

struct WaveSeg {
    uint32_t req;
    uint32_t pixelStart;
    uint32_t pixelCount;
    uint32_t pathOffset;   // first path of the segment within the wave
    uint32_t pixelOffset;  // first pixel of the segment within the wave
    uint32_t pad[3];
};

struct WaveDesc {
    uint32_t segBegin, segCount;
    uint32_t paths, pixels;
};

struct WfRequest {
    DevRequest q;
    AovPtrs aov;
};

// State flag bits (T.w): diffuse depth (bits 0-7), specular depth (8-15),
// previous bounce delta, path done, previous bounce type (18-19), inside a
// transmissive object, its medium attenuating.
constexpr uint32_t kFlagPrevDelta = 1u << 16;
constexpr uint32_t kFlagDone = 1u << 17;
constexpr uint32_t kTypeShift = 18;
constexpr uint32_t kFlagInside = 1u << 20;
constexpr uint32_t kFlagMedium = 1u << 21;

__device__ __forceinline__ uint32_t pack_state(const PathState& ps) {
    return (ps.diffDepth & 0xffu) | ((ps.specDepth & 0xffu) << 8) | (ps.prevDelta ? kFlagPrevDelta : 0u) |
           ((ps.prevType & 3u) << kTypeShift) | (ps.inside ? kFlagInside : 0u) | (ps.mediumActive ? kFlagMedium : 0u);
}

// Work-fetch counters of the persistent stages (slots of WfView::counters).
constexpr uint32_t kFetchExtend = 5, kFetchShade = 6, kFetchOcclude = 7;
// Lengths of the two halves of the shade queue: hits fill it from the front,
// misses from the back.
constexpr uint32_t kHitCount = 8, kMissCount = 9;

struct WfView {
    // path state, one entry per slot of the wave
    float4* ro;      // ro.xyz, unused
    float4* rd;      // rd.xyz, prevPdf
    float4* T;       // T.xyz, bits: diffDepth | specDepth << 8 | flags
    float4* rad;     // radiance.xyz, first-hit depth
    uint4* ident;    // px, py, sample index, request
    float4* hit;     // t, u, v, slot bits
    float4* medium;  // extinction of the medium the path is in (while it attenuates)
    uint32_t* hitGid;
    // shadow records
    float4* shOrigin;  // origin.xyz
    float4* shT;       // throughput at the vertex
    float4* shDir;     // [lightSamples][P]: dir.xyz, reach of the shadow ray (0: no sample / occluded)
    float4* shC;       // [lightSamples][P]: contribution
    uint32_t* rayQ0;
    uint32_t* rayQ1;
    uint32_t* shadowQ;     // paths with light samples to accumulate
    uint32_t* shadowRayQ;  // one item per light sample to test: slot << 3 | sample
    uint32_t* shadeQ;      // rays after extend: hits from the front, misses from the back
    uint32_t* counters;  // 0: ray count A, 1: ray count B, 2: shadow paths, 3: wave index, 4: shadow rays,
                         // 5-7: work fetch, 8: hits, 9: misses
    float4* records;     // 3 per slot
    const WaveDesc* waves;
    const WaveSeg* segs;
    const WfRequest* reqs;
    uint32_t P;
    uint32_t lightSamples;
    int travSteps;     // wide-BVH nodes per lane between refills
    int refillIdle;    // idle lanes that trigger a refill
    uint32_t waveStride;  // waves in flight at once: this pool runs waves k, k + stride, ...
    // queue binning: bucket counters / offsets, the binned queue, and the map
    // of a ray origin to its cell (cell = (o - binLo) * binScale, 8 per axis)
    uint32_t* binCount;
    uint32_t* sortedQ;
    V3 binLo, binScale;
    // non-NULL: instead of resolving pixels, the wave's path records go out
    // per path (radiance, first-hit depth) in request path order
    float4* recordsOut;
    // non-NULL (adjoint waves): the forward stages log, per bounce and slot
    // ([depth][P]), the hit record, the hit triangle and the mask of light
    // samples that were taken and unoccluded; the replay reads them instead
    // of tracing its rays again
    float4* hitLog;
    uint32_t* gidLog;
    uint8_t* visLog;
};

// Buckets of the queue binning: light sample (8) x direction octant (8) x
// origin cell (8 x 8 x 8, Morton-interleaved).
constexpr uint32_t kBins = 8u * 8u * 512u;

// Per-slot state of the adjoint replay, which runs in a wave after the
// wave's forward stages, on the same pool, queues and slots (each path's
// forward record, its total radiance, is still in its slot).
struct AdjWave {
    const AdjView* view;  // device copy (gradient buffers, d_beauty, dome 0's texture), written per call
    float4* lrem;         // radiance of the path not yet accounted for
    float4* delta;        // d loss / d path radiance: d_beauty of its pixel / spp
    float4* vtx;          // 3 per slot: (shading normal, material bits), (coat normal), (view direction)
    float4* cont;         // 2 per slot: (continuation direction, 1 when its gradient is due), (its BSDF value)
    float4* lgrad;        // 3 per light sample and slot, [k][P]: (L w s), (f R w s, 1 for dome 0's texture), (local dir)
    uint32_t on;          // replay stages follow the forward ones
    uint32_t pad;
};
constexpr size_t kAdjSlotFloat4 = 7;      // lrem, delta, vtx (3), cont (2)
constexpr size_t kAdjLightFloat4 = 3;     // per light sample

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

// Appends `item` to a queue when `pred`; one atomicAdd per warp.
__device__ __forceinline__ void warp_push(uint32_t* counter, uint32_t* queue, bool pred, uint32_t item) {
    const uint32_t active = __activemask();
    const uint32_t ballot = __ballot_sync(active, pred);
    if (ballot == 0u) return;
    const uint32_t leader = __ffs(active) - 1u;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, static_cast<uint32_t>(__popc(ballot)));
    base = __shfl_sync(active, base, leader);
    if (pred) queue[base + __popc(ballot & ((1u << lane_id()) - 1u))] = item;
}

// Appends (j << 3 | k) for every bit k < n of `mask` to one queue with a
// single atomicAdd per warp: the warp's entries of sample 0, then of sample
// 1, ... (the order of per-sample pushes, without their atomics).
__device__ __forceinline__ void warp_push_samples(uint32_t* counter, uint32_t* queue, uint32_t mask, uint32_t n,
                                                  uint32_t j) {
    const uint32_t active = __activemask();
    uint32_t total = 0;
    for (uint32_t k = 0; k < n; ++k) total += __popc(__ballot_sync(active, (mask >> k) & 1u));
    if (total == 0u) return;
    const uint32_t leader = __ffs(active) - 1u;
    uint32_t base = 0;
    if (lane_id() == leader) base = atomicAdd(counter, total);
    base = __shfl_sync(active, base, leader);
    const uint32_t lt = (1u << lane_id()) - 1u;
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t b = __ballot_sync(active, (mask >> k) & 1u);
        if ((mask >> k) & 1u) queue[base + __popc(b & lt)] = (j << 3) | k;
        base += __popc(b);
    }
}

__device__ __forceinline__ const WaveDesc& cur_wave(const WfView& v) { return v.waves[v.counters[3]]; }

__device__ __forceinline__ const WaveSeg& find_seg(const WfView& v, const WaveDesc& w, uint32_t j, bool byPixel) {
    uint32_t lo = w.segBegin, hi = w.segBegin + w.segCount - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        const uint32_t key = byPixel ? v.segs[mid].pixelOffset : v.segs[mid].pathOffset;
        if (key <= j) lo = mid; else hi = mid - 1u;
    }
    return v.segs[lo];
}

__device__ __forceinline__ uint32_t bin_key(const WfView& v, const float4& o, const float4& d, uint32_t k) {
    const float f[3] = {(o.x - v.binLo.x) * v.binScale.x, (o.y - v.binLo.y) * v.binScale.y,
                        (o.z - v.binLo.z) * v.binScale.z};
    uint32_t c[3];
    for (int a = 0; a < 3; ++a) {
        const float x = f[a] < 0.0f ? 0.0f : (f[a] > 7.0f ? 7.0f : f[a]);  // NaN -> 7
        c[a] = static_cast<uint32_t>(x);
    }
    uint32_t cell = 0;
    for (int b = 0; b < 3; ++b) cell |= (((c[0] >> b) & 1u) << (3 * b + 2)) | (((c[1] >> b) & 1u) << (3 * b + 1)) |
                                        (((c[2] >> b) & 1u) << (3 * b));
    const uint32_t oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    return ((k & 7u) << 12) | (oct << 9) | cell;
}

// Queue binning (a counting sort into kBins buckets; the order inside a
// bucket is whatever the atomics give - every path's result is independent
// of the order its ray is traced in).  which = 0: the closest-hit queue
// `cur`, 1: the occlusion queue.  Lanes with equal keys add with one atomic.
__device__ __forceinline__ void bin_item(const WfView& v, uint32_t which, uint32_t item, uint32_t* key) {
    if (which) {
        const uint32_t j = item >> 3, k = item & 7u;
        *key = bin_key(v, v.shOrigin[j], v.shDir[static_cast<size_t>(k) * v.P + j], k);
    } else {
        *key = bin_key(v, v.ro[item], v.rd[item], 0u);
    }
}

__global__ void __launch_bounds__(256) wf_bin_count(WfView v, uint32_t which, uint32_t cur) {
    const uint32_t count = which ? v.counters[4] : v.counters[cur];
    const uint32_t* q = which ? v.shadowRayQ : (cur ? v.rayQ1 : v.rayQ0);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < count;
        uint32_t key = 0xffffffffu;
        if (valid) bin_item(v, which, q[i], &key);
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        if (valid && (threadIdx.x & 31u) == static_cast<uint32_t>(__ffs(peers) - 1))
            atomicAdd(&v.binCount[key], static_cast<uint32_t>(__popc(peers)));
    }
}

// Counts -> exclusive offsets, one block of 1024 threads, 32 buckets each.
__global__ void __launch_bounds__(1024) wf_bin_scan(WfView v) {
    __shared__ uint32_t warpSum[32];
    constexpr uint32_t per = kBins / 1024u;
    uint32_t* c = v.binCount + threadIdx.x * per;
    uint32_t local[per];
    uint32_t sum = 0;
    for (uint32_t k = 0; k < per; ++k) {
        local[k] = c[k];
        sum += local[k];
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= static_cast<uint32_t>(o)) x += y;
    }
    if (lane == 31u) warpSum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warpSum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= static_cast<uint32_t>(o)) w += y;
        }
        warpSum[lane] = w;
    }
    __syncthreads();
    uint32_t run = (warp > 0 ? warpSum[warp - 1] : 0u) + x - sum;
    for (uint32_t k = 0; k < per; ++k) {
        c[k] = run;
        run += local[k];
    }
}

__global__ void __launch_bounds__(256) wf_bin_scatter(WfView v, uint32_t which, uint32_t cur) {
    const uint32_t count = which ? v.counters[4] : v.counters[cur];
    const uint32_t* q = which ? v.shadowRayQ : (cur ? v.rayQ1 : v.rayQ0);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t lane = threadIdx.x & 31u;
    for (uint32_t base = blockIdx.x * blockDim.x; base < count; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < count;
        uint32_t key = 0xffffffffu, item = 0;
        if (valid) {
            item = q[i];
            bin_item(v, which, item, &key);
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, key);
        const uint32_t leader = static_cast<uint32_t>(__ffs(peers) - 1);
        uint32_t pos = 0;
        if (valid && lane == leader) pos = atomicAdd(&v.binCount[key], static_cast<uint32_t>(__popc(peers)));
        pos = __shfl_sync(peers, pos, leader);
        if (valid) v.sortedQ[pos + __popc(peers & ((1u << lane) - 1u))] = item;
    }
}

__global__ void wf_begin(WfView v) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const uint32_t w = v.counters[3] + v.waveStride;
        v.counters[3] = w;
        v.counters[0] = v.waves[w].paths;
        v.counters[1] = 0u;
        v.counters[2] = 0u;
        v.counters[4] = 0u;
        v.counters[kFetchExtend] = 0u;
        v.counters[kFetchShade] = 0u;
        v.counters[kFetchOcclude] = 0u;
        v.counters[kHitCount] = 0u;
        v.counters[kMissCount] = 0u;
    }
}

__global__ void __launch_bounds__(128) wf_generate(WfView v) {
    const WaveDesc w = cur_wave(v);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < w.paths; j += gridDim.x * blockDim.x) {
        const WaveSeg& sg = find_seg(v, w, j, false);
        const DevRequest& q = v.reqs[sg.req].q;
        const uint32_t local = j - sg.pathOffset;
        const uint32_t pix = sg.pixelStart + local / q.sampleCount;
        const uint32_t smpIdx = q.sampleStart + (local - (local / q.sampleCount) * q.sampleCount);
        const uint32_t y = pix / q.width, x = pix - y * q.width;
        const Sampler smp{x, y, smpIdx};
        PathState ps;
        init_path(q, smp, ps);
        v.ro[j] = make_float4(ps.ro.x, ps.ro.y, ps.ro.z, 0.0f);
        v.rd[j] = make_float4(ps.rd.x, ps.rd.y, ps.rd.z, ps.prevPdf);
        v.T[j] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(kFlagPrevDelta));
        v.rad[j] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(0x7f800000));
        v.ident[j] = make_uint4(x, y, smpIdx, sg.req);
        v.rayQ0[j] = j;  // albedo / normal records are written by a first hit and read only after one

    }
}

// Persistent warps take their next 32 queue entries from a per-stage counter
// (reset by wf_begin / wf_end_bounce), so rays of very different cost do not
// leave an SM idle behind one slow block.  Returns the first entry for the warp.
__device__ __forceinline__ uint32_t warp_fetch(uint32_t* counter) {
    uint32_t base = 0;
    if (lane_id() == 0) base = atomicAdd(counter, 32u);
    return __shfl_sync(0xffffffffu, base, 0);
}

// Claims a slot per predicated lane of the (converged) warp; one atomicAdd.
__device__ __forceinline__ uint32_t warp_claim(uint32_t* counter, bool pred) {
    const uint32_t ballot = __ballot_sync(0xffffffffu, pred);
    uint32_t base = 0;
    if (ballot != 0u && lane_id() == 0) base = atomicAdd(counter, static_cast<uint32_t>(__popc(ballot)));
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + __popc(ballot & ((1u << lane_id()) - 1u));
}

// Lane-level work distribution for the wide-BVH traversal.  A warp claims
// kFetchChunk queue entries with one atomicAdd and hands them to its lanes;
// once `refillIdle` lanes have finished their rays they take the next
// entries, so a warp is not held back by its slowest ray.  Between refills a
// busy lane visits up to `travSteps` wide nodes (each visit is the same
// 8-child test for every lane, so lanes at different depths still run it
// together).
constexpr uint32_t kFull = 0xffffffffu;
constexpr uint32_t kFetchChunk = 64;

struct LaneFeed {
    uint32_t next = 0, end = 0;  // the warp's claimed entries [next, end)
    bool exhausted = false;
};

// Assigns queue entries to idle lanes (`has` false); warp-uniform call.
// Returns the entry index this lane received, or 0xffffffff.
__device__ __forceinline__ uint32_t feed_lanes(LaneFeed& f, uint32_t* counter, uint32_t count, bool has, int refillIdle) {
    const uint32_t lane = lane_id();
    uint32_t got = 0xffffffffu;
    uint32_t idle = __ballot_sync(kFull, !has);
    if (f.exhausted || __popc(idle) < refillIdle) return got;
    while (idle != 0u) {
        if (f.next >= f.end) {
            uint32_t b = 0;
            if (lane == 0) b = atomicAdd(counter, kFetchChunk);
            b = __shfl_sync(kFull, b, 0);
            if (b >= count) {
                f.exhausted = true;
                break;
            }
            f.next = b;
            f.end = min(b + kFetchChunk, count);
        }
        const uint32_t rank = __popc(idle & ((1u << lane) - 1u));
        const uint32_t take = min(f.end - f.next, static_cast<uint32_t>(__popc(idle)));
        if (((idle >> lane) & 1u) && rank < take) got = f.next + rank;
        f.next += take;
        idle = __ballot_sync(kFull, !has && got == 0xffffffffu);
    }
    return got;
}

// Per-warp staging of finished rays for the shade queue: entries collect in
// shared memory and leave `cnt` at a time with one atomicAdd.
__device__ __forceinline__ void flush_stage(uint32_t* buf, uint32_t& n, uint32_t cnt, uint32_t* counter, uint32_t* shadeQ,
                                            uint32_t P, bool back) {
    const uint32_t lane = lane_id();
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(counter, cnt);
    base = __shfl_sync(kFull, base, 0);
    if (lane < cnt) shadeQ[back ? P - 1u - (base + lane) : base + lane] = buf[lane];
    __syncwarp();
    const uint32_t rest = n - cnt;
    uint32_t x = 0;
    if (lane < rest) x = buf[cnt + lane];
    __syncwarp();
    if (lane < rest) buf[lane] = x;
    __syncwarp();
    n = rest;
}

__device__ __forceinline__ void log_hit(const WfView& v, uint32_t depth, uint32_t j, const float4& h, uint32_t gid) {
    if (v.hitLog) {
        const size_t e = static_cast<size_t>(depth) * v.P + j;
        v.hitLog[e] = h;
        v.gidLog[e] = gid;
    }
}

// ---- warp-cooperative triangle tests ----------------------------------------
// A wide node's leaf triangles are tested by the lanes whose ray reached it;
// tested lane by lane, a step in which a few lanes hold triangles keeps the
// rest of the warp waiting for the longest list.  Here every lane's pending
// triangles are packed into rounds of 32 (lane, triangle) pairs, one pair per
// lane, so a step costs ceil(total / 32) triangle tests instead of the
// longest list.  The hit of a ray is the smallest key (t bits << 32 | global
// triangle id) over its pairs - t > 0, so the float's bits order as the
// float does, and the key order is exactly the (t, mesh order) tie rule -
// which makes the result independent of which lane tested which triangle.
struct CoopTris {
    uint32_t tri[32];              // pair -> triangle (wide order)
    uint32_t src[32];              // pair -> lane whose ray it tests
    unsigned long long best[32];   // lane -> key of its closest hit so far
    float2 uv[32];                 // lane -> barycentrics of that hit
    uint32_t slot[32];             // lane -> its triangle
};

// Packs up to 32 of the warp's pending (lane, triangle) pairs into c.tri /
// c.src, lanes in order, and removes them from `bits`; returns the number of
// pairs (0: none pending anywhere).  Warp-uniform call.
__device__ __forceinline__ uint32_t coop_pack(uint32_t tBase, uint32_t& bits, CoopTris& c) {
    const uint32_t lane = lane_id();
    const uint32_t cnt = __popc(bits);
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += y;
    }
    const uint32_t total = __shfl_sync(kFull, incl, 31);
    if (total == 0u) return 0u;
    const uint32_t excl = incl - cnt;
    const uint32_t take = excl < 32u ? min(cnt, 32u - excl) : 0u;
    for (uint32_t k = 0; k < take; ++k) {
        const uint32_t b = static_cast<uint32_t>(__ffs(bits) - 1);
        bits &= bits - 1u;
        c.tri[excl + k] = tBase + b;
        c.src[excl + k] = lane;
    }
    __syncwarp();
    return min(total, 32u);
}

// Closest hits of the triangles each lane's current node left in
// (tBase, tBits); updates the lane's WideTrav.  Warp-uniform call.
__device__ __forceinline__ void coop_closest(const DevScene& s, WideTrav& t, uint32_t tBase, uint32_t tBits, CoopTris& c) {
    if (!__any_sync(kFull, tBits != 0u)) return;
    const uint32_t lane = lane_id();
    const unsigned long long mine = (static_cast<unsigned long long>(__float_as_uint(t.tmax)) << 32) | t.bestGid;
    c.best[lane] = mine;
    uint32_t bits = tBits;
    for (;;) {
        const uint32_t n = coop_pack(tBase, bits, c);
        if (n == 0u) break;
        const bool pair = lane < n;
        const uint32_t tri = pair ? c.tri[lane] : 0u;
        const uint32_t src = pair ? c.src[lane] : lane;
        const V3 o{__shfl_sync(kFull, t.o.x, src), __shfl_sync(kFull, t.o.y, src), __shfl_sync(kFull, t.o.z, src)};
        const V3 d{__shfl_sync(kFull, t.d.x, src), __shfl_sync(kFull, t.d.y, src), __shfl_sync(kFull, t.d.z, src)};
        unsigned long long key = ~0ull;
        float u = 0.0f, w = 0.0f;
        if (pair) {
            const float4* tp = s.tris + 3 * static_cast<size_t>(tri);
            const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
            float tt;
            if (tri_test(o, d, kRayEpsilon, FLT_MAX, ta, tb, tc, &tt, &u, &w)) {
                key = (static_cast<unsigned long long>(__float_as_uint(tt)) << 32) | __float_as_uint(ta.w);
                atomicMin(&c.best[src], key);
            }
        }
        __syncwarp();
        if (key != ~0ull && c.best[src] == key) {  // one winner per ray: keys are unique
            c.uv[src] = make_float2(u, w);
            c.slot[src] = tri;
        }
        __syncwarp();
    }
    const unsigned long long b = c.best[lane];
    if (b != mine) {
        t.tmax = __uint_as_float(static_cast<uint32_t>(b >> 32));
        t.bestGid = static_cast<uint32_t>(b);
        t.bestSlot = c.slot[lane];
        t.bu = c.uv[lane].x;
        t.bv = c.uv[lane].y;
    }
    __syncwarp();
}

// Any hit in [1e-4, tmax] among the triangles each lane's current node left
// in (tBase, tBits): returns the mask of lanes whose ray is occluded.
// Warp-uniform call.
__device__ __forceinline__ uint32_t coop_any(const DevScene& s, const WideTrav& t, uint32_t tBase, uint32_t tBits,
                                             CoopTris& c) {
    if (!__any_sync(kFull, tBits != 0u)) return 0u;
    const uint32_t lane = lane_id();
    uint32_t bits = tBits, occ = 0u;
    for (;;) {
        const uint32_t n = coop_pack(tBase, bits, c);
        if (n == 0u) break;
        const bool pair = lane < n;
        const uint32_t tri = pair ? c.tri[lane] : 0u;
        const uint32_t src = pair ? c.src[lane] : lane;
        const V3 o{__shfl_sync(kFull, t.o.x, src), __shfl_sync(kFull, t.o.y, src), __shfl_sync(kFull, t.o.z, src)};
        const V3 d{__shfl_sync(kFull, t.d.x, src), __shfl_sync(kFull, t.d.y, src), __shfl_sync(kFull, t.d.z, src)};
        const float tmax = __shfl_sync(kFull, t.tmax, src);
        bool hit = false;
        if (pair) {
            const float4* tp = s.tris + 3 * static_cast<size_t>(tri);
            const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
            float tt, u, w;
            hit = tri_test(o, d, kRayEpsilon, tmax, ta, tb, tc, &tt, &u, &w);
        }
        occ |= __reduce_or_sync(kFull, hit ? (1u << src) : 0u);
        if ((occ >> lane) & 1u) bits = 0u;  // an occluded ray needs no further tests
        __syncwarp();
    }
    return occ;
}

// Closest hit of every queued ray.  The ray is then queued for shading with
// the hits at the front of the shade queue and the misses at its back, so the
// shade stage runs warps of hits and warps of misses instead of warps that
// take both branches.
// kMinBlocks blocks of 256 per SM: 4, 5, 6 cap the registers at 64, 48, 40;
// kLog: an adjoint wave's forward stage, which logs its hits for the replay.
template <bool kCoop, int kMinBlocks, bool kLog = false>
__global__ void __launch_bounds__(256, kMinBlocks) wf_extend(WfView v, DevScene s, uint32_t cur, uint32_t binned,
                                                             uint32_t depth) {
    __shared__ uint32_t stage[8][2][64];
    const uint32_t count = v.counters[cur];
    const uint32_t* q = binned ? v.sortedQ : (cur ? v.rayQ1 : v.rayQ0);
    NullCounter ctr;
    if (kCoop && s.nodes8) {
        // one node per lane and step, the step's triangles tested by the whole warp
        __shared__ CoopTris coop[8];
        CoopTris& c = coop[threadIdx.x >> 5];
        uint32_t* hb = stage[threadIdx.x >> 5][0];
        uint32_t* mb = stage[threadIdx.x >> 5][1];
        const uint32_t ltMask = (1u << lane_id()) - 1u;
        uint2 stack[kStackWide];
        WideTrav t;
        wide_init(t, V3{0.0f, 0.0f, 0.0f}, V3{0.0f, 0.0f, 1.0f}, 0.0f);
        LaneFeed feed;
        bool has = false;
        uint32_t j = 0, hc = 0, mc = 0;
        for (;;) {
            const uint32_t got = feed_lanes(feed, &v.counters[kFetchExtend], count, has, v.refillIdle);
            if (got != 0xffffffffu) {
                j = q[got];
                const float4 o = v.ro[j], d = v.rd[j];
                wide_init(t, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, FLT_MAX);
                has = true;
            }
            if (__ballot_sync(kFull, has) == 0u) break;
            bool fin = false;
            for (int k = 0; k < v.travSteps; ++k) {  // up to travSteps nodes per lane between refills
                const bool step = has && !fin;
                uint32_t gBase = 0, gImask = 0, gInner = 0, tBase = 0, tBits = 0;
                bool bad = false;
                if (step) {
                    if (++t.visits > kMaxVisits) {
                        atomicOr(s.error, kErrTraversalLimit);
                        bad = true;
                    } else {
                        wide_node(s, t.node, t.r, t.tmax, t.octInv, &gBase, &gImask, &gInner, &tBase, &tBits);
                    }
                }
                coop_closest(s, t, tBase, tBits, c);
                if (bad) {
                    t.bestSlot = 0xffffffffu;
                    fin = true;
                } else if (step) {
                    fin = !wide_next(s, t, stack, gBase, gImask, gInner);
                }
                if (!__any_sync(kFull, has && !fin)) break;
            }
            if (fin) {
                const float4 h4 = make_float4(t.tmax, t.bu, t.bv, __uint_as_float(t.bestSlot));
                v.hit[j] = h4;
                v.hitGid[j] = t.bestGid;
                if (kLog) log_hit(v, depth, j, h4, t.bestGid);
                has = false;
            }
            const bool hit = fin && t.bestSlot != 0xffffffffu;
            const uint32_t hbal = __ballot_sync(kFull, hit), mbal = __ballot_sync(kFull, fin && !hit);
            if (hit) hb[hc + __popc(hbal & ltMask)] = j;
            if (fin && !hit) mb[mc + __popc(mbal & ltMask)] = j;
            hc += __popc(hbal);
            mc += __popc(mbal);
            __syncwarp();
            if (hc >= 32u) flush_stage(hb, hc, 32u, &v.counters[kHitCount], v.shadeQ, v.P, false);
            if (mc >= 32u) flush_stage(mb, mc, 32u, &v.counters[kMissCount], v.shadeQ, v.P, true);
        }
        if (hc) flush_stage(hb, hc, hc, &v.counters[kHitCount], v.shadeQ, v.P, false);
        if (mc) flush_stage(mb, mc, mc, &v.counters[kMissCount], v.shadeQ, v.P, true);
        return;
    }
    if (s.nodes8) {
        uint32_t* hb = stage[threadIdx.x >> 5][0];
        uint32_t* mb = stage[threadIdx.x >> 5][1];
        const uint32_t ltMask = (1u << lane_id()) - 1u;
        uint2 stack[kStackWide];
        WideTrav t;
        LaneFeed feed;
        bool has = false;
        uint32_t j = 0, hc = 0, mc = 0;
        for (;;) {
            const uint32_t got = feed_lanes(feed, &v.counters[kFetchExtend], count, has, v.refillIdle);
            if (got != 0xffffffffu) {
                j = q[got];
                const float4 o = v.ro[j], d = v.rd[j];
                wide_init(t, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, FLT_MAX);
                has = true;
            }
            if (__ballot_sync(kFull, has) == 0u) break;
            bool fin = false;
            if (has && wide_closest_advance(s, t, stack, v.travSteps, ctr)) {
                const float4 h4 = make_float4(t.tmax, t.bu, t.bv, __uint_as_float(t.bestSlot));
                v.hit[j] = h4;
                v.hitGid[j] = t.bestGid;
                if (kLog) log_hit(v, depth, j, h4, t.bestGid);
                fin = true;
                has = false;
            }
            const bool hit = fin && t.bestSlot != 0xffffffffu;
            const uint32_t hbal = __ballot_sync(kFull, hit), mbal = __ballot_sync(kFull, fin && !hit);
            if (hit) hb[hc + __popc(hbal & ltMask)] = j;
            if (fin && !hit) mb[mc + __popc(mbal & ltMask)] = j;
            hc += __popc(hbal);
            mc += __popc(mbal);
            __syncwarp();
            if (hc >= 32u) flush_stage(hb, hc, 32u, &v.counters[kHitCount], v.shadeQ, v.P, false);
            if (mc >= 32u) flush_stage(mb, mc, 32u, &v.counters[kMissCount], v.shadeQ, v.P, true);
        }
        if (hc) flush_stage(hb, hc, hc, &v.counters[kHitCount], v.shadeQ, v.P, false);
        if (mc) flush_stage(mb, mc, mc, &v.counters[kMissCount], v.shadeQ, v.P, true);
        return;
    }
    for (;;) {
        const uint32_t base = warp_fetch(&v.counters[kFetchExtend]);
        if (base >= count) break;
        const uint32_t i = base + lane_id();
        const bool valid = i < count;
        uint32_t j = 0;
        bool hit = false;
        if (valid) {
            j = q[i];
            const float4 o = v.ro[j], d = v.rd[j];
            HitRec h;
            trace_closest(s, V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}, &h, ctr);
            const float4 h4 = make_float4(h.t, h.u, h.v, __uint_as_float(h.slot));
            v.hit[j] = h4;
            v.hitGid[j] = h.gid;
            if (kLog) log_hit(v, depth, j, h4, h.gid);
            hit = h.slot != 0xffffffffu;
        }
        const uint32_t hs = warp_claim(&v.counters[kHitCount], valid && hit);
        const uint32_t ms = warp_claim(&v.counters[kMissCount], valid && !hit);
        if (valid) v.shadeQ[hit ? hs : v.P - 1u - ms] = j;
    }
}

__device__ __forceinline__ void write_record(const WfView& v, uint32_t j, const V3& rad, float depth0) {
    v.records[3 * static_cast<size_t>(j)] = make_float4(rad.x, rad.y, rad.z, depth0);
}

// Shade stage, compiled with several register caps (the autotuner picks) and
// with / without the extended lobes (kExt, chosen by the scene).
template <int kRegs, bool kExt>
__global__ void __maxnreg__(kRegs) wf_shade(WfView v, DevScene s, uint32_t cur, uint32_t depth) {
    const uint32_t count = v.counters[kHitCount];
    uint32_t* qout = cur ? v.rayQ0 : v.rayQ1;
    uint32_t* cout = &v.counters[cur ^ 1u];
    NullCounter ctr;
    // whole warps fetch work together, so the warp-aggregated pushes below
    // always see the whole warp; entries [0, hits) of the shade queue
    for (;;) {
        const uint32_t wbase = warp_fetch(&v.counters[kFetchShade]);
        if (wbase >= count) break;
        const uint32_t i = wbase + lane_id();
        const bool valid = i < count;
        bool pushRay = false, pushShadow = false;
        uint32_t lightMask = 0;
        uint32_t j = 0;
        if (valid) {
            j = v.shadeQ[i];
            const uint4 id = v.ident[j];
            const DevRequest& q = v.reqs[id.w].q;
            const float4 o = v.ro[j], d = v.rd[j], t4 = v.T[j], r4 = v.rad[j], h4 = v.hit[j];
            const uint32_t bits = __float_as_uint(t4.w);
            PathState ps;
            ps.ro = V3{o.x, o.y, o.z};
            ps.rd = V3{d.x, d.y, d.z};
            ps.prevPdf = d.w;
            ps.T = V3{t4.x, t4.y, t4.z};
            ps.radiance = V3{r4.x, r4.y, r4.z};
            ps.diffDepth = bits & 0xffu;
            ps.specDepth = (bits >> 8) & 0xffu;
            ps.prevDelta = (bits & kFlagPrevDelta) != 0u;
            ps.prevType = (bits >> kTypeShift) & 3u;
            ps.inside = (bits & kFlagInside) != 0u;
            ps.mediumActive = (bits & kFlagMedium) != 0u;
            ps.extinction = V3{0.0f, 0.0f, 0.0f};
            if (kExt && ps.mediumActive) {
                const float4 m4 = v.medium[j];
                ps.extinction = V3{m4.x, m4.y, m4.z};
            }
            float depth0 = r4.w;
            HitRec h;
            h.t = h4.x;
            h.u = h4.y;
            h.v = h4.z;
            h.slot = __float_as_uint(h4.w);
            h.gid = v.hitGid[j];
            {
                const Vertex vx = make_vertex(s, ps.ro, ps.rd, h);
                const Sampler smp{id.x, id.y, id.z};
                bool anyLight = false, cont;
                if (kExt && !enter_hit(s, smp, depth, vx, h.t, ps)) {
                    cont = depth + 1u < q.maxDepth;  // passes through an opacity cut-out
                } else {
                    if (depth == 0) {
                        const float4 dc = __ldg(bsdf_rec(s, vx.hit.material) + 3);  // DiffuseColor
                        const V3 alb{dc.x, dc.y, dc.z};
                        const V3 nn = vx.n * 0.5f + V3{0.5f, 0.5f, 0.5f};
                        v.records[3 * static_cast<size_t>(j) + 1] = make_float4(alb.x, alb.y, alb.z, 0.0f);
                        v.records[3 * static_cast<size_t>(j) + 2] = make_float4(nn.x, nn.y, nn.z, 0.0f);
                        depth0 = h.t;
                    }
                    if constexpr (kExt) add_emission(s, vx, depth, ps);
                    // this request's light samples (requests of a batch may differ in dome samples)
                    const uint32_t nls = light_sample_count<kExt>(s, q);
                    for (uint32_t k = 0; k < nls; ++k) {
                        V3 dir{0.0f, 0.0f, 0.0f}, c{0.0f, 0.0f, 0.0f};
                        float reach = 0.0f;
                        const bool ok = light_sample<kExt>(s, q, vx, smp, depth, k, &dir, &c, &reach, ctr);
                        anyLight |= ok;
                        lightMask |= ok ? (1u << k) : 0u;
                        const size_t e = static_cast<size_t>(k) * v.P + j;
                        v.shDir[e] = make_float4(dir.x, dir.y, dir.z, ok ? reach : 0.0f);
                        v.shC[e] = make_float4(c.x, c.y, c.z, 0.0f);
                    }
                    if (anyLight) {
                        const V3 org = shadow_origin(vx);
                        v.shOrigin[j] = make_float4(org.x, org.y, org.z, 0.0f);
                        v.shT[j] = make_float4(ps.T.x, ps.T.y, ps.T.z, 0.0f);
                        pushShadow = true;
                    }
                    cont = continue_path<kExt>(s, q, vx, smp, depth, ps, ctr) && depth + 1u < q.maxDepth;
                }
                if (v.visLog && !anyLight) v.visLog[static_cast<size_t>(depth) * v.P + j] = 0u;
                uint32_t nb = pack_state(ps);
                if (!cont && anyLight) {
                    nb |= kFlagDone;
                    v.shT[j].w = 1.0f;  // read by wf_shadow with the throughput (no load of T for the flag)
                }
                v.T[j] = make_float4(ps.T.x, ps.T.y, ps.T.z, __uint_as_float(nb));
                if (kExt && ps.mediumActive)
                    v.medium[j] = make_float4(ps.extinction.x, ps.extinction.y, ps.extinction.z, 0.0f);
                if (cont) {
                    v.ro[j] = make_float4(ps.ro.x, ps.ro.y, ps.ro.z, 0.0f);
                    v.rd[j] = make_float4(ps.rd.x, ps.rd.y, ps.rd.z, ps.prevPdf);
                    pushRay = true;
                }
                v.rad[j] = make_float4(ps.radiance.x, ps.radiance.y, ps.radiance.z, depth0);
                if (!cont && !anyLight) write_record(v, j, ps.radiance, depth0);
            }
        }
        warp_push(cout, qout, pushRay, j);
        warp_push(&v.counters[2], v.shadowQ, pushShadow, j);
        warp_push_samples(&v.counters[4], v.shadowRayQ, lightMask, v.lightSamples, j);
    }
}

// Miss shading (the environment and its MIS weight), one queued miss per
// thread: entries [P - misses, P) of the shade queue.  A kernel of its own so
// that the misses, half of the shade work, run at the occupancy of their own
// small register count instead of the hit shading's.
__global__ void __launch_bounds__(256) wf_miss(WfView v, DevScene s, uint32_t depth) {
    const uint32_t count = v.counters[kMissCount];
    NullCounter ctr;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t j = v.shadeQ[v.P - 1u - i];
        const DevRequest& q = v.reqs[v.ident[j].w].q;
        const float4 d = v.rd[j], t4 = v.T[j], r4 = v.rad[j];
        const uint32_t bits = __float_as_uint(t4.w);
        PathState ps;
        ps.rd = V3{d.x, d.y, d.z};
        ps.prevPdf = d.w;
        ps.T = V3{t4.x, t4.y, t4.z};
        ps.radiance = V3{r4.x, r4.y, r4.z};
        ps.prevDelta = (bits & kFlagPrevDelta) != 0u;
        ps.prevType = (bits >> kTypeShift) & 3u;
        add_miss(s, q, ps, depth, ctr);
        write_record(v, j, ps.radiance, r4.w);
    }
}

// Any hit per queued light sample; an occluded sample's flag is cleared.
// kMode 0: one ray per lane for the warp's 32 entries; 1: cooperative
// triangle tests; 2 (default): lane refill on the wide BVH as in wf_extend (a
// lane takes the next entry of its warp's chunk as soon as enough lanes are
// idle) - on the 1080p field frame the stage takes 30.7 ms per frame instead
// of 38.6 with one ray per lane.
template <int kMode, int kMinBlocks>
__global__ void __launch_bounds__(256, kMinBlocks) wf_occlude(WfView v, DevScene s, uint32_t binned) {
    const uint32_t count = v.counters[4];
    const uint32_t* sq = binned ? v.sortedQ : v.shadowRayQ;
    NullCounter ctr;
    if (kMode == 2 && s.nodes8) {
        uint2 stack[kStackWide];
        WideTrav t;
        wide_init(t, V3{0.0f, 0.0f, 0.0f}, V3{0.0f, 0.0f, 1.0f}, 0.0f);
        LaneFeed feed;
        bool has = false;
        size_t e = 0;
        for (;;) {
            const uint32_t got = feed_lanes(feed, &v.counters[kFetchOcclude], count, has, v.refillIdle);
            if (got != 0xffffffffu) {
                const uint32_t item = sq[got];
                const uint32_t j = item >> 3, k = item & 7u;
                e = static_cast<size_t>(k) * v.P + j;
                const float4 o4 = v.shOrigin[j], d4 = v.shDir[e];
                wide_init(t, V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z}, d4.w);
                has = true;
            }
            if (__ballot_sync(kFull, has) == 0u) break;
            if (has) {
                const int r = wide_occluded_advance(s, t, stack, v.travSteps, ctr);
                if (r >= 0) {
                    if (r == 1) v.shDir[e].w = 0.0f;
                    has = false;
                }
            }
        }
        return;
    }
    if (kMode == 1 && s.nodes8) {
        // one node per lane and step, the step's triangles tested by the whole warp
        __shared__ CoopTris coop[8];
        CoopTris& c = coop[threadIdx.x >> 5];
        uint2 stack[kStackWide];
        for (;;) {
            const uint32_t base = warp_fetch(&v.counters[kFetchOcclude]);
            if (base >= count) break;
            const uint32_t i = base + lane_id();
            bool live = i < count;
            size_t e = 0;
            WideTrav t;
            wide_init(t, V3{0.0f, 0.0f, 0.0f}, V3{0.0f, 0.0f, 1.0f}, 0.0f);
            if (live) {
                const uint32_t item = sq[i];
                const uint32_t j = item >> 3, k = item & 7u;
                e = static_cast<size_t>(k) * v.P + j;
                const float4 o4 = v.shOrigin[j], d4 = v.shDir[e];
                wide_init(t, V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z}, d4.w);
            }
            bool occluded = false;
            while (__ballot_sync(kFull, live) != 0u) {
                uint32_t gBase = 0, gImask = 0, gInner = 0, tBase = 0, tBits = 0;
                if (live) {
                    if (++t.visits > kMaxVisits) {
                        atomicOr(s.error, kErrTraversalLimit);
                        live = false;
                    } else {
                        wide_node(s, t.node, t.r, t.tmax, t.octInv, &gBase, &gImask, &gInner, &tBase, &tBits);
                    }
                }
                const uint32_t occ = coop_any(s, t, tBase, tBits, c);
                if (live) {
                    if ((occ >> lane_id()) & 1u) {
                        occluded = true;
                        live = false;
                    } else if (!wide_next(s, t, stack, gBase, gImask, gInner)) {
                        live = false;
                    }
                }
            }
            if (occluded) v.shDir[e].w = 0.0f;
        }
        return;
    }
    for (;;) {
        const uint32_t base = warp_fetch(&v.counters[kFetchOcclude]);
        if (base >= count) break;
        const uint32_t i = base + lane_id();
        if (i >= count) continue;
        const uint32_t item = sq[i];
        const uint32_t j = item >> 3, k = item & 7u;
        const size_t e = static_cast<size_t>(k) * v.P + j;
        const float4 o4 = v.shOrigin[j], d4 = v.shDir[e];
        if (trace_occluded(s, V3{o4.x, o4.y, o4.z}, V3{d4.x, d4.y, d4.z}, d4.w, ctr)) v.shDir[e].w = 0.0f;
    }
}

// In-order sum of a path's unoccluded light samples (sum_direct's order).
__global__ void __launch_bounds__(256) wf_shadow(WfView v, DevScene s, uint32_t depth) {
    const uint32_t count = v.counters[2];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t j = v.shadowQ[i];
        const DevRequest& q = v.reqs[v.ident[j].w].q;
        const float4 t4 = v.shT[j], r4 = v.rad[j];
        uint32_t visible = 0;
        const V3 direct = sum_direct<true>(s, q, [&](uint32_t k, V3* c) {
            const size_t e = static_cast<size_t>(k) * v.P + j;
            if (v.shDir[e].w == 0.0f) return false;
            const float4 c4 = v.shC[e];
            *c = V3{c4.x, c4.y, c4.z};
            visible |= 1u << k;
            return true;
        });
        if (v.visLog) v.visLog[static_cast<size_t>(depth) * v.P + j] = static_cast<uint8_t>(visible);
        const V3 rad = V3{r4.x, r4.y, r4.z} + V3{t4.x, t4.y, t4.z} * direct;
        v.rad[j] = make_float4(rad.x, rad.y, rad.z, r4.w);
        if (t4.w != 0.0f) write_record(v, j, rad, r4.w);  // the path ends here
    }
}

__global__ void wf_end_bounce(WfView v, uint32_t cur) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        v.counters[cur] = 0u;
        v.counters[2] = 0u;
        v.counters[4] = 0u;
        v.counters[kFetchExtend] = 0u;
        v.counters[kFetchShade] = 0u;
        v.counters[kFetchOcclude] = 0u;
        v.counters[kHitCount] = 0u;
        v.counters[kMissCount] = 0u;
    }
}

// Per-pixel average of the wave's records, same additions as k_resolve.
__global__ void __launch_bounds__(128) wf_resolve(WfView v) {
    const WaveDesc w = cur_wave(v);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < w.pixels; p += gridDim.x * blockDim.x) {
        const WaveSeg& sg = find_seg(v, w, p, true);
        const WfRequest& r = v.reqs[sg.req];
        const uint32_t n = r.q.sampleCount;
        const uint32_t lp = p - sg.pixelOffset;
        const float4* rec = v.records + 3 * (static_cast<size_t>(sg.pathOffset) + static_cast<size_t>(lp) * n);
        float b0 = 0.0f, b1 = 0.0f, b2 = 0.0f, b3 = 0.0f;
        V3 alb{0.0f, 0.0f, 0.0f}, nrm{0.0f, 0.0f, 0.0f};
        float depth = __int_as_float(0x7f800000);
        for (uint32_t k = 0; k < n; ++k) {
            const float4 a = rec[3 * k];
            b0 = b0 + a.x;
            b1 = b1 + a.y;
            b2 = b2 + a.z;
            const bool hit = a.w < __int_as_float(0x7f800000);
            b3 = b3 + (hit ? 1.0f : 0.0f);
            if (hit) {  // albedo and normal of a path whose first ray missed are zero (adding them changes nothing)
                const float4 b = rec[3 * k + 1], c = rec[3 * k + 2];
                alb = alb + V3{b.x, b.y, b.z};
                nrm = nrm + V3{c.x, c.y, c.z};
            }
            if (a.w < depth) depth = a.w;
        }
        const float cnt = static_cast<float>(n);
        const float inv = 1.0f / cnt;
        const size_t px = static_cast<size_t>(sg.pixelStart) + lp;
        if ((reinterpret_cast<uintptr_t>(r.aov.beauty) & 15u) == 0u) {  // one 16-byte store (host planes too)
            reinterpret_cast<float4*>(r.aov.beauty)[px] = make_float4(b0 / cnt, b1 / cnt, b2 / cnt, b3 / cnt);
        } else {
            r.aov.beauty[4 * px + 0] = b0 / cnt;
            r.aov.beauty[4 * px + 1] = b1 / cnt;
            r.aov.beauty[4 * px + 2] = b2 / cnt;
            r.aov.beauty[4 * px + 3] = b3 / cnt;
        }
        const V3 a = alb * inv, nn = nrm * inv;
        r.aov.albedo[3 * px + 0] = a.x;
        r.aov.albedo[3 * px + 1] = a.y;
        r.aov.albedo[3 * px + 2] = a.z;
        r.aov.normal[3 * px + 0] = nn.x;
        r.aov.normal[3 * px + 1] = nn.y;
        r.aov.normal[3 * px + 2] = nn.z;
        r.aov.depth[px] = depth;
    }
}

// ---- adjoint replay stages ---------------------------------------------------
// The estimator of adjoint.cu's path replay (adj_path with the scene's own
// parameters), cut at the same seams as the forward stages: light samples and
// continuation in wa_shade, their occlusion in wf_occlude, the gradients of
// the visible samples and of the continuation in wa_shadow (they need the
// radiance still to come, which is known once the vertex's direct light is),
// the environment gradients of the misses in wa_miss.

__global__ void wa_begin(WfView v) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        for (uint32_t k = 0; k < 10; ++k)
            if (k != 3) v.counters[k] = 0u;  // every queue, keeping the wave index
    }
}

// Paths restart from their QMC seed; those of the adjoint's request (the
// wave's request a.targetReq) whose pixel has a nonzero d_beauty are queued.
__global__ void __launch_bounds__(128) wa_generate(WfView v, AdjWave aw) {
    const WaveDesc w = cur_wave(v);
    const AdjView& a = *aw.view;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < w.paths; base += stride) {
        const uint32_t j = base + threadIdx.x;
        bool push = false;
        const WaveSeg* sgp = j < w.paths ? &find_seg(v, w, j, false) : nullptr;
        if (sgp && sgp->req == a.targetReq) {
            const WaveSeg& sg = *sgp;
            const DevRequest& q = v.reqs[sg.req].q;
            const uint32_t local = j - sg.pathOffset;
            const uint32_t pix = sg.pixelStart + local / q.sampleCount;
            const uint32_t smpIdx = q.sampleStart + (local - (local / q.sampleCount) * q.sampleCount);
            const uint32_t y = pix / q.width, x = pix - y * q.width;
            const Sampler smp{x, y, smpIdx};
            PathState ps;
            init_path(q, smp, ps);
            v.ro[j] = make_float4(ps.ro.x, ps.ro.y, ps.ro.z, 0.0f);
            v.rd[j] = make_float4(ps.rd.x, ps.rd.y, ps.rd.z, ps.prevPdf);
            v.T[j] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(kFlagPrevDelta));
            v.ident[j] = make_uint4(x, y, smpIdx, sg.req);
            const float cnt = static_cast<float>(q.sampleCount);
            const float4 g = reinterpret_cast<const float4*>(a.dBeauty)[pix];
            const float4 r = v.records[3 * static_cast<size_t>(j)];
            aw.delta[j] = make_float4(g.x / cnt, g.y / cnt, g.z / cnt, 0.0f);
            aw.lrem[j] = make_float4(r.x, r.y, r.z, 0.0f);
            push = g.x != 0.0f || g.y != 0.0f || g.z != 0.0f;
        }
        warp_push(&v.counters[0], v.rayQ0, push, j);
    }
}

// The replay's rays of bounce `depth` take the hits the forward stages
// logged for their slots (the same rays: the replay follows the forward's
// decisions), split into the shade queue as wf_extend splits them.
__global__ void __launch_bounds__(256) wa_hits(WfView v, uint32_t cur, uint32_t depth) {
    // one pair of queue atomics per 256 entries (per-warp atomics on the two
    // counters serialised the kernel)
    __shared__ uint32_t wHit[8], wMiss[8], base[2];
    const uint32_t count = v.counters[cur];
    const uint32_t* q = cur ? v.rayQ1 : v.rayQ0;
    const uint32_t lane = lane_id(), w = threadIdx.x >> 5;
    for (uint32_t start = blockIdx.x * 256u; start < count; start += gridDim.x * 256u) {
        const uint32_t i = start + threadIdx.x;
        const bool valid = i < count;
        uint32_t j = 0;
        bool hit = false;
        if (valid) {
            j = q[i];
            const size_t e = static_cast<size_t>(depth) * v.P + j;
            const float4 h4 = v.hitLog[e];
            v.hit[j] = h4;
            v.hitGid[j] = v.gidLog[e];
            hit = __float_as_uint(h4.w) != 0xffffffffu;
        }
        const uint32_t hb = __ballot_sync(kFull, valid && hit), mb = __ballot_sync(kFull, valid && !hit);
        if (lane == 0) {
            wHit[w] = __popc(hb);
            wMiss[w] = __popc(mb);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t th = 0, tm = 0;
            for (int k = 0; k < 8; ++k) {
                const uint32_t a = wHit[k], b = wMiss[k];
                wHit[k] = th;
                wMiss[k] = tm;
                th += a;
                tm += b;
            }
            base[0] = th ? atomicAdd(&v.counters[kHitCount], th) : 0u;
            base[1] = tm ? atomicAdd(&v.counters[kMissCount], tm) : 0u;
        }
        __syncthreads();
        const uint32_t lt = (1u << lane) - 1u;
        if (valid && hit) v.shadeQ[base[0] + wHit[w] + __popc(hb & lt)] = j;
        if (valid && !hit) v.shadeQ[v.P - 1u - (base[1] + wMiss[w] + __popc(mb & lt))] = j;
        __syncthreads();
    }
}

// Light sample k of a vertex with the factors of its gradient: its clamped
// contribution c, gL = L w s (material gradient = delta T gL . df) and
// gE = f R w s (texel gradient of dome 0's texture = delta T gE at `local`),
// with s the clamp scale held constant.  kExt: the scene has emitters or
// cut-outs (the replay stages are compiled for each kind of scene).
template <bool kExt>
__device__ __forceinline__ bool wa_light(const DevScene& s, const DevRequest& q, const AdjView& a, const Vertex& vx,
                                         const Sampler& smp, uint32_t depth, uint32_t k, const float4* rec, const Mat& ms,
                                         V3* ld, V3* c, V3* gL, V3* gE, V3* local, bool* envMark) {
    V3 L, domeRad{0.0f, 0.0f, 0.0f};
    float w;
    int32_t envIdx = -1;
    *local = V3{0.0f, 0.0f, 0.0f};
    if (kExt && k >= s.distantCount + s.domeCount * q.domeSamples) {  // the emissive-triangle sample
        float lp, nl, reach;
        if (!emissive_geometry(s, vx, smp, depth, ld, &L, &lp, &nl, &reach)) return false;
        const float bp = bsdf_pdf_rec(rec, ms, vx.w, vx.n, vx.cn, vx.view, *ld);
        w = nl * power_heuristic(lp, bp) / lp;
    } else if (k < s.distantCount) {
        const DevDistant l = s.distant[k];
        *ld = normalize(l.direction * -1.0f);
        const float nl = sclamp(dot(vx.n, *ld), 0.0f, 1.0f);
        if (nl <= 0.0f) return false;
        L = l.radiance;
        w = nl;
    } else {
        const uint32_t r = k - s.distantCount;
        const uint32_t li = r / q.domeSamples, jj = r - li * q.domeSamples;
        const DevDome& d = s.domes[li];
        const uint32_t dim = kDirectDimBase + depth * kDirectDepthStride + li * kDirectLightStride + jj * kDirectSampleStride;
        const V2 u = smp.next2d(dim);
        float lp;
        if (d.env >= 0) {
            env_sample(s.envs[d.env], u, (q.flags & SHIRO_RENDER_ENV_CDF) != 0u, local, &lp);
            if (lp <= 0.0f) return false;
            L = env_evaluate(env_for_eval(s, a, d.env), *local) * d.radiance;
            envIdx = d.env;
            domeRad = d.radiance;
        } else {
            const float yy = 1.0f - 2.0f * u.y;
            const float rr = sqrtf(smax(0.0f, 1.0f - yy * yy));
            const float phi = 2.0f * kPi * u.x;
            *local = V3{sinf(phi) * rr, yy, cosf(phi) * rr};
            lp = kInvFourPi;
            L = V3{1.0f, 1.0f, 1.0f} * d.radiance;
        }
        *ld = light_to_world(d, *local);
        const float nl = sclamp(dot(vx.n, *ld), 0.0f, 1.0f);
        if (nl <= 0.0f) return false;
        const float bp = bsdf_pdf_rec(rec, ms, vx.w, vx.n, vx.cn, vx.view, *ld);
        const float mis = power_heuristic(lp, bp);
        w = nl * mis / lp;
    }
    const V3 f = bsdf_eval_rec(rec, ms, vx.n, vx.cn, vx.view, *ld);
    const V3 raw = f * L * w;
    *c = clamp24(q, raw);
    const float sc = clamp_scale(q, raw, kDirectSampleClamp);
    *gL = L * (w * sc);
    *gE = f * domeRad * (w * sc);
    *envMark = envIdx >= 0 && envIdx == a.env0;
    return true;
}

template <bool kExt>
__global__ void __launch_bounds__(128) wa_shade(WfView v, DevScene s, AdjWave aw, uint32_t cur, uint32_t depth) {
    const uint32_t count = v.counters[kHitCount];
    uint32_t* qout = cur ? v.rayQ0 : v.rayQ1;
    uint32_t* cout = &v.counters[cur ^ 1u];
    const AdjView& a = *aw.view;
    for (;;) {
        const uint32_t wbase = warp_fetch(&v.counters[kFetchShade]);
        if (wbase >= count) break;
        const uint32_t i = wbase + lane_id();
        bool pushRay = false;
        uint32_t j = 0;
        if (i < count) {
            j = v.shadeQ[i];
            const uint4 id = v.ident[j];
            const DevRequest& q = v.reqs[id.w].q;
            const float4 o = v.ro[j], d = v.rd[j], t4 = v.T[j], h4 = v.hit[j];
            const uint32_t bits = __float_as_uint(t4.w);
            PathState ps;
            ps.ro = V3{o.x, o.y, o.z};
            ps.rd = V3{d.x, d.y, d.z};
            ps.prevPdf = d.w;
            ps.T = V3{t4.x, t4.y, t4.z};
            ps.diffDepth = bits & 0xffu;
            ps.specDepth = (bits >> 8) & 0xffu;
            ps.prevDelta = (bits & kFlagPrevDelta) != 0u;
            ps.prevType = (bits >> kTypeShift) & 3u;
            ps.inside = false;
            ps.mediumActive = false;
            HitRec h;
            h.t = h4.x;
            h.u = h4.y;
            h.v = h4.z;
            h.slot = __float_as_uint(h4.w);
            h.gid = v.hitGid[j];
            const Vertex vx = make_vertex(s, ps.ro, ps.rd, h);
            const uint32_t mat = vx.hit.material;
            const Mat& ms = s.materials[mat];
            const float4* rec = bsdf_rec(s, mat);
            aw.vtx[3 * static_cast<size_t>(j)] = make_float4(vx.n.x, vx.n.y, vx.n.z, __uint_as_float(mat));
            aw.vtx[3 * static_cast<size_t>(j) + 1] = make_float4(vx.cn.x, vx.cn.y, vx.cn.z, 0.0f);
            aw.vtx[3 * static_cast<size_t>(j) + 2] = make_float4(vx.view.x, vx.view.y, vx.view.z, 0.0f);
            const Sampler smp{id.x, id.y, id.z};
            // an opacity cut-out the path passes through (the forward's decision;
            // no media, transmission being refused): the hit is not shaded
            const bool shaded = !kExt || enter_hit(s, smp, depth, vx, h.t, ps);
            if (kExt && shaded) {
                // radiance emitted at this hit: no BSDF value of this vertex or a
                // later one scales it, so it leaves the radiance still to come
                ps.radiance = V3{0.0f, 0.0f, 0.0f};
                add_emission(s, vx, depth, ps);
                if (ps.radiance.x != 0.0f || ps.radiance.y != 0.0f || ps.radiance.z != 0.0f) {
                    const float4 l4 = aw.lrem[j];
                    aw.lrem[j] = make_float4(l4.x - ps.radiance.x, l4.y - ps.radiance.y, l4.z - ps.radiance.z, 0.0f);
                }
            }
            const uint32_t nls = light_sample_count<kExt>(s, q);
            // which samples the forward stages found taken and unoccluded at this vertex
            const uint32_t seen = shaded ? v.visLog[static_cast<size_t>(depth) * v.P + j] : 0u;
            for (uint32_t k = 0; k < nls; ++k) {
                V3 ld{0.0f, 0.0f, 0.0f}, c{0.0f, 0.0f, 0.0f}, gL{0.0f, 0.0f, 0.0f}, gE{0.0f, 0.0f, 0.0f},
                    local{0.0f, 0.0f, 0.0f};
                bool mark = false;
                const bool ok =
                    shaded && wa_light<kExt>(s, q, a, vx, smp, depth, k, rec, ms, &ld, &c, &gL, &gE, &local, &mark);
                const size_t e = static_cast<size_t>(k) * v.P + j;
                v.shDir[e] = make_float4(ld.x, ld.y, ld.z, (ok && ((seen >> k) & 1u)) ? FLT_MAX : 0.0f);
                v.shC[e] = make_float4(c.x, c.y, c.z, 0.0f);
                aw.lgrad[3 * e] = make_float4(gL.x, gL.y, gL.z, 0.0f);
                aw.lgrad[3 * e + 1] = make_float4(gE.x, gE.y, gE.z, mark ? 1.0f : 0.0f);
                aw.lgrad[3 * e + 2] = make_float4(local.x, local.y, local.z, 0.0f);
            }
            v.shT[j] = make_float4(ps.T.x, ps.T.y, ps.T.z, 0.0f);
            // continuation (the reflecting lobes of continue_path); past a cut-out
            // the ray goes on unchanged, with no BSDF value to differentiate
            bool alive = false, due = false, pass = false;
            V3 next{0.0f, 0.0f, 0.0f}, f{0.0f, 0.0f, 0.0f};
            const uint32_t base = depth * kPathDimStride;
            const float rw = vx.w.diffuse + vx.w.spec + vx.w.coat;
            const float tw = rw + 0.0f;
            do {
                if (!shaded) {
                    pass = depth + 1u < q.maxDepth;
                    break;
                }
                if (tw <= 0.0f) break;
                const float sel = smp.next1d(base + 1u) * tw;
                const V2 ds = smp.next2d(base + 2u);
                float pdf;
                bool delta2 = false;
                const float rs = sel - 0.0f;
                uint32_t type = kBounceDiffuse;
                if (rs < vx.w.diffuse) {
                    if (ps.diffDepth >= q.diffuseDepth) break;
                    ++ps.diffDepth;
                    next = cosine_hemisphere(vx.n, ds);
                    const float cpdf = sclamp(dot(vx.n, next), 0.0f, 1.0f) * kInvPi;
                    pdf = smax((rw / tw) * (1.0f * cpdf + 0.0f * 0.0f), 1.0e-6f);
                } else {
                    type = kBounceReflective;
                    const bool coat = !(rs < vx.w.diffuse + vx.w.spec);
                    if (ps.specDepth >= q.specularDepth) break;
                    ++ps.specDepth;
                    const V3 sn = coat ? vx.cn : vx.n;
                    const float sr = coat ? roughness_for(ms.coat_roughness, ms.coat_anisotropy, ms.coat_rotation)
                                          : roughness_for(base_roughness(ms), ms.specular_anisotropy, ms.specular_rotation);
                    const V3 hv = ggx_half(sn, ds, sr);
                    next = normalize(reflect(ps.rd, hv));
                    const float rc = sclamp(dot(sn, next), 0.0f, 1.0f);
                    if (rc <= 0.0f) break;
                    pdf = smax((rw / tw) * bsdf_pdf_rec(rec, ms, vx.w, vx.n, vx.cn, vx.view, next), 1.0e-6f);
                    delta2 = sr <= kDeltaRoughness;
                }
                f = bsdf_eval_rec(rec, ms, vx.n, vx.cn, vx.view, next);
                const float cosT = sclamp(dot(vx.n, next), 0.0f, 1.0f);
                if (cosT <= 0.0f) break;
                ps.T = clamp12(q, ps.T * f * (cosT / pdf));
                const float off = dot(vx.n, next) >= 0.0f ? 1.0f : -1.0f;
                ps.ro = vx.hit.position + vx.n * (kRayEpsilon * off);
                ps.rd = next;
                ps.prevDelta = delta2;
                ps.prevPdf = pdf;
                ps.prevType = type;
                alive = true;
                if (depth >= 2) {
                    const float cp = sclamp(maxc(ps.T), 0.05f, 0.95f);
                    if (smp.next1d(base + 4u) > cp) {
                        alive = false;
                    } else {
                        ps.T = ps.T / cp;
                    }
                }
                due = alive && depth + 1u < q.maxDepth;
            } while (false);
            aw.cont[2 * static_cast<size_t>(j)] = make_float4(next.x, next.y, next.z, due ? 1.0f : 0.0f);
            aw.cont[2 * static_cast<size_t>(j) + 1] = make_float4(f.x, f.y, f.z, 0.0f);
            if (due || pass) {
                v.T[j] = make_float4(ps.T.x, ps.T.y, ps.T.z, __uint_as_float(pack_state(ps)));
                v.ro[j] = make_float4(ps.ro.x, ps.ro.y, ps.ro.z, 0.0f);
                v.rd[j] = make_float4(ps.rd.x, ps.rd.y, ps.rd.z, ps.prevPdf);
                pushRay = true;
            }
        }
        warp_push(cout, qout, pushRay, j);
    }
}

// Gradients of a shaded vertex once its light samples' visibility is known.
template <bool kExt>
__global__ void __launch_bounds__(128, 4) wa_shadow(WfView v, DevScene s, AdjWave aw) {
    const uint32_t count = v.counters[kHitCount];
    const AdjView& a = *aw.view;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t j = v.shadeQ[i];
        const DevRequest& q = v.reqs[v.ident[j].w].q;
        const float4 t4 = v.shT[j], dl4 = aw.delta[j], l4 = aw.lrem[j];
        const float4 v0 = aw.vtx[3 * static_cast<size_t>(j)], v1 = aw.vtx[3 * static_cast<size_t>(j) + 1],
                     v2 = aw.vtx[3 * static_cast<size_t>(j) + 2];
        const V3 T0{t4.x, t4.y, t4.z}, dl{dl4.x, dl4.y, dl4.z};
        const V3 n{v0.x, v0.y, v0.z}, cn{v1.x, v1.y, v1.z}, view{v2.x, v2.y, v2.z};
        const uint32_t mat = __float_as_uint(v0.w);
        const Mat& me = a.evalMats[mat];
        const V3 dT = dl * T0;
        const V3 direct = sum_direct<kExt>(s, q, [&](uint32_t k, V3* c) {
            const size_t e = static_cast<size_t>(k) * v.P + j;
            const float4 d4 = v.shDir[e];
            if (d4.w == 0.0f) return false;
            const float4 c4 = v.shC[e];
            *c = V3{c4.x, c4.y, c4.z};
            const float4 g0 = aw.lgrad[3 * e], g1 = aw.lgrad[3 * e + 1];
            const DV3 fd = bsdf_eval_d(me, n, cn, view, V3{d4.x, d4.y, d4.z});
            add_mat_grad(a, mat, fd, dT * V3{g0.x, g0.y, g0.z});
            if (g1.w != 0.0f) {
                const float4 g2 = aw.lgrad[3 * e + 2];
                add_env_grad(a, a.evalEnv, V3{g2.x, g2.y, g2.z}, dT * V3{g1.x, g1.y, g1.z});
            }
            return true;
        });
        const V3 lrem = V3{l4.x, l4.y, l4.z} - T0 * direct;
        const float4 c0 = aw.cont[2 * static_cast<size_t>(j)];
        if (c0.w != 0.0f) {
            const float4 f4 = aw.cont[2 * static_cast<size_t>(j) + 1];
            const V3 f{f4.x, f4.y, f4.z};
            const DV3 fd = bsdf_eval_d(me, n, cn, view, V3{c0.x, c0.y, c0.z});
            const V3 coef{f.x > 0.0f ? dl.x * lrem.x / f.x : 0.0f, f.y > 0.0f ? dl.y * lrem.y / f.y : 0.0f,
                          f.z > 0.0f ? dl.z * lrem.z / f.z : 0.0f};
            add_mat_grad(a, mat, fd, coef);
        }
        aw.lrem[j] = make_float4(lrem.x, lrem.y, lrem.z, 0.0f);
    }
}

// Texel gradients of dome 0's texture from the paths that left the scene.
__global__ void __launch_bounds__(256) wa_miss(WfView v, DevScene s, AdjWave aw, uint32_t depth) {
    const uint32_t count = v.counters[kMissCount];
    const AdjView& a = *aw.view;
    if (a.env0 < 0 || !a.dEnv4) return;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t j = v.shadeQ[v.P - 1u - i];
        const DevRequest& q = v.reqs[v.ident[j].w].q;
        if (!(depth > 0 || q.backgroundVisible)) continue;
        const float4 d = v.rd[j], t4 = v.T[j], dl4 = aw.delta[j];
        const V3 rd{d.x, d.y, d.z};
        const bool prevDelta = (__float_as_uint(t4.w) & kFlagPrevDelta) != 0u;
        const float mis = (s.domeCount == 0 || depth == 0 || prevDelta) ? 1.0f : env_miss_mis(s, d.w, rd);
        const V3 T{t4.x, t4.y, t4.z}, dl{dl4.x, dl4.y, dl4.z};
        for (uint32_t k = 0; k < s.domeCount; ++k) {
            const DevDome& dm = s.domes[k];
            if (dm.env != a.env0) continue;
            add_env_grad(a, a.evalEnv, world_to_light(dm, rd), dl * T * dm.radiance * mis);
        }
    }
}

// Per-path records of the wave in request path order (pixel-major,
// sample-minor): the radiance a path replay needs (adjoint).
__global__ void __launch_bounds__(128) wf_records_out(WfView v) {
    const WaveDesc w = cur_wave(v);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < w.paths; j += gridDim.x * blockDim.x) {
        const WaveSeg& sg = find_seg(v, w, j, false);
        const uint32_t spp = v.reqs[sg.req].q.sampleCount;
        const size_t path = static_cast<size_t>(sg.pixelStart) * spp + (j - sg.pathOffset);
        v.recordsOut[path] = v.records[3 * static_cast<size_t>(j)];
    }
}

}  // namespace

// ===========================================================================
// host side
// ===========================================================================
// One pool of paths in flight with its queues, and the wave graph it replays.
// An instantiated wave graph and the launch parameters it bakes in (reused
// while a call's parameters are byte-identical: only the tables' contents
// differ between such calls, and the kernels read them from memory).
struct WaveGraph {
    cudaGraphExec_t exec = nullptr;
    std::vector<unsigned char> key;
    uint64_t lastUse = 0;
};

// Graphs kept per pool: a differentiable loop alternates a forward render
// and an adjoint (two different graphs), other callers render one kind.
constexpr int kGraphsPerPool = 4;

struct WavePool {
    DeviceBlock state, shadow, queues, records, adj, adjLog;
    WaveGraph graphs[kGraphsPerPool];
};

constexpr uint32_t kMaxConcurrentWaves = 4;

// A forward render with SHIRO_RENDER_KEEP_PATHS that ran as one wave leaves
// its path records and hit / visibility logs on pool 0; an adjoint of one of
// its requests, before any other wavefront call and any change of scene,
// parameters or configuration (ContextImpl::epoch), replays that request's
// paths of the wave without running the forward stages again.
struct KeptWave {
    bool valid = false;
    std::vector<DevRequest> qs;  // the render's requests, in its order
    uint64_t epoch = 0;
    uint32_t P = 0, depth = 0, lightSamples = 0;
    const void* state = nullptr;  // pool 0's blocks when it was kept
    const void* log = nullptr;
};

struct WavefrontState {
    ShiroWavefrontConfig cfg{};
    WavePool pools[kMaxConcurrentWaves];
    DeviceBlock tables;
    int smCount = 0;
    bool tuned = false;
    // streams of the waves in flight after the first, the event that forks
    // them from the context's stream and the events that join them to it
    cudaStream_t side[kMaxConcurrentWaves - 1] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[kMaxConcurrentWaves - 1] = {};
    DeviceBlock adjView;  // device copy of the adjoint's parameter view
    uint64_t graphClock = 0;
    KeptWave kept;
};

namespace {

WavefrontState* wf_state(ContextImpl* ctx) {
    if (!ctx->wavefront) {
        ctx->wavefront = new WavefrontState();
        ShiroWavefrontConfig& c = ctx->wavefront->cfg;
        // the values the autotuner picks for a 1080p 64-spp frame: pools of
        // 32 M paths (a pool is never larger than its request needs)
        c.paths_in_flight = 1u << 25;
        c.extend_block = 256;
        c.shade_block = 128;
        c.shadow_block = 128;
        c.use_graph = 1;
        c.shade_regs = 96;
        c.extend_steps = 4;
        c.refill_idle = 8;
        c.concurrent_waves = 2;
        c.bin_rays = 2;
        c.bin_shadow = 2;
        c.coop_extend = 2;
        c.coop_occlude = 2;
        c.extend_regs = 64;
        c.occlude_regs = 64;
        c.occlude_refill = 1;
        cudaDeviceGetAttribute(&ctx->wavefront->smCount, cudaDevAttrMultiProcessorCount, ctx->device);
    }
    return ctx->wavefront;
}

bool ensure_pool(ContextImpl* ctx, WavePool* wf, uint32_t P, uint32_t lightSamples) {
    const size_t p = P;
    const size_t stateBytes = p * (7 * sizeof(float4) + sizeof(uint32_t));
    const size_t shadowBytes = p * (2 + 2 * static_cast<size_t>(std::max(1u, lightSamples))) * sizeof(float4);
    const size_t ls = std::max(1u, lightSamples);
    const size_t queueBytes = (p * (4 + ls) + p * ls + kBins) * sizeof(uint32_t) + 64;  // + binned queue, buckets
    const size_t recordBytes = p * 3 * sizeof(float4);
    if (!ensure_block(ctx, &wf->state, stateBytes, "wavefront state")) return false;
    if (!ensure_block(ctx, &wf->shadow, shadowBytes, "wavefront shadow records")) return false;
    if (!ensure_block(ctx, &wf->queues, queueBytes, "wavefront queues")) return false;
    if (!ensure_block(ctx, &wf->records, recordBytes, "wavefront path records")) return false;
    return true;
}

WfView make_view(WavePool* wf, uint32_t P, uint32_t lightSamples, const WaveDesc* waves, const WaveSeg* segs,
                 const WfRequest* reqs) {
    WfView v;
    std::memset(&v, 0, sizeof(v));  // padding too: the bytes key the graph cache
    const size_t p = P;
    char* st = static_cast<char*>(wf->state.ptr);
    v.ro = reinterpret_cast<float4*>(st);
    v.rd = v.ro + p;
    v.T = v.rd + p;
    v.rad = v.T + p;
    v.ident = reinterpret_cast<uint4*>(v.rad + p);
    v.hit = reinterpret_cast<float4*>(v.ident + p);
    v.medium = v.hit + p;
    v.hitGid = reinterpret_cast<uint32_t*>(v.medium + p);
    float4* sh = static_cast<float4*>(wf->shadow.ptr);
    v.shOrigin = sh;
    v.shT = sh + p;
    v.shDir = sh + 2 * p;
    v.shC = sh + (2 + static_cast<size_t>(std::max(1u, lightSamples))) * p;
    uint32_t* qb = static_cast<uint32_t*>(wf->queues.ptr);
    v.counters = qb;
    v.rayQ0 = qb + 16;
    v.rayQ1 = v.rayQ0 + p;
    v.shadowQ = v.rayQ1 + p;
    v.shadowRayQ = v.shadowQ + p;
    v.shadeQ = v.shadowRayQ + p * static_cast<size_t>(std::max(1u, lightSamples));
    v.sortedQ = v.shadeQ + p;
    v.binCount = v.sortedQ + p * static_cast<size_t>(std::max(1u, lightSamples));
    v.records = static_cast<float4*>(wf->records.ptr);
    v.waves = waves;
    v.segs = segs;
    v.reqs = reqs;
    v.P = P;
    v.lightSamples = lightSamples;
    return v;
}

template <typename K>
int grid_for(K kernel, int block, int smCount) {
    int perSm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kernel, block, 0);
    return std::max(1, perSm) * smCount;
}

struct Plan {
    std::vector<WaveDesc> waves;
    std::vector<WaveSeg> segs;
    uint32_t maxDepth = 0;
    uint32_t maxWavePixels = 0;
    uint64_t paths = 0;
};

// Packs whole pixels of the requests, in order, into waves of <= P paths.
Plan plan_waves(const std::vector<DevRequest>& qs, uint32_t P) {
    Plan pl;
    WaveDesc cur{0, 0, 0, 0};
    auto flush = [&]() {
        if (cur.paths) {
            pl.maxWavePixels = std::max(pl.maxWavePixels, cur.pixels);
            pl.waves.push_back(cur);
        }
        cur = WaveDesc{static_cast<uint32_t>(pl.segs.size()), 0, 0, 0};
    };
    cur.segBegin = 0;
    for (uint32_t r = 0; r < qs.size(); ++r) {
        const DevRequest& q = qs[r];
        const uint64_t pixels = static_cast<uint64_t>(q.width) * q.height;
        if (q.sampleCount == 0 || pixels == 0 || q.maxDepth == 0) continue;
        pl.maxDepth = std::max(pl.maxDepth, q.maxDepth);
        pl.paths += pixels * q.sampleCount;
        uint64_t done = 0;
        while (done < pixels) {
            const uint32_t room = (P - cur.paths) / q.sampleCount;
            if (room == 0) {
                flush();
                continue;
            }
            const uint32_t take = static_cast<uint32_t>(std::min<uint64_t>(room, pixels - done));
            WaveSeg sg{};
            sg.req = r;
            sg.pixelStart = static_cast<uint32_t>(done);
            sg.pixelCount = take;
            sg.pathOffset = cur.paths;
            sg.pixelOffset = cur.pixels;
            pl.segs.push_back(sg);
            cur.segCount += 1;
            cur.paths += take * q.sampleCount;
            cur.pixels += take;
            done += take;
        }
    }
    flush();
    return pl;
}

struct Launch {
    WfView v;
    DevScene s;
    int gGen, gExt, gShade, gMiss, gShadow, gOcc, gRes;
    int bExt, bShade, bShadow;
    uint32_t depth;
    uint32_t shadeRegs;
    uint32_t binRays, binShadow;  // queue binning before extend (bounces >= 1) / occlude
    uint32_t coopExt, coopOcc;    // warp-cooperative triangle tests in extend / occlude
    uint32_t extRegs, occRegs;    // register caps of the per-lane traversal stages
    uint32_t occRefill;           // lane refill in the occlusion stage
    int gBin;
    AdjWave aw;                   // aw.on: the adjoint replay follows the forward stages
    uint32_t replayOnly;          // the adjoint replay alone, of a kept forward wave
    int gAdjShade, gAdjShadow, gAdjMiss, gAdjHits;
    bool ext;  // the scene uses transmission, opacity or emitters
};

// The traversal stages' instantiations: cooperative triangle tests (at 64
// registers) or per-lane ones with a register cap of 64, 48 or 40.
template <typename F>
auto with_extend_kernel(uint32_t coop, uint32_t regs, bool log, F&& f) {
    if (log) return f(wf_extend<false, 4, true>);
    if (coop) return f(wf_extend<true, 4>);
    if (regs == 48) return f(wf_extend<false, 5>);
    if (regs == 40) return f(wf_extend<false, 6>);
    return f(wf_extend<false, 4>);
}
template <typename F>
auto with_occlude_kernel(uint32_t coop, uint32_t refill, uint32_t regs, F&& f) {
    if (coop) return f(wf_occlude<1, 4>);
    if (refill) return f(wf_occlude<2, 4>);
    if (regs == 48) return f(wf_occlude<0, 5>);
    if (regs == 40) return f(wf_occlude<0, 6>);
    return f(wf_occlude<0, 4>);
}

void launch_extend(const Launch& L, cudaStream_t st, uint32_t cur, uint32_t binned, uint32_t depth) {
    with_extend_kernel(L.coopExt, L.extRegs, L.v.hitLog != nullptr, [&](auto kern) {
        kern<<<L.gExt, L.bExt, 0, st>>>(L.v, L.s, cur, binned, depth);
        return 0;
    });
}

void launch_occlude(const Launch& L, cudaStream_t st, uint32_t binned) {
    with_occlude_kernel(L.coopOcc, L.occRefill, L.occRegs, [&](auto kern) {
        kern<<<L.gOcc, L.bShadow, 0, st>>>(L.v, L.s, binned);
        return 0;
    });
}

void enqueue_replay(const Launch& L, cudaStream_t st) {
    wa_begin<<<1, 32, 0, st>>>(L.v);
    wa_generate<<<L.gGen, 128, 0, st>>>(L.v, L.aw);
    for (uint32_t d = 0; d < L.depth; ++d) {
        const uint32_t cur = d & 1u;
        wa_hits<<<L.gAdjHits, 256, 0, st>>>(L.v, cur, d);  // no tracing: the forward stages' hits and visibility
        if (L.ext) {
            wa_shade<true><<<L.gAdjShade, 128, 0, st>>>(L.v, L.s, L.aw, cur, d);
        } else {
            wa_shade<false><<<L.gAdjShade, 128, 0, st>>>(L.v, L.s, L.aw, cur, d);
        }
        wa_miss<<<L.gAdjMiss, 256, 0, st>>>(L.v, L.s, L.aw, d);
        if (L.ext) {
            wa_shadow<true><<<L.gAdjShadow, 128, 0, st>>>(L.v, L.s, L.aw);
        } else {
            wa_shadow<false><<<L.gAdjShadow, 128, 0, st>>>(L.v, L.s, L.aw);
        }
        wf_end_bounce<<<1, 32, 0, st>>>(L.v, cur);
    }
}

void enqueue_binning(const Launch& L, cudaStream_t st, uint32_t which, uint32_t cur) {
    cudaMemsetAsync(L.v.binCount, 0, kBins * sizeof(uint32_t), st);
    wf_bin_count<<<L.gBin, 256, 0, st>>>(L.v, which, cur);
    wf_bin_scan<<<1, 1024, 0, st>>>(L.v);
    wf_bin_scatter<<<L.gBin, 256, 0, st>>>(L.v, which, cur);
}

// The shade stage's instantiation for a register cap (80, 96 or 128) and
// the scene's lobe set.
template <typename F>
auto with_shade_kernel(uint32_t regs, bool ext, F&& f) {
    if (ext) {
        if (regs == 80) return f(wf_shade<80, true>);
        if (regs == 96) return f(wf_shade<96, true>);
        return f(wf_shade<128, true>);
    }
    if (regs == 80) return f(wf_shade<80, false>);
    if (regs == 96) return f(wf_shade<96, false>);
    return f(wf_shade<128, false>);
}

void launch_shade(const Launch& L, cudaStream_t st, uint32_t cur, uint32_t d) {
    with_shade_kernel(L.shadeRegs, L.ext, [&](auto kern) {
        kern<<<L.gShade, L.bShade, 0, st>>>(L.v, L.s, cur, d);
        return 0;
    });
    wf_miss<<<L.gMiss, 256, 0, st>>>(L.v, L.s, d);
}

void enqueue_wave(const Launch& L, cudaStream_t st) {
    if (L.replayOnly) {
        enqueue_replay(L, st);
        return;
    }
    wf_begin<<<1, 32, 0, st>>>(L.v);
    wf_generate<<<L.gGen, 128, 0, st>>>(L.v);
    for (uint32_t d = 0; d < L.depth; ++d) {
        const uint32_t cur = d & 1u;
        const uint32_t br = (L.binRays && d > 0) ? 1u : 0u;  // camera rays are coherent already
        if (br) enqueue_binning(L, st, 0u, cur);
        launch_extend(L, st, cur, br, d);
        launch_shade(L, st, cur, d);
        if (L.binShadow) enqueue_binning(L, st, 1u, cur);
        launch_occlude(L, st, L.binShadow);
        wf_shadow<<<L.gShadow, 256, 0, st>>>(L.v, L.s, d);
        wf_end_bounce<<<1, 32, 0, st>>>(L.v, cur);
    }
    if (L.aw.on) enqueue_replay(L, st);
    else if (L.v.recordsOut) wf_records_out<<<L.gRes, 128, 0, st>>>(L.v);
    else wf_resolve<<<L.gRes, 128, 0, st>>>(L.v);
}

// The same wave with events around every stage launch (diagnostic timing).
void enqueue_wave_timed(const Launch& L, cudaStream_t st, std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>>& ev) {
    auto timed = [&](int stage, auto&& launch) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, st);
        launch();
        cudaEventRecord(b, st);
        ev.push_back({stage, {a, b}});
    };
    if (L.replayOnly) {
        timed(4, [&] { enqueue_replay(L, st); });
        return;
    }
    timed(5, [&] { wf_begin<<<1, 32, 0, st>>>(L.v); });
    timed(0, [&] { wf_generate<<<L.gGen, 128, 0, st>>>(L.v); });
    for (uint32_t d = 0; d < L.depth; ++d) {
        const uint32_t cur = d & 1u;
        const uint32_t br = (L.binRays && d > 0) ? 1u : 0u;
        timed(1, [&] {
            if (br) enqueue_binning(L, st, 0u, cur);
            launch_extend(L, st, cur, br, d);
        });
        timed(2, [&] { launch_shade(L, st, cur, d); });
        timed(3, [&] {
            if (L.binShadow) enqueue_binning(L, st, 1u, cur);
            launch_occlude(L, st, L.binShadow);
        });
        timed(5, [&] { wf_shadow<<<L.gShadow, 256, 0, st>>>(L.v, L.s, d); });
        timed(5, [&] { wf_end_bounce<<<1, 32, 0, st>>>(L.v, cur); });
    }
    timed(4, [&] {
        if (L.aw.on) enqueue_replay(L, st);
        else if (L.v.recordsOut) wf_records_out<<<L.gRes, 128, 0, st>>>(L.v);
        else wf_resolve<<<L.gRes, 128, 0, st>>>(L.v);
    });
}

// True when `a` and `b` describe the same paths (SHIRO_RENDER_KEEP_PATHS aside).
bool same_paths(DevRequest a, DevRequest b) {
    a.flags &= ~SHIRO_RENDER_KEEP_PATHS;
    b.flags &= ~SHIRO_RENDER_KEEP_PATHS;
    return std::memcmp(&a, &b, sizeof(DevRequest)) == 0;
}

// Renders the requests (device AOV planes in `aovs`) with configuration
// `cfg`.  maxWaves limits the waves run (autotuning); returns paths traced.
// adj: run the adjoint replay after each wave's forward stages (or alone,
// over a kept forward wave of the same request); keep: log the forward
// stages of a one-wave render and keep its pool for such an adjoint;
// waveDone: called on this thread with each wave's segments once the wave
// has finished on the device, in wave order (not after a failure or cancel).
using WaveDone = std::function<void(const WaveSeg* segs, uint32_t count)>;
int run_waves(ContextImpl* ctx, WavefrontState* wf, const ShiroWavefrontConfig& cfg, const std::vector<DevRequest>& qs,
              const std::vector<AovPtrs>& aovs, const volatile int* cancel, uint32_t maxWaves, uint64_t* pathsOut,
              double* msOut, float4* recordsOut = nullptr, const AdjView* adj = nullptr, bool keep = false,
              const WaveDone* waveDone = nullptr) {
    // every call below reuses the pools: a kept wave serves at most the call that follows it
    KeptWave kept;
    std::swap(kept, wf->kept);
    wf->kept.valid = false;
    // light samples per shading point, pool size and wave plan of a request list
    uint32_t lightSamples = 0;
    Plan pl;
    auto plan_for = [&](const std::vector<DevRequest>& rs) {
        lightSamples = ctx->scene.distantCount;
        uint32_t domeSamplesMax = 1, maxSpp = 1;
        for (const DevRequest& q : rs) {
            domeSamplesMax = std::max(domeSamplesMax, q.domeSamples);
            maxSpp = std::max(maxSpp, q.sampleCount);
        }
        lightSamples += ctx->scene.domeCount * domeSamplesMax;
        if (ctx->scene.emissiveCount > 0 && ctx->scene.emissiveSum > 0.0f) lightSamples += 1;
        pl = plan_waves(rs, std::max(cfg.paths_in_flight, maxSpp));
    };
    // an adjoint of one of the kept wave's requests replays that wave (its
    // plan again: the configuration is unchanged while the epoch is)
    int32_t target = -1;
    if (adj && qs.size() == 1 && kept.valid && kept.epoch == ctx->epoch)
        for (size_t r = 0; r < kept.qs.size() && target < 0; ++r)
            if (same_paths(kept.qs[r], qs[0])) target = static_cast<int32_t>(r);
    if (target >= 0) {
        plan_for(kept.qs);
        if (pl.waves.size() != 1 || maxWaves < 1 || pl.waves[0].paths != kept.P || pl.maxDepth != kept.depth ||
            lightSamples != kept.lightSamples || kept.state != wf->pools[0].state.ptr || kept.log != wf->pools[0].adjLog.ptr)
            target = -1;
    }
    bool replayOnly = target >= 0;
    const std::vector<DevRequest>& rqs = replayOnly ? kept.qs : qs;  // the requests the tables describe
    if (!replayOnly) plan_for(qs);
    if (lightSamples > kMaxLightSamples)
        return fail(ctx, SHIRO_ERR_UNSUPPORTED_SCENE, "wavefront form: more than 8 light samples per shading point");
    if (pl.waves.empty()) {
        *pathsOut = 0;
        return SHIRO_OK;
    }
    uint32_t used = std::min<uint32_t>(static_cast<uint32_t>(pl.waves.size()), maxWaves);
    keep = keep && !adj && !recordsOut && pl.waves.size() == 1 && used == 1;
    const bool logs = adj || keep;  // the forward stages log hits and visibility
    // waves in flight at once: pool k runs waves k, k + nl, ... on its own
    // stream (graphs only; the diagnostic per-stage timing runs one)
    const uint32_t nl = cfg.use_graph ? std::max(1u, std::min({cfg.concurrent_waves, used, kMaxConcurrentWaves})) : 1u;
    uint32_t poolP[kMaxConcurrentWaves] = {};
    for (uint32_t w = 0; w < used; ++w) poolP[w % nl] = std::max(poolP[w % nl], pl.waves[w].paths);
    for (uint32_t k = 0; k < nl; ++k)
        if (!ensure_pool(ctx, &wf->pools[k], poolP[k], lightSamples)) return SHIRO_ERR_OUT_OF_MEMORY;
    for (uint32_t k = 0; k < nl && logs; ++k)  // each pool's hit / visibility logs
        if (!ensure_block(ctx, &wf->pools[k].adjLog,
                          static_cast<size_t>(poolP[k]) * std::max(1u, pl.maxDepth) *
                              (sizeof(float4) + sizeof(uint32_t) + sizeof(uint8_t)), "adjoint hit log"))
            return SHIRO_ERR_OUT_OF_MEMORY;
    // (same sizes as when the wave was kept, so nothing moved; checked all the same)
    replayOnly = replayOnly && kept.state == wf->pools[0].state.ptr && kept.log == wf->pools[0].adjLog.ptr;
    if (target >= 0 && !replayOnly) return fail(ctx, SHIRO_ERR_CUDA, "kept wave moved");  // not reached: sizes are equal
    AdjView adjCopy;  // (pageable source of an asynchronous copy: staged before the call returns)
    if (adj) {  // per-slot replay state of each pool, and the parameter view on the device
        for (uint32_t k = 0; k < nl; ++k)
            if (!ensure_block(ctx, &wf->pools[k].adj,
                              static_cast<size_t>(poolP[k]) * (kAdjSlotFloat4 + kAdjLightFloat4 * std::max(1u, lightSamples)) *
                                  sizeof(float4), "adjoint replay state"))
                return SHIRO_ERR_OUT_OF_MEMORY;
        if (!ensure_block(ctx, &wf->adjView, sizeof(AdjView), "adjoint view")) return SHIRO_ERR_OUT_OF_MEMORY;
        adjCopy = *adj;
        adjCopy.targetReq = replayOnly ? static_cast<uint32_t>(target) : 0u;
        const cudaError_t ce = cudaMemcpyAsync(wf->adjView.ptr, &adjCopy, sizeof(AdjView), cudaMemcpyHostToDevice, ctx->stream);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "adjoint view");
    }
    if (nl > 1 && !wf->fork) {
        const cudaError_t ce = cudaEventCreateWithFlags(&wf->fork, cudaEventDisableTiming);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "wavefront side stream");
    }
    for (uint32_t k = 1; k < nl; ++k) {
        if (wf->side[k - 1]) continue;
        cudaError_t ce = cudaStreamCreateWithFlags(&wf->side[k - 1], cudaStreamNonBlocking);
        if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&wf->join[k - 1], cudaEventDisableTiming);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "wavefront side stream");
    }
    // tables: waves, segments, requests (the replay of a kept wave writes no AOVs)
    std::vector<WfRequest> rq(rqs.size());
    for (size_t r = 0; r < rqs.size(); ++r)
        rq[r] = WfRequest{rqs[r], replayOnly ? AovPtrs{nullptr, nullptr, nullptr, nullptr} : aovs[r]};
    const size_t tb = pl.waves.size() * sizeof(WaveDesc) + pl.segs.size() * sizeof(WaveSeg) + rq.size() * sizeof(WfRequest) + 256;
    if (!ensure_block(ctx, &wf->tables, tb, "wavefront tables")) return SHIRO_ERR_OUT_OF_MEMORY;
    char* t = static_cast<char*>(wf->tables.ptr);
    WaveDesc* dWaves = reinterpret_cast<WaveDesc*>(t);
    WaveSeg* dSegs = reinterpret_cast<WaveSeg*>(t + ((pl.waves.size() * sizeof(WaveDesc) + 63) & ~size_t(63)));
    WfRequest* dReqs = reinterpret_cast<WfRequest*>(reinterpret_cast<char*>(dSegs) +
                                                    ((pl.segs.size() * sizeof(WaveSeg) + 63) & ~size_t(63)));
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(dWaves, pl.waves.data(), pl.waves.size() * sizeof(WaveDesc), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dSegs, pl.segs.data(), pl.segs.size() * sizeof(WaveSeg), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dReqs, rq.data(), rq.size() * sizeof(WfRequest), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "wavefront tables");
    Launch L;
    std::memset(&L, 0, sizeof(L));  // padding too: the bytes key the graph cache
    L.v = make_view(&wf->pools[0], poolP[0], lightSamples, dWaves, dSegs, dReqs);
    L.v.waveStride = nl;
    L.v.recordsOut = recordsOut;
    L.s = ctx->scene;
    if (ctx->bvhWidth != 2 && ctx->nodes8) {  // the wavefront stages traverse the wide BVH unless told otherwise
        L.s.nodes8 = ctx->nodes8;
        L.s.tris = ctx->tris8;
    }
    L.bExt = static_cast<int>(cfg.extend_block);
    L.bShade = static_cast<int>(cfg.shade_block);
    L.bShadow = static_cast<int>(cfg.shadow_block);
    L.gGen = grid_for(wf_generate, 128, wf->smCount);
    L.coopExt = cfg.coop_extend == 1 ? 1u : 0u;
    L.coopOcc = cfg.coop_occlude == 1 ? 1u : 0u;
    L.extRegs = cfg.extend_regs ? cfg.extend_regs : 64;
    L.occRegs = cfg.occlude_regs ? cfg.occlude_regs : 64;
    L.occRefill = cfg.occlude_refill == 1 ? 1u : 0u;
    L.gExt = with_extend_kernel(L.coopExt, L.extRegs, logs,
                                [&](auto kern) { return grid_for(kern, L.bExt, wf->smCount); });
    L.shadeRegs = cfg.shade_regs;
    L.ext = ctx->extendedMaterials;
    L.gShade = with_shade_kernel(L.shadeRegs, L.ext, [&](auto kern) { return grid_for(kern, L.bShade, wf->smCount); });
    L.v.travSteps = static_cast<int>(cfg.extend_steps ? cfg.extend_steps : 4);
    L.v.refillIdle = static_cast<int>(cfg.refill_idle ? cfg.refill_idle : 8);
    L.gMiss = grid_for(wf_miss, 256, wf->smCount);
    L.gShadow = grid_for(wf_shadow, 256, wf->smCount);
    L.gOcc = with_occlude_kernel(L.coopOcc, L.occRefill, L.occRegs, [&](auto kern) { return grid_for(kern, L.bShadow, wf->smCount); });
    L.gRes = grid_for(wf_resolve, 128, wf->smCount);
    L.gBin = grid_for(wf_bin_scatter, 256, wf->smCount);
    L.gAdjShade = L.ext ? grid_for(wa_shade<true>, 128, wf->smCount) : grid_for(wa_shade<false>, 128, wf->smCount);
    L.gAdjShadow = L.ext ? grid_for(wa_shadow<true>, 128, wf->smCount) : grid_for(wa_shadow<false>, 128, wf->smCount);
    L.gAdjMiss = grid_for(wa_miss, 256, wf->smCount);
    L.gAdjHits = grid_for(wa_hits, 256, wf->smCount);
    L.binRays = cfg.bin_rays == 1 ? 1u : 0u;
    L.binShadow = cfg.bin_shadow == 1 ? 1u : 0u;
    {
        const DevScene& sc = ctx->scene;
        const V3 ext{sc.boundsHi.x - sc.boundsLo.x, sc.boundsHi.y - sc.boundsLo.y, sc.boundsHi.z - sc.boundsLo.z};
        L.v.binLo = sc.boundsLo;
        L.v.binScale = V3{ext.x > 0.0f ? 8.0f / ext.x : 0.0f, ext.y > 0.0f ? 8.0f / ext.y : 0.0f,
                          ext.z > 0.0f ? 8.0f / ext.z : 0.0f};
    }
    L.depth = pl.maxDepth;
    auto adj_wave = [&](uint32_t k) {
        AdjWave aw;
        std::memset(&aw, 0, sizeof(aw));
        if (!adj) return aw;
        const size_t p = poolP[k];
        float4* b = static_cast<float4*>(wf->pools[k].adj.ptr);
        aw.view = static_cast<const AdjView*>(wf->adjView.ptr);
        aw.lrem = b;
        aw.delta = b + p;
        aw.vtx = b + 2 * p;
        aw.cont = b + 5 * p;
        aw.lgrad = b + 7 * p;
        aw.on = 1u;
        return aw;
    };
    // the forward stages' hit / visibility logs of each pool; every hit record
    // starts as a miss, so that a replay ray the forward did not trace (it
    // cannot happen when both follow the same decisions) reads a miss, never
    // a triangle of another call's scene (a kept wave's logs are read as they are)
    auto add_logs = [&](WfView& v, uint32_t k) -> cudaError_t {
        if (!logs) return cudaSuccess;
        const size_t n = static_cast<size_t>(poolP[k]) * std::max(1u, pl.maxDepth);
        char* b = static_cast<char*>(wf->pools[k].adjLog.ptr);
        v.hitLog = reinterpret_cast<float4*>(b);
        v.gidLog = reinterpret_cast<uint32_t*>(b + n * sizeof(float4));
        v.visLog = reinterpret_cast<uint8_t*>(b + n * (sizeof(float4) + sizeof(uint32_t)));
        return replayOnly ? cudaSuccess : cudaMemsetAsync(v.hitLog, 0xff, n * sizeof(float4), st);
    };
    if ((e = add_logs(L.v, 0)) != cudaSuccess) return cuda_fail(ctx, e, "adjoint hit log");
    L.aw = adj_wave(0);
    L.replayOnly = replayOnly ? 1u : 0u;
    Launch lanes[kMaxConcurrentWaves];
    for (uint32_t k = 0; k < nl; ++k) {
        std::memcpy(&lanes[k], &L, sizeof(Launch));  // bytes, padding included: they key the graph cache
        if (k > 0) {
            WfView v = make_view(&wf->pools[k], poolP[k], lightSamples, dWaves, dSegs, dReqs);
            v.waveStride = nl;
            v.travSteps = L.v.travSteps;
            v.refillIdle = L.v.refillIdle;
            v.binLo = L.v.binLo;
            v.binScale = L.v.binScale;
            v.recordsOut = recordsOut;
            if ((e = add_logs(v, k)) != cudaSuccess) return cuda_fail(ctx, e, "adjoint hit log");
            std::memcpy(&lanes[k].v, &v, sizeof(WfView));
            const AdjWave aw = adj_wave(k);
            std::memcpy(&lanes[k].aw, &aw, sizeof(AdjWave));
        }
        // wf_begin adds the stride to the wave index: start one stride below k
        // (the replay alone starts at its wave, 0)
        const uint32_t first = replayOnly ? 0u : k - nl;
        e = cudaMemsetAsync(lanes[k].v.counters, 0, 16 * sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(lanes[k].v.counters + 3, &first, 4, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "wavefront counters");
    }

    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> ev;
    cudaGraphExec_t exec[kMaxConcurrentWaves] = {};
    int rc = SHIRO_OK;
    if (cfg.use_graph) {
        for (uint32_t k = 0; k < nl && rc == SHIRO_OK; ++k) {
            WavePool& pool = wf->pools[k];
            const unsigned char* key = reinterpret_cast<const unsigned char*>(&lanes[k]);
            WaveGraph* slot = nullptr;  // the matching graph, else the least recently used slot
            for (WaveGraph& g : pool.graphs) {
                if (g.exec && g.key.size() == sizeof(Launch) && std::memcmp(g.key.data(), key, sizeof(Launch)) == 0) {
                    slot = &g;
                    break;
                }
                if (!slot || (slot->exec && (!g.exec || g.lastUse < slot->lastUse))) slot = &g;
            }
            slot->lastUse = ++wf->graphClock;
            if (slot->exec && slot->key.size() == sizeof(Launch) && std::memcmp(slot->key.data(), key, sizeof(Launch)) == 0) {
                exec[k] = slot->exec;
                continue;
            }
            if (slot->exec) cudaGraphExecDestroy(slot->exec);
            slot->exec = nullptr;
            slot->key.clear();
            cudaGraph_t graph = nullptr;
            e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                enqueue_wave(lanes[k], st);
                e = cudaStreamEndCapture(st, &graph);
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&exec[k], graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                exec[k] = nullptr;
                rc = cuda_fail(ctx, e, "wavefront graph");
            } else {
                slot->exec = exec[k];
                slot->key.assign(key, key + sizeof(Launch));
            }
        }
    }
    // the waves in flight after the first run on side streams, after the
    // tables and counters written above, and the context's stream waits for
    // them at the end
    if (rc == SHIRO_OK && nl > 1) {
        e = cudaEventRecord(wf->fork, st);
        for (uint32_t k = 1; k < nl && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(wf->side[k - 1], wf->fork, 0);
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "wavefront fork");
    }
    auto lane_stream = [&](uint32_t k) { return k == 0 ? st : wf->side[k - 1]; };
    uint64_t launches = 0;
    uint32_t launchedWaves = 0;
    // with a cancel flag, nl + 1 waves are queued at most, so the flag is read
    // between waves that ran (a wave takes milliseconds, a launch microseconds)
    LaunchThrottle throttle(cancel, nl + 1);
    // an event after each wave tells the caller of its finished pixels
    struct Events {
        std::vector<cudaEvent_t> ev;
        ~Events() {
            for (cudaEvent_t x : ev)
                if (x) cudaEventDestroy(x);
        }
    } waveEv;
    if (waveDone && rc == SHIRO_OK) {
        waveEv.ev.assign(used, nullptr);
        for (cudaEvent_t& x : waveEv.ev)
            if (rc == SHIRO_OK && (e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming)) != cudaSuccess)
                rc = cuda_fail(ctx, e, "wave events");
    }
    uint32_t delivered = 0;
    auto deliver = [&](bool wait) {  // the finished waves, in order
        while (waveDone && rc == SHIRO_OK && delivered < launchedWaves) {
            const cudaError_t q = wait ? cudaEventSynchronize(waveEv.ev[delivered]) : cudaEventQuery(waveEv.ev[delivered]);
            if (q != cudaSuccess) {
                if (q != cudaErrorNotReady) rc = cuda_fail(ctx, q, "wavefront render");
                return;
            }
            const WaveDesc& wd = pl.waves[delivered++];
            (*waveDone)(pl.segs.data() + wd.segBegin, wd.segCount);
        }
    };
    for (uint32_t w = 0; w < used && rc == SHIRO_OK; ++w) {
        if (!throttle.before_launch()) {
            rc = fail(ctx, SHIRO_ERR_CANCELLED, "cancelled");
            break;
        }
        const uint32_t k = w % nl;
        if (exec[k]) {
            e = cudaGraphLaunch(exec[k], lane_stream(k));
        } else {
            enqueue_wave_timed(L, st, ev);
            e = cudaGetLastError();
        }
        if (waveDone && e == cudaSuccess) e = cudaEventRecord(waveEv.ev[w], exec[k] ? lane_stream(k) : st);
        throttle.after_launch(exec[k] ? lane_stream(k) : st);
        if (replayOnly)
            launches += 2ull + 5ull * L.depth;
        else
            launches += 3 + 6ull * L.depth + (L.binShadow ? 3ull * L.depth : 0ull) +
                        (L.binRays && L.depth > 1 ? 3ull * (L.depth - 1) : 0ull) + (adj ? 2ull + 5ull * L.depth - 1ull : 0ull);
        ++launchedWaves;
        if (e != cudaSuccess) rc = cuda_fail(ctx, e, "wavefront launch");
        deliver(false);
    }
    deliver(true);
    for (uint32_t k = 1; k < nl; ++k) {  // join (also after a failed launch: side work must end before we return)
        cudaEventRecord(wf->join[k - 1], wf->side[k - 1]);
        cudaStreamWaitEvent(st, wf->join[k - 1], 0);
    }
    cudaEventRecord(e1, st);
    e = cudaEventSynchronize(e1);
    if (e != cudaSuccess && rc == SHIRO_OK) rc = cuda_fail(ctx, e, "wavefront render");
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    double stageMs[6] = {0, 0, 0, 0, 0, 0};
    uint64_t stageN[6] = {0, 0, 0, 0, 0, 0};
    for (auto& x : ev) {
        float v = 0.0f;
        if (rc == SHIRO_OK) cudaEventElapsedTime(&v, x.second.first, x.second.second);
        stageMs[x.first] += v;
        stageN[x.first] += 1;
        cudaEventDestroy(x.second.first);
        cudaEventDestroy(x.second.second);
    }
    ctx->stats.waves = launchedWaves;  // also after a cancel: the waves that ran
    if (rc != SHIRO_OK) {
        cudaStreamSynchronize(st);
        return rc;
    }
    if ((rc = check_device_error(ctx)) != SHIRO_OK) return rc;
    uint64_t paths = 0;
    for (uint32_t w = 0; w < used; ++w) paths += pl.waves[w].paths;
    *pathsOut = paths;
    if (msOut) *msOut = ms;
    ctx->stats.kernel_ms = ms;
    ctx->stats.kernel_launches = launches;
    ctx->stats.paths = paths;
    if (keep) {
        KeptWave& kw = wf->kept;
        kw.valid = true;
        kw.qs = qs;
        kw.epoch = ctx->epoch;
        kw.P = pl.waves[0].paths;
        kw.depth = pl.maxDepth;
        kw.lightSamples = lightSamples;
        kw.state = wf->pools[0].state.ptr;
        kw.log = wf->pools[0].adjLog.ptr;
    }
    if (!ev.empty()) {
        for (int k = 0; k < 6; ++k) {
            ctx->stats.stage_ms[k] = stageMs[k];
            ctx->stats.stage_launches[k] = stageN[k];
        }
        ctx->stats.path_kernel_ms = stageMs[1];
        ctx->stats.path_kernel_launches = stageN[1];
    }
    return SHIRO_OK;
}

}  // namespace

// A host plane the device may write in place: page-locked and mapped at
// the same address (unified addressing).
static bool device_writable_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost && a.devicePointer == p;
}

int wavefront_render(ContextImpl* ctx, const ShiroRenderDesc* reqs, uint32_t count, const volatile int* cancel,
                     ShiroAovs* outs, ShiroPixelsReady ready, void* user) {
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    WavefrontState* wf = wf_state(ctx);
    std::vector<DevRequest> qs(count);
    std::vector<AovPtrs> aov(count);
    // host planes that are page-locked and mapped are written in place by the
    // resolve stage, wave by wave while later waves render (no copy after the
    // last wave); other host planes go through device staging and one copy
    std::vector<char> direct(count, 0);
    uint64_t stagingFloats = 0;
    for (uint32_t r = 0; r < count; ++r) {
        int rc = validate_request(ctx, reqs[r]);
        if (rc != SHIRO_OK) return rc;
        if (!outs[r].beauty || !outs[r].albedo || !outs[r].normal || !outs[r].depth)
            return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "null AOV pointer");
        qs[r] = make_request(reqs[r]);
        const uint64_t px = static_cast<uint64_t>(reqs[r].settings.width) * reqs[r].settings.height;
        direct[r] = !outs[r].on_device && px > 0 && reqs[r].sample_count > 0 && reqs[r].settings.max_depth > 0 &&
                    device_writable_host(outs[r].beauty) &&
                    device_writable_host(outs[r].albedo) && device_writable_host(outs[r].normal) &&
                    device_writable_host(outs[r].depth);
        if (!outs[r].on_device && !direct[r]) stagingFloats += 11ull * px;
    }
    if (stagingFloats && !ensure_block(ctx, &ctx->aovScratch, stagingFloats * sizeof(float), "AOV staging"))
        return SHIRO_ERR_OUT_OF_MEMORY;
    uint64_t off = 0;
    for (uint32_t r = 0; r < count; ++r) {
        const uint64_t px = static_cast<uint64_t>(reqs[r].settings.width) * reqs[r].settings.height;
        if (outs[r].on_device || direct[r]) {
            aov[r] = AovPtrs{outs[r].beauty, outs[r].albedo, outs[r].normal, outs[r].depth};
        } else {
            float* b = static_cast<float*>(ctx->aovScratch.ptr) + off;
            aov[r] = AovPtrs{b, b + 4 * px, b + 7 * px, b + 10 * px};
            off += 11 * px;
        }
        // requests without samples or bounces (the waves hold no paths of
        // them) get cleared planes (FrameBuffer::Clear), what TracePath
        // leaves them with
        if (reqs[r].sample_count == 0 || px == 0 || reqs[r].settings.max_depth == 0) {
            cudaMemsetAsync(aov[r].beauty, 0, px * 16, ctx->stream);
            cudaMemsetAsync(aov[r].albedo, 0, px * 12, ctx->stream);
            cudaMemsetAsync(aov[r].normal, 0, px * 12, ctx->stream);
            std::vector<float> inf(px, __builtin_inff());
            if (px) cudaMemcpyAsync(aov[r].depth, inf.data(), px * 4, cudaMemcpyHostToDevice, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
        }
    }
    ctx->stats.path_kernel_ms = 0.0;
    ctx->stats.path_kernel_launches = 0;
    for (int k = 0; k < 6; ++k) {
        ctx->stats.stage_ms[k] = 0.0;
        ctx->stats.stage_launches[k] = 0;
    }
    uint64_t paths = 0;
    const bool keep = count >= 1 && (reqs[0].flags & SHIRO_RENDER_KEEP_PATHS) != 0;
    // planes the resolve stage writes in place are reported wave by wave,
    // the others (staged, or cleared for want of samples) whole at the end
    auto in_place = [&](uint32_t r) {
        return (outs[r].on_device || direct[r]) && reqs[r].sample_count > 0 && reqs[r].settings.max_depth > 0 &&
               static_cast<uint64_t>(reqs[r].settings.width) * reqs[r].settings.height > 0;
    };
    const WaveDone onWave = [&](const WaveSeg* segs, uint32_t n) {
        for (uint32_t i = 0; i < n; ++i)
            if (in_place(segs[i].req)) ready(user, segs[i].req, segs[i].pixelStart, segs[i].pixelCount);
    };
    int rc = run_waves(ctx, wf, wf->cfg, qs, aov, cancel, 0xffffffffu, &paths, nullptr, nullptr, nullptr, keep,
                       ready ? &onWave : nullptr);
    if (rc == SHIRO_ERR_CANCELLED) {
        // a cancelled batch is discarded (RenderParam.cpp:791-798): cleared
        // planes, as FrameBuffer::Clear leaves them (FrameBuffer.cpp:19-24);
        // no wave may still be writing host planes in place
        cudaStreamSynchronize(ctx->stream);
        for (uint32_t r = 0; r < count; ++r) {
            const uint64_t px = static_cast<uint64_t>(reqs[r].settings.width) * reqs[r].settings.height;
            if (outs[r].on_device) {
                cudaMemsetAsync(outs[r].beauty, 0, px * 16, ctx->stream);
                cudaMemsetAsync(outs[r].albedo, 0, px * 12, ctx->stream);
                cudaMemsetAsync(outs[r].normal, 0, px * 12, ctx->stream);
                std::vector<float> inf(px, __builtin_inff());
                if (px) cudaMemcpyAsync(outs[r].depth, inf.data(), px * 4, cudaMemcpyHostToDevice, ctx->stream);
                cudaStreamSynchronize(ctx->stream);
            } else {
                std::fill(outs[r].beauty, outs[r].beauty + 4 * px, 0.0f);
                std::fill(outs[r].albedo, outs[r].albedo + 3 * px, 0.0f);
                std::fill(outs[r].normal, outs[r].normal + 3 * px, 0.0f);
                std::fill(outs[r].depth, outs[r].depth + px, __builtin_inff());
            }
        }
        return rc;
    }
    if (rc != SHIRO_OK) return rc;
    for (uint32_t r = 0; r < count; ++r) {
        if (outs[r].on_device || direct[r]) continue;
        const uint64_t px = static_cast<uint64_t>(reqs[r].settings.width) * reqs[r].settings.height;
        cudaError_t e = cudaMemcpyAsync(outs[r].beauty, aov[r].beauty, px * 16, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(outs[r].albedo, aov[r].albedo, px * 12, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(outs[r].normal, aov[r].normal, px * 12, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(outs[r].depth, aov[r].depth, px * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "AOV readback");
    }
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "AOV readback");
    ctx->stats.device_bytes = ctx->deviceBytes();
    for (uint32_t r = 0; r < count && ready; ++r) {
        const uint64_t px = static_cast<uint64_t>(reqs[r].settings.width) * reqs[r].settings.height;
        if (px && !in_place(r)) ready(user, r, 0, px);
    }
    return SHIRO_OK;
}

int wavefront_path_records(ContextImpl* ctx, const ShiroRenderDesc& req, float4* out) {
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    WavefrontState* wf = wf_state(ctx);
    std::vector<DevRequest> qs{make_request(req)};
    std::vector<AovPtrs> aov{AovPtrs{nullptr, nullptr, nullptr, nullptr}};
    uint64_t paths = 0;
    return run_waves(ctx, wf, wf->cfg, qs, aov, nullptr, 0xffffffffu, &paths, nullptr, out);
}

int wavefront_adjoint(ContextImpl* ctx, const ShiroRenderDesc& req, const AdjView& adj) {
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    WavefrontState* wf = wf_state(ctx);
    std::vector<DevRequest> qs{make_request(req)};
    std::vector<AovPtrs> aov{AovPtrs{nullptr, nullptr, nullptr, nullptr}};
    uint64_t paths = 0;
    return run_waves(ctx, wf, wf->cfg, qs, aov, nullptr, 0xffffffffu, &paths, nullptr, nullptr, &adj);
}

void wavefront_free(ContextImpl* ctx) {
    if (!ctx->wavefront) return;
    WavefrontState* wf = ctx->wavefront;
    for (cudaStream_t sd : wf->side)
        if (sd) cudaStreamSynchronize(sd);
    for (WavePool& pool : wf->pools) {
        for (WaveGraph& g : pool.graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        for (DeviceBlock* b : {&pool.state, &pool.shadow, &pool.queues, &pool.records, &pool.adj, &pool.adjLog})
            if (b->ptr) cudaFree(b->ptr);
    }
    if (wf->tables.ptr) cudaFree(wf->tables.ptr);
    if (wf->adjView.ptr) cudaFree(wf->adjView.ptr);
    if (wf->fork) cudaEventDestroy(wf->fork);
    for (cudaEvent_t j : wf->join)
        if (j) cudaEventDestroy(j);
    for (cudaStream_t sd : wf->side)
        if (sd) cudaStreamDestroy(sd);
    delete wf;
    ctx->wavefront = nullptr;
}

int wavefront_get_config(const ContextImpl* ctx, ShiroWavefrontConfig* out) {
    WavefrontState* wf = wf_state(const_cast<ContextImpl*>(ctx));
    *out = wf->cfg;
    return SHIRO_OK;
}

int wavefront_set_config(ContextImpl* ctx, const ShiroWavefrontConfig* cfg) {
    WavefrontState* wf = wf_state(ctx);
    auto okBlock = [](uint32_t b) { return b == 0 || (b >= 32 && b <= 1024 && b % 32 == 0); };
    if (!okBlock(cfg->extend_block) || !okBlock(cfg->shade_block) || !okBlock(cfg->shadow_block))
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "block sizes must be multiples of 32 in [32, 1024]");
    if (cfg->extend_block > 256 || cfg->shadow_block > 256)  // per-warp shared buffers for 8 warps
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "extend_block and shadow_block must be at most 256");
    if (cfg->paths_in_flight) {
        if (cfg->paths_in_flight < 1024 || cfg->paths_in_flight > (1u << 27))
            return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "paths_in_flight out of range [1024, 2^27]");
        wf->cfg.paths_in_flight = cfg->paths_in_flight;
    }
    if (cfg->shade_regs && cfg->shade_regs != 80 && cfg->shade_regs != 96 && cfg->shade_regs != 128)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "shade_regs must be 80, 96 or 128");
    if (cfg->extend_steps > 32 || cfg->refill_idle > 32)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "extend_steps and refill_idle must be in [1, 32]");
    if (cfg->extend_block) wf->cfg.extend_block = cfg->extend_block;
    if (cfg->shade_block) wf->cfg.shade_block = cfg->shade_block;
    if (cfg->shadow_block) wf->cfg.shadow_block = cfg->shadow_block;
    if (cfg->shade_regs) wf->cfg.shade_regs = cfg->shade_regs;
    if (cfg->extend_steps) wf->cfg.extend_steps = cfg->extend_steps;
    if (cfg->refill_idle) wf->cfg.refill_idle = cfg->refill_idle;
    if (cfg->concurrent_waves > kMaxConcurrentWaves)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "concurrent_waves must be 1 to 4");
    if (cfg->concurrent_waves) wf->cfg.concurrent_waves = cfg->concurrent_waves;
    if (cfg->bin_rays > 2 || cfg->bin_shadow > 2)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "bin_rays and bin_shadow must be 1 (on), 2 (off) or 0");
    if (cfg->bin_rays) wf->cfg.bin_rays = cfg->bin_rays;
    if (cfg->bin_shadow) wf->cfg.bin_shadow = cfg->bin_shadow;
    if (cfg->coop_extend > 2 || cfg->coop_occlude > 2)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "coop_extend and coop_occlude must be 1 (on), 2 (off) or 0");
    if (cfg->coop_extend) wf->cfg.coop_extend = cfg->coop_extend;
    if (cfg->coop_occlude) wf->cfg.coop_occlude = cfg->coop_occlude;
    auto okRegs = [](uint32_t r) { return r == 0 || r == 40 || r == 48 || r == 64; };
    if (!okRegs(cfg->extend_regs) || !okRegs(cfg->occlude_regs))
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "extend_regs and occlude_regs must be 40, 48 or 64 (0 leaves them)");
    if (cfg->extend_regs) wf->cfg.extend_regs = cfg->extend_regs;
    if (cfg->occlude_regs) wf->cfg.occlude_regs = cfg->occlude_regs;
    if (cfg->occlude_refill > 2)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "occlude_refill must be 1 (on), 2 (off) or 0");
    if (cfg->occlude_refill) wf->cfg.occlude_refill = cfg->occlude_refill;
    wf->cfg.use_graph = cfg->use_graph;
    return SHIRO_OK;
}

// Coordinate descent over the pool size and the three stage block sizes,
// each candidate timed on the first waves of `req` (scratch AOV planes).
int wavefront_autotune(ContextImpl* ctx, const ShiroRenderDesc* req, ShiroWavefrontConfig* chosen) {
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    ++ctx->epoch;  // the configuration changes
    WavefrontState* wf = wf_state(ctx);
    std::vector<DevRequest> qs{make_request(*req)};
    const uint64_t px = static_cast<uint64_t>(req->settings.width) * req->settings.height;
    if (!ensure_block(ctx, &ctx->aovScratch, std::max<uint64_t>(px, 1) * 11 * sizeof(float), "AOV staging"))
        return SHIRO_ERR_OUT_OF_MEMORY;
    float* b = static_cast<float*>(ctx->aovScratch.ptr);
    std::vector<AovPtrs> aov{AovPtrs{b, b + 4 * px, b + 7 * px, b + 10 * px}};
    const uint64_t total = px * qs[0].sampleCount;
    ShiroWavefrontConfig best = wf->cfg;
    best.use_graph = 1;
    double bestRate = 0.0;
    // a candidate's rate: one warm run, then the faster of two timed runs
    // (single timings of a few waves vary by several percent)
    auto measure = [&](const ShiroWavefrontConfig& c, double* rate) -> int {
        // enough waves for ~1/8 of the frame, at least two
        const uint32_t waves = static_cast<uint32_t>(std::max<uint64_t>(2, (total / 8) / std::max<uint32_t>(c.paths_in_flight, 1)));
        uint64_t paths = 0;
        double ms = 0.0;
        int r = run_waves(ctx, wf, c, qs, aov, nullptr, waves, &paths, &ms);  // warm
        if (r != SHIRO_OK) return r;
        *rate = 0.0;
        for (int rep = 0; rep < 2; ++rep) {
            r = run_waves(ctx, wf, c, qs, aov, nullptr, waves, &paths, &ms);
            if (r != SHIRO_OK) return r;
            *rate = std::max(*rate, static_cast<double>(paths) / std::max(ms, 1e-6));
        }
        return SHIRO_OK;
    };
    {  // bring the clocks up before anything is compared
        double warm = 0.0;
        ShiroWavefrontConfig c = best;
        if ((rc = measure(c, &warm)) != SHIRO_OK) return rc;
    }
    auto trial = [&](ShiroWavefrontConfig c) -> int {
        c.use_graph = 1;
        double rate = 0.0;
        const int r = measure(c, &rate);
        if (r == SHIRO_ERR_OUT_OF_MEMORY) return SHIRO_OK;  // a pool that does not fit is no candidate
        if (r != SHIRO_OK) return r;
        if (rate > bestRate) {
            bestRate = rate;
            best = c;
        }
        return SHIRO_OK;
    };
    const uint32_t pools[] = {1u << 20, 1u << 21, 1u << 22, 1u << 23, 1u << 24, 1u << 25};
    for (uint32_t p : pools) {
        if (p > total * 2 && p != pools[0]) break;
        ShiroWavefrontConfig c = best;
        c.paths_in_flight = p;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    for (uint32_t blk : {64u, 128u, 256u}) {
        ShiroWavefrontConfig c = best;
        c.extend_block = blk;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    for (uint32_t blk : {64u, 128u, 256u}) {
        ShiroWavefrontConfig c = best;
        c.shade_block = blk;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    for (uint32_t blk : {64u, 128u, 256u}) {
        ShiroWavefrontConfig c = best;
        c.shadow_block = blk;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    for (uint32_t regs : {80u, 96u, 128u}) {
        ShiroWavefrontConfig c = best;
        c.shade_regs = regs;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    // 2 to 4 waves in flight (each with a pool of the chosen size or half of it)
    if (total > best.paths_in_flight) {
        const uint32_t p1 = best.paths_in_flight;
        for (uint32_t n : {2u, 3u, 4u})
            for (uint32_t p : {p1, p1 / 2}) {
                if (p < (1u << 20) || static_cast<uint64_t>(p) * (n - 1) >= total) continue;
                ShiroWavefrontConfig c = best;
                c.concurrent_waves = n;
                c.paths_in_flight = p;
                if ((rc = trial(c)) != SHIRO_OK) return rc;
            }
    }
    for (uint32_t on : {1u, 2u}) {  // queue binning before the traversal stages
        ShiroWavefrontConfig c = best;
        c.bin_shadow = on;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    for (uint32_t on : {1u, 2u}) {
        ShiroWavefrontConfig c = best;
        c.bin_rays = on;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    for (uint32_t regs : {40u, 48u, 64u}) {  // register caps of the traversal stages
        ShiroWavefrontConfig c = best;
        c.occlude_regs = regs;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    for (uint32_t regs : {48u, 64u}) {
        ShiroWavefrontConfig c = best;
        c.extend_regs = regs;
        if ((rc = trial(c)) != SHIRO_OK) return rc;
    }
    if (ctx->nodes8 && ctx->bvhWidth != 2) {  // lane refill in the occlusion stage
        for (uint32_t on : {1u, 2u}) {
            ShiroWavefrontConfig c = best;
            c.occlude_refill = on;
            if ((rc = trial(c)) != SHIRO_OK) return rc;
        }
    }
    if (ctx->nodes8 && ctx->bvhWidth != 2) {  // warp-cooperative triangle tests
        for (uint32_t on : {1u, 2u}) {
            ShiroWavefrontConfig c = best;
            c.coop_occlude = on;
            if ((rc = trial(c)) != SHIRO_OK) return rc;
        }
        for (uint32_t on : {1u, 2u}) {
            ShiroWavefrontConfig c = best;
            c.coop_extend = on;
            if ((rc = trial(c)) != SHIRO_OK) return rc;
        }
    }
    if (ctx->nodes8 && ctx->bvhWidth != 2) {  // the lane refill of the wide-BVH extend stage
        for (uint32_t steps : {2u, 4u, 8u}) {
            ShiroWavefrontConfig c = best;
            c.extend_steps = steps;
            if ((rc = trial(c)) != SHIRO_OK) return rc;
        }
        for (uint32_t idle : {4u, 8u, 16u}) {
            ShiroWavefrontConfig c = best;
            c.refill_idle = idle;
            if ((rc = trial(c)) != SHIRO_OK) return rc;
        }
    }
    wf->cfg = best;
    wf->tuned = true;
    if (chosen) *chosen = best;
    return SHIRO_OK;
}

}  // namespace shiro_gpu
