// traverse.cuh - BVH traversal with the reference's hit semantics.
//
// The reference (without Embree) intersects every triangle with
// Moller-Trumbore (CpuPathTracer.cpp:386-429) and keeps a new hit only when
// strictly closer, so among equal distances the first (mesh, primitive) wins
// (:431-466).  Here the triangles are reached through a BVH and a hit replaces
// the best one when (t, global index) is lexicographically smaller, which
// selects the same triangle.  The triangle test uses the same operations in
// the same order (compiled without FMA contraction), so t, u, v are
// bit-identical.  Child boxes are inflated at build time by a margin far above
// the rounding error of the box test, so a box is never culled while it holds
// a triangle the exhaustive test would report.
//
// Each traversal loop is bounded by kMaxVisits node visits; past that the
// error word is set and the ray is reported as a miss (a corrupt BVH can never
// hang the kernel).
#pragma once

#include "common.cuh"
#include "scene.cuh"

namespace shiro_gpu {


constexpr uint32_t kMaxVisits = 1u << 22;

// Work counters of the roofline probe (shiro_gpu_count_work).  NullCounter
// compiles every increment away in the render kernels.
struct NullCounter {
    __device__ __forceinline__ void node() {}
    __device__ __forceinline__ void tri() {}
    __device__ __forceinline__ void onode() {}
    __device__ __forceinline__ void otri() {}
    __device__ __forceinline__ void closest() {}
    __device__ __forceinline__ void occlusion() {}
    __device__ __forceinline__ void hit() {}
    __device__ __forceinline__ void env_eval(uint32_t n = 1) {}
    __device__ __forceinline__ void env_sample(uint32_t n = 1) {}
    __device__ __forceinline__ void bsdf_eval() {}
    __device__ __forceinline__ void bsdf_pdf() {}
};
struct LocalCounter {
    uint32_t nodes = 0, tris = 0, onodes = 0, otris = 0, closestRays = 0, occlusionRays = 0, hits = 0, envEvals = 0,
             envSamples = 0, bsdfEvals = 0, bsdfPdfs = 0;
    __device__ __forceinline__ void node() { ++nodes; }
    __device__ __forceinline__ void tri() { ++tris; }
    __device__ __forceinline__ void onode() { ++onodes; }
    __device__ __forceinline__ void otri() { ++otris; }
    __device__ __forceinline__ void closest() { ++closestRays; }
    __device__ __forceinline__ void occlusion() { ++occlusionRays; }
    __device__ __forceinline__ void hit() { ++hits; }
    __device__ __forceinline__ void env_eval(uint32_t n = 1) { envEvals += n; }
    __device__ __forceinline__ void env_sample(uint32_t n = 1) { envSamples += n; }
    __device__ __forceinline__ void bsdf_eval() { ++bsdfEvals; }
    __device__ __forceinline__ void bsdf_pdf() { ++bsdfPdfs; }
};

struct HitRec {
    float t, u, v;
    uint32_t slot;  // leaf-order triangle index, 0xffffffff on a miss
    uint32_t gid;   // global triangle index (meshes in order)
};

struct RayInv {
    V3 inv, ood;
};

__device__ __forceinline__ RayInv ray_inv(const V3& o, const V3& d) {
    RayInv r;
    const float dx = fabsf(d.x) > 1.0e-20f ? d.x : copysignf(1.0e-20f, d.x);
    const float dy = fabsf(d.y) > 1.0e-20f ? d.y : copysignf(1.0e-20f, d.y);
    const float dz = fabsf(d.z) > 1.0e-20f ? d.z : copysignf(1.0e-20f, d.z);
    r.inv = V3{1.0f / dx, 1.0f / dy, 1.0f / dz};
    r.ood = V3{o.x * r.inv.x, o.y * r.inv.y, o.z * r.inv.z};
    return r;
}

// Three-input minimum / maximum (PTX min.f32 / max.f32 with three sources,
// sm_100 and later); for non-NaN inputs equal to two nested fminf / fmaxf.
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Entry / exit of both child boxes of a node (slab test, fused form).
__device__ __forceinline__ void node_boxes(const float4& n0, const float4& n1, const float4& n2, const RayInv& r,
                                           float tmax, float* t0, float* t1, bool* h0, bool* h1) {
    const float ax = __fmaf_rn(n0.x, r.inv.x, -r.ood.x), bx = __fmaf_rn(n0.y, r.inv.x, -r.ood.x);
    const float ay = __fmaf_rn(n0.z, r.inv.y, -r.ood.y), by = __fmaf_rn(n0.w, r.inv.y, -r.ood.y);
    const float az = __fmaf_rn(n2.x, r.inv.z, -r.ood.z), bz = __fmaf_rn(n2.y, r.inv.z, -r.ood.z);
    const float cx = __fmaf_rn(n1.x, r.inv.x, -r.ood.x), dx = __fmaf_rn(n1.y, r.inv.x, -r.ood.x);
    const float cy = __fmaf_rn(n1.z, r.inv.y, -r.ood.y), dy = __fmaf_rn(n1.w, r.inv.y, -r.ood.y);
    const float cz = __fmaf_rn(n2.z, r.inv.z, -r.ood.z), dz = __fmaf_rn(n2.w, r.inv.z, -r.ood.z);
    const float lo0 = fmax3(fminf(ax, bx), fminf(ay, by), fmaxf(fminf(az, bz), 0.0f));
    const float hi0 = fmin3(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), tmax));
    const float lo1 = fmax3(fminf(cx, dx), fminf(cy, dy), fmaxf(fminf(cz, dz), 0.0f));
    const float hi1 = fmin3(fmaxf(cx, dx), fmaxf(cy, dy), fminf(fmaxf(cz, dz), tmax));
    *t0 = lo0;
    *t1 = lo1;
    *h0 = lo0 <= hi0;
    *h1 = lo1 <= hi1;
}

// Moller-Trumbore, IntersectTriangle (CpuPathTracer.cpp:386-429).
__device__ __forceinline__ bool tri_test(const V3& o, const V3& d, float tMin, float tMax, const float4& a,
                                         const float4& b, const float4& c, float* t, float* u, float* v) {
    const V3 p0 = f4xyz(a), e1 = f4xyz(b), e2 = f4xyz(c);
    const V3 pvec = cross(d, e2);
    const float det = dot(e1, pvec);
    if (fabsf(det) < 1.0e-8f) return false;
    const float inv = 1.0f / det;
    const V3 tvec = o - p0;
    const float uu = dot(tvec, pvec) * inv;
    if (uu < 0.0f || uu > 1.0f) return false;
    const V3 qvec = cross(tvec, e1);
    const float vv = dot(d, qvec) * inv;
    if (vv < 0.0f || uu + vv > 1.0f) return false;
    const float tt = dot(e2, qvec) * inv;
    if (tt < tMin || tt > tMax) return false;
    *t = tt;
    *u = uu;
    *v = vv;
    return true;
}

// ---- compressed 8-wide BVH (layout in bvh_build.h) -------------------------


// Children of wide node `node` hit within [0, tmax]: internal ones as bits
// (slot ^ octInv) of *inner (nearest first = lowest bit), leaf triangles as
// bits of *tris relative to *triBase.
//
// A quantised plane q of an axis lies at t = (origin + q * scale - o) * inv
// = (2^23 + q) * A + (B - 2^23 * A) with A = scale * inv (exact: scale is a
// power of two) and B = origin * inv - o * inv.  A byte permute turns q into
// the float 2^23 + q, and the bias B - 2^23 * A is formed once per node, so a
// plane costs one permute and one FMA; the bias rounds to within half a
// quantisation step, which the builder covers by widening every child box by
// one step.  Empty slots hold an inverted box (q_lo = 255, q_hi = 0) and the
// meta byte 0xff.
__device__ __forceinline__ void wide_node(const DevScene& s, uint32_t node, const RayInv& r, float tmax, uint32_t octInv,
                                          uint32_t* childBase, uint32_t* imask, uint32_t* inner, uint32_t* triBase,
                                          uint32_t* tris) {
    const float4* np = s.nodes8 + 5 * static_cast<size_t>(node);
    const float4 a = __ldg(np), b = __ldg(np + 1);
    const float4 q0 = __ldg(np + 2), q1 = __ldg(np + 3), q2 = __ldg(np + 4);
    const uint32_t eb = __float_as_uint(a.w);
    const float sx = __uint_as_float((eb & 0xffu) << 23), sy = __uint_as_float(((eb >> 8) & 0xffu) << 23),
                sz = __uint_as_float(((eb >> 16) & 0xffu) << 23);
    const float ax = sx * r.inv.x, ay = sy * r.inv.y, az = sz * r.inv.z;
    const float bx = __fmaf_rn(-8388608.0f, ax, __fmaf_rn(a.x, r.inv.x, -r.ood.x));
    const float by = __fmaf_rn(-8388608.0f, ay, __fmaf_rn(a.y, r.inv.y, -r.ood.y));
    const float bz = __fmaf_rn(-8388608.0f, az, __fmaf_rn(a.z, r.inv.z, -r.ood.z));
    const uint32_t im = eb >> 24;
    // near / far plane words per axis: a negative direction enters through
    // the upper planes (inv < 0 makes their distances the smaller ones)
    const bool nx = r.inv.x < 0.0f, ny = r.inv.y < 0.0f, nz = r.inv.z < 0.0f;
    const uint32_t lx0 = __float_as_uint(q0.x), lx1 = __float_as_uint(q0.y), ly0 = __float_as_uint(q0.z),
                   ly1 = __float_as_uint(q0.w), lz0 = __float_as_uint(q1.x), lz1 = __float_as_uint(q1.y),
                   hx0 = __float_as_uint(q1.z), hx1 = __float_as_uint(q1.w), hy0 = __float_as_uint(q2.x),
                   hy1 = __float_as_uint(q2.y), hz0 = __float_as_uint(q2.z), hz1 = __float_as_uint(q2.w);
    const uint32_t nw[6] = {nx ? hx0 : lx0, nx ? hx1 : lx1, ny ? hy0 : ly0, ny ? hy1 : ly1, nz ? hz0 : lz0, nz ? hz1 : lz1};
    const uint32_t fw[6] = {nx ? lx0 : hx0, nx ? lx1 : hx1, ny ? ly0 : hy0, ny ? ly1 : hy1, nz ? lz0 : hz0, nz ? lz1 : hz1};
    uint32_t hit = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int h = i >> 2;
        const uint32_t sel = static_cast<uint32_t>(i & 3) | 0x7540u;  // byte i -> float 2^23 + q
        const float x0 = __fmaf_rn(__uint_as_float(__byte_perm(nw[0 + h], 0x4b000000u, sel)), ax, bx);
        const float y0 = __fmaf_rn(__uint_as_float(__byte_perm(nw[2 + h], 0x4b000000u, sel)), ay, by);
        const float z0 = __fmaf_rn(__uint_as_float(__byte_perm(nw[4 + h], 0x4b000000u, sel)), az, bz);
        const float x1 = __fmaf_rn(__uint_as_float(__byte_perm(fw[0 + h], 0x4b000000u, sel)), ax, bx);
        const float y1 = __fmaf_rn(__uint_as_float(__byte_perm(fw[2 + h], 0x4b000000u, sel)), ay, by);
        const float z1 = __fmaf_rn(__uint_as_float(__byte_perm(fw[4 + h], 0x4b000000u, sel)), az, bz);
        const float lo = fmax3(x0, y0, fmaxf(z0, 0.0f));
        const float hi = fmin3(x1, y1, fminf(z1, tmax));
        hit |= (lo <= hi ? 1u : 0u) << i;
    }
    // internal children: bit i moves to bit i ^ octInv
    uint32_t in = hit & im;
    if (octInv & 1u) in = ((in & 0x55u) << 1) | ((in >> 1) & 0x55u);
    if (octInv & 2u) in = ((in & 0x33u) << 2) | ((in >> 2) & 0x33u);
    if (octInv & 4u) in = ((in & 0x0fu) << 4) | ((in >> 4) & 0x0fu);
    // leaf children: their triangles' bits from the meta bytes
    const uint64_t meta = (static_cast<uint64_t>(__float_as_uint(b.w)) << 32) | __float_as_uint(b.z);
    uint32_t lf = hit & ~im, tb = 0;
    while (lf) {
        const uint32_t i = static_cast<uint32_t>(__ffs(lf) - 1);
        lf &= lf - 1u;
        const uint32_t mt = static_cast<uint32_t>(meta >> (8u * i)) & 0xffu;
        // an empty slot's inverted box can only pass when rounding collapses
        // all its planes to one distance; it never contributes triangles
        if (mt != 0xffu) tb |= ((2u << (mt >> 5)) - 1u) << (mt & 31u);
    }
    *childBase = __float_as_uint(b.x);
    *triBase = __float_as_uint(b.y);
    *imask = im;
    *inner = in;
    *tris = tb;
}

__device__ __forceinline__ uint32_t ray_oct_inv(const V3& d) {
    return 7u ^ ((d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u));
}

// Wide-BVH traversal as resumable state (one node and its triangles per
// step), so a caller may interleave rays: the wavefront stages refill a lane
// with a new ray as soon as its ray finishes.  Stack entries are groups of
// sibling wide nodes still to visit: (childBase, remaining inner bits << 8 |
// imask); the caller owns the stack array.
struct WideTrav {
    V3 o, d;
    RayInv r;
    uint32_t octInv;
    float tmax;                 // closest: the best distance so far; occlusion: maxDist
    float bu, bv;
    uint32_t bestGid, bestSlot;
    uint32_t node;              // next node to visit
    int sp;
    uint32_t visits;
};

__device__ __forceinline__ void wide_init(WideTrav& t, const V3& o, const V3& d, float tmax) {
    t.o = o;
    t.d = d;
    t.r = ray_inv(o, d);
    t.octInv = ray_oct_inv(d);
    t.tmax = tmax;
    t.bu = 0.0f;
    t.bv = 0.0f;
    t.bestGid = 0xffffffffu;
    t.bestSlot = 0xffffffffu;
    t.node = 0;
    t.sp = 0;
    t.visits = 0;
}

// Moves to the next node of the traversal; false when none is left (or on a
// violated bound, which also sets the error word and clears the hit).
__device__ __forceinline__ bool wide_next(const DevScene& s, WideTrav& t, uint2* stack, uint32_t gBase, uint32_t gImask,
                                          uint32_t gInner) {
    if (gInner == 0u) {
        if (t.sp == 0) return false;
        --t.sp;
        gBase = stack[t.sp].x;
        gInner = stack[t.sp].y >> 8;
        gImask = stack[t.sp].y & 0xffu;
    }
    const uint32_t slot = static_cast<uint32_t>(__ffs(gInner) - 1) ^ t.octInv;
    gInner &= gInner - 1u;
    t.node = gBase + __popc(gImask & ((1u << slot) - 1u));
    if (gInner) {
        if (t.sp >= kStackWide) {
            atomicOr(s.error, kErrStackOverflow);
            t.bestSlot = 0xffffffffu;
            return false;
        }
        stack[t.sp++] = make_uint2(gBase, (gInner << 8) | gImask);
    }
    return true;
}

// Closest hit: up to `steps` nodes; true when finished (result in t.tmax,
// t.bu, t.bv, t.bestSlot, t.bestGid).
template <typename Ctr>
__device__ __forceinline__ bool wide_closest_advance(const DevScene& s, WideTrav& t, uint2* stack, int steps, Ctr& ctr) {
    for (int k = 0; k < steps; ++k) {
        if (++t.visits > kMaxVisits) {
            atomicOr(s.error, kErrTraversalLimit);
            t.bestSlot = 0xffffffffu;
            return true;
        }
        ctr.node();
        uint32_t gBase, gImask, gInner, tBase, tBits;
        wide_node(s, t.node, t.r, t.tmax, t.octInv, &gBase, &gImask, &gInner, &tBase, &tBits);
        while (tBits) {
            const uint32_t kk = tBase + static_cast<uint32_t>(__ffs(tBits) - 1);
            tBits &= tBits - 1u;
            ctr.tri();
            const float4* tp = s.tris + 3 * static_cast<size_t>(kk);
            const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
            float tt, u, v;
            if (!tri_test(t.o, t.d, kRayEpsilon, FLT_MAX, ta, tb, tc, &tt, &u, &v)) continue;
            const uint32_t gid = __float_as_uint(ta.w);
            if (tt < t.tmax || (tt == t.tmax && gid < t.bestGid)) {
                t.tmax = tt;
                t.bestGid = gid;
                t.bestSlot = kk;
                t.bu = u;
                t.bv = v;
            }
        }
        if (!wide_next(s, t, stack, gBase, gImask, gInner)) return true;
    }
    return false;
}

// Any hit in [1e-4, t.tmax]: up to `steps` nodes; -1 while running, else
// 1 occluded / 0 clear.
template <typename Ctr>
__device__ __forceinline__ int wide_occluded_advance(const DevScene& s, WideTrav& t, uint2* stack, int steps, Ctr& ctr) {
    for (int k = 0; k < steps; ++k) {
        if (++t.visits > kMaxVisits) {
            atomicOr(s.error, kErrTraversalLimit);
            return 0;
        }
        ctr.onode();
        uint32_t gBase, gImask, gInner, tBase, tBits;
        wide_node(s, t.node, t.r, t.tmax, t.octInv, &gBase, &gImask, &gInner, &tBase, &tBits);
        while (tBits) {
            const uint32_t kk = tBase + static_cast<uint32_t>(__ffs(tBits) - 1);
            tBits &= tBits - 1u;
            ctr.otri();
            const float4* tp = s.tris + 3 * static_cast<size_t>(kk);
            const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
            float tt, u, v;
            if (tri_test(t.o, t.d, kRayEpsilon, t.tmax, ta, tb, tc, &tt, &u, &v)) return 1;
        }
        if (!wide_next(s, t, stack, gBase, gImask, gInner)) return 0;
    }
    return -1;
}

template <typename Ctr>
__device__ bool trace_closest_wide(const DevScene& s, const V3& o, const V3& d, HitRec* out, Ctr& ctr) {
    WideTrav t;
    uint2 stack[kStackWide];
    wide_init(t, o, d, FLT_MAX);
    wide_closest_advance(s, t, stack, 0x7fffffff, ctr);
    out->t = t.tmax;
    out->u = t.bu;
    out->v = t.bv;
    out->slot = t.bestSlot;
    out->gid = t.bestGid;
    return t.bestSlot != 0xffffffffu;
}

template <typename Ctr>
__device__ bool trace_occluded_wide(const DevScene& s, const V3& o, const V3& d, float maxDist, Ctr& ctr) {
    WideTrav t;
    uint2 stack[kStackWide];
    wide_init(t, o, d, maxDist);
    return wide_occluded_advance(s, t, stack, 0x7fffffff, ctr) == 1;
}

template <typename Ctr>
__device__ __noinline__ bool trace_closest(const DevScene& s, const V3 o, const V3 d, HitRec* out, Ctr& ctr) {
    ctr.closest();
    if (s.nodes8) return trace_closest_wide(s, o, d, out, ctr);
    const RayInv r = ray_inv(o, d);
    float bestT = FLT_MAX;
    uint32_t bestGid = 0xffffffffu, bestSlot = 0xffffffffu;
    float bu = 0.0f, bv = 0.0f;
    int stackNode[kStack];
    float stackT[kStack];
    int sp = 0;
    int node = 0;
    uint32_t visits = 0;
    for (;;) {
        if (++visits > kMaxVisits) {
            atomicOr(s.error, kErrTraversalLimit);
            bestSlot = 0xffffffffu;
            break;
        }
        if (node >= 0) {
            ctr.node();
            const float4* np = s.nodes + 4 * static_cast<size_t>(node);
            const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3);
            float t0, t1;
            bool h0, h1;
            node_boxes(n0, n1, n2, r, bestT, &t0, &t1, &h0, &h1);
            const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
            if (h0 && h1) {
                const bool swap = t1 < t0;
                if (sp >= kStack) {
                    atomicOr(s.error, kErrStackOverflow);
                    bestSlot = 0xffffffffu;
                    break;
                }
                stackNode[sp] = swap ? c0 : c1;
                stackT[sp] = swap ? t0 : t1;
                ++sp;
                node = swap ? c1 : c0;
                continue;
            }
            if (h0) {
                node = c0;
                continue;
            }
            if (h1) {
                node = c1;
                continue;
            }
        } else {
            const uint32_t enc = ~static_cast<uint32_t>(node);
            const uint32_t first = enc >> 3, cnt = (enc & 7u) + 1u;
            for (uint32_t k = first; k < first + cnt; ++k) {
                ctr.tri();
                const float4* tp = s.tris + 3 * static_cast<size_t>(k);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, u, v;
                if (!tri_test(o, d, kRayEpsilon, FLT_MAX, a, b, c, &t, &u, &v)) continue;
                const uint32_t gid = __float_as_uint(a.w);
                if (t < bestT || (t == bestT && gid < bestGid)) {
                    bestT = t;
                    bestGid = gid;
                    bestSlot = k;
                    bu = u;
                    bv = v;
                }
            }
        }
        // pop the next entry still in range
        bool found = false;
        while (sp > 0) {
            --sp;
            if (stackT[sp] <= bestT) {
                node = stackNode[sp];
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    out->t = bestT;
    out->u = bu;
    out->v = bv;
    out->slot = bestSlot;
    out->gid = bestGid;
    return bestSlot != 0xffffffffu;
}

// Any hit with t in [1e-4, maxDist] (Occluded, CpuPathTracer.cpp:468-475).
template <typename Ctr>
__device__ __noinline__ bool trace_occluded(const DevScene& s, const V3 o, const V3 d, float maxDist, Ctr& ctr) {
    ctr.occlusion();
    if (s.nodes8) return trace_occluded_wide(s, o, d, maxDist, ctr);
    const RayInv r = ray_inv(o, d);
    int stackNode[kStack];
    int sp = 0;
    int node = 0;
    uint32_t visits = 0;
    for (;;) {
        if (++visits > kMaxVisits) {
            atomicOr(s.error, kErrTraversalLimit);
            return false;
        }
        if (node >= 0) {
            ctr.onode();
            const float4* np = s.nodes + 4 * static_cast<size_t>(node);
            const float4 n0 = __ldg(np), n1 = __ldg(np + 1), n2 = __ldg(np + 2), n3 = __ldg(np + 3);
            float t0, t1;
            bool h0, h1;
            node_boxes(n0, n1, n2, r, maxDist, &t0, &t1, &h0, &h1);
            const int c0 = __float_as_int(n3.x), c1 = __float_as_int(n3.y);
            if (h0 && h1) {
                if (sp >= kStack) {
                    atomicOr(s.error, kErrStackOverflow);
                    return false;
                }
                const bool swap = t1 < t0;
                stackNode[sp++] = swap ? c0 : c1;
                node = swap ? c1 : c0;
                continue;
            }
            if (h0) {
                node = c0;
                continue;
            }
            if (h1) {
                node = c1;
                continue;
            }
        } else {
            const uint32_t enc = ~static_cast<uint32_t>(node);
            const uint32_t first = enc >> 3, cnt = (enc & 7u) + 1u;
            for (uint32_t k = first; k < first + cnt; ++k) {
                ctr.otri();
                const float4* tp = s.tris + 3 * static_cast<size_t>(k);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float t, u, v;
                if (tri_test(o, d, kRayEpsilon, maxDist, a, b, c, &t, &u, &v)) return true;
            }
        }
        if (sp == 0) return false;
        node = stackNode[--sp];
    }
}

}  // namespace shiro_gpu
