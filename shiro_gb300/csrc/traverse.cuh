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

// Entry / exit of both child boxes of a node (slab test, fused form).
__device__ __forceinline__ void node_boxes(const float4& n0, const float4& n1, const float4& n2, const RayInv& r,
                                           float tmax, float* t0, float* t1, bool* h0, bool* h1) {
    const float ax = __fmaf_rn(n0.x, r.inv.x, -r.ood.x), bx = __fmaf_rn(n0.y, r.inv.x, -r.ood.x);
    const float ay = __fmaf_rn(n0.z, r.inv.y, -r.ood.y), by = __fmaf_rn(n0.w, r.inv.y, -r.ood.y);
    const float az = __fmaf_rn(n2.x, r.inv.z, -r.ood.z), bz = __fmaf_rn(n2.y, r.inv.z, -r.ood.z);
    const float cx = __fmaf_rn(n1.x, r.inv.x, -r.ood.x), dx = __fmaf_rn(n1.y, r.inv.x, -r.ood.x);
    const float cy = __fmaf_rn(n1.z, r.inv.y, -r.ood.y), dy = __fmaf_rn(n1.w, r.inv.y, -r.ood.y);
    const float cz = __fmaf_rn(n2.z, r.inv.z, -r.ood.z), dz = __fmaf_rn(n2.w, r.inv.z, -r.ood.z);
    const float lo0 = fmaxf(fmaxf(fminf(ax, bx), fminf(ay, by)), fmaxf(fminf(az, bz), 0.0f));
    const float hi0 = fminf(fminf(fmaxf(ax, bx), fmaxf(ay, by)), fminf(fmaxf(az, bz), tmax));
    const float lo1 = fmaxf(fmaxf(fminf(cx, dx), fminf(cy, dy)), fmaxf(fminf(cz, dz), 0.0f));
    const float hi1 = fminf(fminf(fmaxf(cx, dx), fmaxf(cy, dy)), fminf(fmaxf(cz, dz), tmax));
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

// ---- 8-wide BVH with quantised boxes (layout in bvh_build.h) ---------------
constexpr int kStack8 = 128;
constexpr int kEmptyWide = 0x7fffffff;

__device__ __forceinline__ float qbyte(uint32_t lo4, uint32_t hi4, int i) {
    const uint32_t w = i < 4 ? lo4 : hi4;
    return static_cast<float>((w >> (8 * (i & 3))) & 0xffu);
}

// Entry distances of the 8 children of a wide node (+inf for a miss or an
// empty slot) and their links.
__device__ __forceinline__ void wide_children(const DevScene& s, int node, const RayInv& r, float tmax, float t[8], int l[8]) {
    const float4* np = s.nodes8 + 6 * static_cast<size_t>(node);
    const float4 a = __ldg(np), l0 = __ldg(np + 1), l1 = __ldg(np + 2);
    const float4 q0 = __ldg(np + 3), q1 = __ldg(np + 4), q2 = __ldg(np + 5);
    const uint32_t eb = __float_as_uint(a.w);
    const float sx = __uint_as_float((eb & 0xffu) << 23), sy = __uint_as_float(((eb >> 8) & 0xffu) << 23),
                sz = __uint_as_float(((eb >> 16) & 0xffu) << 23);
    // child plane = origin + q * scale:  t = q * (scale * inv) + (origin * inv - o * inv)
    const float ax = sx * r.inv.x, ay = sy * r.inv.y, az = sz * r.inv.z;
    const float bx = __fmaf_rn(a.x, r.inv.x, -r.ood.x), by = __fmaf_rn(a.y, r.inv.y, -r.ood.y),
                bz = __fmaf_rn(a.z, r.inv.z, -r.ood.z);
    const uint32_t qlx0 = __float_as_uint(q0.x), qlx1 = __float_as_uint(q0.y), qly0 = __float_as_uint(q0.z),
                   qly1 = __float_as_uint(q0.w), qlz0 = __float_as_uint(q1.x), qlz1 = __float_as_uint(q1.y),
                   qhx0 = __float_as_uint(q1.z), qhx1 = __float_as_uint(q1.w), qhy0 = __float_as_uint(q2.x),
                   qhy1 = __float_as_uint(q2.y), qhz0 = __float_as_uint(q2.z), qhz1 = __float_as_uint(q2.w);
    const int links[8] = {__float_as_int(l0.x), __float_as_int(l0.y), __float_as_int(l0.z), __float_as_int(l0.w),
                          __float_as_int(l1.x), __float_as_int(l1.y), __float_as_int(l1.z), __float_as_int(l1.w)};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float x0 = __fmaf_rn(qbyte(qlx0, qlx1, i), ax, bx), x1 = __fmaf_rn(qbyte(qhx0, qhx1, i), ax, bx);
        const float y0 = __fmaf_rn(qbyte(qly0, qly1, i), ay, by), y1 = __fmaf_rn(qbyte(qhy0, qhy1, i), ay, by);
        const float z0 = __fmaf_rn(qbyte(qlz0, qlz1, i), az, bz), z1 = __fmaf_rn(qbyte(qhz0, qhz1, i), az, bz);
        const float lo = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), 0.0f));
        const float hi = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tmax));
        const bool hit = links[i] != kEmptyWide && lo <= hi;
        t[i] = hit ? lo : __int_as_float(0x7f800000);
        l[i] = links[i];
    }
}

__device__ __forceinline__ void cswap(float t[8], int l[8], int i, int j) {
    const bool sw = t[j] < t[i];
    const float ti = t[i], tj = t[j];
    const int li = l[i], lj = l[j];
    t[i] = sw ? tj : ti;
    t[j] = sw ? ti : tj;
    l[i] = sw ? lj : li;
    l[j] = sw ? li : lj;
}

// 19-comparator sorting network for 8 entries (ascending distance).
__device__ __forceinline__ void sort8(float t[8], int l[8]) {
    cswap(t, l, 0, 2); cswap(t, l, 1, 3); cswap(t, l, 4, 6); cswap(t, l, 5, 7);
    cswap(t, l, 0, 4); cswap(t, l, 1, 5); cswap(t, l, 2, 6); cswap(t, l, 3, 7);
    cswap(t, l, 0, 1); cswap(t, l, 2, 3); cswap(t, l, 4, 5); cswap(t, l, 6, 7);
    cswap(t, l, 2, 4); cswap(t, l, 3, 5);
    cswap(t, l, 1, 4); cswap(t, l, 3, 6);
    cswap(t, l, 1, 2); cswap(t, l, 3, 4); cswap(t, l, 5, 6);
}

template <typename Ctr>
__device__ bool trace_closest8(const DevScene& s, const V3& o, const V3& d, HitRec* out, Ctr& ctr) {
    const RayInv r = ray_inv(o, d);
    float bestT = FLT_MAX;
    uint32_t bestGid = 0xffffffffu, bestSlot = 0xffffffffu;
    float bu = 0.0f, bv = 0.0f;
    int stackLink[kStack8];
    float stackT[kStack8];
    int sp = 0;
    int cur = 0;
    uint32_t visits = 0;
    for (;;) {
        if (++visits > kMaxVisits) {
            atomicOr(s.error, kErrTraversalLimit);
            bestSlot = 0xffffffffu;
            break;
        }
        if (cur >= 0) {
            ctr.node();
            float t[8];
            int l[8];
            wide_children(s, cur, r, bestT, t, l);
            sort8(t, l);
            if (sp + 8 > kStack8) {
                atomicOr(s.error, kErrStackOverflow);
                bestSlot = 0xffffffffu;
                break;
            }
#pragma unroll
            for (int i = 7; i >= 0; --i) {
                if (t[i] <= bestT) {
                    stackLink[sp] = l[i];
                    stackT[sp] = t[i];
                    ++sp;
                }
            }
        } else {
            const uint32_t enc = ~static_cast<uint32_t>(cur);
            const uint32_t first = enc >> 3, cnt = (enc & 7u) + 1u;
            for (uint32_t k = first; k < first + cnt; ++k) {
                ctr.tri();
                const float4* tp = s.tris + 3 * static_cast<size_t>(k);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float tt, u, v;
                if (!tri_test(o, d, kRayEpsilon, FLT_MAX, a, b, c, &tt, &u, &v)) continue;
                const uint32_t gid = __float_as_uint(a.w);
                if (tt < bestT || (tt == bestT && gid < bestGid)) {
                    bestT = tt;
                    bestGid = gid;
                    bestSlot = k;
                    bu = u;
                    bv = v;
                }
            }
        }
        bool found = false;
        while (sp > 0) {
            --sp;
            if (stackT[sp] <= bestT) {
                cur = stackLink[sp];
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

template <typename Ctr>
__device__ bool trace_occluded8(const DevScene& s, const V3& o, const V3& d, float maxDist, Ctr& ctr) {
    const RayInv r = ray_inv(o, d);
    int stack[kStack8];
    int sp = 0;
    int cur = 0;
    uint32_t visits = 0;
    for (;;) {
        if (++visits > kMaxVisits) {
            atomicOr(s.error, kErrTraversalLimit);
            return false;
        }
        if (cur >= 0) {
            ctr.onode();
            float t[8];
            int l[8];
            wide_children(s, cur, r, maxDist, t, l);
            if (sp + 8 > kStack8) {
                atomicOr(s.error, kErrStackOverflow);
                return false;
            }
#pragma unroll
            for (int i = 0; i < 8; ++i)
                if (t[i] <= maxDist) stack[sp++] = l[i];
        } else {
            const uint32_t enc = ~static_cast<uint32_t>(cur);
            const uint32_t first = enc >> 3, cnt = (enc & 7u) + 1u;
            for (uint32_t k = first; k < first + cnt; ++k) {
                ctr.otri();
                const float4* tp = s.tris + 3 * static_cast<size_t>(k);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float tt, u, v;
                if (tri_test(o, d, kRayEpsilon, maxDist, a, b, c, &tt, &u, &v)) return true;
            }
        }
        if (sp == 0) return false;
        cur = stack[--sp];
    }
}

template <typename Ctr>
__device__ __noinline__ bool trace_closest(const DevScene& s, const V3 o, const V3 d, HitRec* out, Ctr& ctr) {
    ctr.closest();
    if (s.nodes8) return trace_closest8(s, o, d, out, ctr);
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
    if (s.nodes8) return trace_occluded8(s, o, d, maxDist, ctr);
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
