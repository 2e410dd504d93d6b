// common.cuh - device vector arithmetic and constants of the path tracer.
//
// The operators evaluate exactly the expressions of the reference's
// shiro/render/Types.h:28-111 (component-wise, left to right, division by a
// scalar as three divisions).  The whole backend is compiled with
// -fmad=false, so no multiply-add is contracted and, apart from
// transcendental functions, every float result equals the reference's.  Where a
// fused multiply-add is wanted for speed (the BVH box test) it is written
// explicitly with __fmaf_rn.
#pragma once

#include <cfloat>
#include <cstdint>

namespace shiro_gpu {

struct V3 {
    float x, y, z;
};
struct V2 {
    float x, y;
};

__host__ __device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 operator+(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__host__ __device__ __forceinline__ V3 operator-(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__host__ __device__ __forceinline__ V3 operator*(const V3& a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__host__ __device__ __forceinline__ V3 operator*(float s, const V3& a) { return a * s; }
__host__ __device__ __forceinline__ V3 operator*(const V3& a, const V3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__host__ __device__ __forceinline__ V3 operator/(const V3& a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__host__ __device__ __forceinline__ float dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ V3 cross(const V3& a, const V3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float length(const V3& a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalize(const V3& a) {
    const float l = length(a);
    return l > 0.0f ? a / l : V3{0.0f, 0.0f, 0.0f};
}
// std::max / std::min / std::clamp semantics (including the NaN behaviour).
__host__ __device__ __forceinline__ float smax(float a, float b) { return a < b ? b : a; }
__host__ __device__ __forceinline__ float smin(float a, float b) { return b < a ? b : a; }
__host__ __device__ __forceinline__ float sclamp(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }
__host__ __device__ __forceinline__ V3 sclamp3(const V3& v, float lo, float hi) {
    return {sclamp(v.x, lo, hi), sclamp(v.y, lo, hi), sclamp(v.z, lo, hi)};
}
__host__ __device__ __forceinline__ V3 lerp(const V3& a, const V3& b, float t) { return a * (1.0f - t) + b * t; }
__host__ __device__ __forceinline__ float maxc(const V3& v) { return smax(v.x, smax(v.y, v.z)); }
__host__ __device__ __forceinline__ V3 reflect(const V3& i, const V3& n) { return i - 2.0f * dot(i, n) * n; }
__host__ __device__ __forceinline__ V3 ld3(const float* p) { return {p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 f4xyz(const float4& v) { return {v.x, v.y, v.z}; }

// CpuPathTracer.cpp:59-77
constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 2.0f * kPi;
constexpr float kInvPi = 1.0f / kPi;
constexpr float kInvFourPi = 1.0f / (4.0f * kPi);
constexpr float kRayEpsilon = 1.0e-4f;
constexpr float kDirectSampleClamp = 24.0f;
constexpr float kThroughputClamp = 12.0f;
constexpr float kDeltaRoughness = 0.02f;
constexpr uint32_t kPathDimStride = 12u;
constexpr uint32_t kDirectDimBase = 256u;
constexpr uint32_t kDirectDepthStride = 512u;
constexpr uint32_t kDirectLightStride = 128u;
constexpr uint32_t kDirectSampleStride = 2u;
constexpr uint32_t kEmissiveDimBase = 8192u;
constexpr uint32_t kEmissiveDepthStride = 8u;

// Entries of the per-thread BVH traversal stack (the builder rejects deeper trees).
constexpr int kStack = 96;
constexpr int kStackWide = 64;  // entries of the wide-BVH traversal stack (one per level at most)

// Device-side error bits (ShiroGpu error word).
constexpr uint32_t kErrTraversalLimit = 1u;
constexpr uint32_t kErrStackOverflow = 2u;
constexpr uint32_t kErrBadIndex = 4u;
constexpr uint32_t kErrQueueOverflow = 8u;

}  // namespace shiro_gpu
