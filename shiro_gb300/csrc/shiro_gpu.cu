// shiro_gpu.cu - C ABI of the GB300 path-tracing backend (include/shiro_gpu.h).
//
// Host side of the plain form: context management, scene upload (flattening
// of the Scene snapshot, device BVH build, dome importance tables), the
// RenderSampleBatch entry point and the parity probes.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "bvh_build.h"
#include "context.h"
#include "bsdf.cuh"
#include "env.cuh"
#include "kernels.h"

using namespace shiro_gpu;

namespace shiro_gpu {

namespace {
thread_local std::string gCreateError;
constexpr float kHostPi = 3.14159265358979323846f;

void free_block(DeviceBlock* b) {
    if (b->ptr) cudaFree(b->ptr);
    b->ptr = nullptr;
    b->bytes = 0;
}

template <typename T>
int upload(ContextImpl* ctx, const std::vector<T>& v, const T** out, const char* what) {
    DeviceBlock b;
    const size_t bytes = std::max<size_t>(v.size() * sizeof(T), 16);
    cudaError_t e = cudaMalloc(&b.ptr, bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    b.bytes = bytes;
    ctx->sceneBlocks.push_back(b);
    if (!v.empty()) {
        e = cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    }
    *out = static_cast<const T*>(b.ptr);
    return SHIRO_OK;
}

ShiroMaterialDesc default_material() {  // PbrMaterial defaults, Renderer.h:56-102
    ShiroMaterialDesc m;
    std::memset(&m, 0, sizeof(m));
    for (int k = 0; k < 3; ++k) {
        m.base_color[k] = 0.8f;
        m.specular_color[k] = 1.0f;
        m.transmission_color[k] = 1.0f;
        m.coat_color[k] = 1.0f;
        m.subsurface_color[k] = 1.0f;
        m.subsurface_radius[k] = 1.0f;
        m.sheen_color[k] = 1.0f;
    }
    m.base_weight = 1.0f;
    m.specular_weight = 1.0f;
    m.roughness = 0.5f;
    m.opacity = 1.0f;
    m.coat_roughness = 0.03f;
    m.coat_ior = 1.5f;
    m.sheen_roughness = 0.3f;
    m.subsurface_scale = 1.0f;
    m.ior = 1.5f;
    m.thin_film_ior = 1.5f;
    return m;
}

inline float hclamp(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }

}  // namespace

ContextImpl::~ContextImpl() {
    wavefront_free(this);
    adjoint_free(this);
    freeScene();
    free_block(&pathRecords);
    free_block(&aovScratch);
    free_block(&probeScratch);
    if (errorWord) cudaFree(errorWord);
    if (ownStream) cudaStreamDestroy(ownStream);
}

void ContextImpl::freeScene() {
    for (auto& b : sceneBlocks) free_block(&b);
    sceneBlocks.clear();
    geomBlocks = 0;
    geomValid = false;
    envDev.clear();
    envHost.clear();
    domeEnv.clear();
    materialsHost.clear();
    hasScene = false;
    scene = DevScene{};
    nodes8 = tris8 = tris2 = nullptr;
}

void ContextImpl::freeShading() {
    for (size_t i = geomBlocks; i < sceneBlocks.size(); ++i) free_block(&sceneBlocks[i]);
    sceneBlocks.resize(std::min(geomBlocks, sceneBlocks.size()));
    envDev.clear();
    envHost.clear();
    domeEnv.clear();
    materialsHost.clear();
    materialCount = 0;
    extendedMaterials = false;
    hasScene = false;
    DevScene& s = scene;
    s.materials = nullptr;
    s.bsdfRecs = nullptr;
    s.emissive = nullptr;
    s.emissiveCdf = nullptr;
    s.emissiveOf = nullptr;
    s.emissiveCount = 0;
    s.emissiveSum = 0.0f;
    s.distant = nullptr;
    s.distantCount = 0;
    s.domes = nullptr;
    s.domeCount = 0;
    s.envs = nullptr;
    s.extended = 0;
}

size_t ContextImpl::deviceBytes() const {
    size_t n = pathRecords.bytes + aovScratch.bytes + probeScratch.bytes;
    for (const auto& b : sceneBlocks) n += b.bytes;
    return n;
}

bool ensure_block(ContextImpl* ctx, DeviceBlock* b, size_t bytes, const char* what) {
    if (b->bytes >= bytes) return true;
    free_block(b);
    const cudaError_t e = cudaMalloc(&b->ptr, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        ctx->lastError = std::string(what) + ": cudaMalloc(" + std::to_string(bytes) + "): " + cudaGetErrorString(e);
        b->ptr = nullptr;
        return false;
    }
    b->bytes = bytes;
    return true;
}

int fail(ContextImpl* ctx, int code, const std::string& msg) {
    if (ctx) ctx->lastError = msg;
    return code;
}

int cuda_fail(ContextImpl* ctx, cudaError_t e, const char* what) {
    cudaGetLastError();
    return fail(ctx, e == cudaErrorMemoryAllocation ? SHIRO_ERR_OUT_OF_MEMORY : SHIRO_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

DevRequest make_request(const ShiroRenderDesc& r) {
    DevRequest q{};
    const ShiroCameraDesc& c = r.camera;
    q.camPos = ld3(c.position);
    q.camForward = ld3(c.forward);
    q.camRight = ld3(c.right);
    q.camUp = ld3(c.up);
    q.tanHalfFov = std::tan(c.vertical_fov_degrees * 0.5f * kHostPi / 180.0f);
    q.aspect = c.aspect_ratio;
    q.width = r.settings.width;
    q.height = r.settings.height;
    q.sampleStart = r.sample_start;
    q.sampleCount = r.sample_count;
    q.maxDepth = r.settings.max_depth;
    q.diffuseDepth = r.settings.diffuse_depth;
    q.specularDepth = r.settings.specular_depth;
    q.domeSamples = std::max(1u, r.settings.dome_light_samples);
    q.backgroundVisible = r.settings.background_visible ? 1u : 0u;
    q.flags = r.flags;
    return q;
}

int validate_request(ContextImpl* ctx, const ShiroRenderDesc& r) {
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    const uint64_t px = static_cast<uint64_t>(r.settings.width) * r.settings.height;
    if (px > (1ull << 31)) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "frame too large");
    if (r.flags & ~(SHIRO_RENDER_ENV_CDF | SHIRO_RENDER_NO_CLAMP | SHIRO_RENDER_KEEP_PATHS))
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "unknown flags");
    return SHIRO_OK;
}

// Per-texel sample records of a lat-long map (EnvironmentMap::Sample's
// result for each texel): (centre direction, pdf), (radiance there, 0).
__global__ void k_env_samples(DevEnv e, float4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e.w * e.h) return;
    const uint32_t row = i / e.w, col = i - row * e.w;
    V3 d;
    float pdf;
    const V3 rad = env_centre_sample(e, row, col, e.texels[i].w, &d, &pdf);
    out[2 * static_cast<size_t>(i)] = make_float4(d.x, d.y, d.z, pdf);
    out[2 * static_cast<size_t>(i) + 1] = make_float4(rad.x, rad.y, rad.z, 0.0f);
}

__global__ void k_bsdf_recs(const ShiroMaterialDesc* mats, uint32_t n, float4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 r[kBsdfRec];
    make_bsdf_rec(mats[i], r);
    for (int k = 0; k < kBsdfRec; ++k) out[kBsdfRec * static_cast<size_t>(i) + k] = r[k];
}

// Geometric normals of the triangle shading records, from the binary BVH's
// triangle slots (v0 with the global index in w, e1, e2): the same
// normalize(cross(e1, e2)) a hit formed from its slot.  A triangle held in
// several slots is written with the same value by each.
__global__ void k_shade_normals(const float4* __restrict__ tris, uint32_t n, float4* __restrict__ shade) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4* tp = tris + 3 * static_cast<size_t>(i);
    const uint32_t gid = __float_as_uint(tp[0].w);
    const V3 ng = normalize(cross(f4xyz(tp[1]), f4xyz(tp[2])));
    float4* r = shade + kShadeRec * static_cast<size_t>(gid);
    *r = make_float4(ng.x, ng.y, ng.z, r->w);
}

// ---- scene flattening on the device -----------------------------------------
// The upload ships the meshes' own arrays (positions, normals, indices, each
// concatenated over the meshes); these kernels form what the host loop of the
// reference's BuildAccelerationScene forms (CpuPathTracer.cpp:477-598): the
// per-triangle records in global triangle order (meshes in order, triangles
// in order), boxes and centroids, with the same float expressions (the
// backend is compiled without contraction), so every value equals the host
// formulation's.
struct FlatMesh {
    uint32_t vbase, vcount;  // its vertices in the concatenated positions
    uint32_t tbase, tcount;  // its global triangle ids
    uint32_t ibase;          // its first index in the concatenated indices
    uint32_t nbase;          // its first normal (when hasN)
    uint32_t recBits;        // material | kShadeNormals (shading record word)
    uint32_t hasN;
};

// Floats as unsigned integers of the same order (min / max by integer atomics).
__host__ __device__ __forceinline__ uint32_t flat_ord(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float flat_unord(uint32_t u) {
    const uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

__device__ __forceinline__ float host_min(float a, float b) { return b < a ? b : a; }  // std::min
__device__ __forceinline__ float host_max(float a, float b) { return a < b ? b : a; }  // std::max

// Vertices as float4, and the largest coordinate magnitude over all of them.
__global__ void k_flat_verts(const float* __restrict__ pos3, uint32_t n, float4* __restrict__ pos4,
                             unsigned int* __restrict__ magBits) {
    float m = 0.0f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = pos3[3 * static_cast<size_t>(i)], y = pos3[3 * static_cast<size_t>(i) + 1],
                    z = pos3[3 * static_cast<size_t>(i) + 2];
        pos4[i] = make_float4(x, y, z, 0.0f);
        m = host_max(m, host_max(fabsf(x), host_max(fabsf(y), fabsf(z))));
    }
    for (int o = 16; o > 0; o >>= 1) m = host_max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31u) == 0u) atomicMax(magBits, __float_as_uint(m));  // m >= 0: the bits order as the float
}

// Per triangle: vertex indices, shading record (material bits, vertex
// normals; the geometric normal follows after the BVH build), (p0, e1, e2),
// raw box; the scene box as ordered-integer min / max; the first triangle
// with an index out of range in *badTri.
__global__ void k_flat_tris(const FlatMesh* __restrict__ meshes, uint32_t nMesh, const float* __restrict__ pos3,
                            const float* __restrict__ nrm3, const uint32_t* __restrict__ idx, uint32_t ttotal,
                            uint4* __restrict__ triVerts, float4* __restrict__ shade, float4* __restrict__ allTri,
                            float* __restrict__ boxes, unsigned int* __restrict__ sceneBox, uint32_t* __restrict__ badTri) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < ttotal; g += gridDim.x * blockDim.x) {
        uint32_t a = 0, b = nMesh - 1u;  // the last mesh whose first triangle is <= g
        while (a < b) {
            const uint32_t mid = (a + b + 1u) >> 1;
            if (meshes[mid].tbase <= g) a = mid; else b = mid - 1u;
        }
        const FlatMesh m = meshes[a];
        const uint32_t t = g - m.tbase;
        const uint32_t i0 = idx[m.ibase + 3 * t], i1 = idx[m.ibase + 3 * t + 1], i2 = idx[m.ibase + 3 * t + 2];
        if (i0 >= m.vcount || i1 >= m.vcount || i2 >= m.vcount) {
            atomicMin(badTri, g);
            continue;
        }
        triVerts[g] = make_uint4(m.vbase + i0, m.vbase + i1, m.vbase + i2, a);
        float4* rec = shade + 4 * static_cast<size_t>(g);
        rec[0] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(m.recBits));
        const uint32_t vi[3] = {i0, i1, i2};
        for (int k = 0; k < 3; ++k) {
            const float* n = m.hasN ? nrm3 + 3 * (static_cast<size_t>(m.nbase) + vi[k]) : nullptr;
            rec[1 + k] = n ? make_float4(n[0], n[1], n[2], 0.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        const float* p0 = pos3 + 3 * (static_cast<size_t>(m.vbase) + i0);
        const float* p1 = pos3 + 3 * (static_cast<size_t>(m.vbase) + i1);
        const float* p2 = pos3 + 3 * (static_cast<size_t>(m.vbase) + i2);
        allTri[3 * static_cast<size_t>(g)] = make_float4(p0[0], p0[1], p0[2], __uint_as_float(g));
        allTri[3 * static_cast<size_t>(g) + 1] = make_float4(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], 0.0f);
        allTri[3 * static_cast<size_t>(g) + 2] = make_float4(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2], 0.0f);
        for (int k = 0; k < 3; ++k) {
            const float l = host_min(p0[k], host_min(p1[k], p2[k]));
            const float h = host_max(p0[k], host_max(p1[k], p2[k]));
            boxes[6 * static_cast<size_t>(g) + k] = l;
            boxes[6 * static_cast<size_t>(g) + 3 + k] = h;
            lo[k] = fminf(lo[k], l);
            hi[k] = fmaxf(hi[k], h);
        }
    }
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
        if ((threadIdx.x & 31u) == 0u) {
            atomicMin(&sceneBox[k], flat_ord(lo[k]));
            atomicMax(&sceneBox[3 + k], flat_ord(hi[k]));
        }
    }
}

__device__ __forceinline__ float box_area(const float* lo, const float* hi) {
    const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

// Triangles whose box area exceeds `thresh` (candidates for the leaf under
// the root): (area bits, global id).
__global__ void k_large_cands(const float* __restrict__ boxes, uint32_t ttotal, float thresh, uint2* __restrict__ cand,
                              uint32_t* __restrict__ count) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < ttotal; g += gridDim.x * blockDim.x) {
        const float a = box_area(boxes + 6 * static_cast<size_t>(g), boxes + 6 * static_cast<size_t>(g) + 3);
        if (a > thresh) cand[atomicAdd(count, 1u)] = make_uint2(__float_as_uint(a), g);
    }
}

struct FlatLarge {
    uint32_t gid[8];
    uint32_t n;
};

// Inflated boxes; the BVH input of the other triangles in global order (the
// large ones, at most 8, go to largeOut in global order).
__global__ void k_flat_small(const float4* __restrict__ allTri, const float* __restrict__ boxes, uint32_t ttotal,
                             float pad, FlatLarge large, float4* __restrict__ triData, float4* __restrict__ primBoxes,
                             float4* __restrict__ centroids, LargeTri* __restrict__ largeOut) {
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < ttotal; g += gridDim.x * blockDim.x) {
        const float* bx = boxes + 6 * static_cast<size_t>(g);
        float lo[3], hi[3];
        for (int k = 0; k < 3; ++k) {
            const float e = pad + (bx[3 + k] - bx[k]) * 1.0e-5f;
            lo[k] = bx[k] - e;
            hi[k] = bx[3 + k] + e;
        }
        uint32_t rank = 0;
        bool isLarge = false;
        for (uint32_t k = 0; k < large.n; ++k) {
            rank += large.gid[k] < g ? 1u : 0u;
            isLarge |= large.gid[k] == g;
        }
        if (isLarge) {
            LargeTri lt;
            for (int k = 0; k < 3; ++k) {
                lt.tri[k] = allTri[3 * static_cast<size_t>(g) + k];
                lt.lo[k] = lo[k];
                lt.hi[k] = hi[k];
            }
            largeOut[rank] = lt;
            continue;
        }
        const size_t pos = g - rank;
        for (int k = 0; k < 3; ++k) triData[3 * pos + k] = allTri[3 * static_cast<size_t>(g) + k];
        primBoxes[2 * pos] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        primBoxes[2 * pos + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
        centroids[pos] = make_float4(0.5f * (bx[0] + bx[3]), 0.5f * (bx[1] + bx[4]), 0.5f * (bx[2] + bx[5]), 0.0f);
    }
}

// (Re)computes the per-material BSDF records from the resident materials.
int build_bsdf_recs(ContextImpl* ctx) {
    const uint32_t n = ctx->materialCount + 1u;  // + the default material
    if (!ctx->scene.bsdfRecs) {
        DeviceBlock b;
        if (!ensure_block(ctx, &b, kBsdfRec * sizeof(float4) * n, "BSDF records")) return SHIRO_ERR_OUT_OF_MEMORY;
        ctx->sceneBlocks.push_back(b);
        ctx->scene.bsdfRecs = static_cast<const float4*>(b.ptr);
    }
    k_bsdf_recs<<<(n + 127) / 128, 128, 0, ctx->stream>>>(ctx->scene.materials, n, const_cast<float4*>(ctx->scene.bsdfRecs));
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "BSDF records");
}

int finish_env(ContextImpl* ctx, size_t k) {
    DevEnv& d = ctx->envDev[k];
    const size_t n = static_cast<size_t>(d.w) * d.h;
    if (!d.hasTable) return SHIRO_OK;
    int rc = build_env_tables_device(ctx, d);
    if (rc != SHIRO_OK) return rc;
    if (!d.samples) {
        DeviceBlock b;
        if (!ensure_block(ctx, &b, 2 * n * sizeof(float4), "env sample records")) return SHIRO_ERR_OUT_OF_MEMORY;
        ctx->sceneBlocks.push_back(b);
        d.samples = static_cast<const float4*>(b.ptr);
    }
    k_env_samples<<<static_cast<unsigned>((n + 255) / 256), 256, 0, ctx->stream>>>(d, const_cast<float4*>(d.samples));
    const cudaError_t err = cudaGetLastError();
    return err == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, err, "env sample records");
}

__global__ void k_env_texels(const float* __restrict__ rgb, size_t n, float4* __restrict__ tex) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
        tex[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.0f);
}

int upload_envs(ContextImpl* ctx) {
    // the caller's rgb texels go up as they are and become (r, g, b, 0) on
    // the device; the importance tables, the masses in texels.w and the
    // per-texel sample records are built there too
    DeviceBlock rgbStage;
    struct Free {
        DeviceBlock& b;
        ContextImpl* ctx;
        ~Free() {
            if (b.ptr) cudaStreamSynchronize(ctx->stream);  // the conversion read it
            free_block(&b);
        }
    } freeStage{rgbStage, ctx};
    for (size_t k = 0; k < ctx->envHost.size(); ++k) {
        EnvHost& e = ctx->envHost[k];
        const size_t n = static_cast<size_t>(e.w) * e.h;
        DevEnv& d = ctx->envDev[k];
        d.w = e.w;
        d.h = e.h;
        d.latlong = e.latlong ? 1u : 0u;
        d.hasTable = (e.latlong && n > 0) ? 1u : 0u;
        int rc;
        DeviceBlock tb;
        if (!ensure_block(ctx, &tb, std::max<size_t>(n, 1) * sizeof(float4), "env texels")) return SHIRO_ERR_OUT_OF_MEMORY;
        ctx->sceneBlocks.push_back(tb);
        d.texels = static_cast<const float4*>(tb.ptr);
        if (n) {
            if (rgbStage.bytes < 12 * n) {  // grown for the largest texture (a sync frees the old one)
                if (rgbStage.ptr) cudaStreamSynchronize(ctx->stream);
                free_block(&rgbStage);
                if (!ensure_block(ctx, &rgbStage, 12 * n, "env texel staging")) return SHIRO_ERR_OUT_OF_MEMORY;
            }
            cudaError_t ce = cudaMemcpyAsync(rgbStage.ptr, e.rgb, 12 * n, cudaMemcpyHostToDevice, ctx->stream);
            if (ce != cudaSuccess) return cuda_fail(ctx, ce, "env texels");
            k_env_texels<<<static_cast<unsigned>(std::min<size_t>((n + 255) / 256, 4096)), 256, 0, ctx->stream>>>(
                static_cast<const float*>(rgbStage.ptr), n, const_cast<float4*>(d.texels));
            if ((ce = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, ce, "env texels");
        }
        if (d.hasTable) {
            DeviceBlock rb, cb, ab;
            if (!ensure_block(ctx, &rb, (e.h + 1u) * sizeof(float), "env row cdf") ||
                !ensure_block(ctx, &cb, static_cast<size_t>(e.h) * (e.w + 1u) * sizeof(float), "env conditional cdf") ||
                !ensure_block(ctx, &ab, n * sizeof(uint2), "env alias")) {
                for (DeviceBlock* x : {&rb, &cb, &ab}) free_block(x);
                return SHIRO_ERR_OUT_OF_MEMORY;
            }
            for (DeviceBlock* x : {&rb, &cb, &ab}) ctx->sceneBlocks.push_back(*x);
            d.rowCdf = static_cast<const float*>(rb.ptr);
            d.condCdf = static_cast<const float*>(cb.ptr);
            d.alias = static_cast<const uint2*>(ab.ptr);
        }
        if ((rc = finish_env(ctx, k)) != SHIRO_OK) return rc;
        e.rgb = nullptr;  // the caller's array is not ours past the upload
    }
    return SHIRO_OK;
}

bool wait_or_cancel(cudaEvent_t ev, const volatile int* cancel) {
    for (;;) {
        if (cancel && *cancel) return true;
        const cudaError_t e = cudaEventQuery(ev);
        if (e != cudaErrorNotReady) {
            if (e != cudaSuccess) cudaGetLastError();  // reported by the caller's final synchronisation
            return cancel && *cancel;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
}

LaunchThrottle::LaunchThrottle(const volatile int* c, uint32_t depth) : cancel(c) {
    if (!cancel) return;
    ring.resize(std::max(depth, 1u), nullptr);
    for (cudaEvent_t& e : ring)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            e = nullptr;
        }
}

LaunchThrottle::~LaunchThrottle() {
    for (cudaEvent_t e : ring)
        if (e) cudaEventDestroy(e);
}

bool LaunchThrottle::before_launch() {
    if (!cancel) return true;
    if (*cancel) return false;
    if (issued >= ring.size()) {
        cudaEvent_t e = ring[issued % ring.size()];
        if (e && wait_or_cancel(e, cancel)) return false;
    }
    return true;
}

void LaunchThrottle::after_launch(cudaStream_t stream) {
    if (!cancel) return;
    cudaEvent_t e = ring[issued % ring.size()];
    if (e) cudaEventRecord(e, stream);
    ++issued;
}

int check_device_error(ContextImpl* ctx) {
    uint32_t word = 0;
    cudaError_t e = cudaMemcpyAsync(&word, ctx->errorWord, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "kernel execution");
    if (word != 0) {
        cudaMemsetAsync(ctx->errorWord, 0, 4, ctx->stream);
        std::string msg = "device check failed:";
        if (word & kErrTraversalLimit) msg += " traversal visit limit reached;";
        if (word & kErrStackOverflow) msg += " traversal stack overflow;";
        if (word & kErrBadIndex) msg += " index out of range;";
        if (word & kErrQueueOverflow) msg += " queue overflow;";
        return fail(ctx, SHIRO_ERR_DEVICE_CHECK, msg);
    }
    return SHIRO_OK;
}

}  // namespace shiro_gpu

// ===========================================================================
// C ABI
// ===========================================================================
namespace {

int supports(const ShiroSceneDesc* scene, std::string* why) {
    if (!scene) {
        *why = "null scene";
        return 0;
    }
    if (scene->material_count && !scene->materials) {
        *why = "null material array";
        return 0;
    }
    // every lobe of TracePath is implemented (transmission and media,
    // opacity cut-outs, emitters with their light sample)
    return 1;
}

// ---- scene signature -------------------------------------------------------
// 64-bit content hash of a scene descriptor, over everything
// shiro_gpu_upload_scene reads.  Byte ranges are cut into pieces of at most
// 4 MiB, each piece is hashed on its own (seeded by its position) - on
// several host threads when the scene is large - and the piece digests are
// folded in order, so the value does not depend on the thread count.  A
// piece is hashed as 8-byte words in four independent lanes with the round of
// xxHash64 (multiply, rotate, multiply).
struct HashSpan {
    const unsigned char* p;
    size_t n;
};

inline uint64_t hash_round(uint64_t acc, uint64_t w) {
    acc += w * 0xC2B2AE3D27D4EB4Full;
    acc = (acc << 31) | (acc >> 33);
    return acc * 0x9E3779B185EBCA87ull;
}

uint64_t hash_piece(const unsigned char* p, size_t n, uint64_t seed) {
    uint64_t lane[4] = {seed + 0x60EA27EEADC0B5D6ull, seed ^ 0xC2B2AE3D27D4EB4Full, seed, seed - 0x61C8864E7A143579ull};
    const size_t len = n;
    uint64_t w[4];
    while (n >= 32) {
        std::memcpy(w, p, 32);
        for (int k = 0; k < 4; ++k) lane[k] = hash_round(lane[k], w[k]);
        p += 32;
        n -= 32;
    }
    while (n >= 8) {
        std::memcpy(w, p, 8);
        lane[0] = hash_round(lane[0], w[0]);
        p += 8;
        n -= 8;
    }
    uint64_t tail = 0;
    std::memcpy(&tail, p, n);
    lane[1] = hash_round(lane[1], tail ^ (static_cast<uint64_t>(n) << 56));
    uint64_t h = len;
    for (uint64_t l : lane) h = hash_round(h ^ hash_round(0, l), 0x9E3779B97F4A7C15ull);
    h ^= h >> 33;
    h *= 0xC2B2AE3D27D4EB4Full;
    h ^= h >> 29;
    return h;
}

template <typename T>
void put(std::vector<unsigned char>& b, const T& v) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&v);
    b.insert(b.end(), p, p + sizeof(T));
}

uint64_t hash_spans(std::vector<HashSpan> spans);

// The part of the snapshot the geometry depends on: the meshes' arrays and
// counts, each mesh's material index and the material count (they key the
// per-triangle shading records), and the cluster size of the BVH build.
uint64_t geometry_signature(const ShiroSceneDesc& sd, uint32_t sahCluster) {
    std::vector<unsigned char> head;
    put(head, sahCluster);
    put(head, sd.material_count);
    put(head, sd.mesh_count);
    std::vector<HashSpan> spans;
    for (uint32_t i = 0; i < sd.mesh_count && sd.meshes; ++i) {
        const ShiroMeshDesc& m = sd.meshes[i];
        const uint32_t vc = m.positions ? m.vertex_count : 0u, nc = m.normals ? m.normal_count : 0u,
                       ic = m.indices ? m.index_count : 0u;
        put(head, vc);
        put(head, nc);
        put(head, ic);
        put(head, m.material_index);
        spans.push_back({reinterpret_cast<const unsigned char*>(m.positions), 12ull * vc});
        spans.push_back({reinterpret_cast<const unsigned char*>(m.normals), 12ull * nc});
        spans.push_back({reinterpret_cast<const unsigned char*>(m.indices), 4ull * ic});
    }
    spans.insert(spans.begin(), HashSpan{head.data(), head.size()});
    return hash_spans(std::move(spans));
}

uint64_t scene_signature(const ShiroSceneDesc& sd) {
    // every scalar field first (counts, materials, lights, dome frames, sizes),
    // then the large arrays
    std::vector<unsigned char> head;
    put(head, sd.material_count);
    if (sd.material_count && sd.materials)
        head.insert(head.end(), reinterpret_cast<const unsigned char*>(sd.materials),
                    reinterpret_cast<const unsigned char*>(sd.materials + sd.material_count));
    put(head, sd.mesh_count);
    std::vector<HashSpan> spans;
    for (uint32_t i = 0; i < sd.mesh_count && sd.meshes; ++i) {
        const ShiroMeshDesc& m = sd.meshes[i];
        const uint32_t vc = m.positions ? m.vertex_count : 0u, nc = m.normals ? m.normal_count : 0u,
                       ic = m.indices ? m.index_count : 0u;
        put(head, vc);
        put(head, nc);
        put(head, ic);
        put(head, m.material_index);
        spans.push_back({reinterpret_cast<const unsigned char*>(m.positions), 12ull * vc});
        spans.push_back({reinterpret_cast<const unsigned char*>(m.normals), 12ull * nc});
        spans.push_back({reinterpret_cast<const unsigned char*>(m.indices), 4ull * ic});
    }
    put(head, sd.distant_light_count);
    for (uint32_t i = 0; i < sd.distant_light_count && sd.distant_lights; ++i) put(head, sd.distant_lights[i]);
    put(head, sd.dome_light_count);
    for (uint32_t i = 0; i < sd.dome_light_count && sd.dome_lights; ++i) {
        const ShiroDomeLightDesc& d = sd.dome_lights[i];
        for (const float* v : {d.radiance, d.right, d.up, d.forward}) head.insert(head.end(), reinterpret_cast<const unsigned char*>(v), reinterpret_cast<const unsigned char*>(v + 3));
        const uint32_t has = d.env_pixels ? 1u : 0u;
        put(head, d.layout);
        put(head, has ? d.env_width : 0u);
        put(head, has ? d.env_height : 0u);
        if (has) spans.push_back({reinterpret_cast<const unsigned char*>(d.env_pixels), 12ull * d.env_width * d.env_height});
    }
    head.insert(head.end(), reinterpret_cast<const unsigned char*>(sd.environment_top),
                reinterpret_cast<const unsigned char*>(sd.environment_top + 3));
    head.insert(head.end(), reinterpret_cast<const unsigned char*>(sd.environment_bottom),
                reinterpret_cast<const unsigned char*>(sd.environment_bottom + 3));
    spans.insert(spans.begin(), HashSpan{head.data(), head.size()});
    return hash_spans(std::move(spans));
}

// Hashes the spans in pieces of 4 MB, on several host threads for large
// inputs; the value does not depend on the thread count.
uint64_t hash_spans(std::vector<HashSpan> spans) {
    constexpr size_t kPiece = 4u << 20;
    std::vector<HashSpan> pieces;
    size_t total = 0;
    for (const HashSpan& sp : spans) {
        total += sp.n;
        for (size_t off = 0; off < sp.n; off += kPiece) pieces.push_back({sp.p + off, std::min(kPiece, sp.n - off)});
        if (sp.n == 0) pieces.push_back({sp.p, 0});
    }
    std::vector<uint64_t> dig(pieces.size());
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = total < (16u << 20) ? 1 : std::min<size_t>({static_cast<size_t>(hw), pieces.size(), 16});
    if (nt <= 1) {
        for (size_t i = 0; i < pieces.size(); ++i) dig[i] = hash_piece(pieces[i].p, pieces[i].n, i);
    } else {
        std::atomic<size_t> next{0};
        std::vector<std::thread> ts;
        for (size_t t = 0; t < nt; ++t)
            ts.emplace_back([&]() {
                for (size_t i = next.fetch_add(1); i < pieces.size(); i = next.fetch_add(1))
                    dig[i] = hash_piece(pieces[i].p, pieces[i].n, i);
            });
        for (auto& t : ts) t.join();
    }
    uint64_t h = hash_round(0x27D4EB2F165667C5ull, total);
    for (uint64_t d : dig) h = hash_round(h, d);
    return h;
}

// What an upload derives from the materials, lights and environments
// (everything but the geometry): emissive-triangle tables, materials and
// their BSDF records, distant lights, domes with their importance tables.
// The geometry (ctx->scene's BVHs, triangles, per-triangle records) is
// resident.
int upload_shading(ContextImpl* ctx, const ShiroSceneDesc* sd) {
    DevScene& s = ctx->scene;
    int rc;
    ctx->materialsHost.assign(sd->materials, sd->materials + sd->material_count);
    ctx->materialsHost.push_back(default_material());
    ctx->materialCount = sd->material_count;
    size_t ttotal = 0;  // global triangle ids: meshes in order, index_count / 3 each
    for (uint32_t i = 0; i < sd->mesh_count; ++i) ttotal += sd->meshes[i].index_count / 3u;
    // --- emissive triangles (BuildAccelerationScene, CpuPathTracer.cpp:482-522;
    // TriangleArea :198-222), float running sums in mesh / primitive order ----
    std::vector<float4> emissive;
    std::vector<float> emissiveCdf;
    std::vector<int32_t> emissiveOf(ttotal, -1);
    float emissiveSum = 0.0f;
    {
        const ShiroMaterialDesc dflt = default_material();
        uint32_t g = 0;
        for (uint32_t i = 0; i < sd->mesh_count; ++i) {
            const ShiroMeshDesc& m = sd->meshes[i];
            const uint32_t prims = m.index_count / 3u;
            const ShiroMaterialDesc& mat = m.material_index < sd->material_count ? sd->materials[m.material_index] : dflt;
            const float le[3] = {std::max(mat.emission_color[0] * mat.emission_strength, 0.0f),
                                 std::max(mat.emission_color[1] * mat.emission_strength, 0.0f),
                                 std::max(mat.emission_color[2] * mat.emission_strength, 0.0f)};
            const float w = std::max(0.2126f * le[0] + 0.7152f * le[1] + 0.0722f * le[2], 0.0f);
            if (m.index_count < 3 || m.index_count % 3 != 0 || w <= 0.0f) {
                g += prims;
                continue;
            }
            for (uint32_t t = 0; t < prims; ++t, ++g) {
                const float* p0 = m.positions + 3 * static_cast<size_t>(m.indices[3 * t]);
                const float* p1 = m.positions + 3 * static_cast<size_t>(m.indices[3 * t + 1]);
                const float* p2 = m.positions + 3 * static_cast<size_t>(m.indices[3 * t + 2]);
                const float a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
                const float b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
                const float av[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
                const float dbl = std::sqrt(av[0] * av[0] + av[1] * av[1] + av[2] * av[2]);
                if (dbl <= 1.0e-8f) continue;
                const float area = dbl * 0.5f;
                const float sel = area * w;
                emissiveSum += sel;
                emissiveOf[g] = static_cast<int32_t>(emissiveCdf.size());
                float gbits;
                std::memcpy(&gbits, &g, 4);
                emissive.push_back(make_float4(area, sel, emissiveSum, gbits));
                emissive.push_back(make_float4(le[0], le[1], le[2], 0.0f));
                emissive.push_back(make_float4(av[0] / dbl, av[1] / dbl, av[2] / dbl, 0.0f));
                emissiveCdf.push_back(emissiveSum);
            }
        }
    }

    s.emissiveCount = static_cast<uint32_t>(emissiveCdf.size());
    s.emissiveSum = emissiveSum;
    if (s.emissiveCount) {
        if ((rc = upload(ctx, emissive, &s.emissive, "emissive triangles")) != SHIRO_OK) return rc;
        if ((rc = upload(ctx, emissiveCdf, &s.emissiveCdf, "emissive weights")) != SHIRO_OK) return rc;
        if ((rc = upload(ctx, emissiveOf, &s.emissiveOf, "emissive index")) != SHIRO_OK) return rc;
    }
    // A transmission weight, whatever base colour and metalness make of it
    // (they are parameters shiro_gpu_set_params may change; with a zero
    // sample weight the extended stages give the reflecting ones' values).
    ctx->extendedMaterials = false;
    ctx->transmissiveMaterials = false;
    for (uint32_t i = 0; i < sd->material_count; ++i) {
        const ShiroMaterialDesc& m = sd->materials[i];
        const bool transmissive = hclamp(m.transmission, 0.0f, 1.0f) > 0.0f;
        if (transmissive || hclamp(m.opacity, 0.0f, 1.0f) < 0.999f || m.emission_strength > 0.0f)
            ctx->extendedMaterials = true;
        if (transmissive) ctx->transmissiveMaterials = true;
    }
    s.extended = ctx->extendedMaterials ? 1u : 0u;
    if ((rc = upload(ctx, ctx->materialsHost, &s.materials, "materials")) != SHIRO_OK) return rc;
    s.bsdfRecs = nullptr;
    if ((rc = build_bsdf_recs(ctx)) != SHIRO_OK) return rc;
    std::vector<DevDistant> distant(sd->distant_light_count);
    for (uint32_t i = 0; i < sd->distant_light_count; ++i)
        distant[i] = DevDistant{ld3(sd->distant_lights[i].direction), ld3(sd->distant_lights[i].radiance)};
    if ((rc = upload(ctx, distant, &s.distant, "distant lights")) != SHIRO_OK) return rc;
    s.distantCount = sd->distant_light_count;

    std::vector<DevDome> domes(sd->dome_light_count);
    for (uint32_t i = 0; i < sd->dome_light_count; ++i) {
        const ShiroDomeLightDesc& d = sd->dome_lights[i];
        domes[i].radiance = ld3(d.radiance);
        domes[i].right = ld3(d.right);
        domes[i].up = ld3(d.up);
        domes[i].forward = ld3(d.forward);
        domes[i].env = -1;
        if (d.env_pixels && d.env_width && d.env_height) {
            EnvHost e;
            e.w = d.env_width;
            e.h = d.env_height;
            e.latlong = d.layout != SHIRO_ENV_LAYOUT_ANGULAR;
            e.rgb = d.env_pixels;
            domes[i].env = static_cast<int32_t>(ctx->envHost.size());
            ctx->envHost.push_back(std::move(e));
        }
        ctx->domeEnv.push_back(domes[i].env);
    }
    ctx->envDev.assign(ctx->envHost.size(), DevEnv{});
    if ((rc = upload_envs(ctx)) != SHIRO_OK) return rc;
    if ((rc = upload(ctx, ctx->envDev, &s.envs, "env table")) != SHIRO_OK) return rc;
    if ((rc = upload(ctx, domes, &s.domes, "dome lights")) != SHIRO_OK) return rc;
    s.domeCount = sd->dome_light_count;
    s.envTop = ld3(sd->environment_top);
    s.envBottom = ld3(sd->environment_bottom);
    return SHIRO_OK;
}

int finish_upload(ContextImpl* ctx) {
    DevScene& s = ctx->scene;
    s.error = ctx->errorWord;
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "scene upload");
    ctx->hasScene = true;
    ctx->stats = ShiroRenderStats{};
    ctx->stats.bvh_nodes = s.nodes8 ? ctx->node8Count : s.nodeCount;
    ctx->stats.triangles = ctx->noGeometry ? 0u : s.triCount;
    ctx->stats.bvh_depth = s.nodes8 ? ctx->bvh8Depth : ctx->bvhDepth;
    ctx->stats.bvh_max_leaf = ctx->bvhMaxLeaf;
    ctx->stats.device_bytes = ctx->deviceBytes();
    return SHIRO_OK;
}

}  // namespace

extern "C" {

int shiro_gpu_host_alloc(size_t bytes, void** out) {
    if (!out) return SHIRO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (bytes == 0) return SHIRO_OK;
    const cudaError_t e = cudaHostAlloc(out, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return SHIRO_ERR_OUT_OF_MEMORY;
    }
    return SHIRO_OK;
}

void shiro_gpu_host_free(void* ptr) {
    if (ptr) cudaFreeHost(ptr);
}

int shiro_gpu_scene_signature(const ShiroSceneDesc* scene, uint64_t* out) {
    if (!scene || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    *out = scene_signature(*scene);
    return SHIRO_OK;
}

int shiro_gpu_status(ShiroBackendStatus* out) {
    if (!out) return SHIRO_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->kind = SHIRO_BACKEND_GPU;
    std::snprintf(out->name, sizeof(out->name), "gb300");
    out->uses_gpu = 1;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return SHIRO_OK;
    }
    out->device_count = static_cast<uint32_t>(count);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess) {
        std::snprintf(out->device_name, sizeof(out->device_name), "%s", prop.name);
        out->compute_major = prop.major;
        out->compute_minor = prop.minor;
        // the kernels are built for sm_103a only
        out->available = (prop.major == 10 && prop.minor == 3) ? 1u : 0u;
    }
    return SHIRO_OK;
}

int shiro_gpu_create(int device, ShiroGpuContext** out) {
    if (!out) return SHIRO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        gCreateError = "no CUDA device";
        return SHIRO_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) {
        gCreateError = "device index out of range";
        return SHIRO_ERR_INVALID_ARGUMENT;
    }
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        gCreateError = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
        return SHIRO_ERR_CUDA;
    }
    auto* ctx = new (std::nothrow) ShiroGpuContext();
    if (!ctx) return SHIRO_ERR_OUT_OF_MEMORY;
    ContextImpl& c = ctx->impl;
    c.device = device;
    e = cudaStreamCreateWithFlags(&c.ownStream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&c.errorWord, 16);
    if (e == cudaSuccess) e = cudaMemset(c.errorWord, 0, 16);
    if (e != cudaSuccess) {
        gCreateError = std::string("context setup: ") + cudaGetErrorString(e);
        delete ctx;
        return e == cudaErrorMemoryAllocation ? SHIRO_ERR_OUT_OF_MEMORY : SHIRO_ERR_CUDA;
    }
    c.stream = c.ownStream;
    static_scratch_setup(&c);
    *out = ctx;
    return SHIRO_OK;
}

void shiro_gpu_destroy(ShiroGpuContext* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->impl.device);
    if (ctx->impl.stream) cudaStreamSynchronize(ctx->impl.stream);
    delete ctx;
}

const char* shiro_gpu_last_error(const ShiroGpuContext* ctx) {
    if (!ctx) return gCreateError.c_str();
    return ctx->impl.lastError.c_str();
}

int shiro_gpu_set_bvh_width(ShiroGpuContext* ctx, uint32_t width) {
    if (!ctx || (width != 0 && width != 2 && width != 8)) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl& c = ctx->impl;
    c.bvhWidth = width;
    ++c.epoch;
    c.scene.nodes8 = (width == 8 && c.hasScene) ? c.nodes8 : nullptr;
    // hit slots index the triangle array of the BVH that produced them
    if (c.hasScene) c.scene.tris = c.scene.nodes8 ? c.tris8 : c.tris2;
    if (c.hasScene) {
        c.stats.bvh_nodes = c.scene.nodes8 ? c.node8Count : c.scene.nodeCount;
        c.stats.bvh_depth = c.scene.nodes8 ? c.bvh8Depth : c.bvhDepth;
    }
    return SHIRO_OK;
}

int shiro_gpu_set_bvh_build(ShiroGpuContext* ctx, uint32_t sah_cluster_triangles) {
    if (!ctx || sah_cluster_triangles == 1 || sah_cluster_triangles > (1u << 16)) return SHIRO_ERR_INVALID_ARGUMENT;
    ctx->impl.sahClusterSize = sah_cluster_triangles;
    ++ctx->impl.epoch;
    return SHIRO_OK;
}

int shiro_gpu_set_adjoint_form(ShiroGpuContext* ctx, uint32_t wavefront) {
    if (!ctx || wavefront > 1) return SHIRO_ERR_INVALID_ARGUMENT;
    ctx->impl.adjointWavefront = wavefront;
    return SHIRO_OK;
}

int shiro_gpu_set_stream(ShiroGpuContext* ctx, void* stream) {
    if (!ctx) return SHIRO_ERR_INVALID_ARGUMENT;
    ctx->impl.stream = stream ? static_cast<cudaStream_t>(stream) : ctx->impl.ownStream;
    return SHIRO_OK;
}

int shiro_gpu_supports_scene(const ShiroSceneDesc* scene, char* reason, size_t reason_size) {
    std::string why;
    const int ok = supports(scene, &why);
    if (reason && reason_size) std::snprintf(reason, reason_size, "%s", why.c_str());
    return ok;
}

int shiro_gpu_upload_scene(ShiroGpuContext* handle, const ShiroSceneDesc* sd) {
    if (!handle || !sd) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    std::string why;
    if (!supports(sd, &why)) return fail(ctx, SHIRO_ERR_UNSUPPORTED_SCENE, "unsupported scene: " + why);
    if (sd->mesh_count && !sd->meshes) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "null mesh array");
    if (sd->material_count && !sd->materials) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "null material array");
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ++ctx->epoch;
    const uint64_t geom = geometry_signature(*sd, ctx->sahClusterSize);
    if (ctx->hasScene && ctx->geomValid && ctx->geomSignature == geom) {
        // the same geometry (a light, a material or an environment edited):
        // the BVHs, triangles and per-triangle records stay on the device
        ctx->freeShading();
        const int rc = upload_shading(ctx, sd);
        if (rc != SHIRO_OK) {
            ctx->freeScene();
            return rc;
        }
        return finish_upload(ctx);
    }
    ctx->freeScene();

    // --- flatten (on the device) ----------------------------------------------
    // the meshes' own arrays go up concatenated; k_flat_* form the per-triangle
    // data, boxes and centroids there
    size_t vtotal = 0, ttotal = 0, itotal = 0, ntotal = 0;
    std::vector<FlatMesh> fm(sd->mesh_count);
    for (uint32_t i = 0; i < sd->mesh_count; ++i) {
        const ShiroMeshDesc& m = sd->meshes[i];
        if ((m.vertex_count && !m.positions) || (m.index_count && !m.indices))
            return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "mesh " + std::to_string(i) + ": null array");
        const bool hasN = m.normals && m.normal_count == m.vertex_count;
        const uint32_t material = m.material_index < sd->material_count ? m.material_index : sd->material_count;
        fm[i] = FlatMesh{static_cast<uint32_t>(vtotal), m.vertex_count, static_cast<uint32_t>(ttotal), m.index_count / 3u,
                         static_cast<uint32_t>(itotal), static_cast<uint32_t>(ntotal),
                         material | (hasN ? kShadeNormals : 0u), hasN ? 1u : 0u};
        vtotal += m.vertex_count;
        ttotal += m.index_count / 3u;
        itotal += m.index_count;
        if (hasN) ntotal += m.vertex_count;
    }
    if (ttotal >= (1ull << 28) || vtotal >= (1ull << 32))
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "scene exceeds 2^28 triangles");
    if (sd->material_count >= kShadeNormals)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "scene exceeds 2^31 - 1 materials");
    // A scene without triangles renders its lights and environment alone, as
    // the CPU tracer does (every ray misses).  The builders get two zero-area
    // triangles, each collapsed onto one of two points, in a mesh after the
    // caller's with the default material: the triangle test rejects them for
    // every ray (det = 0), so nothing can hit or occlude.
    const bool noGeometry = ttotal == 0;
    static const float kPointPos[18] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1};
    static const uint32_t kPointIdx[6] = {0, 1, 2, 3, 4, 5};
    if (noGeometry) {
        fm.push_back(FlatMesh{0, 6, 0, 2, 0, 0, sd->material_count, 0});
        vtotal = 6;
        ttotal = 2;
        itotal = 6;
    }
    ctx->noGeometry = noGeometry;
    std::vector<float> pos3(3 * vtotal), nrm3(3 * std::max<size_t>(ntotal, 1));
    std::vector<uint32_t> idx(std::max<size_t>(itotal, 1));
    for (uint32_t i = 0; i < sd->mesh_count; ++i) {
        const ShiroMeshDesc& m = sd->meshes[i];
        if (m.vertex_count) std::memcpy(&pos3[3 * static_cast<size_t>(fm[i].vbase)], m.positions, 12ull * m.vertex_count);
        if (fm[i].hasN) std::memcpy(&nrm3[3 * static_cast<size_t>(fm[i].nbase)], m.normals, 12ull * m.vertex_count);
        if (m.index_count) std::memcpy(&idx[fm[i].ibase], m.indices, 4ull * m.index_count);
    }
    if (noGeometry) {
        std::memcpy(pos3.data(), kPointPos, sizeof(kPointPos));
        std::memcpy(idx.data(), kPointIdx, sizeof(kPointIdx));
    }
    struct Temps {  // device scratch of the upload
        std::vector<void*> p;
        ~Temps() {
            for (void* x : p) cudaFree(x);
        }
    } temps;
    auto scratch = [&](size_t bytes, auto** out) -> bool {
        void* v = nullptr;
        if (cudaMalloc(&v, std::max<size_t>(bytes, 16)) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        temps.p.push_back(v);
        *out = static_cast<std::remove_pointer_t<decltype(out)>>(v);
        return true;
    };
    auto keep = [&](size_t bytes, auto** out) -> bool {  // geometry kept with the scene
        DeviceBlock blk;
        if (!ensure_block(ctx, &blk, std::max<size_t>(bytes, 16), "scene geometry")) return false;
        ctx->sceneBlocks.push_back(blk);
        *out = static_cast<std::remove_pointer_t<decltype(out)>>(blk.ptr);
        return true;
    };
    float *dPos3 = nullptr, *dNrm3 = nullptr, *dBoxes = nullptr;
    uint32_t *dIdx = nullptr, *dRed = nullptr;
    FlatMesh* dMeshes = nullptr;
    float4 *dPos4 = nullptr, *dShade = nullptr, *dAllTri = nullptr;
    uint4* dTriVerts = nullptr;
    if (!scratch(pos3.size() * 4, &dPos3) || !scratch(nrm3.size() * 4, &dNrm3) || !scratch(idx.size() * 4, &dIdx) ||
        !scratch(fm.size() * sizeof(FlatMesh), &dMeshes) || !scratch(8 * 4, &dRed) ||
        !scratch(6 * ttotal * sizeof(float), &dBoxes) || !scratch(3 * ttotal * sizeof(float4), &dAllTri) ||
        !keep(vtotal * sizeof(float4), &dPos4) || !keep(ttotal * sizeof(uint4), &dTriVerts) ||
        !keep(kShadeRec * ttotal * sizeof(float4), &dShade))
        return fail(ctx, SHIRO_ERR_OUT_OF_MEMORY, "scene flattening: out of device memory");
    const uint32_t red0[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0xffffffffu};
    cudaError_t ce = cudaMemcpyAsync(dPos3, pos3.data(), pos3.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(dNrm3, nrm3.data(), nrm3.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(dIdx, idx.data(), idx.size() * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (ce == cudaSuccess && !fm.empty())
        ce = cudaMemcpyAsync(dMeshes, fm.data(), fm.size() * sizeof(FlatMesh), cudaMemcpyHostToDevice, ctx->stream);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(dRed, red0, sizeof(red0), cudaMemcpyHostToDevice, ctx->stream);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "scene flattening");
    const unsigned gv = static_cast<unsigned>(std::min<size_t>((vtotal + 255) / 256, 4096));
    const unsigned gt = static_cast<unsigned>(std::min<size_t>((ttotal + 255) / 256, 8192));
    if (vtotal) k_flat_verts<<<gv, 256, 0, ctx->stream>>>(dPos3, static_cast<uint32_t>(vtotal), dPos4, dRed + 6);
    k_flat_tris<<<gt, 256, 0, ctx->stream>>>(dMeshes, static_cast<uint32_t>(fm.size()), dPos3, dNrm3, dIdx,
                                            static_cast<uint32_t>(ttotal),
                                            dTriVerts, dShade, dAllTri, dBoxes, dRed, dRed + 7);
    uint32_t red[8];
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(red, dRed, sizeof(red), cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "scene flattening");
    if (red[7] != 0xffffffffu) {  // the first triangle with an index out of range
        uint32_t i = 0;
        while (i + 1 < sd->mesh_count && fm[i + 1].tbase <= red[7]) ++i;
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT,
                    "mesh " + std::to_string(i) + ": index out of range at triangle " + std::to_string(red[7] - fm[i].tbase));
    }
    float slo[3], shi[3], mag;
    for (int k = 0; k < 3; ++k) {
        slo[k] = flat_unord(red[k]);
        shi[k] = flat_unord(red[3 + k]);
    }
    std::memcpy(&mag, &red[6], 4);

    // --- large triangles (a leaf under the root) + inflated boxes --------------
    auto area = [](const float* lo, const float* hi) {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    };
    const float sceneArea = area(slo, shi);
    FlatLarge fl{};
    if (ttotal > 16) {
        uint2* dCand = nullptr;
        if (!scratch(ttotal * sizeof(uint2), &dCand))
            return fail(ctx, SHIRO_ERR_OUT_OF_MEMORY, "scene flattening: out of device memory");
        uint32_t nc = 0;
        ce = cudaMemsetAsync(dRed, 0, 4, ctx->stream);
        if (ce == cudaSuccess) k_large_cands<<<gt, 256, 0, ctx->stream>>>(dBoxes, static_cast<uint32_t>(ttotal),
                                                                             0.05f * sceneArea, dCand, dRed);
        if (ce == cudaSuccess) ce = cudaGetLastError();
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(&nc, dRed, 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
        std::vector<uint2> cand(nc);
        if (ce == cudaSuccess && nc)
            ce = cudaMemcpyAsync(cand.data(), dCand, nc * sizeof(uint2), cudaMemcpyDeviceToHost, ctx->stream);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "scene flattening");
        auto af = [](const uint2& c) {
            float f;
            std::memcpy(&f, &c.x, 4);
            return f;
        };
        std::sort(cand.begin(), cand.end(), [&](const uint2& x, const uint2& y) {
            return af(x) > af(y) || (af(x) == af(y) && x.y < y.y);
        });
        if (cand.size() > 8) cand.resize(8);
        for (const uint2& c : cand) fl.gid[fl.n++] = c.y;
        std::sort(fl.gid, fl.gid + fl.n);
    }
    const float pad = mag * 1.0e-5f + 1.0e-30f;
    const size_t nSmall = ttotal - fl.n;
    float4 *dTri = nullptr, *dBox = nullptr, *dCen = nullptr;
    LargeTri* dLarge = nullptr;
    if (!scratch(3 * nSmall * sizeof(float4), &dTri) || !scratch(2 * nSmall * sizeof(float4), &dBox) ||
        !scratch(nSmall * sizeof(float4), &dCen) || !scratch(8 * sizeof(LargeTri), &dLarge))
        return fail(ctx, SHIRO_ERR_OUT_OF_MEMORY, "scene flattening: out of device memory");
    k_flat_small<<<gt, 256, 0, ctx->stream>>>(dAllTri, dBoxes, static_cast<uint32_t>(ttotal), pad, fl, dTri, dBox, dCen,
                                             dLarge);
    BvhInput bin;
    bin.largeSlots.resize(fl.n);
    ce = cudaGetLastError();
    if (ce == cudaSuccess && fl.n)
        ce = cudaMemcpyAsync(bin.largeSlots.data(), dLarge, fl.n * sizeof(LargeTri), cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "scene flattening");

    int rc;
    bin.triData = dTri;
    bin.primBoxes = dBox;
    bin.centroids = dCen;
    bin.smallCount = static_cast<uint32_t>(nSmall);
    bin.sahClusterSize = ctx->sahClusterSize;
    BvhOutput bout, bwide;
    std::string berr;
    rc = build_bvh(bin, ctx->stream, &bout, berr);
    // the wide BVH is collapsed from a binary tree with small leaves (the
    // node's triangle bits bound the leaves it can hold); its box test folds
    // 2^23 * scale / direction into a bias, so it is built only while that
    // stays far from float overflow (coordinates below 1e9)
    const bool wideOk = mag < 1.0e9f;
    if (rc == SHIRO_OK && wideOk) {
        BvhInput small = bin;
        small.maxLeaf = kWideLeaf;
        rc = build_bvh(small, ctx->stream, &bwide, berr);
    }
    auto drop = [](BvhOutput& b) {
        if (b.nodes) cudaFree(b.nodes);
        if (b.tris) cudaFree(b.tris);
        b.nodes = nullptr;
        b.tris = nullptr;
    };
    if (rc != SHIRO_OK) {
        drop(bout);
        drop(bwide);
        return fail(ctx, rc, "BVH build: " + berr);
    }
    if (bout.depth + 4 > static_cast<uint32_t>(kStack)) {
        drop(bout);
        drop(bwide);
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "BVH deeper than the traversal stack");
    }
    ctx->sceneBlocks.push_back({bout.nodes, 4 * sizeof(float4) * bout.nodeCount});
    ctx->sceneBlocks.push_back({bout.tris, 3 * sizeof(float4) * bout.triCount});
    WideOutput w8;
    if (wideOk) rc = collapse_wide(bwide.nodes, bwide.nodeCount, bwide.tris, bwide.triCount, ctx->stream, &w8, berr);
    drop(bwide);
    if (rc == SHIRO_OK && w8.depth > static_cast<uint32_t>(kStackWide)) {
        rc = SHIRO_ERR_INVALID_ARGUMENT;
        berr = "deeper than the traversal stack";
    }
    if (rc != SHIRO_OK) {
        if (w8.nodes) cudaFree(w8.nodes);
        if (w8.tris) cudaFree(w8.tris);
        return fail(ctx, rc, "wide BVH: " + berr);
    }
    if (w8.nodes) ctx->sceneBlocks.push_back({w8.nodes, 5 * sizeof(float4) * std::max<uint32_t>(bwide.nodeCount, 1)});
    if (w8.tris) ctx->sceneBlocks.push_back({w8.tris, 3 * sizeof(float4) * std::max<uint32_t>(w8.triCount, 1)});
    ctx->nodes8 = w8.nodes;
    ctx->tris8 = w8.tris;
    ctx->tris2 = bout.tris;
    ctx->node8Count = w8.nodeCount;
    ctx->bvh8Depth = w8.depth;
    ctx->bvhDepth = bout.depth;
    ctx->bvhMaxLeaf = bout.maxLeaf;
    DevScene& s = ctx->scene;
    s.nodes = bout.nodes;
    s.tris = bout.tris;
    s.nodeCount = bout.nodeCount;
    s.triCount = bout.triCount;
    s.nodes8 = ctx->bvhWidth == 8 ? ctx->nodes8 : nullptr;
    s.tris = s.nodes8 ? ctx->tris8 : ctx->tris2;

    // --- per-triangle data (formed by k_flat_tris; the geometric normals now) ---
    s.triVerts = dTriVerts;
    s.positions = dPos4;
    s.shade = dShade;
    k_shade_normals<<<(bout.triCount + 255) / 256, 256, 0, ctx->stream>>>(ctx->tris2, bout.triCount,
                                                                         const_cast<float4*>(s.shade));
    if (const cudaError_t e = cudaGetLastError(); e != cudaSuccess) return cuda_fail(ctx, e, "shading records");
    ctx->geomBlocks = ctx->sceneBlocks.size();  // what follows derives from materials, lights, environments
    if ((rc = upload_shading(ctx, sd)) != SHIRO_OK) return rc;
    s.boundsLo = V3{slo[0], slo[1], slo[2]};
    s.boundsHi = V3{shi[0], shi[1], shi[2]};
    ctx->geomSignature = geom;
    ctx->geomValid = true;
    return finish_upload(ctx);
}

int shiro_gpu_render(ShiroGpuContext* handle, const ShiroRenderDesc* req, const volatile int* cancel, ShiroAovs* out) {
    if (!handle || !req || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    if (!out->beauty || !out->albedo || !out->normal || !out->depth)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "null AOV pointer");
    const DevRequest q = make_request(*req);
    const uint64_t pixels = static_cast<uint64_t>(q.width) * q.height;
    ctx->stats.paths = 0;
    ctx->stats.kernel_launches = 0;
    ctx->stats.kernel_ms = 0.0;
    ctx->stats.path_kernel_ms = 0.0;
    ctx->stats.path_kernel_launches = 0;
    // AOV destination: caller's device planes or the context's staging planes
    AovPtrs aov;
    if (out->on_device) {
        aov = AovPtrs{out->beauty, out->albedo, out->normal, out->depth};
    } else {
        if (!ensure_block(ctx, &ctx->aovScratch, std::max<uint64_t>(pixels, 1) * 11 * sizeof(float), "AOV staging"))
            return SHIRO_ERR_OUT_OF_MEMORY;
        float* b = static_cast<float*>(ctx->aovScratch.ptr);
        aov = AovPtrs{b, b + 4 * pixels, b + 7 * pixels, b + 10 * pixels};
    }
    auto clear_host = [&]() {
        if (out->on_device) return;
        for (uint64_t i = 0; i < pixels; ++i) {
            for (int c = 0; c < 4; ++c) out->beauty[4 * i + c] = 0.0f;
            for (int c = 0; c < 3; ++c) out->albedo[3 * i + c] = out->normal[3 * i + c] = 0.0f;
            out->depth[i] = std::numeric_limits<float>::infinity();
        }
    };
    if (req->sample_count == 0 || pixels == 0) {
        // FrameBuffer::Clear semantics (FrameBuffer.cpp:19-24)
        if (out->on_device) {
            cudaMemsetAsync(out->beauty, 0, pixels * 16, ctx->stream);
            cudaMemsetAsync(out->albedo, 0, pixels * 12, ctx->stream);
            cudaMemsetAsync(out->normal, 0, pixels * 12, ctx->stream);
            std::vector<float> inf(pixels, std::numeric_limits<float>::infinity());
            if (pixels) cudaMemcpyAsync(out->depth, inf.data(), pixels * 4, cudaMemcpyHostToDevice, ctx->stream);
            cudaStreamSynchronize(ctx->stream);
        } else {
            clear_host();
        }
        return SHIRO_OK;
    }
    // paths in flight per launch: whole pixels, at most 2^24 paths (805 MB of records)
    const uint64_t maxPaths = 1ull << 24;
    const uint64_t pixelsPerChunk = std::max<uint64_t>(1, maxPaths / q.sampleCount);
    const uint64_t recBytes = std::min<uint64_t>(pixelsPerChunk, pixels) * q.sampleCount * kPathRecordBytes;
    if (!ensure_block(ctx, &ctx->pathRecords, recBytes, "path records")) return SHIRO_ERR_OUT_OF_MEMORY;
    float4* rec = static_cast<float4*>(ctx->pathRecords.ptr);
    // events around the whole call and around every path-kernel launch
    std::vector<cudaEvent_t> ev;
    auto new_event = [&]() {
        cudaEvent_t x;
        cudaEventCreate(&x);
        ev.push_back(x);
        return x;
    };
    auto drop_events = [&]() {
        for (cudaEvent_t x : ev) cudaEventDestroy(x);
    };
    cudaEvent_t e0 = new_event();
    cudaEventRecord(e0, ctx->stream);
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pathEv;
    LaunchThrottle throttle(cancel, 2);  // two chunks queued at most while a cancel flag is polled
    for (uint64_t p0 = 0; p0 < pixels; p0 += pixelsPerChunk) {
        if (!throttle.before_launch()) {
            cudaStreamSynchronize(ctx->stream);
            drop_events();
            clear_host();
            if (out->on_device) {  // FrameBuffer::Clear semantics for device planes too
                cudaMemsetAsync(out->beauty, 0, pixels * 16, ctx->stream);
                cudaMemsetAsync(out->albedo, 0, pixels * 12, ctx->stream);
                cudaMemsetAsync(out->normal, 0, pixels * 12, ctx->stream);
                std::vector<float> inf(pixels, std::numeric_limits<float>::infinity());
                cudaMemcpyAsync(out->depth, inf.data(), pixels * 4, cudaMemcpyHostToDevice, ctx->stream);
                cudaStreamSynchronize(ctx->stream);
            }
            return fail(ctx, SHIRO_ERR_CANCELLED, "cancelled");
        }
        const uint32_t np = static_cast<uint32_t>(std::min(pixelsPerChunk, pixels - p0));
        const uint64_t paths = static_cast<uint64_t>(np) * q.sampleCount;
        cudaEvent_t a = new_event(), b = new_event();
        cudaEventRecord(a, ctx->stream);
        launch_plain_paths(ctx->scene, q, p0 * q.sampleCount, static_cast<uint32_t>(paths), rec, ctx->stream);
        cudaEventRecord(b, ctx->stream);
        pathEv.emplace_back(a, b);
        launch_resolve_pixels(q, p0, np, rec, aov, ctx->stream);
        throttle.after_launch(ctx->stream);
        ctx->stats.kernel_launches += 2;
        ctx->stats.paths += paths;
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) {
            drop_events();
            return cuda_fail(ctx, le, "render launch");
        }
    }
    cudaEvent_t e1 = new_event();
    cudaEventRecord(e1, ctx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    double pathMs = 0.0;
    if (e == cudaSuccess) {
        cudaEventElapsedTime(&ms, e0, e1);
        for (auto& pe : pathEv) {
            float x = 0.0f;
            cudaEventElapsedTime(&x, pe.first, pe.second);
            pathMs += x;
        }
    }
    drop_events();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render");
    ctx->stats.kernel_ms = ms;
    ctx->stats.path_kernel_ms = pathMs;
    ctx->stats.path_kernel_launches = pathEv.size();
    if ((rc = check_device_error(ctx)) != SHIRO_OK) return rc;
    if (!out->on_device) {
        e = cudaMemcpyAsync(out->beauty, aov.beauty, pixels * 16, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->albedo, aov.albedo, pixels * 12, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->normal, aov.normal, pixels * 12, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(out->depth, aov.depth, pixels * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "AOV readback");
    }
    ctx->stats.device_bytes = ctx->deviceBytes();
    return SHIRO_OK;
}

int shiro_gpu_render_batch(ShiroGpuContext* handle, const ShiroRenderDesc* reqs, uint32_t count, const volatile int* cancel,
                           ShiroAovs* outs) {
    if (!handle || (count && (!reqs || !outs))) return SHIRO_ERR_INVALID_ARGUMENT;
    cudaSetDevice(handle->impl.device);
    return wavefront_render(&handle->impl, reqs, count, cancel, outs);
}

int shiro_gpu_render_batch_ready(ShiroGpuContext* handle, const ShiroRenderDesc* reqs, uint32_t count,
                                 const volatile int* cancel, ShiroAovs* outs, ShiroPixelsReady ready, void* user) {
    if (!handle || !ready || (count && (!reqs || !outs))) return SHIRO_ERR_INVALID_ARGUMENT;
    cudaSetDevice(handle->impl.device);
    return wavefront_render(&handle->impl, reqs, count, cancel, outs, ready, user);
}

int shiro_gpu_get_wavefront_config(const ShiroGpuContext* ctx, ShiroWavefrontConfig* out) {
    if (!ctx || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    return wavefront_get_config(&ctx->impl, out);
}

int shiro_gpu_set_wavefront_config(ShiroGpuContext* ctx, const ShiroWavefrontConfig* cfg) {
    if (!ctx || !cfg) return SHIRO_ERR_INVALID_ARGUMENT;
    ++ctx->impl.epoch;
    return wavefront_set_config(&ctx->impl, cfg);
}

int shiro_gpu_autotune(ShiroGpuContext* ctx, const ShiroRenderDesc* req, ShiroWavefrontConfig* chosen) {
    if (!ctx || !req) return SHIRO_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->impl.device);
    return wavefront_autotune(&ctx->impl, req, chosen);
}

int shiro_gpu_set_params(ShiroGpuContext* ctx, const float* base, const float* rough, const float* metal, const float* env) {
    if (!ctx) return SHIRO_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->impl.device);
    return adjoint_set_params(&ctx->impl, base, rough, metal, env);
}

int shiro_gpu_adjoint(ShiroGpuContext* ctx, const ShiroRenderDesc* req, const float* dBeauty, float* dBase, float* dRough,
                      float* dMetal, float* dEnv) {
    if (!ctx || !req || !dBeauty) return SHIRO_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->impl.device);
    return adjoint_run(&ctx->impl, req, dBeauty, dBase, dRough, dMetal, dEnv);
}

int shiro_gpu_render_frozen(ShiroGpuContext* ctx, const ShiroRenderDesc* req, const float* base, const float* rough,
                            const float* metal, const float* env, float* beauty) {
    if (!ctx || !req || !beauty) return SHIRO_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->impl.device);
    return adjoint_render_frozen(&ctx->impl, req, base, rough, metal, env, beauty);
}

int shiro_gpu_sample(ShiroGpuContext* handle, const uint32_t* px, const uint32_t* py, const uint32_t* index,
                     const uint32_t* branch, uint32_t n, float* out2) {
    if (!handle || (n && (!px || !py || !index || !branch || !out2))) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    if (n == 0) return SHIRO_OK;
    std::vector<uint4> tuples(n);
    for (uint32_t k = 0; k < n; ++k) tuples[k] = make_uint4(px[k], py[k], index[k], branch[k]);
    if (!ensure_block(ctx, &ctx->probeScratch, static_cast<size_t>(n) * (sizeof(uint4) + 2 * sizeof(float)), "probe"))
        return SHIRO_ERR_OUT_OF_MEMORY;
    uint4* dt = static_cast<uint4*>(ctx->probeScratch.ptr);
    float* dout = reinterpret_cast<float*>(dt + n);
    cudaError_t e = cudaMemcpyAsync(dt, tuples.data(), n * sizeof(uint4), cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "sample probe upload");
    launch_sample_probe(dt, n, dout, ctx->stream);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out2, dout, n * 2 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "sample probe");
}

int shiro_gpu_primary_hits(ShiroGpuContext* handle, const ShiroRenderDesc* req, uint32_t* prim, float* t, uint32_t on_device) {
    if (!handle || !req || !prim || !t) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    const DevRequest q = make_request(*req);
    const uint64_t n = static_cast<uint64_t>(q.width) * q.height;
    uint32_t* dp = prim;
    float* dt = t;
    if (!on_device) {
        if (!ensure_block(ctx, &ctx->probeScratch, std::max<uint64_t>(n, 1) * 8, "probe")) return SHIRO_ERR_OUT_OF_MEMORY;
        dp = static_cast<uint32_t*>(ctx->probeScratch.ptr);
        dt = reinterpret_cast<float*>(dp + n);
    }
    launch_primary_hits(ctx->scene, q, dp, dt, ctx->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "primary hits launch");
    if ((rc = check_device_error(ctx)) != SHIRO_OK) return rc;
    if (!on_device) {
        e = cudaMemcpyAsync(prim, dp, n * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(t, dt, n * 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "primary hits readback");
    }
    return SHIRO_OK;
}

int shiro_gpu_trace_rays(ShiroGpuContext* handle, const float* origins, const float* dirs, const float* tmax, uint32_t n,
                         uint32_t* prim, float* t, uint32_t* occ) {
    if (!handle || (n && (!origins || !dirs || !tmax || !prim || !t || !occ))) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    if (n == 0) return SHIRO_OK;
    // host arrays: 7 floats in, 3 words out per ray
    if (!ensure_block(ctx, &ctx->probeScratch, static_cast<size_t>(n) * 10 * 4, "probe")) return SHIRO_ERR_OUT_OF_MEMORY;
    float* base = static_cast<float*>(ctx->probeScratch.ptr);
    float *dO = base, *dD = base + 3 * static_cast<size_t>(n), *dM = base + 6 * static_cast<size_t>(n);
    uint32_t* dP = reinterpret_cast<uint32_t*>(base + 7 * static_cast<size_t>(n));
    float* dT = base + 8 * static_cast<size_t>(n);
    uint32_t* dOcc = reinterpret_cast<uint32_t*>(base + 9 * static_cast<size_t>(n));
    cudaError_t e = cudaMemcpyAsync(dO, origins, 12ull * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dD, dirs, 12ull * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dM, tmax, 4ull * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace rays upload");
    launch_trace_rays(ctx->scene, dO, dD, dM, n, dP, dT, dOcc, ctx->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace rays launch");
    int rc = check_device_error(ctx);
    if (rc != SHIRO_OK) return rc;
    e = cudaMemcpyAsync(prim, dP, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t, dT, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(occ, dOcc, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "trace rays readback");
    return SHIRO_OK;
}

int shiro_gpu_count_work(ShiroGpuContext* handle, const ShiroRenderDesc* req, uint32_t stride, ShiroWorkCounts* out) {
    if (!handle || !req || !out || stride == 0) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    const DevRequest q = make_request(*req);
    if (!ensure_block(ctx, &ctx->probeScratch, 16 * sizeof(unsigned long long), "work counters")) return SHIRO_ERR_OUT_OF_MEMORY;
    auto* totals = static_cast<unsigned long long*>(ctx->probeScratch.ptr);
    cudaError_t e = cudaMemsetAsync(totals, 0, 12 * sizeof(unsigned long long), ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "work counters");
    if (req->sample_count > 0) launch_count_paths(ctx->scene, q, stride, totals, ctx->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "count launch");
    if ((rc = check_device_error(ctx)) != SHIRO_OK) return rc;
    unsigned long long h[12];
    e = cudaMemcpyAsync(h, totals, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "work counters readback");
    out->paths = h[0];
    out->closest_rays = h[1];
    out->occlusion_rays = h[2];
    out->node_visits = h[3];
    out->tri_tests = h[4];
    out->hits = h[5];
    out->env_evals = h[6];
    out->env_samples = h[7];
    out->bsdf_evals = h[8];
    out->bsdf_pdfs = h[9];
    out->occlusion_node_visits = h[10];
    out->occlusion_tri_tests = h[11];
    return SHIRO_OK;
}

int shiro_gpu_env_tables(ShiroGpuContext* handle, uint32_t env, uint32_t* wOut, uint32_t* hOut, float* rowCdf,
                         float* condCdf, float* mass, uint32_t* aliasThreshold, uint32_t* aliasIndex) {
    if (!handle) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    if (env >= ctx->envDev.size()) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "no such dome texture");
    const DevEnv& d = ctx->envDev[env];
    if (wOut) *wOut = d.w;
    if (hOut) *hOut = d.h;
    const size_t n = static_cast<size_t>(d.w) * d.h;
    const bool table = d.hasTable != 0;
    if (!table && (rowCdf || condCdf || aliasThreshold || aliasIndex))
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "this dome texture has no importance table (angular layout)");
    cudaError_t e = cudaSuccess;
    if (rowCdf) e = cudaMemcpyAsync(rowCdf, d.rowCdf, (d.h + 1u) * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && condCdf)
        e = cudaMemcpyAsync(condCdf, d.condCdf, static_cast<size_t>(d.h) * (d.w + 1u) * sizeof(float),
                            cudaMemcpyDeviceToHost, ctx->stream);
    std::vector<float4> tex(mass ? n : 0);
    if (e == cudaSuccess && mass)
        e = cudaMemcpyAsync(tex.data(), d.texels, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream);
    std::vector<uint2> al((aliasThreshold || aliasIndex) ? n : 0);
    if (e == cudaSuccess && !al.empty())
        e = cudaMemcpyAsync(al.data(), d.alias, n * sizeof(uint2), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "env table readback");
    for (size_t i = 0; i < tex.size(); ++i) mass[i] = tex[i].w;
    for (size_t i = 0; i < al.size(); ++i) {
        if (aliasThreshold) aliasThreshold[i] = al[i].x;
        if (aliasIndex) aliasIndex[i] = al[i].y;
    }
    return SHIRO_OK;
}

int shiro_gpu_env_sample(ShiroGpuContext* handle, uint32_t env, uint32_t n, const float* u2, uint32_t flags,
                         uint32_t* texel, float* pdf) {
    if (!handle || (n && (!u2 || !texel || !pdf))) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    if (env >= ctx->envDev.size() || !ctx->envDev[env].hasTable)
        return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "no such dome texture with an importance table");
    if (n == 0) return SHIRO_OK;
    if (!ensure_block(ctx, &ctx->probeScratch, static_cast<size_t>(n) * 16, "probe")) return SHIRO_ERR_OUT_OF_MEMORY;
    float2* du = static_cast<float2*>(ctx->probeScratch.ptr);
    uint32_t* dt = reinterpret_cast<uint32_t*>(du + n);
    float* dp = reinterpret_cast<float*>(dt + n);
    cudaError_t e = cudaMemcpyAsync(du, u2, static_cast<size_t>(n) * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "env sample upload");
    launch_env_pick(ctx->envDev[env], du, n, (flags & SHIRO_RENDER_ENV_CDF) != 0u, dt, dp, ctx->stream);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(texel, dt, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pdf, dp, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "env sample probe");
}

int shiro_gpu_render_paths(ShiroGpuContext* handle, const ShiroRenderDesc* req, const uint32_t* pixels, uint32_t n,
                           const uint32_t* sampleIndex, float* out) {
    if (!handle || !req || (n && (!pixels || !sampleIndex || !out))) return SHIRO_ERR_INVALID_ARGUMENT;
    ContextImpl* ctx = &handle->impl;
    cudaSetDevice(ctx->device);
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    const uint64_t px = static_cast<uint64_t>(req->settings.width) * req->settings.height;
    for (uint32_t i = 0; i < n; ++i)
        if (pixels[i] >= px) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "pixel index out of range");
    if (n == 0) return SHIRO_OK;
    if (!ensure_block(ctx, &ctx->probeScratch, static_cast<size_t>(n) * 12 * 4, "probe")) return SHIRO_ERR_OUT_OF_MEMORY;
    uint32_t* dpx = static_cast<uint32_t*>(ctx->probeScratch.ptr);
    uint32_t* dsi = dpx + n;
    float* dout = reinterpret_cast<float*>(dsi + n);
    cudaError_t e = cudaMemcpyAsync(dpx, pixels, static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dsi, sampleIndex, static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render paths upload");
    launch_render_paths(ctx->scene, make_request(*req), dpx, dsi, n, dout, ctx->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render paths launch");
    if ((rc = check_device_error(ctx)) != SHIRO_OK) return rc;
    e = cudaMemcpyAsync(out, dout, static_cast<size_t>(n) * 40, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "render paths readback");
}

int shiro_gpu_last_stats(const ShiroGpuContext* ctx, ShiroRenderStats* out) {
    if (!ctx || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    *out = ctx->impl.stats;
    return SHIRO_OK;
}

}  // extern "C"
