// shiro_oracle.cpp - CPU restatement of Shiro's reference path tracer.
//
// TEST INFRASTRUCTURE ONLY (checker for the GPU backend and the timed CPU
// baseline).  Every function states the reference lines it restates
// (ichin0se/Shiro; CpuPathTracer.cpp = src/backend/cpu/CpuPathTracer.cpp,
// EnvironmentMap.cpp / OpenQmcSampler.cpp = src/render/...).  Expressions are
// written in the reference's evaluation order and the file is compiled with
// -ffp-contract=off, so on the same libm the results are bit-identical to the
// reference (checked against tests/golden).
//
// Intersection: the reference's brute-force closest hit (CpuPathTracer.cpp:
// 431-466) keeps the first (mesh, primitive) among equal distances.  Here a
// binned-SAH BVH with conservatively inflated boxes is traversed and hits are
// ordered by (t, global primitive index), which selects the same triangle.

#include "shiro_oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// Vector arithmetic with the reference's operator semantics (Types.h:28-111)
// ---------------------------------------------------------------------------
struct V3 {
    float x = 0.0f, y = 0.0f, z = 0.0f;
};
struct V2 {
    float x = 0.0f, y = 0.0f;
};

inline V3 operator+(const V3& a, const V3& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(const V3& a, const V3& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(const V3& a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, const V3& a) { return a * s; }
inline V3 operator*(const V3& a, const V3& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 operator/(const V3& a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float Dot(const V3& a, const V3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 Cross(const V3& a, const V3& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float Length(const V3& a) { return std::sqrt(Dot(a, a)); }
inline V3 Normalize(const V3& a) {
    const float l = Length(a);
    return l > 0.0f ? a / l : V3{};
}
inline float Clampf(float v, float lo, float hi) { return std::clamp(v, lo, hi); }
inline V3 Clamp3(const V3& v, float lo, float hi) { return {Clampf(v.x, lo, hi), Clampf(v.y, lo, hi), Clampf(v.z, lo, hi)}; }
inline V3 Lerp(const V3& a, const V3& b, float t) { return a * (1.0f - t) + b * t; }
inline float MaxComponent(const V3& v) { return std::max(v.x, std::max(v.y, v.z)); }
inline V3 Reflect(const V3& i, const V3& n) { return i - 2.0f * Dot(i, n) * n; }
inline V3 L3(const float* p) { return {p[0], p[1], p[2]}; }

constexpr float kPi = 3.14159265358979323846f;  // CpuPathTracer.cpp:59-77
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

// ---------------------------------------------------------------------------
// QMC fallback sampler (OpenQmcSampler.cpp:20-71, 110-135)
// ---------------------------------------------------------------------------
constexpr uint32_t kPrimes[24] = {2u, 3u, 5u, 7u, 11u, 13u, 17u, 19u, 23u, 29u, 31u, 37u,
                                  41u, 43u, 47u, 53u, 59u, 61u, 67u, 71u, 73u, 79u, 83u, 89u};
constexpr float kR2Step[2] = {0.7548776662466927f, 0.5698402909980532f};

inline uint32_t Scramble(uint32_t s) {  // MixBits, :30-37
    s ^= s >> 16;
    s *= 0x7feb352du;
    s ^= s >> 15;
    s *= 0x846ca68bu;
    s ^= s >> 16;
    return s;
}

inline float RadicalInv(uint32_t base, uint32_t i) {  // :43-54
    const float invBase = 1.0f / static_cast<float>(base);
    float scale = invBase;
    float acc = 0.0f;
    while (i > 0u) {
        acc += static_cast<float>(i % base) * scale;
        i /= base;
        scale *= invBase;
    }
    return acc;
}

inline float QmcDim(uint32_t px, uint32_t py, uint32_t index, uint32_t dim) {  // :56-71
    if (dim < 2u) {
        const float v = 0.5f + kR2Step[dim] * static_cast<float>(index);
        return v - std::floor(v);
    }
    const float seq = RadicalInv(kPrimes[dim % 24u], index + 1u);
    const uint32_t key = px * 0x8da6b343u ^ py * 0xd8163841u ^ dim * 0xcb1ab31fu ^ 0x9e3779b9u;
    const float rot = static_cast<float>(Scramble(key) & 0x00ffffffu) / 16777216.0f;
    const float v = seq + rot;
    return v - std::floor(v);
}

struct Sampler {
    uint32_t px, py, index;
    V2 Next2D(uint32_t branch) const {
        return {QmcDim(px, py, index, branch * 2u), QmcDim(px, py, index, branch * 2u + 1u)};
    }
    float Next1D(uint32_t branch) const { return QmcDim(px, py, index, branch * 2u); }
};

// ---------------------------------------------------------------------------
// Environment map (EnvironmentMap.cpp)
// ---------------------------------------------------------------------------
struct Env {
    uint32_t w = 0, h = 0;
    bool latlong = true;
    std::vector<V3> px;
    std::vector<float> rowCdf, condCdf;
    // Optional alias table of the GPU backend (not part of the reference):
    // per texel the acceptance threshold (float bits) and the alias texel.
    // When present and the render does not ask for the CDF search, a sample
    // picks its texel as the backend's alias lookup does; everything after
    // the pick is EnvironmentMap::Sample's.
    std::vector<uint32_t> aliasThr, aliasIdx;

    static float Wrap(float v) {  // :23-26
        v = std::fmod(v, 1.0f);
        return v < 0.0f ? v + 1.0f : v;
    }

    void Build() {  // BuildImportanceTable, :185-236
        rowCdf.clear();
        condCdf.clear();
        if (px.empty() || w == 0 || h == 0 || !latlong) return;
        rowCdf.assign(h + 1u, 0.0f);
        condCdf.assign(static_cast<size_t>(h) * (w + 1u), 0.0f);
        float total = 0.0f;
        for (uint32_t y = 0; y < h; ++y) {
            const float theta = (static_cast<float>(y) + 0.5f) * kPi / static_cast<float>(h);
            const float sinT = std::max(std::sin(theta), 1.0e-6f);
            const size_t off = static_cast<size_t>(y) * (w + 1u);
            float row = 0.0f;
            for (uint32_t x = 0; x < w; ++x) {
                const V3& c = px[static_cast<size_t>(y) * w + x];
                const float lum = c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f;
                row += std::max(0.0f, lum) * sinT;
                condCdf[off + x + 1u] = row;
            }
            if (row > 0.0f) {
                for (uint32_t x = 1; x <= w; ++x) condCdf[off + x] /= row;
            } else {
                for (uint32_t x = 1; x <= w; ++x) condCdf[off + x] = static_cast<float>(x) / static_cast<float>(w);
                row = 1.0f;
            }
            total += row;
            rowCdf[y + 1u] = total;
        }
        if (total <= 0.0f) {
            for (uint32_t y = 1; y <= h; ++y) rowCdf[y] = static_cast<float>(y) / static_cast<float>(h);
            return;
        }
        for (uint32_t y = 1; y <= h; ++y) rowCdf[y] /= total;
    }

    V3 Bilinear(float u, float v) const {  // :266-300
        if (px.empty() || w == 0 || h == 0) return {};
        u = Wrap(u) * static_cast<float>(w) - 0.5f;
        v = Clampf(v, 0.0f, 1.0f) * static_cast<float>(h) - 0.5f;
        const int x0 = static_cast<int>(std::floor(u));
        const int y0 = static_cast<int>(std::floor(v));
        const int x1 = x0 + 1;
        const int y1 = std::min(y0 + 1, static_cast<int>(h) - 1);
        const float tx = u - static_cast<float>(x0);
        const float ty = v - static_cast<float>(y0);
        auto at = [&](int x, int y) {
            int xx = x % static_cast<int>(w);
            if (xx < 0) xx += static_cast<int>(w);
            const int yy = std::clamp(y, 0, static_cast<int>(h) - 1);
            return px[static_cast<size_t>(yy) * w + static_cast<size_t>(xx)];
        };
        const V3 c0 = Lerp(at(x0, y0), at(x1, y0), tx);
        const V3 c1 = Lerp(at(x0, y1), at(x1, y1), tx);
        return Lerp(c0, c1, ty);
    }

    V3 Evaluate(const V3& local) const {  // :94-107, 238-264
        if (px.empty()) return {};
        const V3 d = Normalize(local);
        if (!latlong) {
            const float rl = std::sqrt(d.x * d.x + d.y * d.y);
            if (rl <= 1.0e-6f) return Bilinear(0.5f, 0.5f);
            const float angle = std::acos(Clampf(d.z, -1.0f, 1.0f));
            const float radius = angle / kPi;
            const float nx = d.x / rl;
            const float ny = d.y / rl;
            const float u = 0.5f + 0.5f * radius * nx;
            const float v = 0.5f + 0.5f * radius * ny;
            if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f) return {};
            return Bilinear(u, v);
        }
        const float phi = std::atan2(d.x, d.z);
        const float theta = std::acos(Clampf(d.y, -1.0f, 1.0f));
        return Bilinear(Wrap(phi / kTwoPi), Clampf(theta / kPi, 0.0f, 1.0f));
    }

    uint32_t SampleCdf(const std::vector<float>& cdf, uint32_t begin, uint32_t end, float s, float* mass) const {
        // :315-330 - first entry of cdf[begin+1 .. end] not below s.
        const float key = Clampf(s, 0.0f, std::nextafter(1.0f, 0.0f));
        const auto first = cdf.begin() + static_cast<std::ptrdiff_t>(begin + 1u);
        const auto last = cdf.begin() + static_cast<std::ptrdiff_t>(end + 1u);
        const uint32_t idx = static_cast<uint32_t>(std::lower_bound(first, last, key) - cdf.begin()) - 1u;
        *mass = cdf[idx + 1u] - cdf[idx];
        return idx - begin;
    }

    float PixelPdf(uint32_t x, uint32_t y, float sinT) const {  // LatLongPdf, :302-313
        if (rowCdf.empty() || condCdf.empty() || w == 0 || h == 0 || sinT <= 1.0e-6f) return 0.0f;
        const float rowMass = rowCdf[y + 1u] - rowCdf[y];
        const size_t off = static_cast<size_t>(y) * (w + 1u);
        const float colMass = condCdf[off + x + 1u] - condCdf[off + x];
        return rowMass * colMass * static_cast<float>(w * h) / (2.0f * kPi * kPi * sinT);
    }

    V3 Sample(const V2& u, V3* dir, float* pdf, bool useAlias = false) const {  // :109-163
        if (px.empty()) {
            *dir = {0.0f, 1.0f, 0.0f};
            *pdf = 0.0f;
            return {};
        }
        if (latlong && !rowCdf.empty() && w > 0 && h > 0) {
            float rowMass = 0.0f, colMass = 0.0f;
            uint32_t row, col;
            if (useAlias && aliasThr.size() == static_cast<size_t>(w) * h) {
                // the backend's texel pick: bucket floor(u.y * n), accepted
                // when u.x is below its threshold, else its alias
                const uint32_t n = w * h;
                uint32_t i = static_cast<uint32_t>(u.y * static_cast<float>(n));
                i = i >= n ? n - 1u : i;
                float thr;
                std::memcpy(&thr, &aliasThr[i], 4);
                const uint32_t t = u.x < thr ? i : aliasIdx[i];
                row = t / w;
                col = t - row * w;
                rowMass = rowCdf[row + 1u] - rowCdf[row];
                const size_t off = static_cast<size_t>(row) * (w + 1u);
                colMass = condCdf[off + col + 1u] - condCdf[off + col];
            } else {
                row = SampleCdf(rowCdf, 0, h, u.y, &rowMass);
                const uint32_t off = row * (w + 1u);
                col = SampleCdf(condCdf, off, off + w, u.x, &colMass);
            }
            const float uu = (static_cast<float>(col) + 0.5f) / static_cast<float>(w);
            const float vv = (static_cast<float>(row) + 0.5f) / static_cast<float>(h);
            const float theta = vv * kPi;
            const float phi = uu * kTwoPi;
            const float sinT = std::sin(theta);
            const V3 d{std::sin(phi) * sinT, std::cos(theta), std::cos(phi) * sinT};
            *dir = d;
            const float mass = rowMass * colMass;
            *pdf = sinT > 1.0e-6f ? mass * static_cast<float>(w * h) / (2.0f * kPi * kPi * sinT) : 0.0f;
            return Evaluate(d);
        }
        const float y = 1.0f - 2.0f * u.y;
        const float r = std::sqrt(std::max(0.0f, 1.0f - y * y));
        const float phi = kTwoPi * u.x;
        const V3 d{std::sin(phi) * r, y, std::cos(phi) * r};
        *dir = d;
        *pdf = kInvFourPi;
        return Evaluate(d);
    }

    float Pdf(const V3& local) const {  // :165-183
        if (px.empty()) return 0.0f;
        if (!latlong || rowCdf.empty() || w == 0 || h == 0) return kInvFourPi;
        const V3 d = Normalize(local);
        const float phi = std::atan2(d.x, d.z);
        const float theta = std::acos(Clampf(d.y, -1.0f, 1.0f));
        const float u = Wrap(phi / kTwoPi);
        const float v = Clampf(theta / kPi, 0.0f, 1.0f);
        const uint32_t x = std::min(static_cast<uint32_t>(u * static_cast<float>(w)), w - 1u);
        const uint32_t y = std::min(static_cast<uint32_t>(v * static_cast<float>(h)), h - 1u);
        return PixelPdf(x, y, std::sin(theta));
    }
};

std::shared_ptr<Env> MakeEnv(uint32_t w, uint32_t h, const float* rgb, uint32_t layout) {
    auto e = std::make_shared<Env>();
    e->w = w;
    e->h = h;
    e->latlong = layout != SHIRO_ENV_LAYOUT_ANGULAR;
    e->px.resize(static_cast<size_t>(w) * h);
    for (size_t i = 0; i < e->px.size(); ++i) e->px[i] = L3(rgb + 3 * i);
    e->Build();
    return e;
}

// ---------------------------------------------------------------------------
// Scene
// ---------------------------------------------------------------------------
struct Dome {
    V3 radiance, right, up, forward;
    std::shared_ptr<Env> env;
};
struct Distant {
    V3 direction, radiance;
};
struct MeshData {
    std::vector<V3> pos, nrm;
    std::vector<uint32_t> idx;
    uint32_t material = 0;
};

ShiroMaterialDesc DefaultMaterial() {  // PbrMaterial defaults, Renderer.h:56-102
    ShiroMaterialDesc m;
    std::memset(&m, 0, sizeof(m));
    auto s3 = [](float* d, float a, float b, float c) { d[0] = a; d[1] = b; d[2] = c; };
    s3(m.base_color, 0.8f, 0.8f, 0.8f);
    s3(m.specular_color, 1, 1, 1);
    s3(m.transmission_color, 1, 1, 1);
    s3(m.coat_color, 1, 1, 1);
    s3(m.subsurface_color, 1, 1, 1);
    s3(m.subsurface_radius, 1, 1, 1);
    s3(m.sheen_color, 1, 1, 1);
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

struct Node {
    float lo[3], hi[3];
    uint32_t left = 0, right = 0;  // internal: children; leaf: first prim, count
    bool leaf = false;
};

struct SceneData {
    std::vector<ShiroMaterialDesc> materials;  // last entry = default material
    std::vector<MeshData> meshes;
    std::vector<Distant> distant;
    std::vector<Dome> domes;
    V3 envTop, envBottom;
    // flattened triangles, global index = mesh-major order
    std::vector<uint32_t> triMesh, triPrim;
    std::vector<V3> tv0, te1, te2;
    std::vector<uint32_t> bvhPrims;
    std::vector<Node> nodes;
    // emissive triangles (AccelerationScene::emissiveTriangles,
    // CpuPathTracer.cpp:482-522) and, per global triangle, its entry or -1
    struct Emissive {
        uint32_t mesh, prim, gid;
        float area, weight, cumulative;
        V3 radiance, ng;
    };
    std::vector<Emissive> emissive;
    float emissiveSum = 0.0f;
    std::vector<int32_t> emissiveOf;
};

struct Ray {
    V3 o, d;
    float tMin = kRayEpsilon;
    float tMax = FLT_MAX;
};

struct Hit {
    bool hit = false;
    float t = FLT_MAX;
    uint32_t gid = 0xffffffffu;
    float u = 0.0f, v = 0.0f;
};

// Moller-Trumbore as in IntersectTriangle (CpuPathTracer.cpp:386-429).
inline bool TriTest(const Ray& r, const V3& p0, const V3& e1, const V3& e2, float* t, float* u, float* v) {
    const V3 pvec = Cross(r.d, e2);
    const float det = Dot(e1, pvec);
    if (std::fabs(det) < 1.0e-8f) return false;
    const float inv = 1.0f / det;
    const V3 tvec = r.o - p0;
    const float uu = Dot(tvec, pvec) * inv;
    if (uu < 0.0f || uu > 1.0f) return false;
    const V3 qvec = Cross(tvec, e1);
    const float vv = Dot(r.d, qvec) * inv;
    if (vv < 0.0f || uu + vv > 1.0f) return false;
    const float tt = Dot(e2, qvec) * inv;
    if (tt < r.tMin || tt > r.tMax) return false;
    *t = tt;
    *u = uu;
    *v = vv;
    return true;
}

// ---- binned SAH BVH ------------------------------------------------------
struct BuildPrim {
    float lo[3], hi[3], c[3];
};

void BuildBvh(SceneData& s) {
    const size_t n = s.tv0.size();
    s.nodes.clear();
    s.bvhPrims.resize(n);
    if (n == 0) return;
    std::vector<BuildPrim> bp(n);
    float mag = 0.0f;
    for (size_t i = 0; i < n; ++i) {
        const V3 a = s.tv0[i], b = a + s.te1[i], c = a + s.te2[i];
        // exact vertex positions are p0, p0 + e1, p0 + e2 only up to rounding;
        // boxes are widened below to cover that and the intersector's error.
        const float xs[3] = {a.x, b.x, c.x}, ys[3] = {a.y, b.y, c.y}, zs[3] = {a.z, b.z, c.z};
        bp[i].lo[0] = std::min({xs[0], xs[1], xs[2]});
        bp[i].hi[0] = std::max({xs[0], xs[1], xs[2]});
        bp[i].lo[1] = std::min({ys[0], ys[1], ys[2]});
        bp[i].hi[1] = std::max({ys[0], ys[1], ys[2]});
        bp[i].lo[2] = std::min({zs[0], zs[1], zs[2]});
        bp[i].hi[2] = std::max({zs[0], zs[1], zs[2]});
        for (int k = 0; k < 3; ++k) {
            bp[i].c[k] = 0.5f * (bp[i].lo[k] + bp[i].hi[k]);
            mag = std::max(mag, std::max(std::fabs(bp[i].lo[k]), std::fabs(bp[i].hi[k])));
        }
        s.bvhPrims[i] = static_cast<uint32_t>(i);
    }
    const float pad = mag * 1.0e-5f + 1.0e-30f;
    for (auto& p : bp) {
        for (int k = 0; k < 3; ++k) {
            const float e = pad + (p.hi[k] - p.lo[k]) * 1.0e-5f;
            p.lo[k] -= e;
            p.hi[k] += e;
        }
    }
    struct Task {
        uint32_t node, begin, end, depth;
    };
    s.nodes.reserve(2 * n / 2 + 1);
    s.nodes.push_back(Node{});
    std::vector<Task> stack{{0u, 0u, static_cast<uint32_t>(n), 0u}};
    constexpr int kBins = 16;
    auto area = [](const float* lo, const float* hi) {
        const float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return dx * dy + dy * dz + dz * dx;
    };
    while (!stack.empty()) {
        const Task t = stack.back();
        stack.pop_back();
        Node nd;
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int k = 0; k < 3; ++k) {
            nd.lo[k] = FLT_MAX;
            nd.hi[k] = -FLT_MAX;
        }
        for (uint32_t i = t.begin; i < t.end; ++i) {
            const BuildPrim& p = bp[s.bvhPrims[i]];
            for (int k = 0; k < 3; ++k) {
                nd.lo[k] = std::min(nd.lo[k], p.lo[k]);
                nd.hi[k] = std::max(nd.hi[k], p.hi[k]);
                clo[k] = std::min(clo[k], p.c[k]);
                chi[k] = std::max(chi[k], p.c[k]);
            }
        }
        const uint32_t count = t.end - t.begin;
        int bestAxis = -1, bestSplit = 0;
        float bestCost = FLT_MAX;
        if (count > 2) {
            for (int k = 0; k < 3; ++k) {
                const float ext = chi[k] - clo[k];
                if (!(ext > 0.0f)) continue;
                uint32_t cnt[kBins] = {};
                float blo[kBins][3], bhi[kBins][3];
                for (int b = 0; b < kBins; ++b)
                    for (int j = 0; j < 3; ++j) {
                        blo[b][j] = FLT_MAX;
                        bhi[b][j] = -FLT_MAX;
                    }
                for (uint32_t i = t.begin; i < t.end; ++i) {
                    const BuildPrim& p = bp[s.bvhPrims[i]];
                    int b = static_cast<int>((p.c[k] - clo[k]) / ext * kBins);
                    b = std::min(std::max(b, 0), kBins - 1);
                    cnt[b]++;
                    for (int j = 0; j < 3; ++j) {
                        blo[b][j] = std::min(blo[b][j], p.lo[j]);
                        bhi[b][j] = std::max(bhi[b][j], p.hi[j]);
                    }
                }
                float rA[kBins];
                uint32_t rC[kBins];
                float alo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, ahi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                uint32_t acc = 0;
                for (int b = kBins - 1; b > 0; --b) {
                    acc += cnt[b];
                    for (int j = 0; j < 3; ++j) {
                        alo[j] = std::min(alo[j], blo[b][j]);
                        ahi[j] = std::max(ahi[j], bhi[b][j]);
                    }
                    rA[b] = acc ? area(alo, ahi) : 0.0f;
                    rC[b] = acc;
                }
                for (int j = 0; j < 3; ++j) {
                    alo[j] = FLT_MAX;
                    ahi[j] = -FLT_MAX;
                }
                acc = 0;
                for (int b = 0; b < kBins - 1; ++b) {
                    acc += cnt[b];
                    for (int j = 0; j < 3; ++j) {
                        alo[j] = std::min(alo[j], blo[b][j]);
                        ahi[j] = std::max(ahi[j], bhi[b][j]);
                    }
                    if (acc == 0 || rC[b + 1] == 0) continue;
                    const float cost = area(alo, ahi) * acc + rA[b + 1] * rC[b + 1];
                    if (cost < bestCost) {
                        bestCost = cost;
                        bestAxis = k;
                        bestSplit = b;
                    }
                }
            }
        }
        const float leafCost = area(nd.lo, nd.hi) * count;
        const uint32_t self = t.node;
        if (count <= 4 && (bestAxis < 0 || bestCost >= leafCost)) {
            nd.leaf = true;
            nd.left = t.begin;
            nd.right = count;
            s.nodes[self] = nd;
            continue;
        }
        uint32_t mid;
        if (bestAxis >= 0 && t.depth < 96) {
            const int k = bestAxis;
            const float ext = chi[k] - clo[k];
            auto it = std::partition(s.bvhPrims.begin() + t.begin, s.bvhPrims.begin() + t.end, [&](uint32_t id) {
                int b = static_cast<int>((bp[id].c[k] - clo[k]) / ext * kBins);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= bestSplit;
            });
            mid = static_cast<uint32_t>(it - s.bvhPrims.begin());
        } else {
            mid = t.begin + count / 2;
        }
        if (mid == t.begin || mid == t.end) mid = t.begin + count / 2;
        const uint32_t l = static_cast<uint32_t>(s.nodes.size());
        s.nodes.push_back(Node{});
        s.nodes.push_back(Node{});
        nd.leaf = false;
        nd.left = l;
        nd.right = l + 1;
        s.nodes[self] = nd;
        stack.push_back({l, t.begin, mid, t.depth + 1});
        stack.push_back({l + 1, mid, t.end, t.depth + 1});
    }
}

inline bool BoxHit(const Node& nd, const V3& o, const float inv[3], float tmax, float* tEnter) {
    float t0 = 0.0f, t1 = tmax;
    const float oo[3] = {o.x, o.y, o.z};
    for (int k = 0; k < 3; ++k) {
        float a = (nd.lo[k] - oo[k]) * inv[k];
        float b = (nd.hi[k] - oo[k]) * inv[k];
        if (a > b) std::swap(a, b);
        if (a > t0) t0 = a;
        if (b < t1) t1 = b;
        if (!(t0 <= t1)) return false;
    }
    *tEnter = t0;
    return true;
}

void InvDir(const V3& d, float inv[3]) {
    const float c[3] = {d.x, d.y, d.z};
    for (int k = 0; k < 3; ++k) {
        const float v = std::fabs(c[k]) > 1.0e-20f ? c[k] : std::copysign(1.0e-20f, c[k]);
        inv[k] = 1.0f / v;
    }
}

// Closest hit with the brute-force tie rule: smallest (t, global index).
bool Closest(const SceneData& s, const Ray& r, Hit* out) {
    if (s.nodes.empty()) return false;
    float inv[3];
    InvDir(r.d, inv);
    Hit best;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const Node& nd = s.nodes[stack[--sp]];
        float te;
        const float bound = best.hit ? best.t * 1.0000005f + 1e-30f : FLT_MAX;
        if (!BoxHit(nd, r.o, inv, bound, &te)) continue;
        if (nd.leaf) {
            for (uint32_t i = nd.left; i < nd.left + nd.right; ++i) {
                const uint32_t id = s.bvhPrims[i];
                float t, u, v;
                if (!TriTest(r, s.tv0[id], s.te1[id], s.te2[id], &t, &u, &v)) continue;
                if (!best.hit || t < best.t || (t == best.t && id < best.gid)) {
                    best.hit = true;
                    best.t = t;
                    best.gid = id;
                    best.u = u;
                    best.v = v;
                }
            }
            continue;
        }
        float ta, tb;
        const bool ha = BoxHit(s.nodes[nd.left], r.o, inv, bound, &ta);
        const bool hb = BoxHit(s.nodes[nd.right], r.o, inv, bound, &tb);
        if (ha && hb) {
            if (ta <= tb) {
                stack[sp++] = nd.right;
                stack[sp++] = nd.left;
            } else {
                stack[sp++] = nd.left;
                stack[sp++] = nd.right;
            }
        } else if (ha) {
            stack[sp++] = nd.left;
        } else if (hb) {
            stack[sp++] = nd.right;
        }
    }
    *out = best;
    return best.hit;
}

bool ClosestBrute(const SceneData& s, const Ray& r, Hit* out) {
    Hit best;
    for (uint32_t id = 0; id < s.tv0.size(); ++id) {
        float t, u, v;
        if (!TriTest(r, s.tv0[id], s.te1[id], s.te2[id], &t, &u, &v) || t >= best.t) continue;
        best.hit = true;
        best.t = t;
        best.gid = id;
        best.u = u;
        best.v = v;
    }
    *out = best;
    return best.hit;
}

// Occluded (CpuPathTracer.cpp:468-475, 697-709): any hit in [1e-4, maxDist].
bool Occluded(const SceneData& s, const V3& o, const V3& d, float maxDist) {
    if (s.nodes.empty()) return false;
    Ray r;
    r.o = o;
    r.d = d;
    r.tMax = maxDist;
    float inv[3];
    InvDir(d, inv);
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    const float bound = maxDist * 1.0000005f + 1e-30f;
    while (sp) {
        const Node& nd = s.nodes[stack[--sp]];
        float te;
        if (!BoxHit(nd, o, inv, bound, &te)) continue;
        if (nd.leaf) {
            for (uint32_t i = nd.left; i < nd.left + nd.right; ++i) {
                const uint32_t id = s.bvhPrims[i];
                float t, u, v;
                if (TriTest(r, s.tv0[id], s.te1[id], s.te2[id], &t, &u, &v)) return true;
            }
            continue;
        }
        stack[sp++] = nd.left;
        stack[sp++] = nd.right;
    }
    return false;
}

bool OccludedBrute(const SceneData& s, const V3& o, const V3& d, float maxDist) {
    Ray r;
    r.o = o;
    r.d = d;
    r.tMax = maxDist;
    for (uint32_t id = 0; id < s.tv0.size(); ++id) {
        float t, u, v;
        if (TriTest(r, s.tv0[id], s.te1[id], s.te2[id], &t, &u, &v)) return true;
    }
    return false;
}

struct SurfaceHit {
    float t;
    V3 position, ng, ns;
    uint32_t material;
    uint32_t gid;
};

// Hit record of IntersectSceneBruteForce (CpuPathTracer.cpp:448-456) and
// TriangleShadingNormal (:142-168).
SurfaceHit MakeSurface(const SceneData& s, const Ray& r, const Hit& h) {
    SurfaceHit sh;
    sh.t = h.t;
    sh.gid = h.gid;
    sh.position = r.o + r.d * h.t;
    const uint32_t mesh = s.triMesh[h.gid], prim = s.triPrim[h.gid];
    const MeshData& m = s.meshes[mesh];
    const uint32_t i0 = m.idx[3 * prim], i1 = m.idx[3 * prim + 1], i2 = m.idx[3 * prim + 2];
    const V3 p0 = m.pos[i0], p1 = m.pos[i1], p2 = m.pos[i2];
    sh.ng = Normalize(Cross(p1 - p0, p2 - p0));
    const float b0 = 1.0f - h.u - h.v, b1 = h.u, b2 = h.v;
    V3 ns = Normalize(Cross(p1 - p0, p2 - p0));
    if (m.nrm.size() == m.pos.size()) {
        const V3 interp = m.nrm[i0] * b0 + m.nrm[i1] * b1 + m.nrm[i2] * b2;
        if (Length(interp) > 0.0f) ns = Normalize(interp);
    }
    sh.ns = ns;
    sh.material = m.material;
    return sh;
}

// ---------------------------------------------------------------------------
// BSDF (CpuPathTracer.cpp:836-1132, 1218-1354, 1376-1389)
// ---------------------------------------------------------------------------
using Mat = ShiroMaterialDesc;

inline float Sq(float v) { return v * v; }
inline V3 SafeNormalized(const V3& v, const V3& fb) {  // :836-839
    const float l = Length(v);
    return l > 0.0f ? v / l : fb;
}
inline V3 OrthoX(const V3& n) {  // BuildOrthonormalX, :255-258
    const V3 axis = std::fabs(n.z) < 0.999f ? V3{0.0f, 0.0f, 1.0f} : V3{0.0f, 1.0f, 0.0f};
    return Normalize(Cross(axis, n));
}
inline float F0Dielectric(float ior) {  // :895-899
    const float s = std::max(ior, 1.0f);
    return Sq((s - 1.0f) / (s + 1.0f));
}
inline V3 DiffuseColor(const Mat& m) {  // :901-909
    const float metal = Clampf(m.metallic, 0.0f, 1.0f);
    const float trans = Clampf(m.transmission, 0.0f, 1.0f);
    const float sss = Clampf(m.subsurface, 0.0f, 1.0f);
    const float blend = Clampf(MaxComponent(L3(m.subsurface_radius)) / 3.0f, 0.0f, 1.0f);
    const V3 tint = Lerp(L3(m.base_color), L3(m.subsurface_color), blend);
    const V3 base = Lerp(L3(m.base_color), tint, sss);
    return base * (Clampf(m.base_weight, 0.0f, 1.0f) * (1.0f - metal) * (1.0f - trans));
}
inline float BaseRoughness(const Mat& m) {  // :911-916
    return Clampf(m.roughness + m.coat_affect_roughness * m.coat_weight * m.coat_roughness, 0.0f, 1.0f);
}
inline V3 SpecF0(const Mat& m) {  // :918-924
    const float metal = Clampf(m.metallic, 0.0f, 1.0f);
    const V3 d = L3(m.specular_color) * (Clampf(m.specular_weight, 0.0f, 1.0f) * F0Dielectric(m.ior));
    return Lerp(d, L3(m.base_color), metal);
}
inline V3 CoatF0(const Mat& m) {  // :926-928
    return L3(m.coat_color) * (Clampf(m.coat_weight, 0.0f, 1.0f) * F0Dielectric(m.coat_ior));
}
inline V3 OneMinusClamped(const V3& v) {  // :1035-1041
    return {Clampf(1.0f - v.x, 0.0f, 1.0f), Clampf(1.0f - v.y, 0.0f, 1.0f), Clampf(1.0f - v.z, 0.0f, 1.0f)};
}
inline V3 Schlick(const V3& f0, float vDotH) {  // :1005-1009
    const float c = Clampf(1.0f - vDotH, 0.0f, 1.0f);
    const float f = c * c * c * c * c;
    return f0 + (V3{1.0f, 1.0f, 1.0f} - f0) * f;
}
inline V3 CoatTint(const Mat& m) {  // CoatUnderlayerTint, :1043-1046
    const float a = Clampf(m.coat_affect_color * m.coat_weight, 0.0f, 1.0f);
    return Lerp(V3{1.0f, 1.0f, 1.0f}, Clamp3(L3(m.coat_color), 0.0f, 1.0f), a);
}
inline V3 LayerTransmittance(const V3& f0, float nDotV, float nDotL) {  // :1048-1052
    const V3 fv = Schlick(f0, Clampf(nDotV, 0.0f, 1.0f));
    const V3 fl = Schlick(f0, Clampf(nDotL, 0.0f, 1.0f));
    return OneMinusClamped((fv + fl) * 0.5f);
}
inline float GgxD(float nDotH, float r) {  // :988-993
    const float a = std::max(0.02f, r * r);
    const float a2 = a * a;
    const float den = std::max(1.0e-6f, Sq(nDotH * nDotH * (a2 - 1.0f) + 1.0f));
    return a2 / (kPi * den);
}
inline float GgxVis(float nDotV, float nDotL, float r) {  // :995-1003
    const float a = std::max(0.02f, r * r);
    const float a2 = a * a;
    auto lambda = [&](float x) {
        const float c = std::max(x, 1.0e-6f);
        return (-1.0f + std::sqrt(1.0f + a2 * (1.0f - c * c) / (c * c))) * 0.5f;
    };
    return 1.0f / (1.0f + lambda(nDotV) + lambda(nDotL));
}
inline V3 SpecLobe(const V3& n, const V3& v, const V3& l, const V3& f0, float r) {  // :1096-1115
    const float nv = Clampf(Dot(n, v), 0.0f, 1.0f);
    const float nl = Clampf(Dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return {};
    const V3 h = SafeNormalized(v + l, n);
    const float nh = Clampf(Dot(n, h), 0.0f, 1.0f);
    const float vh = Clampf(Dot(v, h), 0.0f, 1.0f);
    const float d = GgxD(nh, r);
    const float g = GgxVis(nv, nl, r);
    return Schlick(f0, vh) * (d * g / std::max(4.0f * nv * nl, 1.0e-6f));
}
inline float SpecPdf(const V3& n, const V3& v, const V3& l, float r) {  // :1117-1132
    const float nv = Clampf(Dot(n, v), 0.0f, 1.0f);
    const float nl = Clampf(Dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return 0.0f;
    const V3 h = SafeNormalized(v + l, n);
    const float nh = Clampf(Dot(n, h), 0.0f, 1.0f);
    const float vh = Clampf(Dot(v, h), 1.0e-6f, 1.0f);
    return GgxD(nh, r) * nh / std::max(4.0f * vh, 1.0e-6f);
}
inline V3 ProjTangent(const Mat& m, const V3& n) {  // :852-860
    if (m.has_tangent_override) {
        const V3 t = L3(m.tangent_override) - n * Dot(L3(m.tangent_override), n);
        if (Length(t) > 0.0f) return Normalize(t);
    }
    return OrthoX(n);
}
// AdjustedRoughness with the anisotropy phase of the half vector (:862-893).
// With zero anisotropy the phase term is multiplied by zero, so it is skipped.
inline float RoughnessFor(float r, float aniso, float rot, const V3& n, const V3& tangent, const V3& v,
                          const V3& l) {
    const float ca = Clampf(aniso, -0.95f, 0.95f);
    float phase = 0.0f;
    if (ca != 0.0f) {
        const V3 td = SafeNormalized(tangent - n * Dot(tangent, n), OrthoX(n));
        const V3 bt = Normalize(Cross(n, td));
        const V3 h = SafeNormalized(v + l, n);
        const V3 hp = h - n * Dot(n, h);
        if (Length(hp) <= 1.0e-6f) {
            phase = std::cos(rot * 2.0f * kPi);
        } else {
            const V3 hd = Normalize(hp);
            const float ang = std::atan2(Dot(hd, bt), Dot(hd, td));
            phase = std::cos(ang - rot * 2.0f * kPi);
        }
    }
    return Clampf(r * (1.0f - 0.35f * ca * phase), 0.02f, 1.0f);
}
inline float RoughnessFor(float r, float aniso, float rot) {  // :845-850
    const float ca = Clampf(aniso, -0.95f, 0.95f);
    const float phase = std::cos(rot * 2.0f * kPi);
    return Clampf(r * (1.0f - 0.35f * ca * phase), 0.02f, 1.0f);
}
inline V3 FilmColor(float thickness, float ior, float vDotH) {  // :934-953
    if (thickness <= 0.0f) return {1.0f, 1.0f, 1.0f};
    const float si = std::max(ior, 1.0f);
    const float op = 2.0f * si * thickness * Clampf(vDotH, 0.05f, 1.0f);
    auto band = [&](float wl) {
        const float phase = 4.0f * kPi * op / std::max(wl, 1.0f);
        return 0.5f + 0.5f * std::cos(phase);
    };
    const V3 iri{band(650.0f), band(510.0f), band(475.0f)};
    const float strength = Clampf(thickness / 1200.0f, 0.0f, 1.0f);
    return Lerp(V3{1.0f, 1.0f, 1.0f}, (V3{1.0f, 1.0f, 1.0f} + iri) * 0.5f, strength);
}
inline V3 ThinFilm(const V3& lobe, const Mat& m, const V3& n, const V3& v, const V3& l) {  // :955-968
    if (m.thin_film_thickness <= 0.0f) return lobe;
    const V3 h = SafeNormalized(v + l, n);
    const float vh = Clampf(Dot(v, h), 0.0f, 1.0f);
    return lobe * FilmColor(m.thin_film_thickness, m.thin_film_ior, vh);
}
inline V3 ResolveNormal(const Mat& m, const V3& fb, bool coat) {  // :970-986
    const bool has = coat ? m.has_coat_normal_override != 0 : m.has_normal_override != 0;
    if (!has) return fb;
    const V3 c = coat ? L3(m.coat_normal_override) : L3(m.normal_override);
    if (Length(c) <= 0.0f) return fb;
    V3 n = Normalize(c);
    if (Dot(n, fb) < 0.0f) n = n * -1.0f;
    return n;
}
inline float DiffuseWeight(const Mat& m) {  // :1376-1380
    const V3 uc = CoatTint(m) * OneMinusClamped(CoatF0(m));
    const V3 ub = OneMinusClamped(SpecF0(m));
    return std::max(0.0f, MaxComponent(DiffuseColor(m) * uc * ub));
}
inline float SpecWeight(const Mat& m) {  // :1382-1385
    const V3 uc = CoatTint(m) * OneMinusClamped(CoatF0(m));
    return std::max(0.0f, MaxComponent(uc * SpecF0(m)));
}
inline float CoatWeight(const Mat& m) { return std::max(0.0f, MaxComponent(CoatF0(m))); }  // :1387-1389
inline float TransmissionWeight(const Mat& m) {  // :1391-1403
    const float tr = Clampf(m.transmission, 0.0f, 1.0f);
    const float metal = Clampf(m.metallic, 0.0f, 1.0f);
    if (tr <= 0.0f || metal >= 0.999f) return 0.0f;
    const V3 uc = CoatTint(m) * OneMinusClamped(CoatF0(m));
    const V3 ub = OneMinusClamped(SpecF0(m));
    return std::max(0.0f, MaxComponent(Clamp3(L3(m.transmission_color), 0.0f, 1.0f) * uc * ub)) * tr * (1.0f - metal);
}

float BsdfPdf(const Mat& m, const V3& n, const V3& cn, const V3& v, const V3& l) {  // :1232-1273
    const float nl = Clampf(Dot(n, l), 0.0f, 1.0f);
    if (nl <= 0.0f) return 0.0f;
    const float dw = DiffuseWeight(m), bw = SpecWeight(m), cw = CoatWeight(m);
    const float rw = dw + bw + cw;
    if (rw <= 0.0f) return 0.0f;
    const float dp = dw / rw, bp = bw / rw, cp = cw / rw;
    const float sr = RoughnessFor(BaseRoughness(m), m.specular_anisotropy, m.specular_rotation, n, ProjTangent(m, n), v, l);
    const float cr = RoughnessFor(m.coat_roughness, m.coat_anisotropy, m.coat_rotation, cn, ProjTangent(m, cn), v, l);
    return dp * nl * kInvPi + bp * SpecPdf(n, v, l, sr) + cp * SpecPdf(cn, v, l, cr);
}

V3 Bsdf(const Mat& m, const V3& n, const V3& cn, const V3& v, const V3& l) {  // :1275-1354
    const float nv = Clampf(Dot(n, v), 0.0f, 1.0f);
    const float nl = Clampf(Dot(n, l), 0.0f, 1.0f);
    if (nv <= 0.0f || nl <= 0.0f) return {};
    const V3 baseF0 = SpecF0(m);
    const V3 coatF0 = CoatF0(m);
    const V3 underCoat = CoatTint(m) * LayerTransmittance(coatF0, Dot(cn, v), Dot(cn, l));
    const V3 underBase = LayerTransmittance(baseF0, nv, nl);
    const V3 tangent = ProjTangent(m, n);
    const V3 coatTangent = ProjTangent(m, cn);
    const V3 vp = Normalize(v - n * nv);
    const V3 lp = Normalize(l - n * nl);
    const float cosPhi = Length(vp) > 0.0f && Length(lp) > 0.0f ? Clampf(Dot(vp, lp), -1.0f, 1.0f) : 0.0f;
    const float sigma = Clampf(m.diffuse_roughness, 0.0f, 1.0f);
    const float s2 = sigma * sigma;
    const float orenA = 1.0f - (s2 / (2.0f * (s2 + 0.33f)));
    const float orenB = 0.45f * s2 / (s2 + 0.09f);
    const float sinV = std::sqrt(std::max(0.0f, 1.0f - nv * nv));
    const float sinL = std::sqrt(std::max(0.0f, 1.0f - nl * nl));
    const float sinAlpha = std::max(sinV, sinL);
    const float tanBeta = std::min(sinV / std::max(nv, 1.0e-6f), sinL / std::max(nl, 1.0e-6f));
    const float wrap = Clampf(m.subsurface * m.subsurface_scale *
                                  (0.35f + 0.15f * Clampf(m.subsurface_anisotropy, -1.0f, 1.0f) +
                                   0.1f * Clampf(MaxComponent(L3(m.subsurface_radius)) / 3.0f, 0.0f, 1.0f)),
                              0.0f, 0.9f);
    const float wrapped = Clampf((nl + wrap) / (1.0f + wrap), 0.0f, 1.0f);
    const float term = (orenA + orenB * std::max(0.0f, cosPhi) * sinAlpha * tanBeta) * (wrapped / std::max(nl, 1.0e-6f));
    const V3 diffuse = DiffuseColor(m) * underCoat * underBase * (kInvPi * term);
    const float sr = RoughnessFor(BaseRoughness(m), m.specular_anisotropy, m.specular_rotation, n, tangent, v, l);
    const V3 spec = underCoat * ThinFilm(SpecLobe(n, v, l, baseF0, sr), m, n, v, l);
    const float cr = RoughnessFor(m.coat_roughness, m.coat_anisotropy, m.coat_rotation, cn, coatTangent, v, l);
    const V3 coat = ThinFilm(SpecLobe(cn, v, l, coatF0, cr), m, cn, v, l);
    const V3 h = SafeNormalized(v + l, n);
    const float sw = Clampf(m.sheen, 0.0f, 1.0f);
    const float lh = Clampf(Dot(l, h), 0.0f, 1.0f);
    const float sf = std::pow(1.0f - lh, 5.0f) * (1.0f - 0.5f * Clampf(m.sheen_roughness, 0.0f, 1.0f));
    const V3 sheen = L3(m.sheen_color) * sw * sf * underCoat * underBase;
    return diffuse + spec + coat + sheen;
}

inline V3 CosineHemisphere(const V3& n, const V2& s) {  // :276-286
    const float phi = 2.0f * kPi * s.x;
    const float r = std::sqrt(s.y);
    const float x = r * std::cos(phi);
    const float y = r * std::sin(phi);
    const float z = std::sqrt(std::max(0.0f, 1.0f - s.y));
    const V3 t = OrthoX(n);
    const V3 b = Cross(n, t);
    return Normalize(t * x + b * y + n * z);
}
inline V3 GgxHalf(const V3& n, const V2& s, float rough) {  // :288-302
    const float a = std::max(0.02f, rough * rough);
    const float a2 = a * a;
    const float phi = 2.0f * kPi * s.x;
    const float ct = std::sqrt(std::max(0.0f, (1.0f - s.y) / std::max(1.0e-6f, 1.0f + (a2 - 1.0f) * s.y)));
    const float st = std::sqrt(std::max(0.0f, 1.0f - ct * ct));
    const float x = st * std::cos(phi);
    const float y = st * std::sin(phi);
    const float z = ct;
    const V3 t = OrthoX(n);
    const V3 b = Cross(n, t);
    return Normalize(t * x + b * y + n * z);
}
inline V3 ClampMax(const V3& v, float mx) {  // :1224-1230
    const float c = MaxComponent(v);
    if (c <= mx || c <= 0.0f) return v;
    return v * (mx / c);
}
inline float Power(float a, float b) {  // :1218-1222
    const float a2 = a * a, b2 = b * b;
    return a2 / std::max(a2 + b2, 1.0e-6f);
}

// --- transmission, media and emitters -------------------------------------
inline float TransmissionRoughness(const Mat& m) {  // :930-932
    return Clampf(m.roughness + m.transmission_extra_roughness, 0.0f, 1.0f);
}
float FresnelDielectric(float cosThetaI, float etaI, float etaT) {  // :1011-1033
    float c = Clampf(cosThetaI, -1.0f, 1.0f);
    float ei = std::max(etaI, 1.0e-6f);
    float et = std::max(etaT, 1.0e-6f);
    if (c <= 0.0f) {
        std::swap(ei, et);
        c = std::fabs(c);
    }
    const float sinI = std::sqrt(std::max(0.0f, 1.0f - c * c));
    const float sinT = ei / et * sinI;
    if (sinT >= 1.0f) return 1.0f;
    const float cosT = std::sqrt(std::max(0.0f, 1.0f - sinT * sinT));
    const float rPar = ((et * c) - (ei * cosT)) / std::max((et * c) + (ei * cosT), 1.0e-6f);
    const float rPer = ((ei * c) - (et * cosT)) / std::max((ei * c) + (et * cosT), 1.0e-6f);
    return 0.5f * (rPar * rPar + rPer * rPer);
}
inline V3 InterfaceTransmittance(const V3& f0, float a, float b) {  // TransmissionInterfaceTransmittance, :1059-1063
    const V3 fa = Schlick(f0, Clampf(std::fabs(a), 0.0f, 1.0f));
    const V3 fb = Schlick(f0, Clampf(std::fabs(b), 0.0f, 1.0f));
    return OneMinusClamped((fa + fb) * 0.5f);
}
inline V3 CoatTransmissionScale(const Mat& m, const V3& cn, const V3& v, const V3& l) {  // :1084-1094
    return CoatTint(m) * InterfaceTransmittance(CoatF0(m), Dot(cn, v), Dot(cn, l));
}
inline V3 TransmissionSurfaceTint(const Mat& m) {  // :1405-1410
    if (!m.thin_walled && m.transmission_depth > 0.0f) return {1.0f, 1.0f, 1.0f};
    return Clamp3(L3(m.transmission_color), 0.0f, 1.0f);
}
inline float ThinPaneTransmittance(float r) {  // ThinWalledPaneTransmittance, :1412-1418
    const float c = Clampf(r, 0.0f, 1.0f);
    return Clampf((1.0f - c) / std::max(1.0f + c, 1.0e-6f), 0.0f, 1.0f);
}
V3 MediumExtinction(const Mat& m) {  // :1420-1437
    V3 e{std::max(m.transmission_scatter[0], 0.0f), std::max(m.transmission_scatter[1], 0.0f),
         std::max(m.transmission_scatter[2], 0.0f)};
    if (m.thin_walled || m.transmission_depth <= 0.0f) return e;
    const float depth = std::max(m.transmission_depth, 1.0e-3f);
    const V3 tint = Clamp3(L3(m.transmission_color), 1.0e-4f, 1.0f);
    e.x += -std::log(tint.x) / depth;
    e.y += -std::log(tint.y) / depth;
    e.z += -std::log(tint.z) / depth;
    return e;
}
inline V3 MediumAttenuation(const V3& e, float d) {  // :1439-1441, Exp :841-843
    return {std::exp(-e.x * d), std::exp(-e.y * d), std::exp(-e.z * d)};
}
bool Refract(const V3& i, const V3& n, float eta, V3* out) {  // RefractDirection, :1355-1373
    const float c = Clampf(-Dot(i, n), -1.0f, 1.0f);
    const float sin2 = std::max(0.0f, 1.0f - c * c);
    const float k = 1.0f - eta * eta * sin2;
    if (k <= 0.0f) return false;
    *out = Normalize(i * eta + n * (eta * c - std::sqrt(k)));
    return true;
}
V3 TransmissionLobe(const Mat& m, const V3& n, const V3& cn, const V3& v, const V3& l, float etaI, float etaT,
                    float r) {  // EvaluateTransmissionLobe, :1136-1181
    const float cosWo = Dot(n, v), cosWi = Dot(n, l);
    const float aWo = std::fabs(cosWo), aWi = std::fabs(cosWi);
    if (aWo <= 0.0f || aWi <= 0.0f || cosWo * cosWi >= 0.0f) return {};
    const float rel = etaT / std::max(etaI, 1.0e-6f);
    V3 h = SafeNormalized(v + l * rel, n);
    if (Dot(n, h) < 0.0f) h = h * -1.0f;
    const float woH = Dot(v, h), wiH = Dot(l, h);
    if (woH * wiH >= 0.0f) return {};
    const float nh = Clampf(Dot(n, h), 0.0f, 1.0f);
    const float sd = woH + rel * wiH;
    if (nh <= 0.0f || std::fabs(sd) <= 1.0e-6f) return {};
    const float dist = GgxD(nh, r);
    const float vis = GgxVis(aWo, aWi, r);
    const float fres = 1.0f - FresnelDielectric(std::fabs(woH), etaI, etaT);
    const V3 scale = TransmissionSurfaceTint(m) * CoatTransmissionScale(m, cn, v, l) *
                     (Clampf(m.transmission, 0.0f, 1.0f) * (1.0f - Clampf(m.metallic, 0.0f, 1.0f)));
    const float factor = std::fabs(dist * vis * std::fabs(wiH) * std::fabs(woH) / std::max(aWo * aWi * Sq(sd), 1.0e-6f));
    const float transport = 1.0f / std::max(rel * rel, 1.0e-6f);
    return scale * fres * (factor * transport);
}
float TransmissionPdf(const V3& n, const V3& v, const V3& l, float eta, float r) {  // :1183-1212
    const float cosWo = Dot(n, v), cosWi = Dot(n, l);
    if (std::fabs(cosWo) <= 0.0f || std::fabs(cosWi) <= 0.0f || cosWo * cosWi >= 0.0f) return 0.0f;
    V3 h = SafeNormalized(v + l * eta, n);
    if (Dot(n, h) < 0.0f) h = h * -1.0f;
    const float woH = Dot(v, h), wiH = Dot(l, h);
    const float sd = woH + eta * wiH;
    if (woH * wiH >= 0.0f || std::fabs(sd) <= 1.0e-6f) return 0.0f;
    const float nh = Clampf(Dot(n, h), 0.0f, 1.0f);
    const float pdfWh = GgxD(nh, r) * nh;
    const float dwh = std::fabs((eta * eta * wiH) / Sq(sd));
    return pdfWh * dwh;
}
inline V3 EmittedRadiance(const Mat& m) {  // :1722-1727, :486-490
    return {std::max(m.emission_color[0] * m.emission_strength, 0.0f),
            std::max(m.emission_color[1] * m.emission_strength, 0.0f),
            std::max(m.emission_color[2] * m.emission_strength, 0.0f)};
}
// SampleEmissiveTriangleLight (:1443-1460): first entry whose cumulative
// weight is not below the target, else the last.
const SceneData::Emissive* SampleEmitter(const SceneData& s, float u) {
    if (s.emissive.empty() || s.emissiveSum <= 0.0f) return nullptr;
    const float target = Clampf(u, 0.0f, 0.99999994f) * s.emissiveSum;
    size_t lo = 0, hi = s.emissive.size();
    while (lo < hi) {
        const size_t mid = (lo + hi) / 2;
        if (s.emissive[mid].cumulative < target) lo = mid + 1; else hi = mid;
    }
    return lo == s.emissive.size() ? &s.emissive.back() : &s.emissive[lo];
}
// EmissiveTrianglePdf (:1475-1495) of global triangle `gid`.
float EmitterPdf(const SceneData& s, uint32_t gid, const V3& origin, const V3& position) {
    const int32_t k = s.emissiveOf[gid];
    if (k < 0 || s.emissive[k].area <= 0.0f || s.emissiveSum <= 0.0f) return 0.0f;
    const SceneData::Emissive& e = s.emissive[k];
    const V3 to = position - origin;
    const float d2 = Dot(to, to);
    if (d2 <= 1.0e-10f) return 0.0f;
    const V3 ld = Normalize(to);
    const float cosL = std::max(std::fabs(Dot(e.ng, ld * -1.0f)), 1.0e-6f);
    const float sel = e.weight / s.emissiveSum;
    const float areaPdf = sel / e.area;
    return areaPdf * d2 / cosL;
}


// ---------------------------------------------------------------------------
// Lights (CpuPathTracer.cpp:315-384, 1497-1509)
// ---------------------------------------------------------------------------
inline V3 WorldToLight(const Dome& d, const V3& v) {
    return Normalize({Dot(v, d.right), Dot(v, d.up), Dot(v, d.forward)});
}
inline V3 LightToWorld(const Dome& d, const V3& v) { return Normalize(d.right * v.x + d.up * v.y + d.forward * v.z); }
inline V3 DomeRadiance(const Dome& d, const V3& dir) {
    if (d.env) return d.env->Evaluate(WorldToLight(d, dir)) * d.radiance;
    return d.radiance;
}
V3 EnvRadiance(const SceneData& s, const V3& dir) {
    if (!s.domes.empty()) {
        V3 r{};
        for (const Dome& d : s.domes) r = r + DomeRadiance(d, dir);
        return r;
    }
    const float t = Clampf(dir.y * 0.5f + 0.5f, 0.0f, 1.0f);
    return Lerp(s.envBottom, s.envTop, t);
}
inline float DomePdf(const Dome& d, const V3& dir) {
    if (d.env) return d.env->Pdf(WorldToLight(d, dir));
    return kInvFourPi;
}
bool SampleDome(const Dome& d, const V2& u, V3* dir, V3* rad, float* pdf, bool useAlias) {
    V3 ld{};
    float lp = 0.0f;
    V3 lr{};
    if (d.env) {
        lr = d.env->Sample(u, &ld, &lp, useAlias);
    } else {
        const float y = 1.0f - 2.0f * u.y;
        const float r = std::sqrt(std::max(0.0f, 1.0f - y * y));
        const float phi = 2.0f * kPi * u.x;
        ld = {std::sin(phi) * r, y, std::cos(phi) * r};
        lp = kInvFourPi;
        lr = {1.0f, 1.0f, 1.0f};
    }
    if (lp <= 0.0f) return false;
    *dir = LightToWorld(d, ld);
    *rad = lr * d.radiance;
    *pdf = lp;
    return true;
}

struct PathResult {
    V3 radiance, albedo, normal;
    float depth = std::numeric_limits<float>::infinity();
};

struct Tracer {
    const SceneData& s;
    uint32_t flags;
    bool brute = false;

    bool Intersect(const Ray& r, SurfaceHit* out) const {
        Hit h;
        const bool ok = brute ? ClosestBrute(s, r, &h) : Closest(s, r, &h);
        if (!ok) return false;
        *out = MakeSurface(s, r, h);
        return true;
    }
    bool Blocked(const V3& o, const V3& d, float maxDist) const {
        return brute ? OccludedBrute(s, o, d, maxDist) : Occluded(s, o, d, maxDist);
    }
    V3 Clamp24(const V3& v) const { return (flags & SHIRO_RENDER_NO_CLAMP) ? v : ClampMax(v, kDirectSampleClamp); }
    V3 Clamp12(const V3& v) const { return (flags & SHIRO_RENDER_NO_CLAMP) ? v : ClampMax(v, kThroughputClamp); }

    // DirectLighting (CpuPathTracer.cpp:1511-1631).
    V3 Direct(const ShiroSettingsDesc& st, const SurfaceHit& hit, const V3& n, const V3& cn, const Mat& m,
              const V3& view, const Sampler& smp, uint32_t depth) const {
        V3 out{};
        const V3 origin = hit.position + n * kRayEpsilon;
        for (const Distant& l : s.distant) {
            const V3 ld = Normalize(l.direction * -1.0f);
            const float nl = Clampf(Dot(n, ld), 0.0f, 1.0f);
            if (nl <= 0.0f || Blocked(origin, ld, FLT_MAX)) continue;
            out = out + Clamp24(Bsdf(m, n, cn, view, ld) * l.radiance * nl);
        }
        const uint32_t spl = std::max(1u, st.dome_light_samples);
        for (size_t li = 0; li < s.domes.size(); ++li) {
            V3 acc{};
            for (uint32_t k = 0; k < spl; ++k) {
                const uint32_t dim = kDirectDimBase + depth * kDirectDepthStride +
                                     static_cast<uint32_t>(li) * kDirectLightStride + k * kDirectSampleStride;
                V3 ld, lr;
                float lp = 0.0f;
                if (!SampleDome(s.domes[li], smp.Next2D(dim), &ld, &lr, &lp, !(flags & SHIRO_RENDER_ENV_CDF)) ||
                    lp <= 0.0f)
                    continue;
                const float nl = Clampf(Dot(n, ld), 0.0f, 1.0f);
                if (nl <= 0.0f || Blocked(origin, ld, FLT_MAX)) continue;
                const float bp = BsdfPdf(m, n, cn, view, ld);
                const float mis = Power(lp, bp);
                acc = acc + Clamp24(Bsdf(m, n, cn, view, ld) * lr * (nl * mis / lp));
            }
            out = out + acc / static_cast<float>(spl);
        }
        // one emissive-triangle sample (:1578-1628)
        if (!s.emissive.empty() && s.emissiveSum > 0.0f) {
            const uint32_t db = kEmissiveDimBase + depth * kEmissiveDepthStride;
            const SceneData::Emissive* e = SampleEmitter(s, smp.Next1D(db + 0u));
            if (e && e->gid != hit.gid) {
                const MeshData& md = s.meshes[e->mesh];
                const V2 u = smp.Next2D(db + 1u);
                const float su = std::sqrt(Clampf(u.x, 0.0f, 1.0f));  // UniformTriangleBarycentrics, :240-253
                const float b0 = 1.0f - su;
                const float b1 = Clampf(u.y, 0.0f, 1.0f) * su;
                const float b2 = 1.0f - b0 - b1;
                const V3 p = md.pos[md.idx[3 * e->prim]] * b0 + md.pos[md.idx[3 * e->prim + 1]] * b1 +
                             md.pos[md.idx[3 * e->prim + 2]] * b2;  // TrianglePoint, :224-238
                const V3 to = p - hit.position;
                const float d2 = Dot(to, to);
                if (d2 > 1.0e-10f) {
                    const float dist = std::sqrt(d2);
                    const V3 ld = to / dist;
                    const float nl = Clampf(Dot(n, ld), 0.0f, 1.0f);
                    const float cosL = std::fabs(Dot(e->ng, ld * -1.0f));
                    if (nl > 0.0f && cosL > 0.0f &&
                        !Blocked(origin, ld, std::max(dist - 2.0f * kRayEpsilon, kRayEpsilon))) {
                        const float sel = e->weight / s.emissiveSum;
                        const float areaPdf = sel / std::max(e->area, 1.0e-6f);
                        const float lp = areaPdf * d2 / std::max(cosL, 1.0e-6f);
                        if (lp > 0.0f) {
                            const float bp = BsdfPdf(m, n, cn, view, ld);
                            const float mis = Power(lp, bp);
                            out = out + Clamp24(Bsdf(m, n, cn, view, ld) * e->radiance * (nl * mis / lp));
                        }
                    }
                }
            }
        }
        return out;
    }

    // TracePath (CpuPathTracer.cpp:1650-2017); the path guide is empty in
    // the first batch of a scene (:2054-2062) and is not restated.
    PathResult Trace(const ShiroSettingsDesc& st, Ray ray, const Sampler& smp) const {
        enum Bounce { kNone, kDiffuse, kReflective, kTransmission };
        PathResult res;
        V3 T{1.0f, 1.0f, 1.0f};
        uint32_t diffDepth = 0, specDepth = 0;
        Bounce prevType = kNone;
        bool prevDelta = true;
        float prevPdf = 0.0f;
        bool inside = false, mediumActive = false;
        V3 extinction{};
        for (uint32_t depth = 0; depth < st.max_depth; ++depth) {
            const uint32_t base = depth * kPathDimStride;
            SurfaceHit hit;
            if (!Intersect(ray, &hit)) {
                if (depth > 0 || st.background_visible) {
                    const V3 env = EnvRadiance(s, ray.d);
                    V3 delta;
                    if (s.domes.empty() || depth == 0 || prevDelta || prevType == kTransmission) {
                        delta = T * env;
                    } else {
                        float sum = 0.0f;
                        for (const Dome& d : s.domes) {
                            const float p = DomePdf(d, ray.d);
                            sum += p * p;
                        }
                        const float b2 = prevPdf * prevPdf;
                        const float mis = b2 / std::max(b2 + sum, 1.0e-6f);
                        delta = T * env * mis;
                    }
                    res.radiance = res.radiance + delta;
                }
                break;
            }
            if (mediumActive) T = T * MediumAttenuation(extinction, hit.t);
            const Mat& m = s.materials[hit.material];
            const bool front = Dot(hit.ng, ray.d) < 0.0f;
            const V3 ng = front ? hit.ng : hit.ng * -1.0f;
            V3 sb = front ? hit.ns : hit.ns * -1.0f;
            if (Dot(sb, ng) < 0.0f) sb = sb * -1.0f;
            V3 n = ResolveNormal(m, sb, false);
            if (Dot(n, ng) < 0.0f) n = n * -1.0f;
            const V3 cn = ResolveNormal(m, n, true);
            const V3 view = ray.d * -1.0f;
            const float opacity = Clampf(m.opacity, 0.0f, 1.0f);
            if (opacity < 0.999f) {  // :1713-1720
                if (smp.Next1D(base + 0u) > opacity) {
                    ray.o = hit.position + ray.d * kRayEpsilon;
                    continue;
                }
                T = T / std::max(opacity, 1.0e-4f);
            }
            if (depth == 0) {
                res.albedo = DiffuseColor(m);
                res.normal = n * 0.5f + V3{0.5f, 0.5f, 0.5f};
                res.depth = hit.t;
            }
            if (m.emission_strength > 0.0f) {  // :1728-1744
                const V3 le = EmittedRadiance(m);
                V3 delta;
                if (depth == 0 || prevDelta || prevType == kTransmission) {
                    delta = T * le;
                } else {
                    const float lp = EmitterPdf(s, hit.gid, ray.o, hit.position);
                    const float mis = lp > 0.0f ? Power(prevPdf, lp) : 1.0f;
                    delta = T * le * mis;
                }
                res.radiance = res.radiance + delta;
            }
            res.radiance = res.radiance + T * Direct(st, hit, n, cn, m, view, smp, depth);

            const float dw = DiffuseWeight(m), cw = CoatWeight(m), rawTw = TransmissionWeight(m);
            float bw = SpecWeight(m);
            float tw = rawTw;
            if (rawTw > 0.0f) {  // :1763-1772
                const float etaI = inside ? std::max(m.ior, 1.0f) : 1.0f;
                const float etaT = inside ? 1.0f : std::max(m.ior, 1.0f);
                const float refl = FresnelDielectric(std::fabs(Dot(ng, view)), etaI, etaT);
                const float pass = m.thin_walled ? ThinPaneTransmittance(refl) : (1.0f - refl);
                tw = rawTw * pass;
                bw += rawTw * (1.0f - pass);
            }
            const float rw = dw + bw + cw;
            const float total = rw + tw;
            if (total <= 0.0f) break;
            const float sel = smp.Next1D(base + 1u) * total;
            const V2 ds = smp.Next2D(base + 2u);
            V3 next{}, f{};
            float pdf = 1.0f;
            Bounce type = kDiffuse;
            bool delta = false;
            bool chooseT = false, chooseB = false, chooseC = false;
            if (sel < tw) {
                chooseT = true;
            } else {
                const float rs = sel - tw;
                if (rs < dw) {
                } else if (rs < dw + bw) {
                    chooseB = true;
                } else {
                    chooseC = true;
                }
            }
            if (chooseT) {  // :1811-1925
                if (specDepth >= st.specular_depth) break;
                ++specDepth;
                type = kTransmission;
                const float tp = std::max(tw / total, 1.0e-6f);
                const float tr = m.thin_walled
                                     ? 0.0f
                                     : RoughnessFor(TransmissionRoughness(m), m.specular_anisotropy, m.specular_rotation);
                if (m.thin_walled) {
                    next = ray.d;
                    const float refl = FresnelDielectric(std::fabs(Dot(ng, view)), 1.0f, std::max(m.ior, 1.0f));
                    const float pane = ThinPaneTransmittance(refl);
                    const V3 scale = TransmissionSurfaceTint(m) * CoatTransmissionScale(m, cn, view, next) *
                                     (Clampf(m.transmission, 0.0f, 1.0f) * (1.0f - Clampf(m.metallic, 0.0f, 1.0f)));
                    const float ac = std::max(std::fabs(Dot(ng, next)), 1.0e-4f);
                    f = scale * pane / ac;
                    pdf = tp;
                    delta = true;
                } else {
                    const float etaI = inside ? std::max(m.ior, 1.0f) : 1.0f;
                    const float etaT = inside ? 1.0f : std::max(m.ior, 1.0f);
                    const float ratio = etaI / etaT;
                    const float rel = etaT / std::max(etaI, 1.0f);
                    const float refl = FresnelDielectric(std::fabs(Dot(ng, view)), etaI, etaT);
                    const float mt = Clampf(m.transmission, 0.0f, 1.0f) * (1.0f - Clampf(m.metallic, 0.0f, 1.0f));
                    if (tr <= kDeltaRoughness) {
                        if (!Refract(ray.d, ng, ratio, &next)) {
                            next = Normalize(Reflect(ray.d, ng));
                            if (rw <= 0.0f) break;
                            f = Bsdf(m, n, cn, view, next);
                            pdf = std::max((rw / total) * BsdfPdf(m, n, cn, view, next), 1.0e-6f);
                            type = kReflective;
                            delta = true;
                            chooseT = false;
                            chooseB = true;
                        } else {
                            const V3 scale = TransmissionSurfaceTint(m) * CoatTransmissionScale(m, cn, view, next) * mt;
                            const float ac = std::max(std::fabs(Dot(ng, next)), 1.0e-4f);
                            const float transport = 1.0f / std::max(rel * rel, 1.0e-6f);
                            f = scale * (1.0f - refl) * transport / ac;
                            pdf = tp;
                            inside = !inside;
                            if (inside) {
                                extinction = MediumExtinction(m);
                                mediumActive = m.transmission_depth > 0.0f ||
                                               MaxComponent(L3(m.transmission_scatter)) > 0.0f;
                            } else {
                                mediumActive = false;
                            }
                            delta = true;
                        }
                    } else {
                        V3 mn = GgxHalf(ng, ds, tr);
                        if (Dot(mn, view) < 0.0f) mn = mn * -1.0f;
                        if (!Refract(ray.d, mn, ratio, &next)) {
                            next = Normalize(Reflect(ray.d, mn));
                            if (rw <= 0.0f) break;
                            f = Bsdf(m, n, cn, view, next);
                            pdf = std::max((rw / total) * BsdfPdf(m, n, cn, view, next), 1.0e-6f);
                            type = kReflective;
                            delta = false;
                            chooseT = false;
                            chooseB = true;
                        } else {
                            f = TransmissionLobe(m, ng, cn, view, next, etaI, etaT, tr);
                            pdf = std::max(tp * TransmissionPdf(ng, view, next, etaT / etaI, tr), 1.0e-6f);
                            inside = !inside;
                            if (inside) {
                                extinction = MediumExtinction(m);
                                mediumActive = m.transmission_depth > 0.0f ||
                                               MaxComponent(L3(m.transmission_scatter)) > 0.0f;
                            } else {
                                mediumActive = false;
                            }
                            delta = tr <= kDeltaRoughness;
                        }
                    }
                }
            } else if (chooseB || chooseC) {
                if (specDepth >= st.specular_depth) break;
                ++specDepth;
                type = kReflective;
                const V3 sn = chooseC ? cn : n;
                const float sr = chooseC ? RoughnessFor(m.coat_roughness, m.coat_anisotropy, m.coat_rotation)
                                         : RoughnessFor(BaseRoughness(m), m.specular_anisotropy, m.specular_rotation);
                const V3 h = GgxHalf(sn, ds, sr);
                next = Normalize(Reflect(ray.d, h));
                const float rc = Clampf(Dot(sn, next), 0.0f, 1.0f);
                if (rc <= 0.0f) break;
                pdf = std::max((rw / total) * BsdfPdf(m, n, cn, view, next), 1.0e-6f);
                f = Bsdf(m, n, cn, view, next);
                delta = sr <= kDeltaRoughness;
            } else {
                if (diffDepth >= st.diffuse_depth) break;
                ++diffDepth;
                next = CosineHemisphere(n, ds);
                const float cpdf = Clampf(Dot(n, next), 0.0f, 1.0f) * kInvPi;
                pdf = std::max((rw / total) * (1.0f * cpdf + 0.0f * 0.0f), 1.0e-6f);
                f = Bsdf(m, n, cn, view, next);
            }
            const float cosT = chooseT ? std::max(std::fabs(Dot(ng, next)), 1.0e-4f) : Clampf(Dot(n, next), 0.0f, 1.0f);
            if (cosT <= 0.0f) break;
            T = Clamp12(T * f * (cosT / pdf));
            const V3 rn = chooseT ? ng : n;
            const float off = Dot(rn, next) >= 0.0f ? 1.0f : -1.0f;
            ray.o = hit.position + rn * (kRayEpsilon * off);
            ray.d = next;
            prevType = type;
            prevDelta = delta;
            prevPdf = pdf;
            if (depth >= 2) {
                const float cp = Clampf(MaxComponent(T), 0.05f, 0.95f);
                if (smp.Next1D(base + 4u) > cp) break;
                T = T / cp;
            }
        }
        return res;
    }
};

// GenerateCameraRay (CpuPathTracer.cpp:1633-1648).
Ray CameraRay(const ShiroCameraDesc& c, const ShiroSettingsDesc& st, uint32_t x, uint32_t y, const V2& s) {
    const float fx = ((static_cast<float>(x) + s.x) / static_cast<float>(st.width)) * 2.0f - 1.0f;
    const float fy = ((static_cast<float>(y) + s.y) / static_cast<float>(st.height)) * 2.0f - 1.0f;
    const float th = std::tan(c.vertical_fov_degrees * 0.5f * kPi / 180.0f);
    const V3 dir = L3(c.forward) + L3(c.right) * (fx * c.aspect_ratio * th) + L3(c.up) * (fy * th);
    Ray r;
    r.o = L3(c.position);
    r.d = Normalize(dir);
    return r;
}

// Every material is handled (transmission, media, opacity, emitters); only
// the progressive path guide, empty in a scene's first batch, is not.
bool Supported(const ShiroSceneDesc& d) { return d.material_count == 0 || d.materials != nullptr; }

int Convert(const ShiroSceneDesc& d, SceneData* s) {
    if (!Supported(d)) return SHIRO_ERR_UNSUPPORTED_SCENE;
    s->materials.assign(d.materials, d.materials + d.material_count);
    s->materials.push_back(DefaultMaterial());
    const uint32_t defaultMat = d.material_count;
    for (uint32_t i = 0; i < d.mesh_count; ++i) {
        const ShiroMeshDesc& md = d.meshes[i];
        MeshData m;
        m.pos.resize(md.vertex_count);
        for (uint32_t v = 0; v < md.vertex_count; ++v) m.pos[v] = L3(md.positions + 3 * v);
        if (md.normals) {
            m.nrm.resize(md.normal_count);
            for (uint32_t v = 0; v < md.normal_count; ++v) m.nrm[v] = L3(md.normals + 3 * v);
        }
        m.idx.assign(md.indices, md.indices + md.index_count);
        for (uint32_t v : m.idx)
            if (v >= md.vertex_count) return SHIRO_ERR_INVALID_ARGUMENT;
        m.material = md.material_index < d.material_count ? md.material_index : defaultMat;
        const uint32_t tris = md.index_count / 3u;
        for (uint32_t t = 0; t < tris; ++t) {
            const V3 p0 = m.pos[m.idx[3 * t]], p1 = m.pos[m.idx[3 * t + 1]], p2 = m.pos[m.idx[3 * t + 2]];
            s->tv0.push_back(p0);
            s->te1.push_back(p1 - p0);
            s->te2.push_back(p2 - p0);
            s->triMesh.push_back(i);
            s->triPrim.push_back(t);
        }
        s->meshes.push_back(std::move(m));
    }
    for (uint32_t i = 0; i < d.distant_light_count; ++i)
        s->distant.push_back({L3(d.distant_lights[i].direction), L3(d.distant_lights[i].radiance)});
    for (uint32_t i = 0; i < d.dome_light_count; ++i) {
        const ShiroDomeLightDesc& dl = d.dome_lights[i];
        Dome dm{L3(dl.radiance), L3(dl.right), L3(dl.up), L3(dl.forward), nullptr};
        if (dl.env_pixels && dl.env_width && dl.env_height) dm.env = MakeEnv(dl.env_width, dl.env_height, dl.env_pixels, dl.layout);
        s->domes.push_back(dm);
    }
    s->envTop = L3(d.environment_top);
    s->envBottom = L3(d.environment_bottom);
    BuildBvh(*s);
    // emissive triangles in mesh / primitive order with float running sums
    // (BuildAccelerationScene, CpuPathTracer.cpp:482-522; TriangleArea :198-222)
    s->emissiveOf.assign(s->triMesh.size(), -1);
    uint32_t gid = 0;
    for (uint32_t i = 0; i < s->meshes.size(); ++i) {
        const MeshData& md = s->meshes[i];
        const uint32_t prims = static_cast<uint32_t>(md.idx.size() / 3u);
        const V3 le = EmittedRadiance(s->materials[md.material]);
        const float w = std::max(0.2126f * le.x + 0.7152f * le.y + 0.0722f * le.z, 0.0f);
        if (md.idx.size() < 3 || md.idx.size() % 3 != 0 || w <= 0.0f) {
            gid += prims;
            continue;
        }
        for (uint32_t t = 0; t < prims; ++t, ++gid) {
            const V3 p0 = md.pos[md.idx[3 * t]], p1 = md.pos[md.idx[3 * t + 1]], p2 = md.pos[md.idx[3 * t + 2]];
            const V3 av = Cross(p1 - p0, p2 - p0);
            const float dbl = Length(av);
            if (dbl <= 1.0e-8f) continue;
            const float area = dbl * 0.5f;
            const float sel = area * w;
            s->emissiveSum += sel;
            s->emissiveOf[gid] = static_cast<int32_t>(s->emissive.size());
            s->emissive.push_back({i, t, gid, area, sel, s->emissiveSum, le, av / dbl});
        }
    }
    return SHIRO_OK;
}

std::atomic<uint32_t> gThreads{0};

uint32_t ThreadCount() {
    const uint32_t hw = std::max(1u, std::thread::hardware_concurrency());
    const uint32_t t = gThreads.load();
    if (t > 0) return std::min(t, 4096u);
    return hw > 1 ? hw - 1 : 1;
}

template <typename F>
void ParallelRows(uint32_t y0, uint32_t y1, F&& fn) {
    std::atomic<uint32_t> next{y0};
    const uint32_t tc = std::max(1u, std::min(ThreadCount(), y1 > y0 ? y1 - y0 : 1u));
    std::vector<std::thread> ws;
    for (uint32_t w = 0; w < tc; ++w) {
        ws.emplace_back([&]() {
            for (;;) {
                const uint32_t y = next.fetch_add(1);
                if (y >= y1) return;
                fn(y);
            }
        });
    }
    for (auto& t : ws) t.join();
}

// One row of pixels (the per-pixel loop of RenderSampleBatch,
// CpuPathTracer.cpp:2093-2137).
void RenderRow(const Tracer& tr, const ShiroRenderDesc& req, uint32_t y, ShiroAovs* out) {
    const ShiroSettingsDesc& st = req.settings;
    {
        for (uint32_t x = 0; x < st.width; ++x) {
            float b[4] = {0, 0, 0, 0};
            V3 alb{}, nrm{};
            float depth = std::numeric_limits<float>::infinity();
            for (uint32_t k = 0; k < req.sample_count; ++k) {
                const Sampler smp{x, y, req.sample_start + k};
                const Ray r = CameraRay(req.camera, st, x, y, smp.Next2D(0));
                const PathResult pr = tr.Trace(st, r, smp);
                b[0] = b[0] + pr.radiance.x;
                b[1] = b[1] + pr.radiance.y;
                b[2] = b[2] + pr.radiance.z;
                b[3] = b[3] + (pr.depth < std::numeric_limits<float>::infinity() ? 1.0f : 0.0f);
                alb = alb + pr.albedo;
                nrm = nrm + pr.normal;
                if (pr.depth < depth) depth = pr.depth;
            }
            const float cnt = static_cast<float>(req.sample_count);
            const float inv = 1.0f / cnt;
            const size_t i = static_cast<size_t>(y) * st.width + x;
            for (int c = 0; c < 4; ++c) out->beauty[4 * i + c] = b[c] / cnt;
            const V3 a = alb * inv, nn = nrm * inv;
            out->albedo[3 * i + 0] = a.x;
            out->albedo[3 * i + 1] = a.y;
            out->albedo[3 * i + 2] = a.z;
            out->normal[3 * i + 0] = nn.x;
            out->normal[3 * i + 1] = nn.y;
            out->normal[3 * i + 2] = nn.z;
            out->depth[i] = depth;
        }
    }
}

int64_t RenderRows(const SceneData& s, const ShiroRenderDesc& req, uint32_t y0, uint32_t y1, ShiroAovs* out,
                   bool brute = false) {
    if (req.sample_count == 0) return 0;
    Tracer tr{s, req.flags, brute};
    ParallelRows(y0, y1, [&](uint32_t y) { RenderRow(tr, req, y, out); });
    return static_cast<int64_t>(y1 - y0) * req.settings.width * req.sample_count;
}

}  // namespace

struct OracleScene {
    SceneData data;
};

extern "C" {

void oracle_set_threads(uint32_t threads) { gThreads.store(threads); }

int oracle_supports_scene(const ShiroSceneDesc* scene) { return scene && Supported(*scene) ? 1 : 0; }

int oracle_sampler(uint32_t n, const uint32_t* px, const uint32_t* py, const uint32_t* index, const uint32_t* branch,
                   float* out2) {
    for (uint32_t i = 0; i < n; ++i) {
        const V2 v = Sampler{px[i], py[i], index[i]}.Next2D(branch[i]);
        out2[2 * i] = v.x;
        out2[2 * i + 1] = v.y;
    }
    return 0;
}

int oracle_camera_rays(const ShiroRenderDesc* req, float* origins, float* dirs) {
    const ShiroSettingsDesc& st = req->settings;
    for (uint32_t y = 0; y < st.height; ++y)
        for (uint32_t x = 0; x < st.width; ++x) {
            const Sampler smp{x, y, req->sample_start};
            const Ray r = CameraRay(req->camera, st, x, y, smp.Next2D(0));
            const size_t i = static_cast<size_t>(y) * st.width + x;
            origins[3 * i] = r.o.x;
            origins[3 * i + 1] = r.o.y;
            origins[3 * i + 2] = r.o.z;
            dirs[3 * i] = r.d.x;
            dirs[3 * i + 1] = r.d.y;
            dirs[3 * i + 2] = r.d.z;
        }
    return 0;
}

static int TraceRaysImpl(const ShiroSceneDesc* sd, const float* o, const float* d, const float* tmax, uint32_t n,
                         uint32_t* prim, float* t, uint32_t* occ, bool brute) {
    // Geometry only: unsupported materials do not matter for ray queries.
    SceneData s;
    ShiroSceneDesc geo = *sd;
    geo.material_count = 0;
    const int rc = Convert(geo, &s);
    if (rc != SHIRO_OK) return rc;
    const uint32_t rows = (n + 1023u) / 1024u;
    ParallelRows(0, rows, [&](uint32_t r) {
        for (uint32_t i = r * 1024u; i < std::min(n, (r + 1u) * 1024u); ++i) {
            Ray ray;
            ray.o = L3(o + 3 * i);
            ray.d = L3(d + 3 * i);
            Hit h;
            const bool ok = brute ? ClosestBrute(s, ray, &h) : Closest(s, ray, &h);
            prim[i] = ok ? h.gid : 0xffffffffu;
            t[i] = ok ? h.t : FLT_MAX;
            occ[i] = (brute ? OccludedBrute(s, ray.o, ray.d, tmax[i]) : Occluded(s, ray.o, ray.d, tmax[i])) ? 1u : 0u;
        }
    });
    return 0;
}

int oracle_trace_rays(const ShiroSceneDesc* sd, const float* o, const float* d, const float* tmax, uint32_t n,
                      uint32_t* prim, float* t, uint32_t* occ) {
    return TraceRaysImpl(sd, o, d, tmax, n, prim, t, occ, false);
}

int oracle_trace_rays_bruteforce(const ShiroSceneDesc* sd, const float* o, const float* d, const float* tmax,
                                 uint32_t n, uint32_t* prim, float* t, uint32_t* occ) {
    return TraceRaysImpl(sd, o, d, tmax, n, prim, t, occ, true);
}

int oracle_primary_hits(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, uint32_t* prim, float* t) {
    SceneData s;
    ShiroSceneDesc geo = *sd;
    geo.material_count = 0;
    const int rc = Convert(geo, &s);
    if (rc != SHIRO_OK) return rc;
    const ShiroSettingsDesc& st = req->settings;
    ParallelRows(0, st.height, [&](uint32_t y) {
        for (uint32_t x = 0; x < st.width; ++x) {
            const Sampler smp{x, y, req->sample_start};
            const Ray r = CameraRay(req->camera, st, x, y, smp.Next2D(0));
            Hit h;
            const size_t i = static_cast<size_t>(y) * st.width + x;
            const bool ok = Closest(s, r, &h);
            prim[i] = ok ? h.gid : 0xffffffffu;
            t[i] = ok ? h.t : FLT_MAX;
        }
    });
    return 0;
}

int oracle_bsdf(const ShiroMaterialDesc* md, uint32_t n, const float* normals, const float* views,
                const float* lights, float* f_out, float* pdf_out, float* w_out) {
    const Mat& m = *md;
    for (uint32_t i = 0; i < n; ++i) {
        const V3 nn = L3(normals + 3 * i);
        const V3 sn = ResolveNormal(m, nn, false);
        const V3 cn = ResolveNormal(m, sn, true);
        const V3 f = Bsdf(m, sn, cn, L3(views + 3 * i), L3(lights + 3 * i));
        f_out[3 * i] = f.x;
        f_out[3 * i + 1] = f.y;
        f_out[3 * i + 2] = f.z;
        pdf_out[i] = BsdfPdf(m, sn, cn, L3(views + 3 * i), L3(lights + 3 * i));
    }
    w_out[0] = DiffuseWeight(m);
    w_out[1] = SpecWeight(m);
    w_out[2] = CoatWeight(m);
    w_out[3] = TransmissionWeight(m);
    const V3 dc = DiffuseColor(m);
    w_out[4] = dc.x;
    w_out[5] = dc.y;
    w_out[6] = dc.z;
    return 0;
}

int oracle_env_tables(uint32_t w, uint32_t h, const float* rgb, float* row_cdf, float* cond_cdf) {
    auto e = MakeEnv(w, h, rgb, SHIRO_ENV_LAYOUT_LATLONG);
    std::copy(e->rowCdf.begin(), e->rowCdf.end(), row_cdf);
    std::copy(e->condCdf.begin(), e->condCdf.end(), cond_cdf);
    return 0;
}

// The GPU backend's alias table over the reference masses (its own sampler;
// the reference has none), built by the sequential sweep the backend's
// parallel construction must reproduce: weights floor(mass * 2^60), buckets
// of C = ceil(T / n) units with the slack on the first heaviest texel; lights
// are topped up from the current heavy while it holds more than C, otherwise
// the heavy closes its own bucket and draws the rest from the next heavy.
int oracle_env_alias(uint32_t w, uint32_t h, const float* rgb, uint32_t* threshold_bits, uint32_t* alias) {
    auto e = MakeEnv(w, h, rgb, SHIRO_ENV_LAYOUT_LATLONG);
    const uint64_t n = static_cast<uint64_t>(w) * h;
    if (n == 0 || e->rowCdf.empty()) return SHIRO_ERR_INVALID_ARGUMENT;
    using u64 = unsigned long long;
    std::vector<u64> q(n);
    u64 total = 0, best = 0;
    uint64_t imax = 0;
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            const size_t i = static_cast<size_t>(y) * w + x;
            const float rowMass = e->rowCdf[y + 1u] - e->rowCdf[y];
            const size_t off = static_cast<size_t>(y) * (w + 1u);
            const float colMass = e->condCdf[off + x + 1u] - e->condCdf[off + x];
            const float m = rowMass * colMass;
            q[i] = m > 0.0f ? static_cast<u64>(static_cast<double>(m) * 1152921504606846976.0) : 0ull;
            total += q[i];
            if (q[i] > best) {
                best = q[i];
                imax = i;
            }
        }
    auto put = [&](uint64_t i, u64 units, u64 cap, uint64_t to) {
        const float t = static_cast<float>(static_cast<double>(units) / static_cast<double>(cap));
        std::memcpy(&threshold_bits[i], &t, 4);
        alias[i] = static_cast<uint32_t>(to);
    };
    if (total == 0) {
        for (uint64_t i = 0; i < n; ++i) put(i, 1, 1, i);
        return 0;
    }
    const u64 cap = (total + n - 1u) / n;
    q[imax] += cap * n - total;
    std::vector<uint64_t> lights, heavies;
    for (uint64_t i = 0; i < n; ++i) (q[i] < cap ? lights : heavies).push_back(i);
    size_t i = 0, j = 0;
    u64 rest = q[heavies[0]];  // units the current heavy still holds
    while (i < lights.size()) {
        if (rest > cap || j + 1 == heavies.size()) {
            put(lights[i], q[lights[i]], cap, heavies[j]);
            rest -= cap - q[lights[i]];
            ++i;
        } else {
            put(heavies[j], rest, cap, heavies[j + 1]);
            rest = q[heavies[j + 1]] - (cap - rest);
            ++j;
        }
    }
    for (; j + 1 < heavies.size(); ++j) {
        put(heavies[j], rest, cap, heavies[j + 1]);
        rest = q[heavies[j + 1]] - (cap - rest);
    }
    put(heavies[j], 1, 1, heavies[j]);
    return 0;
}

int oracle_env_query(uint32_t w, uint32_t h, const float* rgb, uint32_t layout, uint32_t n, const float* u2,
                     const float* dirs, float* sdir, float* spdf, float* srgb, float* pdf, float* rgb_out) {
    auto e = MakeEnv(w, h, rgb, layout);
    for (uint32_t i = 0; i < n; ++i) {
        V3 d;
        float p = 0.0f;
        const V3 c = e->Sample({u2[2 * i], u2[2 * i + 1]}, &d, &p);
        sdir[3 * i] = d.x;
        sdir[3 * i + 1] = d.y;
        sdir[3 * i + 2] = d.z;
        spdf[i] = p;
        srgb[3 * i] = c.x;
        srgb[3 * i + 1] = c.y;
        srgb[3 * i + 2] = c.z;
        const V3 q = L3(dirs + 3 * i);
        pdf[i] = e->Pdf(q);
        const V3 ev = e->Evaluate(q);
        rgb_out[3 * i] = ev.x;
        rgb_out[3 * i + 1] = ev.y;
        rgb_out[3 * i + 2] = ev.z;
    }
    return 0;
}

int oracle_render(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, ShiroAovs* out) {
    SceneData s;
    const int rc = Convert(*sd, &s);
    if (rc != SHIRO_OK) return rc;
    RenderRows(s, *req, 0, req->settings.height, out);
    return 0;
}

static int RenderPathsImpl(const SceneData& s, const ShiroRenderDesc* req, const uint32_t* pixels, uint32_t n,
                           const uint32_t* sample_index, float* out) {
    const ShiroSettingsDesc& st = req->settings;
    Tracer tr{s, req->flags, false};
    const uint32_t rows = (n + 255u) / 256u;
    ParallelRows(0, rows, [&](uint32_t r) {
        for (uint32_t i = r * 256u; i < std::min(n, (r + 1u) * 256u); ++i) {
            const uint32_t x = pixels[i] % st.width, y = pixels[i] / st.width;
            const Sampler smp{x, y, sample_index[i]};
            const Ray ray = CameraRay(req->camera, st, x, y, smp.Next2D(0));
            const PathResult pr = tr.Trace(st, ray, smp);
            float* o = out + 10 * static_cast<size_t>(i);
            o[0] = pr.radiance.x;
            o[1] = pr.radiance.y;
            o[2] = pr.radiance.z;
            o[3] = pr.albedo.x;
            o[4] = pr.albedo.y;
            o[5] = pr.albedo.z;
            o[6] = pr.normal.x;
            o[7] = pr.normal.y;
            o[8] = pr.normal.z;
            o[9] = pr.depth;
        }
    });
    return 0;
}

int oracle_render_paths(const ShiroSceneDesc* sd, const ShiroRenderDesc* req, const uint32_t* pixels, uint32_t n,
                        const uint32_t* sample_index, float* out, void*, void*) {
    SceneData s;
    const int rc = Convert(*sd, &s);
    if (rc != SHIRO_OK) return rc;
    return RenderPathsImpl(s, req, pixels, n, sample_index, out);
}

int oracle_scene_create(const ShiroSceneDesc* sd, OracleScene** out) {
    if (!sd || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    auto* s = new (std::nothrow) OracleScene();
    if (!s) return SHIRO_ERR_OUT_OF_MEMORY;
    const int rc = Convert(*sd, &s->data);
    if (rc != SHIRO_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return SHIRO_OK;
}

void oracle_scene_destroy(OracleScene* s) { delete s; }

int64_t oracle_scene_render_rows(OracleScene* s, const ShiroRenderDesc* req, uint32_t y0, uint32_t y1, ShiroAovs* out) {
    if (!s || !req || !out || y1 > req->settings.height || y0 > y1) return SHIRO_ERR_INVALID_ARGUMENT;
    return RenderRows(s->data, *req, y0, y1, out);
}

// An arbitrary set of rows, rendered in parallel (a sample of a frame).
int64_t oracle_scene_render_row_list(OracleScene* s, const ShiroRenderDesc* req, const uint32_t* rows, uint32_t n,
                                     ShiroAovs* out) {
    if (!s || !req || !out || (n && !rows)) return SHIRO_ERR_INVALID_ARGUMENT;
    for (uint32_t k = 0; k < n; ++k)
        if (rows[k] >= req->settings.height) return SHIRO_ERR_INVALID_ARGUMENT;
    if (req->sample_count == 0) return 0;
    Tracer tr{s->data, req->flags, false};
    ParallelRows(0, n, [&](uint32_t k) { RenderRow(tr, *req, rows[k], out); });
    return static_cast<int64_t>(n) * req->settings.width * req->sample_count;
}

int oracle_scene_render_paths(OracleScene* s, const ShiroRenderDesc* req, const uint32_t* pixels, uint32_t n,
                              const uint32_t* sample_index, float* out) {
    if (!s || !req || (n && (!pixels || !sample_index || !out))) return SHIRO_ERR_INVALID_ARGUMENT;
    const uint64_t px = static_cast<uint64_t>(req->settings.width) * req->settings.height;
    for (uint32_t i = 0; i < n; ++i)
        if (pixels[i] >= px) return SHIRO_ERR_INVALID_ARGUMENT;
    return RenderPathsImpl(s->data, req, pixels, n, sample_index, out);
}

int oracle_scene_set_env_alias(OracleScene* s, uint32_t dome, const uint32_t* threshold_bits, const uint32_t* alias,
                               uint32_t n) {
    if (!s || dome >= s->data.domes.size() || !s->data.domes[dome].env) return SHIRO_ERR_INVALID_ARGUMENT;
    Env& e = *s->data.domes[dome].env;
    if (n != static_cast<uint64_t>(e.w) * e.h || (n && (!threshold_bits || !alias))) return SHIRO_ERR_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < n; ++i)
        if (alias[i] >= n) return SHIRO_ERR_INVALID_ARGUMENT;
    e.aliasThr.assign(threshold_bits, threshold_bits + n);
    e.aliasIdx.assign(alias, alias + n);
    return SHIRO_OK;
}

}  // extern "C"
