// env_tables.cu - a dome texture's importance tables, built on the device.
//
// 1. The reference table (EnvironmentMap::BuildImportanceTable,
//    src/render/EnvironmentMap.cpp:185-236) in the reference's float
//    arithmetic and order: per row a running sum of
//    max(0, luminance) * sin(theta_centre) (one thread per row, so each row's
//    conditional CDF is summed left to right exactly as the reference does),
//    the rows' normalisation, the row CDF (one thread: H additions in order),
//    then the texel masses rowMass * columnMass (LatLongPdf, :302-313).  Only
//    the H per-row sines come from the host, from the same std::sin the
//    reference calls, so the tables equal the reference's bit for bit.
//
// 2. The alias table over those masses (this backend's O(1) sampler; the
//    reference has none), built in exact integer arithmetic:
//      * each mass becomes q_i = floor(mass_i * 2^60); T = sum q_i;
//      * every bucket holds C = ceil(T / n) units; the R = n C - T units of
//        slack go to the heaviest texel (the first of equal ones), which
//        moves its probability by at most n^2 / 2^60 of itself;
//      * texels below C are "light", the others "heavy"; each light bucket is
//        topped up from the heavies in order, and a heavy whose remainder
//        drops to C or below closes its own bucket and takes the rest from
//        the next heavy.  In sequence this is a merge of two sorted lists, the
//        lights' deficit prefix sums LD(i) and the heavies' excess prefix sums
//        HE(j): light i is topped up by the first heavy j with HE(j+1) > LD(i),
//        and heavy j closes after the LD(i) < HE(j+1) lights.  Both are found
//        by binary search, so every bucket is filled independently, in
//        parallel, with the same integers a sequential sweep produces;
//      * threshold = own units / C (rounded once, through double, to float).
//    All sums are integers, so the result does not depend on the order the
//    GPU forms them in (the oracle's sequential sweep checks it bit for bit).
#include <cub/cub.cuh>

#include <cmath>
#include <vector>

#include "context.h"
#include "env.cuh"

namespace shiro_gpu {

namespace {

using u64 = unsigned long long;
constexpr double kMassScale = 1152921504606846976.0;  // 2^60

inline unsigned grid_of(uint64_t n, unsigned b) { return static_cast<unsigned>((n + b - 1) / b); }

// Row sums and unnormalised conditional CDFs, one thread per row.
__global__ void k_env_rows(const float4* __restrict__ tex, const float* __restrict__ sines, uint32_t w, uint32_t h,
                           float* __restrict__ cond, float* __restrict__ rowSum) {
    const uint32_t y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= h) return;
    const float sinT = sines[y];
    const size_t off = static_cast<size_t>(y) * (w + 1u);
    const float4* t = tex + static_cast<size_t>(y) * w;
    float row = 0.0f;
    cond[off] = 0.0f;
    for (uint32_t x = 0; x < w; ++x) {
        const float4 c = t[x];
        const float lum = c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f;
        row += (0.0f < lum ? lum : 0.0f) * sinT;  // std::max(0.0f, lum)
        cond[off + x + 1u] = row;
    }
    rowSum[y] = row;
}

__global__ void k_env_cond_normalize(float* __restrict__ cond, const float* __restrict__ rowSum, uint32_t w,
                                     uint32_t h) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i >= static_cast<uint64_t>(h) * w) return;
    const uint32_t y = static_cast<uint32_t>(i / w), x = static_cast<uint32_t>(i - static_cast<uint64_t>(y) * w) + 1u;
    const float row = rowSum[y];
    float& c = cond[static_cast<size_t>(y) * (w + 1u) + x];
    c = row > 0.0f ? c / row : static_cast<float>(x) / static_cast<float>(w);
}

// Row CDF: H additions in row order (a row without weight counts 1), then
// the normalisation - one thread, as the reference's loop.
__global__ void k_env_row_cdf(const float* __restrict__ rowSum, uint32_t h, float* __restrict__ rowCdf) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float total = 0.0f;
    rowCdf[0] = 0.0f;
    for (uint32_t y = 0; y < h; ++y) {
        const float r = rowSum[y];
        total += r > 0.0f ? r : 1.0f;
        rowCdf[y + 1u] = total;
    }
    for (uint32_t y = 1; y <= h; ++y)
        rowCdf[y] = total <= 0.0f ? static_cast<float>(y) / static_cast<float>(h) : rowCdf[y] / total;
}

// Texel masses (into texels.w) and their fixed-point weights; stats[0] +=
// weights, stats[1] = max weight.
__global__ void k_env_mass(float4* __restrict__ tex, const float* __restrict__ rowCdf, const float* __restrict__ cond,
                           uint32_t w, uint32_t h, u64* __restrict__ q, u64* __restrict__ stats) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    const uint64_t n = static_cast<uint64_t>(w) * h;
    u64 v = 0;
    if (i < n) {
        const uint32_t y = static_cast<uint32_t>(i / w), x = static_cast<uint32_t>(i - static_cast<uint64_t>(y) * w);
        const float rowMass = rowCdf[y + 1u] - rowCdf[y];
        const size_t off = static_cast<size_t>(y) * (w + 1u);
        const float colMass = cond[off + x + 1u] - cond[off + x];
        const float m = rowMass * colMass;
        tex[i].w = m;
        v = m > 0.0f ? static_cast<u64>(static_cast<double>(m) * kMassScale) : 0ull;
        q[i] = v;
    }
    u64 sum = v, mx = v;
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const u64 other = __shfl_xor_sync(0xffffffffu, mx, o);
        mx = other > mx ? other : mx;
    }
    if ((threadIdx.x & 31u) == 0u) {
        if (sum) atomicAdd(&stats[0], sum);
        atomicMax(&stats[1], mx);
    }
}

// First index holding the largest weight.
__global__ void k_env_first_max(const u64* __restrict__ q, uint64_t n, const u64* __restrict__ stats,
                                unsigned int* __restrict__ first) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i < n && q[i] == stats[1]) atomicMin(first, static_cast<unsigned int>(i));
}

// Bucket weights (slack on the heaviest texel) and the light flags.
__global__ void k_alias_classify(const u64* __restrict__ q, uint64_t n, uint32_t imax, u64 slack, u64 cap,
                                 u64* __restrict__ s, uint32_t* __restrict__ light) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const u64 v = q[i] + (i == imax ? slack : 0ull);
    s[i] = v;
    light[i] = v < cap ? 1u : 0u;
}

// The light and the heavy texels, each in index order (lpos = exclusive
// prefix count of lights).
__global__ void k_alias_split(const uint32_t* __restrict__ light, const uint32_t* __restrict__ lpos, uint64_t n,
                              uint32_t* __restrict__ lights, uint32_t* __restrict__ heavies) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = lpos[i];
    if (light[i]) lights[p] = static_cast<uint32_t>(i);
    else heavies[i - p] = static_cast<uint32_t>(i);
}

// Deficits of the lights and excesses of the heavies, in list order.
__global__ void k_alias_gaps(const u64* __restrict__ s, const uint32_t* __restrict__ lights, uint32_t nL,
                             const uint32_t* __restrict__ heavies, uint32_t nH, u64 cap, u64* __restrict__ d,
                             u64* __restrict__ e) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nL) d[k] = cap - s[lights[k]];
    if (k < nH) e[k] = s[heavies[k]] - cap;
}

__device__ __forceinline__ uint32_t entry_bits(u64 units, u64 cap) {
    return __float_as_uint(static_cast<float>(static_cast<double>(units) / static_cast<double>(cap)));
}

// Light k: own units s / C; topped up by the first heavy j with HEinc[j] > LD[k].
__global__ void k_alias_lights(const u64* __restrict__ s, const uint32_t* __restrict__ lights, uint32_t nL,
                               const uint32_t* __restrict__ heavies, uint32_t nH, const u64* __restrict__ ld,
                               const u64* __restrict__ heInc, u64 cap, uint2* __restrict__ alias) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nL) return;
    const u64 key = ld[k];
    uint32_t lo = 0, hi = nH;  // upper_bound: first j with heInc[j] > key
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (heInc[mid] <= key) lo = mid + 1u; else hi = mid;
    }
    const uint32_t j = lo < nH ? lo : nH - 1u;
    const uint32_t t = lights[k];
    alias[t] = make_uint2(entry_bits(s[t], cap), heavies[j]);
}

// Heavy j (not the last): closes after the lights with LD < HEinc[j], keeping
// w = s + HE(j) - LD(i*) of its own units and taking the rest from heavy j+1.
__global__ void k_alias_heavies(const u64* __restrict__ s, uint32_t nL, const uint32_t* __restrict__ heavies, uint32_t nH,
                                const u64* __restrict__ ld, const u64* __restrict__ heInc, const u64* __restrict__ e,
                                u64 deficitTotal, u64 cap, uint2* __restrict__ alias) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nH) return;
    const uint32_t t = heavies[j];
    if (j + 1u == nH) {  // the last heavy keeps its whole bucket
        alias[t] = make_uint2(__float_as_uint(1.0f), t);
        return;
    }
    const u64 key = heInc[j];
    uint32_t lo = 0, hi = nL;  // lower_bound: first i with ld[i] >= key
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (ld[mid] < key) lo = mid + 1u; else hi = mid;
    }
    const u64 ldStar = lo < nL ? ld[lo] : deficitTotal;
    const u64 own = s[t] + (key - e[j]) - ldStar;
    alias[t] = make_uint2(entry_bits(own, cap), heavies[j + 1u]);
}

__global__ void k_alias_identity(uint2* __restrict__ alias, uint64_t n) {
    const uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    if (i < n) alias[i] = make_uint2(__float_as_uint(1.0f), static_cast<uint32_t>(i));
}

// Scratch of one build, freed when it goes out of scope.
struct Scratch {
    std::vector<void*> blocks;
    ~Scratch() {
        for (void* p : blocks) cudaFree(p);
    }
    template <typename T>
    cudaError_t get(T** p, size_t count) {
        void* v = nullptr;
        const cudaError_t e = cudaMalloc(&v, std::max<size_t>(count * sizeof(T), 16));
        if (e == cudaSuccess) blocks.push_back(v);
        *p = static_cast<T*>(v);
        return e;
    }
};

}  // namespace

#define ENV_CHECK(x)                                   \
    do {                                               \
        const cudaError_t err_ = (x);                  \
        if (err_ != cudaSuccess) return cuda_fail(ctx, err_, "env tables: " #x); \
    } while (0)

int build_env_tables_device(ContextImpl* ctx, DevEnv& d) {
    const uint32_t w = d.w, h = d.h;
    const uint64_t n = static_cast<uint64_t>(w) * h;
    if (n == 0 || !d.latlong) return SHIRO_OK;
    if (n >= (1ull << 31)) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "environment texture too large");
    cudaStream_t st = ctx->stream;
    // per-row sines from the host's std::sin, as the reference evaluates them
    constexpr float kHostPi = 3.14159265358979323846f;
    std::vector<float> sines(h);
    for (uint32_t y = 0; y < h; ++y) {
        const float theta = (static_cast<float>(y) + 0.5f) * kHostPi / static_cast<float>(h);
        sines[y] = std::max(std::sin(theta), 1.0e-6f);
    }
    Scratch sc;
    float *dSin, *rowSum;
    u64 *q, *s, *gapD, *gapE, *ld, *heInc, *stats;
    uint32_t *lightFlag, *lpos, *lights, *heavies;
    unsigned int* first;
    ENV_CHECK(sc.get(&dSin, h));
    ENV_CHECK(sc.get(&rowSum, h));
    ENV_CHECK(sc.get(&q, n));
    ENV_CHECK(sc.get(&s, n));
    ENV_CHECK(sc.get(&gapD, n));
    ENV_CHECK(sc.get(&gapE, n));
    ENV_CHECK(sc.get(&ld, n));
    ENV_CHECK(sc.get(&heInc, n));
    ENV_CHECK(sc.get(&stats, 2));
    ENV_CHECK(sc.get(&lightFlag, n));
    ENV_CHECK(sc.get(&lpos, n));
    ENV_CHECK(sc.get(&lights, n));
    ENV_CHECK(sc.get(&heavies, n));
    ENV_CHECK(sc.get(&first, 1));
    float* rowCdf = const_cast<float*>(d.rowCdf);
    float* cond = const_cast<float*>(d.condCdf);
    float4* tex = const_cast<float4*>(d.texels);
    uint2* alias = const_cast<uint2*>(d.alias);

    // 1. the reference table and the masses
    ENV_CHECK(cudaMemcpyAsync(dSin, sines.data(), h * sizeof(float), cudaMemcpyHostToDevice, st));
    ENV_CHECK(cudaMemsetAsync(stats, 0, 2 * sizeof(u64), st));
    ENV_CHECK(cudaMemsetAsync(first, 0xff, sizeof(unsigned int), st));
    k_env_rows<<<grid_of(h, 128), 128, 0, st>>>(tex, dSin, w, h, cond, rowSum);
    k_env_cond_normalize<<<grid_of(n, 256), 256, 0, st>>>(cond, rowSum, w, h);
    k_env_row_cdf<<<1, 32, 0, st>>>(rowSum, h, rowCdf);
    k_env_mass<<<grid_of(n, 256), 256, 0, st>>>(tex, rowCdf, cond, w, h, q, stats);
    k_env_first_max<<<grid_of(n, 256), 256, 0, st>>>(q, n, stats, first);
    ENV_CHECK(cudaGetLastError());
    u64 hs[2];
    unsigned int imax = 0;
    ENV_CHECK(cudaMemcpyAsync(hs, stats, sizeof(hs), cudaMemcpyDeviceToHost, st));
    ENV_CHECK(cudaMemcpyAsync(&imax, first, sizeof(imax), cudaMemcpyDeviceToHost, st));
    ENV_CHECK(cudaStreamSynchronize(st));
    const u64 total = hs[0];
    if (total == 0) {  // no texel has weight: every bucket keeps itself
        k_alias_identity<<<grid_of(n, 256), 256, 0, st>>>(alias, n);
        ENV_CHECK(cudaGetLastError());
        return SHIRO_OK;
    }
    // 2. the alias table
    const u64 cap = (total + n - 1u) / n;
    const u64 slack = cap * n - total;
    k_alias_classify<<<grid_of(n, 256), 256, 0, st>>>(q, n, imax, slack, cap, s, lightFlag);
    ENV_CHECK(cudaGetLastError());
    size_t tmpBytes = 0, need = 0;
    const int nn = static_cast<int>(n);
    ENV_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, need, lightFlag, lpos, nn, st));
    tmpBytes = std::max(tmpBytes, need);
    ENV_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, need, gapD, ld, nn, st));
    tmpBytes = std::max(tmpBytes, need);
    ENV_CHECK(cub::DeviceScan::InclusiveSum(nullptr, need, gapE, heInc, nn, st));
    tmpBytes = std::max(tmpBytes, need);
    unsigned char* tmp = nullptr;
    ENV_CHECK(sc.get(&tmp, tmpBytes));
    ENV_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, lightFlag, lpos, nn, st));
    k_alias_split<<<grid_of(n, 256), 256, 0, st>>>(lightFlag, lpos, n, lights, heavies);
    ENV_CHECK(cudaGetLastError());
    uint32_t lastPos = 0, lastFlag = 0;
    ENV_CHECK(cudaMemcpyAsync(&lastPos, lpos + (n - 1u), 4, cudaMemcpyDeviceToHost, st));
    ENV_CHECK(cudaMemcpyAsync(&lastFlag, lightFlag + (n - 1u), 4, cudaMemcpyDeviceToHost, st));
    ENV_CHECK(cudaStreamSynchronize(st));
    const uint32_t nL = lastPos + lastFlag, nH = static_cast<uint32_t>(n - nL);
    if (nH == 0 || static_cast<uint64_t>(nL) + nH != n)
        return fail(ctx, SHIRO_ERR_DEVICE_CHECK, "env tables: inconsistent light / heavy split");
    k_alias_gaps<<<grid_of(std::max(nL, nH), 256), 256, 0, st>>>(s, lights, nL, heavies, nH, cap, gapD, gapE);
    ENV_CHECK(cudaGetLastError());
    if (nL) ENV_CHECK(cub::DeviceScan::ExclusiveSum(tmp, tmpBytes, gapD, ld, static_cast<int>(nL), st));
    ENV_CHECK(cub::DeviceScan::InclusiveSum(tmp, tmpBytes, gapE, heInc, static_cast<int>(nH), st));
    // sum of all deficits = sum of all excesses = heInc[nH - 1]
    u64 deficitTotal = 0;
    ENV_CHECK(cudaMemcpyAsync(&deficitTotal, heInc + (nH - 1u), sizeof(u64), cudaMemcpyDeviceToHost, st));
    ENV_CHECK(cudaStreamSynchronize(st));
    if (nL) k_alias_lights<<<grid_of(nL, 256), 256, 0, st>>>(s, lights, nL, heavies, nH, ld, heInc, cap, alias);
    k_alias_heavies<<<grid_of(nH, 256), 256, 0, st>>>(s, nL, heavies, nH, ld, heInc, gapE, deficitTotal, cap, alias);
    ENV_CHECK(cudaGetLastError());
    ENV_CHECK(cudaStreamSynchronize(st));  // the scratch is freed on return
    return SHIRO_OK;
}

}  // namespace shiro_gpu
