// adjoint.cu - the differentiable form (no counterpart in the reference).
//
// Gradients of an image loss with respect to per-material base colour,
// specular roughness and metalness and to the texels of dome light 0's
// environment map, by path replay: every path is traced twice from its QMC
// seed - once by the plain megakernel for its radiance L (its path record),
// once here to push the adjoint radiance dL/dL_path = d_beauty(pixel) / spp
// into the parameters - so no path vertex is stored.
//
// Estimator: the one of integrator.cuh (same sample dimensions, lobe
// choice, MIS, clamps, Russian roulette).  Sampling decisions, pdfs, MIS
// weights, Russian-roulette probabilities and clamp scales are held constant
// (detached); the parameters enter through the BSDF values (continuation and
// light samples) and the environment radiance (light samples and misses):
//   * a light sample's contribution c = s * f * L * w  contributes
//     delta * T * s * (df * L * w + f * dL * w);
//   * a continuation BSDF value f_k scales every later contribution, which
//     is the radiance not yet accounted for, L_rem: delta * L_rem * df_k / f_k;
//   * a miss adds delta * T * mis * dL_env.
// BSDF derivatives come from bsdf_eval_d (forward-mode dual numbers).
//
// shiro_gpu_render_frozen evaluates the same estimator with the sampling
// taken from the scene's parameters and the BSDF / environment values from a
// second parameter set; its central finite differences are exactly the
// quantity the adjoint computes, which is how the adjoint is checked.
#include <algorithm>
#include <cstring>
#include <vector>

#include "adjoint.cuh"
#include "bsdf_diff.cuh"
#include "context.h"
#include "integrator.cuh"

namespace shiro_gpu {

namespace {

// One path of the estimator with sampling from the scene and values from
// (a.evalMats, a.evalEnv).  kGrad = false returns the radiance; kGrad = true
// replays it and accumulates the gradients of delta . radiance, given the
// path's total radiance Ltot.  One out-of-line body serves both passes (the
// flag is a run-time argument): two inlined copies of the whole estimator
// overflowed the instruction cache.
__device__ __noinline__ V3 adj_path(const DevScene& s, const DevRequest& q, const AdjView& a, uint32_t x, uint32_t y,
                                    uint32_t sampleIndex, const V3 delta, const V3 Ltot, float* depthOut,
                                    const bool kGrad) {
    NullCounter ctr;
    const Sampler smp{x, y, sampleIndex};
    PathState ps;
    init_path(q, smp, ps);
    // throughput under the sampling parameters: Russian roulette decides on it
    V3 Ts = ps.T;
    V3 Lrem = Ltot;
    float depth0 = __int_as_float(0x7f800000);
    const bool useCdf = (q.flags & SHIRO_RENDER_ENV_CDF) != 0u;
    for (uint32_t depth = 0; depth < q.maxDepth; ++depth) {
        HitRec h;
        if (!trace_closest(s, ps.ro, ps.rd, &h, ctr)) {
            if (depth > 0 || q.backgroundVisible) {
                const V3 env = env_radiance_eval(s, a, ps.rd);
                float mis = 1.0f;
                if (s.domeCount == 0 || depth == 0 || ps.prevDelta) {
                    ps.radiance = ps.radiance + ps.T * env;
                } else {
                    mis = env_miss_mis(s, ps.prevPdf, ps.rd);
                    ps.radiance = ps.radiance + ps.T * env * mis;
                }
                if (kGrad && a.env0 >= 0) {
                    for (uint32_t i = 0; i < s.domeCount; ++i) {
                        const DevDome& d = s.domes[i];
                        if (d.env != a.env0) continue;
                        const V3 coef = delta * ps.T * d.radiance * mis;
                        add_env_grad(a, a.evalEnv, world_to_light(d, ps.rd), coef);
                    }
                }
            }
            break;
        }
        const Vertex v = make_vertex(s, ps.ro, ps.rd, h);
        // an opacity cut-out the path passes through (no media: transmission
        // is refused) - the hit is not shaded; a partly opaque hit that is
        // shaded scales the throughput by 1 / opacity, the sampling one too
        if (s.extended) {
            if (!enter_hit(s, smp, depth, v, h.t, ps)) continue;
            const float op = sclamp(s.materials[v.hit.material].opacity, 0.0f, 1.0f);
            if (op < 0.999f) Ts = Ts / smax(op, 1.0e-4f);
        }
        const Mat& me = a.evalMats[v.hit.material];
        const Mat& ms = s.materials[v.hit.material];
        // the scene's materials have their BSDF records on the device; values
        // from a second parameter set (frozen renders) build theirs per call
        const float4* rec = bsdf_rec(s, v.hit.material);
        auto evalE = [&](const V3& l) {
            return a.distinctEval ? bsdf_eval(me, v.n, v.cn, v.view, l) : bsdf_eval_rec(rec, ms, v.n, v.cn, v.view, l);
        };
        if (depth == 0) depth0 = h.t;
        if (s.extended) {
            // emitted radiance at this hit: no parameter scales it here, and
            // no later BSDF value does either
            const V3 before = ps.radiance;
            add_emission(s, v, depth, ps);
            if (kGrad) Lrem = Lrem - (ps.radiance - before);
        }
        const V3 origin = shadow_origin(v);
        // light samples, in sum_direct's order
        const V3 dT = delta * ps.T;
        const uint32_t firstEmissive = s.distantCount + s.domeCount * q.domeSamples;
        const V3 direct = sum_direct<true>(s, q, [&](uint32_t k, V3* c) {
            V3 ld, L;
            V3 Ls;  // the radiance under the sampling (scene) parameters: the clamp's scale comes from it
            float w;
            float reach = FLT_MAX;
            int32_t envIdx = -1;
            V3 local{0.0f, 0.0f, 0.0f};
            V3 domeRad{0.0f, 0.0f, 0.0f};
            if (k >= firstEmissive) {  // the emissive-triangle sample (emission is not a parameter)
                float lp, nl;
                if (!emissive_geometry(s, v, smp, depth, &ld, &L, &lp, &nl, &reach)) return false;
                Ls = L;
                const float bp = bsdf_pdf_rec(rec, ms, v.w, v.n, v.cn, v.view, ld);
                w = nl * power_heuristic(lp, bp) / lp;
            } else if (k < s.distantCount) {
                const DevDistant l = s.distant[k];
                ld = normalize(l.direction * -1.0f);
                const float nl = sclamp(dot(v.n, ld), 0.0f, 1.0f);
                if (nl <= 0.0f) return false;
                L = l.radiance;
                Ls = L;
                w = nl;
            } else {
                const uint32_t r = k - s.distantCount;
                const uint32_t li = r / q.domeSamples, j = r - li * q.domeSamples;
                const DevDome& d = s.domes[li];
                const uint32_t dim = kDirectDimBase + depth * kDirectDepthStride + li * kDirectLightStride + j * kDirectSampleStride;
                const V2 u = smp.next2d(dim);
                float lp;
                if (d.env >= 0) {
                    env_sample(s.envs[d.env], u, useCdf, &local, &lp);
                    if (lp <= 0.0f) return false;
                    L = env_evaluate(env_for_eval(s, a, d.env), local) * d.radiance;
                    Ls = a.distinctEval ? env_evaluate(s.envs[d.env], local) * d.radiance : L;
                    envIdx = d.env;
                    domeRad = d.radiance;
                } else {
                    const float yy = 1.0f - 2.0f * u.y;
                    const float rr = sqrtf(smax(0.0f, 1.0f - yy * yy));
                    const float phi = 2.0f * kPi * u.x;
                    local = V3{sinf(phi) * rr, yy, cosf(phi) * rr};
                    lp = kInvFourPi;
                    L = V3{1.0f, 1.0f, 1.0f} * d.radiance;
                }
                if (d.env < 0) Ls = L;
                ld = light_to_world(d, local);
                const float nl = sclamp(dot(v.n, ld), 0.0f, 1.0f);
                if (nl <= 0.0f) return false;
                const float bp = bsdf_pdf_rec(rec, ms, v.w, v.n, v.cn, v.view, ld);
                const float mis = power_heuristic(lp, bp);
                w = nl * mis / lp;
            }
            if (trace_occluded(s, origin, ld, reach, ctr)) return false;
            const V3 f = evalE(ld);
            const V3 raw = f * L * w;
            if (a.distinctEval) {
                // frozen render: the clamp scale of the sampling parameters'
                // contribution (held constant, as the adjoint holds it)
                const V3 rawS = bsdf_eval_rec(rec, ms, v.n, v.cn, v.view, ld) * Ls * w;
                *c = raw * clamp_scale(q, rawS, kDirectSampleClamp);
            } else {
                *c = clamp24(q, raw);
            }
            if (kGrad) {
                const float sc = clamp_scale(q, raw, kDirectSampleClamp);
                const DV3 fd = bsdf_eval_d(me, v.n, v.cn, v.view, ld);
                add_mat_grad(a, v.hit.material, fd, dT * L * (w * sc));
                if (envIdx >= 0 && envIdx == a.env0) add_env_grad(a, a.evalEnv, local, dT * f * domeRad * (w * sc));
            }
            return true;
        });
        ps.radiance = ps.radiance + ps.T * direct;
        if (kGrad) Lrem = Lrem - ps.T * direct;
        // continuation (continue_path with the BSDF value from the eval material)
        const uint32_t base = depth * kPathDimStride;
        const float rw = v.w.diffuse + v.w.spec + v.w.coat;
        const float tw = rw + 0.0f;
        if (tw <= 0.0f) break;
        const float sel = smp.next1d(base + 1u) * tw;
        const V2 ds = smp.next2d(base + 2u);
        V3 next, f;
        float pdf;
        bool delta2 = false;
        const float rs = sel - 0.0f;
        if (rs < v.w.diffuse) {
            if (ps.diffDepth >= q.diffuseDepth) break;
            ++ps.diffDepth;
            next = cosine_hemisphere(v.n, ds);
            const float cpdf = sclamp(dot(v.n, next), 0.0f, 1.0f) * kInvPi;
            pdf = smax((rw / tw) * (1.0f * cpdf + 0.0f * 0.0f), 1.0e-6f);
            f = evalE(next);
        } else {
            const bool coat = !(rs < v.w.diffuse + v.w.spec);
            if (ps.specDepth >= q.specularDepth) break;
            ++ps.specDepth;
            const V3 sn = coat ? v.cn : v.n;
            const float sr = coat ? roughness_for(ms.coat_roughness, ms.coat_anisotropy, ms.coat_rotation)
                                  : roughness_for(base_roughness(ms), ms.specular_anisotropy, ms.specular_rotation);
            const V3 hv = ggx_half(sn, ds, sr);
            next = normalize(reflect(ps.rd, hv));
            const float rc = sclamp(dot(sn, next), 0.0f, 1.0f);
            if (rc <= 0.0f) break;
            pdf = smax((rw / tw) * bsdf_pdf_rec(rec, ms, v.w, v.n, v.cn, v.view, next), 1.0e-6f);
            f = evalE(next);
            delta2 = sr <= kDeltaRoughness;
        }
        const float cosT = sclamp(dot(v.n, next), 0.0f, 1.0f);
        if (cosT <= 0.0f) break;
        if (a.distinctEval) {
            // frozen render: the throughput clamp's scale comes from the
            // sampling throughput (clamp_max(v) == v * clamp_scale(v))
            const V3 tsRaw = Ts * bsdf_eval_rec(rec, ms, v.n, v.cn, v.view, next) * (cosT / pdf);
            const float sc = clamp_scale(q, tsRaw, kThroughputClamp);
            Ts = tsRaw * sc;
            ps.T = ps.T * f * (cosT / pdf) * sc;
        } else {
            ps.T = clamp12(q, ps.T * f * (cosT / pdf));
            Ts = ps.T;
        }
        const float off = dot(v.n, next) >= 0.0f ? 1.0f : -1.0f;
        ps.ro = v.hit.position + v.n * (kRayEpsilon * off);
        const V3 prevDir = ps.rd;
        ps.rd = next;
        ps.prevDelta = delta2;
        ps.prevPdf = pdf;
        bool alive = true;
        if (depth >= 2) {
            const float cp = sclamp(maxc(Ts), 0.05f, 0.95f);
            if (smp.next1d(base + 4u) > cp) {
                alive = false;
            } else {
                ps.T = ps.T / cp;
                Ts = Ts / cp;
            }
        }
        if (kGrad && alive && depth + 1u < q.maxDepth) {
            // every later contribution scales with f (per channel)
            const DV3 fd = bsdf_eval_d(me, v.n, v.cn, v.view, next);
            const V3 coef{f.x > 0.0f ? delta.x * Lrem.x / f.x : 0.0f, f.y > 0.0f ? delta.y * Lrem.y / f.y : 0.0f,
                          f.z > 0.0f ? delta.z * Lrem.z / f.z : 0.0f};
            add_mat_grad(a, v.hit.material, fd, coef);
        }
        (void)prevDir;
        if (!alive) break;
    }
    if (depthOut) *depthOut = depth0;
    return ps.radiance;
}

// The gradient pass.  Each path's total radiance comes from the record of the
// same path (same estimator, same sample) rendered just before by the
// wavefront form into `records` (one float4 per path, request path order), so
// only the replay that accumulates gradients runs here.  (4 blocks per SM: 128 registers measured faster than
// the 168 the compiler otherwise takes.)
__global__ void __launch_bounds__(128, 4) k_adjoint(const __grid_constant__ DevScene s, const __grid_constant__ DevRequest q,
                                                    const __grid_constant__ AdjView a, uint64_t pathBase, uint32_t count,
                                                    const float4* __restrict__ records) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) {
        const uint64_t path = pathBase + i;
        const uint64_t pixel = path / q.sampleCount;
        const uint32_t smp = static_cast<uint32_t>(path - pixel * q.sampleCount);
        const uint32_t y = static_cast<uint32_t>(pixel / q.width);
        const uint32_t x = static_cast<uint32_t>(pixel - static_cast<uint64_t>(y) * q.width);
        const float cnt = static_cast<float>(q.sampleCount);
        const float4 g = reinterpret_cast<const float4*>(a.dBeauty)[pixel];
        const V3 delta{g.x / cnt, g.y / cnt, g.z / cnt};
        if (delta.x != 0.0f || delta.y != 0.0f || delta.z != 0.0f) {
            const float4 r = records[path];
            adj_path(s, q, a, x, y, q.sampleStart + smp, delta, V3{r.x, r.y, r.z}, nullptr, true);
        }
    }
}

// Adds the float4 texel accumulators into the caller's rgb gradient.
__global__ void k_env_grad_out(const float4* __restrict__ acc, float* __restrict__ dEnv, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 g = acc[i];
    dEnv[3 * static_cast<size_t>(i)] += g.x;
    dEnv[3 * static_cast<size_t>(i) + 1] += g.y;
    dEnv[3 * static_cast<size_t>(i) + 2] += g.z;
}

// Frozen-sampling forward: radiance + first-hit depth per path as a record.
__global__ void __launch_bounds__(128) k_frozen(const __grid_constant__ DevScene s, const __grid_constant__ DevRequest q,
                                                const __grid_constant__ AdjView a, uint64_t pathBase,
                                                uint32_t count, float4* __restrict__ records) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const uint64_t path = pathBase + i;
    const uint64_t pixel = path / q.sampleCount;
    const uint32_t smp = static_cast<uint32_t>(path - pixel * q.sampleCount);
    const uint32_t y = static_cast<uint32_t>(pixel / q.width);
    const uint32_t x = static_cast<uint32_t>(pixel - static_cast<uint64_t>(y) * q.width);
    float depth0;
    const V3 L = adj_path(s, q, a, x, y, q.sampleStart + smp, V3{0, 0, 0}, V3{0, 0, 0}, &depth0, false);
    float4* o = records + 3 * static_cast<size_t>(i);
    o[0] = make_float4(L.x, L.y, L.z, depth0);
    o[1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void k_scatter_params(Mat* mats, uint32_t n, const float* base, const float* rough, const float* metal) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (base) {
        mats[i].base_color[0] = base[3 * i];
        mats[i].base_color[1] = base[3 * i + 1];
        mats[i].base_color[2] = base[3 * i + 2];
    }
    if (rough) mats[i].roughness = rough[i];
    if (metal) mats[i].metallic = metal[i];
}

__global__ void k_rgb_to_texels(const float* rgb, float4* tex, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    tex[i] = make_float4(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2], 0.0f);
}

inline unsigned grid(uint64_t n, unsigned b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace

struct AdjointState {
    DeviceBlock evalMats, evalTexels, envGrad;
};

namespace {

AdjointState* adj_state(ContextImpl* ctx) {
    if (!ctx->adjoint) ctx->adjoint = new AdjointState();
    return ctx->adjoint;
}

int32_t dome0_env(const ContextImpl* ctx) { return ctx->domeEnv.empty() ? -1 : ctx->domeEnv[0]; }

AdjView base_view(ContextImpl* ctx) {
    AdjView a{};
    a.evalMats = ctx->scene.materials;
    a.env0 = dome0_env(ctx);
    if (a.env0 >= 0) a.evalEnv = ctx->envDev[a.env0];
    a.materialCount = ctx->materialCount;
    return a;
}

}  // namespace

int adjoint_set_params(ContextImpl* ctx, const float* base, const float* rough, const float* metal, const float* env) {
    if (!ctx->hasScene) return fail(ctx, SHIRO_ERR_NO_SCENE, "no scene uploaded");
    ++ctx->epoch;
    if ((base || rough || metal) && ctx->materialCount) {
        k_scatter_params<<<grid(ctx->materialCount, 128), 128, 0, ctx->stream>>>(
            const_cast<Mat*>(ctx->scene.materials), ctx->materialCount, base, rough, metal);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(ctx, e, "set material params");
        const int rc = build_bsdf_recs(ctx);
        if (rc != SHIRO_OK) return rc;
    }
    if (env) {
        const int32_t e0 = dome0_env(ctx);
        if (e0 < 0) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "dome light 0 has no environment texture");
        const DevEnv& de = ctx->envDev[e0];
        const uint64_t n = static_cast<uint64_t>(de.w) * de.h;
        // resident texels take the new radiance (masses are rebuilt below)
        k_rgb_to_texels<<<grid(n, 256), 256, 0, ctx->stream>>>(env, const_cast<float4*>(de.texels), static_cast<uint32_t>(n));
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(ctx, e, "set env params");
        const int rc = finish_env(ctx, static_cast<size_t>(e0));  // rebuilt importance table + sample records
        if (rc != SHIRO_OK) return rc;
    }
    const cudaError_t e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? SHIRO_OK : cuda_fail(ctx, e, "set params");
}

int adjoint_run(ContextImpl* ctx, const ShiroRenderDesc* req, const float* dBeauty, float* dBase, float* dRough, float* dMetal,
                float* dEnv) {
    if (ctx->hasScene && ctx->transmissiveMaterials)
        return fail(ctx, SHIRO_ERR_UNSUPPORTED_SCENE,
                    "the differentiable form covers reflecting, emitting and cut-out materials (no transmission)");
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    const DevRequest q = make_request(*req);
    AdjView a = base_view(ctx);
    a.dBeauty = dBeauty;
    a.dBase = dBase;
    a.dRough = dRough;
    a.dMetal = dMetal;
    const uint32_t texels = a.env0 >= 0 ? a.evalEnv.w * a.evalEnv.h : 0u;
    if (dEnv && texels) {
        AdjointState* st = adj_state(ctx);
        if (!ensure_block(ctx, &st->envGrad, texels * sizeof(float4), "environment gradient")) return SHIRO_ERR_OUT_OF_MEMORY;
        const cudaError_t e = cudaMemsetAsync(st->envGrad.ptr, 0, texels * sizeof(float4), ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "environment gradient");
        a.dEnv4 = static_cast<float4*>(st->envGrad.ptr);
    }
    const uint64_t total = static_cast<uint64_t>(q.width) * q.height * q.sampleCount;
    const uint64_t chunk = 1ull << 24;
    // one record (radiance, depth) per path of the request (one-thread-per-path replay)
    if (!ctx->adjointWavefront &&
        !ensure_block(ctx, &ctx->pathRecords, std::max<uint64_t>(total, 1) * sizeof(float4), "path records"))
        return SHIRO_ERR_OUT_OF_MEMORY;
    float4* rec = static_cast<float4*>(ctx->pathRecords.ptr);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, ctx->stream);
    uint64_t launches = 0;
    if (total && ctx->adjointWavefront) {
        // forward and replay stages per wave of the wavefront form
        rc = wavefront_adjoint(ctx, *req, a);
        if (rc != SHIRO_OK) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc;
        }
        launches += ctx->stats.kernel_launches;
    } else if (total) {  // the paths' radiance, by the wavefront form, then one thread per path
        rc = wavefront_path_records(ctx, *req, rec);
        if (rc != SHIRO_OK) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return rc;
        }
        launches += ctx->stats.kernel_launches;
    }
    for (uint64_t p0 = 0; p0 < total && !ctx->adjointWavefront; p0 += chunk) {
        const uint32_t n = static_cast<uint32_t>(std::min(chunk, total - p0));
        k_adjoint<<<grid(n, 128), 128, 0, ctx->stream>>>(ctx->scene, q, a, p0, n, rec);
        launches += 1;
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return cuda_fail(ctx, e, "adjoint launch");
        }
    }
    if (a.dEnv4) {
        k_env_grad_out<<<grid(texels, 256), 256, 0, ctx->stream>>>(a.dEnv4, dEnv, texels);
        ++launches;
    }
    cudaEventRecord(e1, ctx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "adjoint");
    ctx->stats.kernel_ms = ms;
    ctx->stats.path_kernel_ms = ms;
    ctx->stats.path_kernel_launches = launches;
    ctx->stats.kernel_launches = launches;
    ctx->stats.paths = total;
    return check_device_error(ctx);
}

void adjoint_free(ContextImpl* ctx) {
    if (!ctx->adjoint) return;
    for (DeviceBlock* b : {&ctx->adjoint->evalMats, &ctx->adjoint->evalTexels, &ctx->adjoint->envGrad})
        if (b->ptr) cudaFree(b->ptr);
    delete ctx->adjoint;
    ctx->adjoint = nullptr;
}

int adjoint_render_frozen(ContextImpl* ctx, const ShiroRenderDesc* req, const float* base, const float* rough,
                          const float* metal, const float* env, float* beauty) {
    if (ctx->hasScene && ctx->transmissiveMaterials)
        return fail(ctx, SHIRO_ERR_UNSUPPORTED_SCENE,
                    "the differentiable form covers reflecting, emitting and cut-out materials (no transmission)");
    int rc = validate_request(ctx, *req);
    if (rc != SHIRO_OK) return rc;
    AdjointState* st = adj_state(ctx);
    const DevRequest q = make_request(*req);
    AdjView a = base_view(ctx);
    const uint32_t nm = ctx->materialCount + 1;
    if (!ensure_block(ctx, &st->evalMats, nm * sizeof(Mat), "eval materials")) return SHIRO_ERR_OUT_OF_MEMORY;
    Mat* em = static_cast<Mat*>(st->evalMats.ptr);
    cudaError_t e = cudaMemcpyAsync(em, ctx->scene.materials, nm * sizeof(Mat), cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "eval materials");
    if ((base || rough || metal) && ctx->materialCount)
        k_scatter_params<<<grid(ctx->materialCount, 128), 128, 0, ctx->stream>>>(em, ctx->materialCount, base, rough, metal);
    a.evalMats = em;
    a.distinctEval = 1u;
    if (env && a.env0 >= 0) {
        const uint32_t n = a.evalEnv.w * a.evalEnv.h;
        if (!ensure_block(ctx, &st->evalTexels, std::max<size_t>(n, 1) * sizeof(float4), "eval texels"))
            return SHIRO_ERR_OUT_OF_MEMORY;
        k_rgb_to_texels<<<grid(n, 256), 256, 0, ctx->stream>>>(env, static_cast<float4*>(st->evalTexels.ptr), n);
        a.evalEnv.texels = static_cast<const float4*>(st->evalTexels.ptr);
    }
    const uint64_t pixels = static_cast<uint64_t>(q.width) * q.height;
    if (q.sampleCount == 0 || pixels == 0) return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "empty request");
    const uint64_t pixelsPerChunk = std::max<uint64_t>(1, (1ull << 24) / q.sampleCount);
    const uint64_t recBytes = std::min<uint64_t>(pixelsPerChunk, pixels) * q.sampleCount * kPathRecordBytes;
    if (!ensure_block(ctx, &ctx->pathRecords, recBytes, "path records")) return SHIRO_ERR_OUT_OF_MEMORY;
    if (!ensure_block(ctx, &ctx->aovScratch, pixels * 11 * sizeof(float), "AOV staging")) return SHIRO_ERR_OUT_OF_MEMORY;
    float* sc = static_cast<float*>(ctx->aovScratch.ptr);
    const AovPtrs aov{beauty, sc + 4 * pixels, sc + 7 * pixels, sc + 10 * pixels};
    float4* rec = static_cast<float4*>(ctx->pathRecords.ptr);
    for (uint64_t p0 = 0; p0 < pixels; p0 += pixelsPerChunk) {
        const uint32_t np = static_cast<uint32_t>(std::min(pixelsPerChunk, pixels - p0));
        const uint32_t paths = np * q.sampleCount;
        k_frozen<<<grid(paths, 128), 128, 0, ctx->stream>>>(ctx->scene, q, a, p0 * q.sampleCount, paths, rec);
        launch_resolve_pixels(q, p0, np, rec, aov, ctx->stream);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_fail(ctx, e, "frozen render launch");
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "frozen render");
    return check_device_error(ctx);
}

}  // namespace shiro_gpu
