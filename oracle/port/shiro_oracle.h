// shiro_oracle.h - C ABI of the CPU restatement of Shiro's reference path
// tracer.  TEST INFRASTRUCTURE ONLY: the oracle is the checker of the GPU
// backend (tests, smoke) and the timed CPU baseline of bench.py; the product
// never links it.
//
// Scope: the reference CpuPathTracer (src/backend/cpu/CpuPathTracer.cpp) for
// every scene the GPU backend accepts (shiro_gpu_supports_scene): reflective
// layered BSDF (diffuse / Oren-Nayar, GGX base specular, coat, sheen, thin
// film, subsurface wrap, anisotropy, normal overrides), distant lights, dome
// lights (lat-long with importance table, angular, constant), gradient
// environment, MIS, clamps, Russian roulette, AOVs.  Transmission, opacity,
// emissive triangles and the progressive path guide are rejected.
// Intersection follows the reference's brute-force fallback exactly
// (CpuPathTracer.cpp:386-475: Moller-Trumbore, first (mesh, prim) wins a tie)
// but is accelerated by a binned-SAH BVH whose traversal reproduces the same
// closest hit.
#ifndef SHIRO_ORACLE_H_
#define SHIRO_ORACLE_H_

#include <stdint.h>

#include "../../include/shiro_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Same signatures as oracle/ref/ref_harness.cpp (prefix ref_). */
int oracle_sampler(uint32_t n, const uint32_t* px, const uint32_t* py, const uint32_t* index,
                   const uint32_t* branch, float* out2);
int oracle_camera_rays(const ShiroRenderDesc* req, float* origins, float* dirs);
int oracle_trace_rays(const ShiroSceneDesc* scene, const float* origins, const float* dirs, const float* tmax,
                      uint32_t n, uint32_t* prim, float* t, uint32_t* occluded);
int oracle_trace_rays_bruteforce(const ShiroSceneDesc* scene, const float* origins, const float* dirs,
                                 const float* tmax, uint32_t n, uint32_t* prim, float* t, uint32_t* occluded);
int oracle_primary_hits(const ShiroSceneDesc* scene, const ShiroRenderDesc* req, uint32_t* prim, float* t);
int oracle_bsdf(const ShiroMaterialDesc* m, uint32_t n, const float* normals, const float* views,
                const float* lights, float* f_out, float* pdf_out, float* weights_out);
int oracle_env_tables(uint32_t w, uint32_t h, const float* rgb, float* row_cdf, float* cond_cdf);
int oracle_env_query(uint32_t w, uint32_t h, const float* rgb, uint32_t layout, uint32_t n, const float* u2,
                     const float* dirs, float* sample_dir, float* sample_pdf, float* sample_rgb, float* pdf,
                     float* rgb_out);
int oracle_render(const ShiroSceneDesc* scene, const ShiroRenderDesc* req, ShiroAovs* out);
/* The GPU backend's alias table (not part of the reference) over the
 * reference's texel masses of a w x h lat-long texture, by a sequential sweep:
 * the checker of the backend's parallel construction.  threshold_bits,
 * alias: w * h entries each. */
int oracle_env_alias(uint32_t w, uint32_t h, const float* rgb, uint32_t* threshold_bits, uint32_t* alias);

/* Worker threads of the render calls (0 = hardware_concurrency - 1, as the
 * reference, CpuPathTracer.cpp:2064-2067). */
void oracle_set_threads(uint32_t threads);

/* Per-path results: for path i, pixel pixels[i] (y * width + x) and sample
 * index sample_index[i]; out[i*10 + 0..9] = radiance rgb, albedo rgb,
 * normal rgb, depth. */
int oracle_render_paths(const ShiroSceneDesc* scene, const ShiroRenderDesc* req, const uint32_t* pixels,
                        uint32_t n, const uint32_t* sample_index, float* out, void* reserved0, void* reserved1);

/* Handle API for timing: build once, render bounded row ranges. */
typedef struct OracleScene OracleScene;
int oracle_scene_create(const ShiroSceneDesc* scene, OracleScene** out);
void oracle_scene_destroy(OracleScene* s);
/* Renders rows [y0, y1) of the request's frame into out (full-frame
 * planes); returns the number of paths traced or a negative error. */
int64_t oracle_scene_render_rows(OracleScene* s, const ShiroRenderDesc* req, uint32_t y0, uint32_t y1,
                                 ShiroAovs* out);
/* Renders the n listed rows (each < height) with all host threads into
 * out (full-frame planes); returns the number of paths traced or a
 * negative error. */
int64_t oracle_scene_render_row_list(OracleScene* s, const ShiroRenderDesc* req, const uint32_t* rows, uint32_t n,
                                     ShiroAovs* out);
/* Per-path results as oracle_render_paths, on a created scene (with its
 * alias tables, if set). */
int oracle_scene_render_paths(OracleScene* s, const ShiroRenderDesc* req, const uint32_t* pixels, uint32_t n,
                              const uint32_t* sample_index, float* out);
/* Gives dome `dome`'s environment the GPU backend's alias table (n = w * h
 * entries: acceptance threshold as float bits, alias texel).  Renders without
 * SHIRO_RENDER_ENV_CDF then pick dome-sample texels by that table (bucket
 * floor(u.y * n), accepted when u.x < threshold, else the alias) and follow
 * EnvironmentMap::Sample from the picked texel on: the backend's timed
 * sampler, checked path by path.  Not part of the reference. */
int oracle_scene_set_env_alias(OracleScene* s, uint32_t dome, const uint32_t* threshold_bits, const uint32_t* alias,
                               uint32_t n);
/* 1 if the scene is within the restated scope (see above), else 0. */
int oracle_supports_scene(const ShiroSceneDesc* scene);

#ifdef __cplusplus
}
#endif

#endif
