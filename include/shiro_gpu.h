/*
 * shiro_gpu.h - C ABI of the GB300 path-tracing backend for Shiro.
 *
 * This is the drop-in boundary that replaces Shiro's OptiX backend behind
 * shiro::backend::RenderBackend (include/shiro/backend/RenderBackend.h:28-34 in
 * ichin0se/Shiro).  The reference has no C ABI of its own: its backends are C++
 * classes called through
 *     virtual BackendStatus GetStatus() const;                    (RenderBackend.h:32)
 *     virtual FrameBuffer RenderSampleBatch(const RenderRequest&); (RenderBackend.h:33)
 *     bool SupportsScene(const Scene&) const;                      (OptixBackend.h:16)
 * The entry points below are what a C++ adapter (shiro_gb300/backend/GpuBackend.cpp)
 * binds to implement that class; every struct is plain data (pointers, sizes,
 * floats), no C++ or torch types.
 *
 * Ownership: the caller owns every host array passed in; the context owns all
 * device memory it allocates.  Calls on one context must be serialised by the
 * caller (the reference serialises RenderSampleBatch with a mutex,
 * OptixBackend.h:24-26).  Errors are reported as a negative status; the
 * message is available from shiro_gpu_last_error().  The backend never falls
 * back to a CPU path: a missing device or a failed launch is an error.
 */
#ifndef SHIRO_GPU_H_
#define SHIRO_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SHIRO_GPU_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------- */
#define SHIRO_OK 0
#define SHIRO_ERR_INVALID_ARGUMENT (-1)
#define SHIRO_ERR_NO_DEVICE (-2)
#define SHIRO_ERR_CUDA (-3)
#define SHIRO_ERR_OUT_OF_MEMORY (-4)
#define SHIRO_ERR_UNSUPPORTED_SCENE (-5)
#define SHIRO_ERR_CANCELLED (-6)
#define SHIRO_ERR_NO_SCENE (-7)
#define SHIRO_ERR_TIMEOUT (-8)
#define SHIRO_ERR_DEVICE_CHECK (-9)

/* ---- enums mirrored from shiro/render/Renderer.h ------------------------- */
/* BackendKind, Renderer.h:23-27 */
#define SHIRO_BACKEND_CPU 0
#define SHIRO_BACKEND_GPU 1
#define SHIRO_BACKEND_HYBRID 2
/* EnvironmentMapLayout, Renderer.h:17-21 */
#define SHIRO_ENV_LAYOUT_AUTOMATIC 0
#define SHIRO_ENV_LAYOUT_LATLONG 1
#define SHIRO_ENV_LAYOUT_ANGULAR 2

/* Render flags (ShiroRenderDesc.flags). */
/* Sample the dome light by binary search over the reference's row / column
 * CDFs (EnvironmentMap.cpp:109-163) instead of the O(1) alias table.  Both
 * give the same per-pixel probability; the CDF mode also maps a given 2-D
 * sample to the same texel as the reference does, so paths match the CPU
 * tracer sample for sample. */
#define SHIRO_RENDER_ENV_CDF 0x1u
/* Differentiable mode: the direct-sample (24) and throughput (12) clamps of
 * the reference (CpuPathTracer.cpp:63-64) are disabled, in the forward and
 * in the adjoint, so that the rendered estimate is smooth in the parameters. */
#define SHIRO_RENDER_NO_CLAMP 0x2u
/* Forward pass of the differentiable form, batched wavefront form only
 * (shiro_gpu_render_batch; the flag of the call's first request decides):
 * when all the call's paths fit one pool (ShiroWavefrontConfig.
 * paths_in_flight), the forward stages also log every bounce's hits and
 * light-sample visibility (21 bytes per path and bounce of device memory),
 * and the paths' radiance records and logs stay on the device.  A
 * shiro_gpu_adjoint of one of the call's requests (this flag aside) that
 * follows it, with no wavefront render, adjoint, autotuning, upload,
 * parameter, BVH or configuration change in between, replays that
 * request's paths instead of running the forward stages again; otherwise
 * the adjoint runs them as usual.  Images and gradients are the same either
 * way.  (A loss gradient that replays samples independent of the image's
 * renders both sample ranges in one call, two requests, and the adjoint
 * takes the second.)  Ignored by the plain form. */
#define SHIRO_RENDER_KEEP_PATHS 0x4u

/* ---- scene snapshot (shiro/render/Renderer.h:29-133) --------------------- */

/* PbrMaterial, Renderer.h:56-102; same fields in the same order. Booleans are
 * uint32 (0/1). */
typedef struct ShiroMaterialDesc {
    float base_color[3];
    float emission_color[3];
    float specular_color[3];
    float transmission_color[3];
    float transmission_scatter[3];
    float coat_color[3];
    float subsurface_color[3];
    float subsurface_radius[3];
    float sheen_color[3];
    float normal_override[3];
    float coat_normal_override[3];
    float tangent_override[3];
    float base_weight;
    float emission_strength;
    float specular_weight;
    float metallic;
    float roughness;
    float diffuse_roughness;
    float opacity;
    float specular_anisotropy;
    float specular_rotation;
    float coat_weight;
    float coat_roughness;
    float coat_ior;
    float coat_anisotropy;
    float coat_rotation;
    float sheen;
    float sheen_roughness;
    float subsurface;
    float subsurface_scale;
    float subsurface_anisotropy;
    float transmission;
    float transmission_depth;
    float transmission_scatter_anisotropy;
    float transmission_dispersion;
    float transmission_extra_roughness;
    float ior;
    float coat_affect_color;
    float coat_affect_roughness;
    float thin_film_thickness;
    float thin_film_ior;
    uint32_t thin_walled;
    uint32_t has_normal_override;
    uint32_t has_coat_normal_override;
    uint32_t has_tangent_override;
} ShiroMaterialDesc;

/* TriangleMesh, Renderer.h:104-109.  positions / normals are xyz float
 * triples; normals may be absent (normal_count 0) and are only used when
 * normal_count == vertex_count, as in TriangleShadingNormal
 * (CpuPathTracer.cpp:156). */
typedef struct ShiroMeshDesc {
    const float* positions;
    uint32_t vertex_count;
    const float* normals;
    uint32_t normal_count;
    const uint32_t* indices;
    uint32_t index_count;
    uint32_t material_index;
} ShiroMeshDesc;

/* DirectionalLight, Renderer.h:111-114 */
typedef struct ShiroDistantLightDesc {
    float direction[3];
    float radiance[3];
} ShiroDistantLightDesc;

/* DomeLight, Renderer.h:116-124.  The texture is passed as decoded RGB float
 * pixels (row-major, env_width * env_height * 3), i.e. the contents of
 * EnvironmentMap::Pixels() (EnvironmentMap.h:24); env_pixels NULL means a
 * constant dome (DomeLight without environment). */
typedef struct ShiroDomeLightDesc {
    float radiance[3];
    float right[3];
    float up[3];
    float forward[3];
    uint32_t layout; /* SHIRO_ENV_LAYOUT_* */
    uint32_t env_width;
    uint32_t env_height;
    const float* env_pixels;
} ShiroDomeLightDesc;

/* Scene, Renderer.h:126-133 */
typedef struct ShiroSceneDesc {
    const ShiroMaterialDesc* materials;
    uint32_t material_count;
    const ShiroMeshDesc* meshes;
    uint32_t mesh_count;
    const ShiroDistantLightDesc* distant_lights;
    uint32_t distant_light_count;
    const ShiroDomeLightDesc* dome_lights;
    uint32_t dome_light_count;
    float environment_top[3];
    float environment_bottom[3];
} ShiroSceneDesc;

/* Camera, Renderer.h:47-54 */
typedef struct ShiroCameraDesc {
    float position[3];
    float forward[3];
    float right[3];
    float up[3];
    float vertical_fov_degrees;
    float aspect_ratio;
} ShiroCameraDesc;

/* RenderSettings, Renderer.h:29-45 (booleans as uint32). */
typedef struct ShiroSettingsDesc {
    uint32_t width;
    uint32_t height;
    uint32_t samples_per_pixel;
    uint32_t samples_per_update;
    uint32_t dome_light_samples;
    uint32_t max_depth;
    uint32_t diffuse_depth;
    uint32_t specular_depth;
    uint32_t thread_limit;
    uint32_t max_subdiv_level;
    uint32_t backend;
    uint32_t background_visible;
    uint32_t enable_headlight;
    uint32_t enable_caustics;
    uint32_t enable_sss;
} ShiroSettingsDesc;

/* RenderRequest, RenderBackend.h:12-19 (scene is bound separately through
 * shiro_gpu_upload_scene; the cancel flag is a call argument). */
typedef struct ShiroRenderDesc {
    ShiroCameraDesc camera;
    ShiroSettingsDesc settings;
    uint32_t sample_start;
    uint32_t sample_count;
    uint32_t flags; /* SHIRO_RENDER_* */
    uint32_t reserved;
} ShiroRenderDesc;

/* FrameBuffer, FrameBuffer.h:10-37: beauty RGBA (alpha = hit fraction),
 * albedo RGB, normal RGB (n * 0.5 + 0.5), depth (min hit distance, +inf on
 * miss); row-major y * width + x.  on_device != 0 means the four pointers
 * are device pointers (no host copy is made). */
typedef struct ShiroAovs {
    float* beauty;
    float* albedo;
    float* normal;
    float* depth;
    uint32_t on_device;
    uint32_t reserved;
} ShiroAovs;

/* BackendStatus, RenderBackend.h:21-26 */
typedef struct ShiroBackendStatus {
    uint32_t kind; /* SHIRO_BACKEND_* */
    uint32_t available;
    uint32_t uses_gpu;
    uint32_t device_count;
    char name[32];
    char device_name[96];
    int32_t compute_major;
    int32_t compute_minor;
} ShiroBackendStatus;

typedef struct ShiroGpuContext ShiroGpuContext;

/* ---- entry points -------------------------------------------------------- */

/* BackendStatus RenderBackend::GetStatus() (RenderBackend.h:32;
 * OptixBackend.cpp:1036-1060): device present and an sm_103 part. */
int shiro_gpu_status(ShiroBackendStatus* out);

/* Creates a context on a device (OptixBackend::EnsureRuntime,
 * OptixBackend.cpp:1071-1139, minus the NVRTC / OptiX pipeline). */
int shiro_gpu_create(int device, ShiroGpuContext** out);
void shiro_gpu_destroy(ShiroGpuContext* ctx);

/* Last error message of this context (or of the last failed create when ctx
 * is NULL). Never NULL. */
const char* shiro_gpu_last_error(const ShiroGpuContext* ctx);

/* Selects the acceleration structure the kernels traverse: 2 the binary
 * BVH, 8 the compressed 8-wide BVH (quantised child boxes, octant-ordered
 * slots), 0 (default) each form its faster one on GB300: the wavefront
 * stages the wide BVH, the one-thread-per-path kernels (plain, adjoint,
 * probes) the binary one.  Both give identical hits; the choice only changes
 * speed. */
int shiro_gpu_set_bvh_width(ShiroGpuContext* ctx, uint32_t width);

/* How the next shiro_gpu_upload_scene builds its binary BVHs (the wide one
 * is collapsed from them): sah_cluster_triangles > 1 keeps the Morton (LBVH)
 * subtrees of at most that many triangles as clusters and rebuilds the tree
 * above them by binned SAH over the clusters' boxes (16 bins per axis, on the
 * device); 0 keeps the Morton hierarchy throughout.  Default 2.  Both give
 * identical hits; the choice only changes speed. */
int shiro_gpu_set_bvh_build(ShiroGpuContext* ctx, uint32_t sah_cluster_triangles);

/* Renders on this CUDA stream (cudaStream_t cast to void*; NULL = the
 * context's own stream). */
int shiro_gpu_set_stream(ShiroGpuContext* ctx, void* stream);

/* bool SupportsScene(const Scene&) (OptixBackend.h:16, Renderer.cpp:20).
 * Returns 1 when every material and light of the scene is handled by the GPU
 * integrator, 0 otherwise (the renderer then falls back to the CPU tracer,
 * Renderer.cpp:19-30).  reason (may be NULL) receives a short explanation. */
int shiro_gpu_supports_scene(const ShiroSceneDesc* scene, char* reason, size_t reason_size);

/* 64-bit content signature of a scene snapshot: a hash of everything
 * shiro_gpu_upload_scene reads (every material field, each mesh's material
 * index, positions, normals and indices, the lights, each dome's radiance,
 * frame, layout and texels, the gradient environment).  Callers that cache the
 * uploaded scene compare it to decide whether to upload again, as the OptiX
 * backend compares ComputeSceneSignature (OptixBackend.cpp:150-232,
 * 1079-1092): a snapshot edited in place, or a new one built at a freed
 * address (RenderParam.cpp:614-659), gets a new signature.  Large scenes are
 * hashed on several host threads (about 20 GB/s); the value does not depend on
 * the thread count. */
int shiro_gpu_scene_signature(const ShiroSceneDesc* scene, uint64_t* out);

/* Page-locked host memory (no counterpart in the reference).  AOV planes
 * inside it are written in place by the wavefront form's resolve stage, wave
 * by wave, so a render into them needs no copy after its last wave; a host
 * that must hand frames over in its own (pageable) buffers, as
 * RenderBackend::RenderSampleBatch returns a FrameBuffer by value, renders
 * into such a buffer and copies out.  Free with shiro_gpu_host_free. */
int shiro_gpu_host_alloc(size_t bytes, void** out);
void shiro_gpu_host_free(void* ptr);

/* Environment images from disk: EnvironmentMap::Load (EnvironmentMap.cpp:
 * 49-92) without OpenImageIO, for hosts whose EnvironmentMap is built without
 * it (it then loads nothing).  Reads a Radiance RGBE file (.hdr: flat,
 * old- and new-style run-length scanlines, all eight orientations; a texel is
 * mantissa * 2^(exponent - 136)) or a single-part scanline OpenEXR file
 * (.exr: HALF / FLOAT / UINT channels; NONE, RLE, ZIPS, ZIP compression; R, G,
 * B used when present, else Y, else the first non-alpha channels), told apart
 * by their magic bytes.  *pixels receives width * height RGB float triples,
 * row 0 at the top (EnvironmentMap::Pixels()'s layout, ready for
 * ShiroDomeLightDesc.env_pixels); free it with shiro_hdri_free.  On failure
 * returns SHIRO_ERR_INVALID_ARGUMENT (SHIRO_ERR_OUT_OF_MEMORY) with the reason
 * in error (may be NULL).  Host code only: no device is needed. */
int shiro_hdri_load(const char* path, uint32_t* width, uint32_t* height, float** pixels, char* error,
                    size_t error_size);
int shiro_hdri_decode(const void* data, size_t size, uint32_t* width, uint32_t* height, float** pixels, char* error,
                      size_t error_size);
void shiro_hdri_free(float* pixels);

/* Uploads a scene snapshot: flattens meshes, builds the device BVH, the
 * material table and the dome-light importance tables (CDF and alias).
 * Counterpart of OptixBackend::UploadSceneData (OptixBackend.cpp:751-1026) and
 * CpuPathTracer::BuildAccelerationScene (CpuPathTracer.cpp:477-598).  When the
 * geometry equals the resident scene's (mesh positions, normals, indices and
 * material indices, the material count, the BVH build setting), the BVHs and
 * per-triangle records are kept and only what derives from materials, lights
 * and environments is replaced.  A scene without triangles is accepted and
 * renders as the CPU tracer renders it: every ray misses (the environment,
 * unoccluded lights). */
int shiro_gpu_upload_scene(ShiroGpuContext* ctx, const ShiroSceneDesc* scene);

/* FrameBuffer RenderSampleBatch(const RenderRequest&)
 * (RenderBackend.h:33; CpuPathTracer.cpp:2043-2170) with the plain
 * one-thread-per-path megakernel.  cancel (may be NULL) is polled between
 * launches of at most 2^24 paths while they run (with a flag given, two
 * launches are queued at most, so another host thread may set it mid-frame);
 * a set flag returns SHIRO_ERR_CANCELLED and leaves the AOVs cleared, as the
 * reference discards a cancelled batch (RenderParam.cpp:791-798). */
int shiro_gpu_render(ShiroGpuContext* ctx, const ShiroRenderDesc* request,
                     const volatile int* cancel, ShiroAovs* out);

/* Batched wavefront form: renders `count` requests (each with its own
 * camera, resolution, spp and depth) against the uploaded scene with
 * persistent stage kernels and per-stage queues.  Results equal those of
 * shiro_gpu_render for each request.  cancel (may be NULL) is polled between
 * waves while they run (with a flag given, at most waves-in-flight + 1 waves
 * are queued ahead); a set flag returns SHIRO_ERR_CANCELLED with every
 * request's AOVs cleared, and last_stats().waves counts the waves that ran. */
int shiro_gpu_render_batch(ShiroGpuContext* ctx, const ShiroRenderDesc* requests, uint32_t count,
                           const volatile int* cancel, ShiroAovs* outs);

/* Wavefront tuning (tile of paths in flight per wave, waves in flight, block
 * sizes, register cap, lane refill).  Zero fields leave the current value
 * (use_graph is always taken).  Defaults: 8 388 608 paths per wave, two waves
 * in flight, blocks of 128, graphs on, 128 registers, refill every 4 nodes
 * once 8 lanes are idle.  The autotuner sets these itself when
 * shiro_gpu_autotune is called. */
typedef struct ShiroWavefrontConfig {
    uint32_t paths_in_flight;
    uint32_t extend_block;
    uint32_t shade_block;
    uint32_t shadow_block;
    uint32_t use_graph;
    uint32_t shade_regs;    /* register cap of the shade stage: 128, 96 or 80 */
    uint32_t extend_steps;  /* wide-BVH nodes a lane visits between refills, 1-32 */
    uint32_t refill_idle;   /* idle lanes that make a warp refill, 1-32 */
    uint32_t concurrent_waves; /* 1 to 4: waves in flight at once, each with its own pool of
                                  paths_in_flight paths and its own stream (2 fills one wave's
                                  stage tails with the other's work); 0 leaves the current value */
    uint32_t bin_rays;         /* 1: before each bounce after the first, the closest-hit queue is
                                  counting-sorted into buckets of ray direction octant x origin
                                  cell, so a warp's rays traverse similar nodes; 2: off; 0 leaves
                                  the current value */
    uint32_t bin_shadow;       /* the same for the occlusion queue (buckets of light sample x
                                  octant x origin cell): 1 on, 2 off, 0 leaves the current value */
    uint32_t coop_extend;      /* 1: the closest-hit stage visits one wide node per lane and step
                                  and tests the step's leaf triangles with the whole warp (up to
                                  32 ray-triangle pairs per round); 2: each lane tests its own;
                                  0 leaves the current value.  Hits are identical either way. */
    uint32_t coop_occlude;     /* the same for the occlusion stage: 1 on, 2 off, 0 leaves it */
    uint32_t extend_regs;      /* register cap of the closest-hit stage (per-lane triangle tests):
                                  64, 48 or 40 (more resident warps, some spilling); 0 leaves it */
    uint32_t occlude_regs;     /* the same for the occlusion stage */
    uint32_t occlude_refill;   /* 1 (default): the occlusion stage refills a warp's idle lanes from
                                  its chunk of the queue (extend_steps, refill_idle as in the
                                  closest-hit stage); 2: one ray per lane for 32 entries; 0 leaves it.
                                  Visibility is identical either way. */
} ShiroWavefrontConfig;
int shiro_gpu_get_wavefront_config(const ShiroGpuContext* ctx, ShiroWavefrontConfig* out);
int shiro_gpu_set_wavefront_config(ShiroGpuContext* ctx, const ShiroWavefrontConfig* cfg);
/* Told that pixels [first_pixel, first_pixel + pixel_count) of request
 * `request` (its index in the call) are final in that request's AOV planes. */
typedef void (*ShiroPixelsReady)(void* user, uint32_t request, uint64_t first_pixel, uint64_t pixel_count);

/* shiro_gpu_render_batch that reports finished pixel ranges while later
 * waves still render, so that a caller can consume them (copy a frame out,
 * say) during the render: `ready` is called on the calling thread before
 * the call returns.  Planes the device writes in place (device planes, or
 * page-locked host planes mapped at the same address) are reported wave by
 * wave as each wave finishes; other host planes, and requests without
 * samples or bounces, whole once their planes are written.  Of a call that succeeds
 * every pixel of every request is reported exactly once, the ranges of one
 * request in increasing order; a call that fails or is cancelled stops
 * reporting (ranges reported before held final values; a cancelled call
 * then clears its planes).  `ready` must not call into this context. */
int shiro_gpu_render_batch_ready(ShiroGpuContext* ctx, const ShiroRenderDesc* requests, uint32_t count,
                                 const volatile int* cancel, ShiroAovs* outs, ShiroPixelsReady ready, void* user);

/* Times candidate configurations on `request` and keeps the fastest. */
int shiro_gpu_autotune(ShiroGpuContext* ctx, const ShiroRenderDesc* request, ShiroWavefrontConfig* chosen);

/* Differentiable form.  Parameters live on the device (float32):
 *   base_color [material_count * 3], roughness [material_count],
 *   metallic [material_count], env texels [env_height * env_width * 3] of
 *   dome light 0.
 * shiro_gpu_set_params overrides those material fields / texels of the
 * uploaded scene (and rebuilds the dome importance table when env changes).
 * shiro_gpu_adjoint replays every path of `request` from its QMC seed and
 * accumulates d(sum over pixels of d_beauty . beauty)/d(param) into the
 * gradient buffers (added, not overwritten).  All pointers are device
 * pointers; any may be NULL to skip that parameter group.  Scenes with
 * emitters and opacity cut-outs are covered; a scene with a transmission
 * weight on any material is refused (SHIRO_ERR_UNSUPPORTED_SCENE), as by
 * shiro_gpu_render_frozen. */
int shiro_gpu_set_params(ShiroGpuContext* ctx, const float* base_color, const float* roughness,
                         const float* metallic, const float* env_rgb);
int shiro_gpu_adjoint(ShiroGpuContext* ctx, const ShiroRenderDesc* request, const float* d_beauty,
                      float* d_base_color, float* d_roughness, float* d_metallic, float* d_env_rgb);

/* How shiro_gpu_adjoint replays paths: 1 (default) with the wavefront form -
 * each wave of paths runs its forward stages, which also log every bounce's
 * hits and light-sample visibility, then replays its paths with gradient
 * stages on the same pool and queues (the logged hits instead of tracing
 * again; light-sample and continuation gradients once the vertex's direct
 * light is known); 0 one thread per path (the whole replay, tracing
 * included, in one kernel, after a wavefront pass for the paths' radiance).
 * Both accumulate the same gradients (up to the order of their float
 * atomics).  The wavefront form holds 21 bytes per path slot and bounce of
 * device memory for its logs. */
int shiro_gpu_set_adjoint_form(ShiroGpuContext* ctx, uint32_t wavefront);

/* Frozen-sampling forward of the differentiable form: renders the beauty
 * plane (device pointer, 4 floats per pixel) with every sampling decision,
 * pdf and MIS weight taken from the uploaded scene's parameters and the BSDF
 * values / dome-0 radiance taken from the given parameter arrays (device
 * pointers, NULL = the scene's own).  Central finite differences of this
 * render are exactly the derivative shiro_gpu_adjoint estimates. */
int shiro_gpu_render_frozen(ShiroGpuContext* ctx, const ShiroRenderDesc* request, const float* base_color,
                            const float* roughness, const float* metallic, const float* env_rgb, float* beauty);

/* Per-path debugging / parity probes (device or host arrays per on_device).
 * Primary closest hit of every pixel's camera ray for sample sample_start:
 * prim_out[i] = global triangle index (meshes in order, triangles in order)
 * or 0xffffffff on a miss; t_out[i] = hit distance. */
/* OpenQmcSampler::Next2D (OpenQmcSampler.cpp:110-135; fallback sequence
 * :56-71) on the device for n host tuples (px, py, sample index, branch):
 * out2 receives 2 floats per tuple.  Diagnostic: the sampler the kernels use,
 * for bit-exact checks against the reference's values. */
int shiro_gpu_sample(ShiroGpuContext* ctx, const uint32_t* px, const uint32_t* py, const uint32_t* index,
                     const uint32_t* branch, uint32_t n, float* out2);
int shiro_gpu_primary_hits(ShiroGpuContext* ctx, const ShiroRenderDesc* request, uint32_t* prim_out,
                           float* t_out, uint32_t on_device);
/* Closest hit / occlusion for arbitrary rays: origins, directions [n*3];
 * t_max [n] (FLT_MAX for unbounded).  prim_out, t_out as above;
 * occluded_out[i] = 1 when any hit in [1e-4, t_max]. */
int shiro_gpu_trace_rays(ShiroGpuContext* ctx, const float* origins, const float* directions,
                         const float* t_max, uint32_t n, uint32_t* prim_out, float* t_out,
                         uint32_t* occluded_out);

/* Importance tables of dome texture `env` (the domes that carry a texture,
 * counted in dome order from 0), copied from device memory into the caller's
 * host arrays; any array may be NULL.  row_cdf: h + 1 floats, cond_cdf:
 * h * (w + 1) floats (EnvironmentMap::BuildImportanceTable,
 * EnvironmentMap.cpp:185-236), mass: w * h per-texel probabilities
 * rowMass * columnMass (LatLongPdf, :302-313), alias_threshold / alias_index:
 * w * h entries of the alias table (acceptance threshold as float bits, alias
 * texel).  Diagnostic: lets tests check the tables the kernels sample. */
int shiro_gpu_env_tables(ShiroGpuContext* ctx, uint32_t env, uint32_t* w_out, uint32_t* h_out, float* row_cdf,
                         float* cond_cdf, float* mass, uint32_t* alias_threshold, uint32_t* alias_index);
/* The texel the kernels' dome sampler picks (EnvironmentMap::Sample's row and
 * column, :109-163) for n host 2-D points u2 (u.x, u.y pairs): the alias
 * lookup, or the CDF search when flags has SHIRO_RENDER_ENV_CDF.  texel_out[i]
 * = row * w + column, pdf_out[i] = the reference's pdf of that sample. */
int shiro_gpu_env_sample(ShiroGpuContext* ctx, uint32_t env, uint32_t n, const float* u2, uint32_t flags,
                         uint32_t* texel_out, float* pdf_out);
/* Per-path results of the plain form for listed paths (TracePath,
 * CpuPathTracer.cpp:1650-2017): out[10 i .. 10 i + 9] = radiance rgb, albedo
 * rgb, normal rgb, depth of the path of pixel pixels[i] (y * width + x) with
 * sample index sample_index[i].  Diagnostic: pins differing pixels to paths. */
int shiro_gpu_render_paths(ShiroGpuContext* ctx, const ShiroRenderDesc* request, const uint32_t* pixels, uint32_t n,
                           const uint32_t* sample_index, float* out);

/* Render without allocating device memory.  No counterpart in the reference:
 * this entry point exists for callers that must not allocate device memory
 * while they render - e.g. a process that hands all device memory to its own
 * allocator at start-up, or a render loop that must not stall on the
 * allocator's implicit device synchronisation while other streams run.  It
 * renders exactly like shiro_gpu_render (same kernels and results) but draws
 * the per-path scratch from an array reserved in the library's device image
 * (1 048 576 path records = 48 MiB, held by every device that loads the
 * library until the process exits) and calls no cudaMalloc / cudaFree.
 * Rules: the AOV planes must be device pointers (on_device = 1); a request
 * with sample_count > 1 048 576 is refused (SHIRO_ERR_INVALID_ARGUMENT);
 * all calls share the array, so calls that overlap on the GPU race and must be
 * serialised by the caller.  shiro_gpu_create sets the array up for its device
 * (looks its address up and loads its module and the plain-form kernels), so
 * the device memory this entry point relies on is taken when the context is
 * made, before a caller's allocator claims the rest; if that set-up failed,
 * this entry point returns SHIRO_ERR_CUDA with the reason.  The thread-local
 * memory the kernels use is sized by the CUDA driver at the first launch of a
 * kernel that needs it: a caller that must see no allocation at all renders
 * once with shiro_gpu_render (or this entry point) before claiming the
 * device's memory. */
int shiro_gpu_render_static(ShiroGpuContext* ctx, const ShiroRenderDesc* request, const volatile int* cancel,
                            ShiroAovs* out);

/* Statistics of the last render (for the roofline and tests). */
typedef struct ShiroRenderStats {
    double kernel_ms;           /* device time of all kernels of the last call */
    double path_kernel_ms;      /* device time of the path-tracing kernel(s) alone */
    uint64_t path_kernel_launches;
    uint64_t paths;             /* paths traced */
    uint64_t kernel_launches;   /* kernels launched by the last call */
    uint64_t bvh_nodes;         /* BVH nodes of the uploaded scene */
    uint64_t triangles;         /* triangles of the uploaded scene */
    uint32_t bvh_depth;
    uint32_t bvh_max_leaf;
    uint64_t device_bytes;      /* device memory held by the context */
    /* wavefront stages (filled by an event-timed run, use_graph = 0):
     * 0 generate, 1 extend (closest hit), 2 shade, 3 occlusion rays,
     * 4 resolve, 5 light-sample accumulation and queue bookkeeping */
    double stage_ms[6];
    uint64_t stage_launches[6];
    uint64_t waves;             /* waves of the last wavefront call */
} ShiroRenderStats;
int shiro_gpu_last_stats(const ShiroGpuContext* ctx, ShiroRenderStats* out);

/* Work counts of the estimator, for the algorithmic-bytes roofline: traces
 * every `stride`-th path of `request` with counting kernels (same paths, same
 * decisions as the render) and returns the totals over the traced paths. */
typedef struct ShiroWorkCounts {
    uint64_t paths;
    uint64_t closest_rays;
    uint64_t occlusion_rays;
    uint64_t node_visits;       /* BVH nodes fetched (both kinds of ray) */
    uint64_t tri_tests;         /* triangles fetched and tested */
    uint64_t hits;              /* surface hits shaded */
    uint64_t env_evals;         /* bilinear environment lookups (4 texels) */
    uint64_t env_samples;       /* importance-table lookups */
    uint64_t bsdf_evals;
    uint64_t bsdf_pdfs;
    uint64_t occlusion_node_visits;  /* part of node_visits spent on occlusion rays */
    uint64_t occlusion_tri_tests;    /* part of tri_tests spent on occlusion rays */
} ShiroWorkCounts;
int shiro_gpu_count_work(ShiroGpuContext* ctx, const ShiroRenderDesc* request, uint32_t stride,
                         ShiroWorkCounts* out);

/* ---- device-resident progressive accumulation --------------------------
 * Renderer::FrameAccumulator (Renderer.cpp:47-110) kept in device memory:
 * the per-pixel running sums of a progressive render stay on the GPU, each
 * batch is folded in where it was rendered, and a resolved frame is copied
 * out only when the caller asks for one (instead of one host frame per batch
 * plus the host accumulation of HdShiroRenderParam's worker,
 * RenderParam.cpp:790-806).  The sums use the reference's float32 arithmetic
 * (sum + frame * sampleCount; resolve by 1 / total samples; depth averaged
 * over the samples that hit).  An accumulator belongs to the context it was
 * created on and uses its stream; once the context is destroyed only
 * shiro_gpu_accum_destroy may still be called on it. */
typedef struct ShiroAccumulator ShiroAccumulator;
int shiro_gpu_accum_create(ShiroGpuContext* ctx, ShiroAccumulator** out);
void shiro_gpu_accum_destroy(ShiroAccumulator* acc);
/* FrameAccumulator::Reset (Renderer.cpp:47-58). */
int shiro_gpu_accum_reset(ShiroAccumulator* acc, uint32_t width, uint32_t height);
/* FrameAccumulator::Accumulate (Renderer.cpp:60-84): folds a width x height
 * frame (host or device planes, per frame->on_device) rendered with
 * sample_count samples per pixel; a frame of another size resets the sums
 * first; an empty frame or sample_count 0 is ignored. */
int shiro_gpu_accum_add(ShiroAccumulator* acc, const ShiroAovs* frame, uint32_t width, uint32_t height,
                        uint32_t sample_count);
/* One step of the progressive loop (RenderParam.cpp:790-806): renders the
 * request's batch into device planes (wavefront != 0: the batched wavefront
 * form, else the plain one); unless the batch was cancelled, resets the sums
 * when it starts at sample 0 or nothing is accumulated yet, then folds it in.
 * Returns the render's status (a cancelled batch is not accumulated). */
int shiro_gpu_accum_render(ShiroAccumulator* acc, const ShiroRenderDesc* request, const volatile int* cancel,
                           uint32_t wavefront);
/* The same step in two halves, for callers that decide after the render
 * whether the batch counts (RenderParam.cpp:791-798 reads its cancel flag
 * once the batch returns): _stage renders the batch into the accumulator's
 * pending frame, _commit folds the pending frame in with the rule above
 * (SHIRO_ERR_INVALID_ARGUMENT when nothing is pending).  A new _stage
 * replaces an uncommitted pending frame. */
int shiro_gpu_accum_stage(ShiroAccumulator* acc, const ShiroRenderDesc* request, const volatile int* cancel,
                          uint32_t wavefront);
int shiro_gpu_accum_commit(ShiroAccumulator* acc);
/* FrameAccumulator::Resolve (Renderer.cpp:86-110) into host or device planes
 * (per out->on_device) of the accumulated size; with nothing accumulated the
 * frame is cleared (FrameBuffer::Resize: zeros, depth +inf). */
int shiro_gpu_accum_resolve(ShiroAccumulator* acc, ShiroAovs* out);
/* FrameAccumulator::SampleCount and the accumulated size. */
int shiro_gpu_accum_info(const ShiroAccumulator* acc, uint32_t* sample_count, uint32_t* width, uint32_t* height);

#ifdef __cplusplus
}
#endif

#endif /* SHIRO_GPU_H_ */
