// fake_device.cpp - TEST INFRASTRUCTURE: a stand-in for libshiro_gpu.so that
// renders with the CPU oracle (oracle/port), so that the reference's own
// Renderer (src/render/Renderer.cpp) can route requests to the C++ adapter
// GpuBackend on a machine without a GPU.  It implements the C ABI entry
// points the adapter calls; renders go to oracle_scene_render_rows (the CPU
// restatement of the reference tracer), so a frame routed through
// Renderer -> GpuBackend -> this library must equal the reference CPU
// tracer's frame bit for bit.
//
// Environment switches: SHIRO_FAKE_UNAVAILABLE=1 makes shiro_gpu_status
// report no usable device, SHIRO_FAKE_UNSUPPORTED=1 makes
// shiro_gpu_supports_scene decline every scene (both must send the Renderer
// to its CPU tracer, Renderer.cpp:16-31).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/shiro_gpu.h"
#include "../../oracle/port/shiro_oracle.h"

extern "C" {
int shiro_fake_render_calls = 0;
int shiro_fake_uploads = 0;
}

namespace {

bool Flag(const char* name) {
    const char* v = std::getenv(name);
    return v && v[0] == '1';
}

std::string gError;

}  // namespace

struct ShiroGpuContext {
    OracleScene* scene = nullptr;
    std::string error;
};

extern "C" {

int shiro_gpu_status(ShiroBackendStatus* out) {
    if (!out) return SHIRO_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->kind = SHIRO_BACKEND_GPU;
    std::snprintf(out->name, sizeof(out->name), "fake");
    out->uses_gpu = 1;
    out->available = Flag("SHIRO_FAKE_UNAVAILABLE") ? 0u : 1u;
    out->device_count = out->available;
    return SHIRO_OK;
}

int shiro_gpu_create(int, ShiroGpuContext** out) {
    if (!out) return SHIRO_ERR_INVALID_ARGUMENT;
    *out = new ShiroGpuContext();
    return SHIRO_OK;
}

void shiro_gpu_destroy(ShiroGpuContext* ctx) {
    if (!ctx) return;
    if (ctx->scene) oracle_scene_destroy(ctx->scene);
    delete ctx;
}

const char* shiro_gpu_last_error(const ShiroGpuContext* ctx) { return ctx ? ctx->error.c_str() : gError.c_str(); }

int shiro_gpu_supports_scene(const ShiroSceneDesc* scene, char* reason, size_t reason_size) {
    if (reason && reason_size) reason[0] = 0;
    return scene && !Flag("SHIRO_FAKE_UNSUPPORTED") ? 1 : 0;
}

// FNV-1a over the small fields and the mesh arrays (a test stand-in for the
// real signature).
int shiro_gpu_scene_signature(const ShiroSceneDesc* s, uint64_t* out) {
    if (!s || !out) return SHIRO_ERR_INVALID_ARGUMENT;
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    };
    mix(&s->material_count, 4);
    if (s->material_count) mix(s->materials, sizeof(ShiroMaterialDesc) * s->material_count);
    for (uint32_t i = 0; i < s->mesh_count; ++i) {
        const ShiroMeshDesc& m = s->meshes[i];
        mix(&m.vertex_count, 4);
        mix(&m.index_count, 4);
        mix(&m.material_index, 4);
        if (m.positions) mix(m.positions, 12ull * m.vertex_count);
        if (m.indices) mix(m.indices, 4ull * m.index_count);
    }
    for (uint32_t i = 0; i < s->distant_light_count; ++i) mix(&s->distant_lights[i], sizeof(ShiroDistantLightDesc));
    for (uint32_t i = 0; i < s->dome_light_count; ++i) {
        const ShiroDomeLightDesc& d = s->dome_lights[i];
        mix(d.radiance, 48);
        mix(&d.env_width, 8);
        if (d.env_pixels) mix(d.env_pixels, 12ull * d.env_width * d.env_height);
    }
    *out = h;
    return SHIRO_OK;
}

int shiro_gpu_host_alloc(size_t bytes, void** out) {
    if (!out) return SHIRO_ERR_INVALID_ARGUMENT;
    *out = bytes ? std::malloc(bytes) : nullptr;
    return bytes && !*out ? SHIRO_ERR_OUT_OF_MEMORY : SHIRO_OK;
}

void shiro_gpu_host_free(void* ptr) { std::free(ptr); }

int shiro_gpu_upload_scene(ShiroGpuContext* ctx, const ShiroSceneDesc* scene) {
    if (!ctx || !scene) return SHIRO_ERR_INVALID_ARGUMENT;
    if (ctx->scene) oracle_scene_destroy(ctx->scene);
    ctx->scene = nullptr;
    const int rc = oracle_scene_create(scene, &ctx->scene);
    if (rc != 0) ctx->error = "oracle scene build failed";
    ++shiro_fake_uploads;
    return rc;
}

int shiro_gpu_render_batch(ShiroGpuContext* ctx, const ShiroRenderDesc* reqs, uint32_t count, const volatile int* cancel,
                           ShiroAovs* outs) {
    if (!ctx || !ctx->scene) return SHIRO_ERR_NO_SCENE;
    for (uint32_t r = 0; r < count; ++r) {
        if (cancel && *cancel) return SHIRO_ERR_CANCELLED;
        if (outs[r].on_device) return SHIRO_ERR_INVALID_ARGUMENT;
        const int64_t n = oracle_scene_render_rows(ctx->scene, &reqs[r], 0, reqs[r].settings.height, &outs[r]);
        if (n < 0) return static_cast<int>(n);
        ++shiro_fake_render_calls;
    }
    return SHIRO_OK;
}

int shiro_gpu_render_batch_ready(ShiroGpuContext* ctx, const ShiroRenderDesc* reqs, uint32_t count,
                                 const volatile int* cancel, ShiroAovs* outs, ShiroPixelsReady ready, void* user) {
    const int rc = shiro_gpu_render_batch(ctx, reqs, count, cancel, outs);
    if (rc != SHIRO_OK) return rc;
    for (uint32_t r = 0; r < count; ++r) {
        const uint64_t px = static_cast<uint64_t>(reqs[r].settings.width) * reqs[r].settings.height;
        if (px) ready(user, r, 0, px);
    }
    return SHIRO_OK;
}

// The device accumulator is not part of what the Renderer calls.
int shiro_gpu_accum_create(ShiroGpuContext*, ShiroAccumulator**) { return SHIRO_ERR_UNSUPPORTED_SCENE; }
void shiro_gpu_accum_destroy(ShiroAccumulator*) {}
int shiro_gpu_accum_stage(ShiroAccumulator*, const ShiroRenderDesc*, const volatile int*, uint32_t) {
    return SHIRO_ERR_UNSUPPORTED_SCENE;
}
int shiro_gpu_accum_commit(ShiroAccumulator*) { return SHIRO_ERR_UNSUPPORTED_SCENE; }
int shiro_gpu_accum_info(const ShiroAccumulator*, uint32_t*, uint32_t*, uint32_t*) { return SHIRO_ERR_UNSUPPORTED_SCENE; }
int shiro_gpu_accum_resolve(ShiroAccumulator*, ShiroAovs*) { return SHIRO_ERR_UNSUPPORTED_SCENE; }

}  // extern "C"
