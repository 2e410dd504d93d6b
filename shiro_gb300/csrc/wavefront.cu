// wavefront.cu - batched wavefront form (placeholder until implemented).
#include "context.h"

namespace shiro_gpu {

int wavefront_render(ContextImpl* ctx, const ShiroRenderDesc*, uint32_t, const volatile int*, ShiroAovs*) {
    return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "wavefront form not built");
}
void wavefront_free(ContextImpl*) {}
int wavefront_get_config(const ContextImpl*, ShiroWavefrontConfig* out) {
    *out = ShiroWavefrontConfig{};
    return SHIRO_OK;
}
int wavefront_set_config(ContextImpl*, const ShiroWavefrontConfig*) { return SHIRO_OK; }
int wavefront_autotune(ContextImpl* ctx, const ShiroRenderDesc*, ShiroWavefrontConfig*) {
    return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "wavefront form not built");
}

}  // namespace shiro_gpu
