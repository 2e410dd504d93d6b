// adjoint.cu - differentiable form (placeholder until implemented).
#include "context.h"

namespace shiro_gpu {

int adjoint_run(ContextImpl* ctx, const ShiroRenderDesc*, const float*, float*, float*, float*, float*) {
    return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "adjoint form not built");
}
int adjoint_set_params(ContextImpl* ctx, const float*, const float*, const float*, const float*) {
    return fail(ctx, SHIRO_ERR_INVALID_ARGUMENT, "adjoint form not built");
}
void adjoint_free(ContextImpl*) {}

}  // namespace shiro_gpu
