"""torch.autograd binding of the differentiable form.

``render(backend, camera, settings, base_color, roughness, metallic, env)``
returns the beauty image [H, W, 4] as a differentiable function of the
per-material base colour [M, 3], roughness [M], metalness [M] and the texels
[H_env, W_env, 3] of dome light 0.  The forward renders with the batched
wavefront form (or the plain form) after writing the parameters into the
resident scene; the backward runs the
adjoint path replay (shiro_gpu_adjoint), which follows every path again from
its QMC seed.  The wavefront forward keeps the paths the backward replays on
the device - their radiance records and hit / visibility logs
(SHIRO_RENDER_KEEP_PATHS) - so the backward does not run the forward stages
a second time: its own paths when the backward replays the forward's
samples, else the replayed sample range, rendered in the same call as a
second request.

For a loss that is non-linear in the image (an L2 loss), replaying the same
samples in the backward pass as in the forward one correlates the upstream
gradient with the image noise: the expected gradient then also carries the
derivative of the image variance, which with bright environments pushes
materials darker.  `adjoint_sample_start` replays an independent range of
sample indices instead (a decorrelated gradient estimate).
"""
from __future__ import annotations

import torch

from .abi import RENDER_KEEP_PATHS, Camera, RenderSettings


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, base_color, roughness, metallic, env, backend, camera, settings, sample_start, flags, adj_start,
                wavefront):
        tensors = [t.detach().contiguous().float() if t is not None else None
                   for t in (base_color, roughness, metallic, env)]
        backend.set_params(*tensors)
        also = adj_start if wavefront and adj_start is not None and adj_start != sample_start else None
        beauty = backend.render_device(camera, settings, sample_start, settings.samples_per_pixel,
                                       flags | (RENDER_KEEP_PATHS if wavefront else 0), wavefront=wavefront,
                                       also_start=also)
        ctx.backend = backend
        ctx.camera = camera
        ctx.settings = settings
        ctx.sample_start = sample_start if adj_start is None else adj_start
        ctx.flags = flags
        ctx.shapes = [None if t is None else t.shape for t in (base_color, roughness, metallic, env)]
        return beauty

    @staticmethod
    def backward(ctx, d_beauty):
        grads = {}
        names = ("base_color", "roughness", "metallic", "env")
        for name, shape, need in zip(names, ctx.shapes, ctx.needs_input_grad[:4]):
            if shape is not None and need:
                grads[name] = torch.zeros(shape, dtype=torch.float32, device="cuda")
        ctx.backend.adjoint(ctx.camera, ctx.settings, d_beauty.contiguous().float(), grads, ctx.sample_start,
                            ctx.settings.samples_per_pixel, ctx.flags)
        return tuple(grads.get(n) for n in names) + (None, None, None, None, None, None, None)


def render(backend, camera: Camera, settings: RenderSettings, base_color, roughness, metallic, env=None,
           sample_start: int = 0, flags: int = 0, adjoint_sample_start=None, wavefront: bool = True):
    """Differentiable render of the backend's uploaded scene (see module doc).
    The forward runs the batched wavefront form (wavefront=True, the faster
    one; its frames equal the plain form's bit for bit) or the plain
    one-thread-per-path form."""
    return _Render.apply(base_color, roughness, metallic, env, backend, camera, settings, sample_start, flags,
                         adjoint_sample_start, wavefront)
