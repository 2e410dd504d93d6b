"""Converged reference images and error measurement.

The reference renders progressively: each batch traces `sampleCount`
consecutive sample indices starting at `sampleStart` and the batches are
averaged per pixel (Renderer.cpp:47-110, CpuPathTracer.cpp:2093-2137).  A
converged image here is the same estimator run for many samples per pixel:
`converged` renders batches of `batch_spp` consecutive sample indices with the
plain GPU form (one CUDA thread per path) and accumulates the batch means in
float64 on the device.  The spread of the batch means estimates the per-pixel
variance of one sample, which turns the difference between an image and the
converged one into z-scores.

These are the measurements behind "equal RMSE": the plain and wavefront forms
trace the same paths, so at equal samples per pixel they have the same error
against the converged image; the CPU tracer traces the same paths too.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

from .abi import Camera, RenderSettings


@dataclass
class Converged:
    mean: "object"        # torch.float64 [H, W, 3], device
    var: "object"         # torch.float64 [H, W, 3], per-sample variance estimate
    spp: int
    first: int            # first sample index
    batch_spp: int


def converged(backend, camera: Camera, settings: RenderSettings, total_spp: int = 65536, batch_spp: int = 256,
              first: int = 0, flags: int = 0) -> Converged:
    """Mean of `total_spp` samples per pixel (sample indices first ..
    first + total_spp - 1) of the uploaded scene, accumulated in float64.

    Keep the indices small (below ~2^18): the sampler's first two dimensions
    are frac(0.5 + a * i) evaluated in float32 (OpenQmcSampler.cpp:56-71), so
    large indices quantise the sub-pixel jitter and bias the image."""
    import torch

    if total_spp % batch_spp or total_spp // batch_spp < 2:
        raise ValueError("total_spp must be a multiple of batch_spp with at least two batches")
    nb = total_spp // batch_spp
    s = torch.zeros((settings.height, settings.width, 3), dtype=torch.float64, device="cuda")
    s2 = torch.zeros_like(s)
    for k in range(nb):
        b = backend.render_device(camera, settings, first + k * batch_spp, batch_spp, flags)[..., :3].double()
        s += b
        s2 += b * b
    mean = s / nb
    var_batch = (s2 / nb - mean * mean).clamp_min(0.0) * (nb / (nb - 1))
    return Converged(mean=mean, var=var_batch * batch_spp, spp=total_spp, first=first, batch_spp=batch_spp)


def rmse(image, ref) -> float:
    """Root mean square difference over the RGB channels of [H, W, >=3] images
    (torch tensors or numpy arrays)."""
    import torch

    a = torch.as_tensor(image)[..., :3].double()
    b = torch.as_tensor(ref)[..., :3].double().to(a.device)
    return float(torch.sqrt(((a - b) ** 2).mean()))


def z_scores(image, spp: int, ref: Converged):
    """Per-pixel, per-channel z-scores of an `spp`-sample estimate against the
    converged image, with the converged image's own variance included."""
    import torch

    a = torch.as_tensor(image)[..., :3].double().to(ref.mean.device)
    sd = torch.sqrt(ref.var / spp + ref.var / ref.spp)
    z = (a - ref.mean) / sd.clamp_min(1e-12)
    return torch.where(sd > 1e-12, z, torch.zeros_like(z))


def expected_mc_rmse(ref: Converged, spp: int) -> float:
    """RMSE a plain Monte-Carlo estimate of `spp` samples would have."""
    return math.sqrt(float((ref.var / spp).mean()))
