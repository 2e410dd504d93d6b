"""Inverse rendering with the differentiable form.

Recovers the per-material base colour, roughness and metalness and the
texels of dome light 0 from images of several views: target images are
rendered with the true parameters (more samples, disjoint sample indices),
the optimisation starts from neutral parameters and minimises the mean
squared error over all views with Adam.  Gradients come from the adjoint path
replay (autograd.render), decorrelated from the forward render's samples.  Material parameters are optimised directly and
projected back into their valid ranges after each step; environment texels
are optimised as logarithms (a step is a relative change of radiance).

Run as a module for the 16-view field-scene configuration:

    python -m shiro_gb300.inverse [--steps 200] [--views 16] [--size 512]

which prints one JSON line (parameter RMSE before / after, loss, gradient
throughput).
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import time
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import scenes
from .abi import Camera, RenderSettings, Scene


def orbit_views(count: int, radius: float, height: float, target=(0.0, 0.0, 0.0), seed: int = 0,
                aspect: float = 1.0) -> List[Camera]:
    """`count` cameras on a jittered ring around `target`."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        az = 2.0 * math.pi * (k + rng.uniform(0.0, 0.5)) / count
        h = height * rng.uniform(0.7, 1.3)
        r = radius * rng.uniform(0.8, 1.1)
        out.append(scenes.look_at((r * math.sin(az), h, r * math.cos(az)), target, 45.0, aspect))
    return out


@dataclass
class InverseResult:
    steps: int
    views: int
    paths_per_step: int
    seconds: float
    loss: List[float] = field(default_factory=list)
    rmse_start: dict = field(default_factory=dict)
    rmse_end: dict = field(default_factory=dict)

    @property
    def steps_per_s(self) -> float:
        return self.steps / max(self.seconds, 1e-9)


def _param_rmse(p, truth) -> dict:
    import torch

    out = {}
    for k in ("base_color", "roughness", "metallic"):
        out[k] = float(torch.sqrt(((p[k] - truth[k]) ** 2).mean()))
    out["env_log"] = float(torch.sqrt(((p["env_log"] - truth["env_log"]) ** 2).mean()))
    return out


PARAMS = ("base_color", "roughness", "metallic", "env")


def inverse_render(backend, scene: Scene, views: List[Camera], settings: RenderSettings, steps: int = 200,
                   lr: float = 1e-2, target_spp: int = 64, log_every: int = 0,
                   optimize: tuple = PARAMS, decorrelate: bool = True, autotune: bool = False) -> InverseResult:
    """Optimises the parameter groups `optimize` (all material parameters
    and the dome texels of `scene` by default; the others keep their true
    values) against targets rendered from `views`.  With both the lighting
    and the albedo unknown the problem is ambiguous (a brighter environment
    and darker materials give the same images), so the image loss falls
    faster than the parameter error.  `decorrelate` replays the adjoint from
    sample indices independent of the forward render's (see autograd).
    `autotune` picks the wavefront configuration (pool size, waves in flight,
    block sizes) on one view's forward request before the first step; off by
    default: for the 512x512 16-spp views it picks two waves of 2 M paths in
    flight, which suits the forward render but made the whole step (forward
    + adjoint) slower than the default single 4 M-path wave (2.0 vs 3.3
    steps/s)."""
    import torch

    from .autograd import render

    backend.upload_scene(scene, force=True)
    if autotune:
        backend.autotune(scene, views[0], settings)
    mats = scene.materials
    truth = dict(
        base_color=torch.tensor([m.base_color for m in mats], dtype=torch.float32, device="cuda"),
        roughness=torch.tensor([m.roughness for m in mats], dtype=torch.float32, device="cuda"),
        metallic=torch.tensor([m.metallic for m in mats], dtype=torch.float32, device="cuda"),
    )
    env_true = torch.tensor(scene.dome_lights[0].env, dtype=torch.float32, device="cuda")
    truth["env_log"] = torch.log(env_true.clamp_min(1e-4))
    # targets: true parameters, more samples, sample indices disjoint from the
    # optimisation's (all indices stay small: the sampler's first dimensions
    # lose sub-pixel resolution at large indices)
    backend.set_params(truth["base_color"], truth["roughness"], truth["metallic"], env_true)
    tst = dataclasses.replace(settings, samples_per_pixel=target_spp)
    targets = [backend.render_device(cam, tst, 0, target_spp)[..., :3].clone() for cam in views]

    # neutral start for the unknown groups, the truth for the known ones
    p = dict(
        base_color=torch.full_like(truth["base_color"], 0.5),
        roughness=torch.full_like(truth["roughness"], 0.5),
        metallic=torch.full_like(truth["metallic"], 0.5),
        env_log=torch.full_like(truth["env_log"], float(truth["env_log"].mean())),
    )
    for k in ("base_color", "roughness", "metallic"):
        if k not in optimize:
            p[k] = truth[k].clone()
    if "env" not in optimize:
        p["env_log"] = truth["env_log"].clone()
    unknown = [p[k] for k in ("base_color", "roughness", "metallic") if k in optimize]
    if "env" in optimize:
        unknown.append(p["env_log"])
    for t in unknown:
        t.requires_grad_()
    res = InverseResult(steps=steps, views=len(views),
                        paths_per_step=len(views) * settings.width * settings.height * settings.samples_per_pixel,
                        seconds=0.0)
    res.rmse_start = _param_rmse({k: v.detach() for k, v in p.items()}, truth)
    opt = torch.optim.Adam(unknown, lr=lr)
    spp = settings.samples_per_pixel
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(steps):
        opt.zero_grad(set_to_none=True)
        total = 0.0
        env = torch.exp(p["env_log"]) if "env" in optimize else None  # None: keep the resident texels
        for v, (cam, tgt) in enumerate(zip(views, targets)):
            start = target_spp + 2 * (it * len(views) + v) * spp
            img = render(backend, cam, settings, p["base_color"], p["roughness"], p["metallic"], env,
                         sample_start=start, adjoint_sample_start=start + spp if decorrelate else None)
            loss = ((img[..., :3] - tgt) ** 2).mean() / len(views)
            loss.backward(retain_graph=v + 1 < len(views) and "env" in optimize)
            total += float(loss.detach())
        opt.step()
        with torch.no_grad():
            p["base_color"].clamp_(0.0, 1.0)
            p["roughness"].clamp_(0.02, 1.0)
            p["metallic"].clamp_(0.0, 1.0)
            p["env_log"].clamp_(-9.0, 9.0)
        res.loss.append(total)
        if log_every and (it % log_every == 0 or it + 1 == steps):
            print(f"step {it:4d} loss {total:.6g}", flush=True)
    torch.cuda.synchronize()
    res.seconds = time.perf_counter() - t0
    res.rmse_end = _param_rmse({k: v.detach() for k, v in p.items()}, truth)
    return res


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--views", type=int, default=16)
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-2)
    ap.add_argument("--env-width", type=int, default=1024)
    ap.add_argument("--log-every", type=int, default=20)
    ap.add_argument("--autotune", action="store_true", help="autotune the wavefront configuration on one view first")
    a = ap.parse_args(argv)
    from .backend import GpuBackend

    scene = scenes.field_scene(env_width=a.env_width, env_height=a.env_width // 2)
    st = RenderSettings(width=a.size, height=a.size, samples_per_pixel=a.spp, max_depth=a.depth, diffuse_depth=a.depth,
                        specular_depth=a.depth, dome_light_samples=1, background_visible=True, backend=1)
    views = orbit_views(a.views, 30.0, 12.0, seed=11)
    with GpuBackend(0) as gpu:
        r = inverse_render(gpu, scene, views, st, steps=a.steps, lr=a.lr, log_every=a.log_every,
                           autotune=a.autotune)
        wf_config = gpu.wavefront_config()
    line = {"metric": "inverse rendering: Adam steps/s (forward + adjoint over all views)",
            "value": r.steps_per_s, "unit": "steps/s", "views": r.views, "steps": r.steps,
            "paths_per_step": r.paths_per_step, "gradient_views_per_s": r.steps_per_s * r.views,
            "Mpaths_per_s_forward_plus_adjoint": r.steps_per_s * r.paths_per_step / 1e6, "seconds": r.seconds,
            "loss_first": r.loss[0], "loss_last": r.loss[-1], "param_rmse_start": r.rmse_start,
            "param_rmse_end": r.rmse_end, "unknowns": {"materials": len(scene.materials),
                                                       "env_texels": a.env_width * (a.env_width // 2) * 3},
            "config": {"scene": "field 1310720 tris", "size": a.size, "spp": a.spp, "depth": a.depth, "lr": a.lr,
                       "wavefront_config": wf_config}}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
