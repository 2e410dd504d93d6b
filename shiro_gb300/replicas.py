"""Replicas: one process per GPU, each rendering its own sample range.

Paths are independent, so the frame shards by sample index with no exchange
on the data path: rank r renders the pixels' samples
[sampleStart + offset_r, sampleStart + offset_r + count_r) and the ranks'
frame buffers are combined once at the end, host-staged (device-to-host copy,
gather to rank 0 over a CPU process group, accumulation on the host).

The differentiable form shards the same way: each rank renders and replays
its own sample range, the whole job's image is the ranks' images weighted by
their sample counts (`allreduce_image`), and one host-staged all-reduce of
the gradient buffers per step sums the ranks' adjoints (`replica_gradient`).

The combination is the reference's progressive accumulation
(Renderer::FrameAccumulator, src/render/Renderer.cpp:47-110) applied to the
ranks' frames in rank order: beauty / albedo / normal weighted by the sample
count, depth averaged over the frames that hit.  The arithmetic is float32 in
the accumulator's order, so the combined frame equals the one the reference
accumulator would produce from the same batches.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np

from .abi import FrameBuffer


def sample_range(rank: int, world: int, sample_start: int, sample_count: int) -> Tuple[int, int]:
    """(first sample index, count) of `rank`: consecutive ranges in rank
    order, the first sample_count % world ranks taking one extra sample."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(sample_count, world)
    count = base + (1 if rank < extra else 0)
    first = sample_start + rank * base + min(rank, extra)
    return first, count


class FrameAccumulator:
    """Restatement of Renderer::FrameAccumulator (Renderer.cpp:47-110)."""

    def __init__(self):
        self.width = self.height = 0
        self.samples = 0

    def reset(self, width: int, height: int):  # :47-58
        self.width, self.height = width, height
        self.samples = 0
        n = width * height
        self.beauty = np.zeros((n, 4), np.float32)
        self.albedo = np.zeros((n, 3), np.float32)
        self.normal = np.zeros((n, 3), np.float32)
        self.depth_sum = np.zeros(n, np.float32)
        self.depth_samples = np.zeros(n, np.uint32)

    def accumulate(self, fb: FrameBuffer, sample_count: int):  # :60-84
        if fb.width == 0 or fb.height == 0 or sample_count == 0:
            return
        if fb.width != self.width or fb.height != self.height:
            self.reset(fb.width, fb.height)
        w = np.float32(sample_count)
        self.beauty = self.beauty + fb.beauty.reshape(-1, 4) * w
        self.albedo = self.albedo + fb.albedo.reshape(-1, 3) * w
        self.normal = self.normal + fb.normal.reshape(-1, 3) * w
        d = fb.depth.reshape(-1)
        hit = d < np.float32(np.inf)
        self.depth_sum = np.where(hit, self.depth_sum + np.where(hit, d, 0).astype(np.float32) * w, self.depth_sum)
        self.depth_samples = self.depth_samples + np.where(hit, np.uint32(sample_count), np.uint32(0))
        self.samples += sample_count

    def resolve(self) -> FrameBuffer:  # :86-110
        out = FrameBuffer(self.width, self.height)
        if self.samples == 0:
            return out
        inv = np.float32(1.0) / np.float32(self.samples)
        out.beauty[:] = (self.beauty * inv).reshape(out.beauty.shape)
        out.albedo[:] = (self.albedo * inv).reshape(out.albedo.shape)
        out.normal[:] = (self.normal * inv).reshape(out.normal.shape)
        has = self.depth_samples > 0
        with np.errstate(divide="ignore", invalid="ignore"):
            dep = np.where(has, self.depth_sum / self.depth_samples.astype(np.float32), np.float32(np.inf))
        out.depth[:] = dep.astype(np.float32).reshape(out.depth.shape)
        return out


def accumulate(frames: Sequence[FrameBuffer], counts: Sequence[int]) -> FrameBuffer:
    acc = FrameAccumulator()
    for fb, n in zip(frames, counts):
        acc.accumulate(fb, n)
    return acc.resolve()


def _planes(fb: FrameBuffer):
    import torch

    return torch.from_numpy(np.concatenate([fb.beauty.reshape(-1), fb.albedo.reshape(-1), fb.normal.reshape(-1),
                                            fb.depth.reshape(-1)]).astype(np.float32))


def _from_planes(flat, width: int, height: int) -> FrameBuffer:
    n = width * height
    a = flat.numpy()
    fb = FrameBuffer(width, height)
    fb.beauty[:] = a[:4 * n].reshape(fb.beauty.shape)
    fb.albedo[:] = a[4 * n:7 * n].reshape(fb.albedo.shape)
    fb.normal[:] = a[7 * n:10 * n].reshape(fb.normal.shape)
    fb.depth[:] = a[10 * n:11 * n].reshape(fb.depth.shape)
    return fb


def combine(fb: FrameBuffer, sample_count: int, group=None, dst: int = 0):
    """Host-staged combination of every rank's frame: gathers the AOV planes
    and sample counts to `dst` over `group` (a CPU-capable process group,
    e.g. gloo) and returns the accumulated frame there (None elsewhere)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    flat = _planes(fb)
    cnt = torch.tensor([sample_count], dtype=torch.int64)
    gathered = [torch.empty_like(flat) for _ in range(world)] if rank == dst else None
    counts = [torch.empty_like(cnt) for _ in range(world)] if rank == dst else None
    dist.gather(flat, gathered, dst=dst, group=group)
    dist.gather(cnt, counts, dst=dst, group=group)
    if rank != dst:
        return None
    frames: List[FrameBuffer] = [_from_planes(g, fb.width, fb.height) for g in gathered]
    return accumulate(frames, [int(c.item()) for c in counts])


def _host_allreduce(flat, group=None):
    """Sums a flat float32 tensor over the ranks of `group` (a CPU-capable
    process group), staged through host memory; returns it on its device."""
    import torch.distributed as dist

    host = flat.detach().to("cpu", copy=True)
    dist.all_reduce(host, op=dist.ReduceOp.SUM, group=group)
    return host.to(flat.device)


def allreduce_image(beauty, sample_count: int, total: int, group=None):
    """The whole job's image on every rank: this rank's image (the mean of
    its `sample_count` samples) weighted by sample_count / total and summed
    over the ranks.  Returns a tensor shaped and placed like `beauty`."""
    w = float(sample_count) / float(total) if total else 0.0
    return _host_allreduce((beauty.float() * w).reshape(-1), group).reshape(beauty.shape)


def allreduce_gradients(grads: dict, group=None) -> dict:
    """Sums every rank's gradient tensors in place: all groups in one
    host-staged all-reduce (the one exchange of a replica step)."""
    import torch

    keys = [k for k in sorted(grads) if grads[k] is not None]
    if not keys:
        return grads
    flat = torch.cat([grads[k].detach().reshape(-1).float() for k in keys])
    flat = _host_allreduce(flat, group)
    off = 0
    for k in keys:
        n = grads[k].numel()
        grads[k].copy_(flat[off:off + n].reshape(grads[k].shape))
        off += n
    return grads


def replica_gradient(backend, camera, settings, d_beauty, grads: dict, group=None, sample_start: int = 0,
                     sample_count=None, flags: int = 0) -> dict:
    """Adds the adjoint of the whole job's image into `grads` on every rank
    (as one adjoint over all samples adds it): this rank replays its sample
    range (`sample_range`) with d_beauty weighted by its share of the
    samples, so each path carries d_beauty / total, into zeroed buffers; the
    ranks' buffers are summed (`allreduce_gradients`) and added to `grads`."""
    import torch
    import torch.distributed as dist

    total = settings.samples_per_pixel if sample_count is None else sample_count
    first, count = sample_range(dist.get_rank(group), dist.get_world_size(group), sample_start, total)
    local = {k: torch.zeros_like(v) for k, v in grads.items() if v is not None}
    if count:
        backend.adjoint(camera, settings, d_beauty * (float(count) / float(total)), local, first, count, flags)
    allreduce_gradients(local, group)
    for k, v in local.items():
        grads[k] += v
    return grads
