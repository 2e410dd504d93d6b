"""Replica host logic on CPU: sample-range partition, the reference's frame
accumulation, and the host-staged combination over two gloo ranks.

The ranks render their sample ranges with the CPU oracle (the same paths the
GPU traces); rank 0's combined frame must equal the frame accumulated from
the same batches in one process, bit for bit, and agree with a single render
of all samples to float rounding.
"""
import os
import socket
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_sample_range_partitions():
    from shiro_gb300.replicas import sample_range

    for world in (1, 2, 3, 4, 8):
        for count in (0, 1, 5, 16, 64, 67):
            got = [sample_range(r, world, 100, count) for r in range(world)]
            assert sum(c for _, c in got) == count
            nxt = 100
            for first, c in got:
                assert first == nxt
                nxt += c
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        sample_range(2, 2, 0, 4)


def test_accumulator_semantics():
    """Known answers of FrameAccumulator (Renderer.cpp:60-110): weighted
    means, depth averaged over the batches that hit, +inf without hits."""
    from shiro_gb300.abi import FrameBuffer
    from shiro_gb300.replicas import accumulate

    a, b = FrameBuffer(2, 1), FrameBuffer(2, 1)
    a.beauty[:] = [[1, 2, 3, 1], [0, 0, 0, 0]]
    b.beauty[:] = [[3, 2, 1, 0], [4, 4, 4, 1]]
    a.albedo[:] = 0.5
    b.albedo[:] = 0.25
    a.depth[:] = [2.0, np.inf]
    b.depth[:] = [5.0, np.inf]
    out = accumulate([a, b], [1, 3])
    np.testing.assert_array_equal(out.beauty[0], np.float32([2.5, 2.0, 1.5, 0.25]))
    np.testing.assert_array_equal(out.beauty[1], np.float32([3.0, 3.0, 3.0, 0.75]))
    np.testing.assert_array_equal(out.albedo, np.full((2, 3), 0.3125, np.float32))
    assert out.depth[0] == np.float32((2.0 * 1 + 5.0 * 3) / 4) and np.isinf(out.depth[1])
    empty = accumulate([a], [0])
    assert (empty.beauty == 0).all()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _workload():
    from shiro_gb300 import scenes

    return scenes.sphere_workload(16, 12, 8, 3, env_width=32, env_height=16)


def _rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    import oracle
    from oracle import api
    from shiro_gb300.replicas import combine, sample_range

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = _workload()
        st = w.settings
        first, count = sample_range(rank, world, 0, st.samples_per_pixel)
        ck = oracle.port_checker()
        fb = api.render(ck, w.scene, w.camera, st, first, count)
        out = combine(fb, count)
        if rank == 0:
            np.savez(out_path, beauty=out.beauty, albedo=out.albedo, normal=out.normal, depth=out.depth)
        else:
            assert out is None
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine():
    import torch.multiprocessing as mp

    import oracle
    from oracle import api
    from shiro_gb300.replicas import accumulate, sample_range

    oracle.build_port()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "combined.npz")
        mp.start_processes(_rank_main, args=(2, _free_port(), path), nprocs=2, join=True, start_method="spawn")
        got = np.load(path)
    w = _workload()
    st = w.settings
    ck = oracle.port_checker()
    parts = [sample_range(r, 2, 0, st.samples_per_pixel) for r in range(2)]
    frames = [api.render(ck, w.scene, w.camera, st, f, c) for f, c in parts]
    want = accumulate(frames, [c for _, c in parts])
    for k in ("beauty", "albedo", "normal", "depth"):
        assert np.array_equal(got[k], getattr(want, k)), k
    full = api.render(ck, w.scene, w.camera, st, 0, st.samples_per_pixel)
    np.testing.assert_allclose(got["beauty"], full.beauty, rtol=1e-5, atol=1e-6)
    hit = np.isfinite(full.depth)
    assert np.array_equal(np.isfinite(got["depth"]), hit)


class _LinearRenderer:
    """A stand-in backend whose image is linear in its parameters: pixel p's
    sample s has radiance a * phi(p, s) (per channel, phi a fixed hash), so a
    sample range's image and its adjoint have closed forms."""

    def __init__(self, pixels=6):
        self.pixels = pixels

    def phi(self, first, count):
        s = torch.arange(first, first + count, dtype=torch.float64)
        p = torch.arange(self.pixels, dtype=torch.float64)
        c = torch.arange(3, dtype=torch.float64)
        return torch.sin(p[:, None, None] * 1.3 + s[None, :, None] * 0.7 + c[None, None, :] * 2.1) + 1.5

    def render(self, a, first, count):  # [pixels, 4]: rgb = a * mean_s phi, alpha 0
        img = torch.zeros(self.pixels, 4, dtype=torch.float32)
        img[:, :3] = (a.double() * self.phi(first, count).mean(1)).float()
        return img

    def adjoint(self, camera, settings, d_beauty, grads, first, count, flags):
        g = (d_beauty[:, :3].double() * self.phi(first, count).mean(1)).sum(0)
        grads["a"] += g.float()


def _grad_rank_main(rank, world, port, out_path):
    import torch.distributed as dist

    from shiro_gb300.abi import RenderSettings
    from shiro_gb300.replicas import allreduce_gradients, allreduce_image, replica_gradient, sample_range

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        st = RenderSettings(width=3, height=2, samples_per_pixel=7)
        be = _LinearRenderer()
        a = torch.tensor([0.3, 0.8, 0.5])
        first, count = sample_range(rank, world, 4, st.samples_per_pixel)
        img = allreduce_image(be.render(a, first, count), count, st.samples_per_pixel)
        target = torch.full((6, 4), 0.9)
        d = 2.0 * (img - target) / target.numel()
        d[:, 3] = 0.0
        grads = {"a": torch.full((3,), 0.25)}  # what the buffer held before stays, once
        replica_gradient(be, None, st, d, grads, sample_start=4)
        mixed = {"x": torch.full((2, 2), float(rank + 1)), "y": torch.arange(3.0) * (rank + 1), "z": None}
        allreduce_gradients(mixed)
        np.savez(out_path % rank, img=img.numpy(), grad=grads["a"].numpy(), x=mixed["x"].numpy(), y=mixed["y"].numpy())
    finally:
        dist.destroy_process_group()


def test_three_gloo_ranks_replica_gradient():
    """The differentiable form over replicas (three gloo ranks, 7 samples split
    3 / 2 / 2): every rank ends with the whole job's image and with the
    gradient of one adjoint over all samples, gradient buffers summed in one
    host-staged all-reduce and added to what the buffers held."""
    import torch.multiprocessing as mp

    world = 3
    with tempfile.TemporaryDirectory() as dname:
        path = os.path.join(dname, "rank%d.npz")
        mp.start_processes(_grad_rank_main, args=(world, _free_port(), path), nprocs=world, join=True,
                           start_method="spawn")
        got = [np.load(path % r) for r in range(world)]
    be = _LinearRenderer()
    a = torch.tensor([0.3, 0.8, 0.5])
    img = be.render(a, 4, 7)
    d = 2.0 * (img - 0.9) / img.numel()
    d[:, 3] = 0.0
    want = {"a": torch.zeros(3)}
    be.adjoint(None, None, d, want, 4, 7, 0)
    for g in got:
        np.testing.assert_allclose(g["img"], img.numpy(), rtol=1e-6, atol=1e-7)
        np.testing.assert_allclose(g["grad"], want["a"].numpy() + 0.25, rtol=1e-5, atol=1e-7)
        assert np.array_equal(g["x"], np.full((2, 2), 6.0, np.float32))
        assert np.array_equal(g["y"], np.arange(3.0, dtype=np.float32) * 6.0)
