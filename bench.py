#!/usr/bin/env python
"""Throughput benchmark of the GB300 path-tracing backend.

Workload (default): the 1M-triangle field scene at 1080p - 256 noise-displaced
icospheres (1 310 720 triangles) + a 50x50 ground quad, 64 standard_surface
materials, 2048x1024 HDRI dome + one directional light, 1920x1080, 64 spp,
max depth 12.  One step renders the whole frame (132 710 400 paths).

Metric: Mpaths/s (whole job).  ``value`` is timed with CUDA events on the
render stream with the scene resident in HBM and the AOVs written to device
memory; ``e2e`` goes through the public API (GpuBackend.render with host
FrameBuffer planes), so the device->host copy of the four AOV planes is inside
the timed region.  Between timed steps L2 is flushed (a 512 MiB memset).

--impl reference times the reference's CPU path on the host cores: the CPU
restatement of CpuPathTracer (oracle/port; the reference's own sources are not
present on the GPU machine) with every host thread, on a bounded sample of rows of
the same frame.

Multi-GPU (torchrun): paths are independent, so every rank renders the full
frame with its own sample range (sampleStart = rank * spp): replicas with no
data-path collective, weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Mpaths/s 1080p 1M-tri (plain vs wavefront) at equal RMSE; adjoint grads/s"
UNIT = "Mpaths/s"

# Bytes moved per unit of counted work in this backend's layout (the
# algorithmic-bytes model of the roofline): a binary node (64) or wide node
# (80), a triangle (48), a hit (its 64-byte shading record + the 276-byte
# material), a bilinear environment lookup (4 texels), an environment sample
# (alias entry + per-texel sample record), the plain form's path record.
BYTES = dict(node=64, tri=48, hit=64 + 276, env_eval=4 * 16, env_sample=8 + 32, record=2 * 48)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", choices=["field", "sphere"], default="field")
    p.add_argument("--form", choices=["auto", "plain", "wavefront"], default="auto")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--width", type=int, default=0, help="override the frame width (profiling cases)")
    p.add_argument("--height", type=int, default=0)
    p.add_argument("--spp", type=int, default=0)
    p.add_argument("--no-adjoint", action="store_true")
    p.add_argument("--bvh-width", type=int, choices=[0, 2, 8], default=0,
                   help="2 binary, 8 compressed 8-wide BVH, 0 each form its faster one (wavefront: wide, plain: binary)")
    p.add_argument("--no-rmse", action="store_true", help="skip the equal-RMSE check against a converged image")
    p.add_argument("--no-batch", action="store_true", help="skip the 48-request batch measurement")
    p.add_argument("--no-autotune", action="store_true", help="keep the current wavefront configuration")
    p.add_argument("--adjoint-only", type=int, default=0, metavar="SIZE",
                   help="only the adjoint measurement, on a SIZE x SIZE frame (profiling cases); prints its JSON")
    p.add_argument("--adjoint-form", choices=["wavefront", "thread"], default="wavefront",
                   help="adjoint replay: wavefront stages (default) or one thread per path")
    p.add_argument("--wf-config", default="",
                   help="wavefront configuration to set before measuring (with --no-autotune: the one measured), "
                        "e.g. paths_in_flight=33554432,concurrent_waves=2")
    return p.parse_args()


def workload(name: str, args=None):
    from shiro_gb300 import scenes

    if name == "field":
        w = scenes.field_workload(1920, 1080, 64, 12)
    else:
        w = scenes.sphere_workload(256, 256, 16, 8)
    if args is not None and (args.width or args.height or args.spp):
        s = w.settings
        s.width = args.width or s.width
        s.height = args.height or s.height
        s.samples_per_pixel = args.spp or s.samples_per_pixel
        w.camera.aspect_ratio = s.width / s.height
        w.name += f" (profiling case {s.width}x{s.height} {s.samples_per_pixel}spp)"
    return w


def workload_config(w, flush: str) -> dict:
    s = w.settings
    return {"workload": w.name, "triangles": int(w.scene.triangle_count), "width": s.width, "height": s.height,
            "spp": s.samples_per_pixel, "max_depth": s.max_depth, "dome_light_samples": s.dome_light_samples,
            "env": list(w.scene.dome_lights[0].env.shape[:2][::-1]), "distant_lights": len(w.scene.distant_lights),
            "paths_per_step": w.paths, "l2": flush}


class ClockSampler:
    """nvidia-smi sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,clocks.mem,clocks.max.mem")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout: float = 5.0):
        """nvidia-smi's start-up takes driver locks; start timing only once it
        is sampling."""
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.05)
        time.sleep(0.3)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.t:
                self.t.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, mem, memx, power, reasons = [], [], [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            try:
                power.append(float(parts[3]))
                mem.append(float(parts[9]))
                memx.append(float(parts[10]))
            except (ValueError, IndexError):
                pass
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active") or v == "1":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}
        if mem:
            out.update({"mem_mhz": statistics.median(mem), "mem_min_mhz": min(mem), "mem_max_mhz": max(memx)})
        if power:
            out["power_w_median"] = statistics.median(power)
        return out


def peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def ncu_traffic(kernel: str, workload_name: str):
    """DRAM bytes per path of `kernel` from the committed ncu summary (a
    smaller case of the same kernel, scaled per path)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload_name}.json")
    if not os.path.exists(path):
        return None
    d = json.load(open(path))
    return d.get("dram_bytes_per_path")


def cpu_baseline(w, seconds: float, rank: int = 0) -> dict:
    """The CPU path tracer (oracle restatement of CpuPathTracer) on every host
    thread (rows handed out dynamically), over rows spread evenly over the
    same frame."""
    import ctypes as C

    import oracle
    from shiro_gb300.abi import FrameBuffer, MarshalledScene, render_desc

    lib = oracle.load_port()
    lib.oracle_scene_create.argtypes = [C.c_void_p, C.c_void_p]
    lib.oracle_scene_create.restype = C.c_int
    lib.oracle_scene_render_row_list.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    lib.oracle_scene_render_row_list.restype = C.c_int64
    lib.oracle_scene_destroy.argtypes = [C.c_void_p]
    threads = os.cpu_count() or 1
    lib.oracle_set_threads(threads)
    ms = MarshalledScene(w.scene)
    h = C.c_void_p()
    t0 = time.perf_counter()
    rc = lib.oracle_scene_create(ms.ref(), C.byref(h))
    build_s = time.perf_counter() - t0
    if rc != 0:
        raise RuntimeError(f"oracle scene build failed: {rc}")
    st = w.settings
    req = render_desc(w.camera, st, 0, st.samples_per_pixel)
    fb = FrameBuffer(st.width, st.height)
    aovs = fb.aovs()

    def spread(n):
        # n rows spread evenly over the frame (rows differ widely in cost: sky
        # rows are cheap), so the sample's mix of sky and field does not
        # depend on the time budget
        return (C.c_uint32 * n)(*[min(st.height - 1, int((k + 0.5) * st.height / n)) for k in range(n)])

    def render(n):
        rows_n = spread(n)
        t0 = time.perf_counter()
        got = lib.oracle_scene_render_row_list(h, C.byref(req), rows_n, n, C.byref(aovs))
        dt = time.perf_counter() - t0
        if got < 0:
            raise RuntimeError(f"oracle render failed: {got}")
        return got, dt

    # calibrate on two rows per thread (one row per thread leaves the slowest
    # row alone at the end), then render the sized sample in one call
    paths, t_render = render(min(st.height, 2 * threads))
    rate = paths / max(t_render, 1e-6)
    rows = int(min(st.height, max(threads, seconds * rate / (st.width * st.samples_per_pixel))))
    paths, t_render = render(rows)
    lib.oracle_scene_destroy(h)
    value = paths / t_render / 1e6
    cpu = ""
    try:
        cpu = [ln.split(":", 1)[1].strip() for ln in open("/proc/cpuinfo") if ln.lower().startswith(("model name", "cpu part"))][0]
    except Exception:
        pass
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{rows} rows evenly spread over the frame x {st.width} px x {st.samples_per_pixel} spp ({paths} paths, "
                      f"{rows / st.height:.1%} of the frame), {t_render:.1f} s render + {build_s:.1f} s BVH build",
            "cpu": cpu, "seconds": t_render, "paths": int(paths)}


def adjoint_bench(local: int, iters: int = 5, warmup: int = 2, bvh_width: int = 2, size: int = 512,
                  form: str = "wavefront") -> dict:
    """Gradient throughput of the differentiable form on the 256-material
    sphere scene: 512x512 (`size` for profiling cases), 32 spp, depth 6, L2
    loss against a seeded target, gradients for 256 x (base colour, roughness,
    metalness) and the 512x256x3 environment texels.  One gradient = one
    forward render + one adjoint pass (which replays the forward's kept paths)."""
    import torch

    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import RENDER_KEEP_PATHS, RenderSettings

    scene = scenes.split_sphere_scene(parts=256, env_width=512, env_height=256, seed=4)
    st = RenderSettings(width=size, height=size, samples_per_pixel=32, max_depth=6, diffuse_depth=6, specular_depth=6,
                        backend=1)
    cam = scenes.sphere_camera(1.0)
    gpu = GpuBackend(local)
    gpu.set_bvh_width(bvh_width)
    gpu.set_adjoint_form(form == "wavefront")
    stream = torch.cuda.current_stream()
    gpu.lib.shiro_gpu_set_stream(gpu.handle, stream.cuda_stream)
    gpu.upload_scene(scene)
    p = dict(base_color=torch.tensor([m.base_color for m in scene.materials], dtype=torch.float32, device="cuda"),
             roughness=torch.tensor([m.roughness for m in scene.materials], dtype=torch.float32, device="cuda"),
             metallic=torch.tensor([m.metallic for m in scene.materials], dtype=torch.float32, device="cuda"),
             env=torch.tensor(scene.dome_lights[0].env, dtype=torch.float32, device="cuda"))
    target = torch.rand((size, size, 3), generator=torch.Generator().manual_seed(9)).cuda()
    grads = {k: torch.zeros_like(v) for k, v in p.items()}

    def step():
        # the forward autograd.render runs (its paths kept for the adjoint)
        img = gpu.render_device(cam, st, flags=RENDER_KEEP_PATHS, wavefront=True)
        fwd_ms = gpu.last_stats()["kernel_ms"]
        d = torch.zeros_like(img)
        d[..., :3] = 2.0 * (img[..., :3] - target) / target.numel()
        for g in grads.values():
            g.zero_()
        gpu.adjoint(cam, st, d, grads)
        return fwd_ms, gpu.last_stats()["kernel_ms"]

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    adj_ms = fwd_total = 0.0
    e0.record(stream)
    for _ in range(iters):
        f, a = step()
        fwd_total += f
        adj_ms += a
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / iters
    nparams = sum(v.numel() for v in p.values())
    paths = size * size * 32
    gpu.close()
    return {"workload": f"256-material sphere scene, 512x256 env, {size}x{size}, 32 spp, depth 6, L2 loss",
            "replay": form, "forward": "wavefront", "forward_ms": fwd_total / iters, "params": int(nparams), "ms_per_gradient": ms, "grads_per_s": 1000.0 / ms,
            "adjoint_ms": adj_ms / iters, "adjoint_Mpaths_s": paths / (adj_ms / iters / 1000.0) / 1e6,
            "param_gradients_per_s": nparams * 1000.0 / ms}


def rmse_check(local: int, bvh_width: int, with_cpu: bool) -> dict:
    """The equal-RMSE rule on the sphere frame (256x256, 16 spp, depth 8):
    RMSE of the plain and wavefront renders (and of the CPU oracle, which
    traces the same paths) against a 65 536-spp float64-accumulated image
    rendered from disjoint sample indices."""
    import torch

    from shiro_gb300 import GpuBackend
    from shiro_gb300.converge import converged, expected_mc_rmse, rmse

    w = workload("sphere")
    st = w.settings
    gpu = GpuBackend(local)
    gpu.set_bvh_width(bvh_width)
    gpu.upload_scene(w.scene)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ref = converged(gpu, w.camera, st, total_spp=65536, batch_spp=256, first=st.samples_per_pixel)
    torch.cuda.synchronize()
    ref_s = time.perf_counter() - t0
    plain = gpu.render_device(w.camera, st, 0, st.samples_per_pixel)
    wave = gpu.render_device(w.camera, st, 0, st.samples_per_pixel, wavefront=True)
    plain_cdf = gpu.render_device(w.camera, st, 0, st.samples_per_pixel, flags=1)
    a, b = rmse(plain, ref.mean), rmse(wave, ref.mean)
    out = {"workload": w.name, "reference_spp": ref.spp, "reference_first_sample": ref.first,
           "reference_accumulation": "float64 over 256-spp batch means", "reference_seconds": ref_s,
           "plain": a, "wavefront": b, "relative_difference": abs(a - b) / max(a, 1e-30),
           "identical_images": bool((plain == wave).all()), "expected_mc_rmse": expected_mc_rmse(ref, st.samples_per_pixel),
           "plain_env_cdf": rmse(plain_cdf, ref.mean),
           "note": "plain / wavefront pick dome-sample texels by the alias table (the timed path), plain_env_cdf by "
                   "the reference's CDF search; cpu_oracle (CDF search, as the reference) pairs with plain_env_cdf and "
                   "cpu_oracle_alias (the port given the backend's alias table) with plain: like for like, same paths"}
    if with_cpu:
        import oracle
        from oracle import api

        oracle.build_port()
        ck = oracle.port_checker()
        ps = api.PortScene(ck, w.scene)
        rows = np.arange(st.height)

        def cpu_rmse(fb):
            return rmse(torch.from_numpy(fb.beauty.reshape(st.height, st.width, 4).copy()), ref.mean.cpu())

        cpu_cdf = ps.render_rows(w.camera, st, rows, 0, st.samples_per_pixel, flags=1)
        tab = gpu.env_tables(0)
        ps.set_alias(0, tab["alias_threshold_bits"], tab["alias_index"])
        cpu_alias = ps.render_rows(w.camera, st, rows, 0, st.samples_per_pixel, flags=0)
        ps.close()
        out["cpu_oracle"] = cpu_rmse(cpu_cdf)
        out["cpu_oracle_alias"] = cpu_rmse(cpu_alias)

        def differing(gimg, fb):
            g = gimg.cpu().numpy().reshape(-1, 4)
            c = fb.beauty.reshape(-1, 4)
            return int((~np.isclose(g, c, rtol=1e-3, atol=1e-4).all(1)).sum())

        out["pixels_differing_cdf"] = differing(plain_cdf, cpu_cdf)
        out["pixels_differing_alias"] = differing(plain, cpu_alias)
    gpu.close()
    return out


def adapter_e2e(w, steps: int, warmup: int) -> dict:
    """End to end through the C++ RenderBackend adapter (GpuBackend), the call
    Shiro's Renderer makes: RenderSampleBatch with the renderer-owned scene
    snapshot in and a host FrameBuffer (the AOVs in the FrameBuffer's own
    storage) out, timed on the host clock around each call; the adapter's
    default wavefront configuration, no tuning.  Driven through the test
    harness's C entry point (tests/cpp)."""
    import ctypes as C

    from tests.cpp.harness import load_harness
    from shiro_gb300.abi import FrameBuffer, MarshalledScene, render_desc

    lib = load_harness()
    st = w.settings
    ms = MarshalledScene(w.scene)
    req = render_desc(w.camera, st, 0, st.samples_per_pixel)
    times = (C.c_double * steps)()
    fb = FrameBuffer(st.width, st.height)
    aov = fb.aovs()
    rc = lib.shiro_harness_time_render(ms.ref(), C.byref(req), warmup, steps, times, C.byref(aov))
    if rc != 1:
        return {"unavailable": f"adapter harness returned {rc}"}
    ms_steps = [times[k] for k in range(steps)]
    mean = statistics.mean(ms_steps)
    return {"value": w.paths / (mean / 1000.0) / 1e6, "unit": UNIT, "ms_per_step": mean, "ms_steps": ms_steps,
            "h2d_bytes_per_step": C.sizeof(req), "d2h_bytes_per_step": st.width * st.height * 44,
            "note": "GpuBackend::RenderSampleBatch (C++ adapter) -> FrameBuffer in pageable host memory; the scene "
                    "signature is checked every call, the scene uploaded once"}


def c5_bench(local: int, steps: int = 3) -> dict:
    """Inverse rendering (the 16-view configuration: 1.31 M-triangle field
    scene, 512 x 512, 16 spp, depth 8, 65 materials + a 1024 x 512 dome as
    unknowns, Adam lr 1e-2): a few optimisation steps with the wavefront
    forward and the adjoint backward, for steps/s; the 200-step run's parameter
    errors are recorded separately (python -m shiro_gb300.inverse)."""
    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import RenderSettings
    from shiro_gb300.inverse import inverse_render, orbit_views

    scene = scenes.field_scene(env_width=1024, env_height=512)
    st = RenderSettings(width=512, height=512, samples_per_pixel=16, max_depth=8, diffuse_depth=8, specular_depth=8,
                        dome_light_samples=1, background_visible=True, backend=1)
    views = orbit_views(16, 30.0, 12.0, seed=11)
    with GpuBackend(local) as gpu:
        inverse_render(gpu, scene, views, st, steps=1)  # warm-up (targets, pools, graphs)
        r = inverse_render(gpu, scene, views, st, steps=steps)
    return {"workload": "field 1310720 tris, 16 views 512x512, 16 spp, depth 8, 65 materials + 1024x512 env",
            "forward": "wavefront", "steps": steps, "steps_per_s": r.steps_per_s,
            "gradient_views_per_s": r.steps_per_s * r.views,
            "Mpaths_s_forward_plus_adjoint": r.steps_per_s * r.paths_per_step / 1e6}


def batch_bench(local: int, bvh_width: int, reps: int = 2) -> dict:
    """48 requests of uneven resolution / spp / depth on the sphere scene in
    one wavefront call, against the same requests rendered one by one with
    the plain form (device AOV planes, CUDA events)."""
    import ctypes as C

    import torch

    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import Aovs, RenderDesc, render_desc

    reqs = scenes.batch_requests(48)
    scene = scenes.sphere_scene()
    gpu = GpuBackend(local)
    gpu.set_bvh_width(bvh_width)
    stream = torch.cuda.current_stream()
    gpu.lib.shiro_gpu_set_stream(gpu.handle, stream.cuda_stream)
    gpu.upload_scene(scene)
    n = len(reqs)
    descs = (RenderDesc * n)()
    outs = (Aovs * n)()
    keep = []
    paths = 0
    for i, r in enumerate(reqs):
        st = r.settings
        npx = st.width * st.height
        planes = [torch.empty(npx * c, dtype=torch.float32, device="cuda") for c in (4, 3, 3, 1)]
        keep.append(planes)
        outs[i] = Aovs(*[C.cast(C.c_void_p(p.data_ptr()), C.POINTER(C.c_float)) for p in planes], 1, 0)
        descs[i] = render_desc(r.camera, st, 0, st.samples_per_pixel)
        paths += npx * st.samples_per_pixel

    def batched():
        if gpu.lib.shiro_gpu_render_batch(gpu.handle, descs, n, None, outs) != 0:
            raise RuntimeError(gpu.lib.shiro_gpu_last_error(gpu.handle).decode())

    def sequential():
        for i in range(n):
            if gpu.lib.shiro_gpu_render(gpu.handle, C.byref(descs[i]), None, C.byref(outs[i])) != 0:
                raise RuntimeError(gpu.lib.shiro_gpu_last_error(gpu.handle).decode())

    res = {}
    for name, fn in (("wavefront_batch", batched), ("plain_sequential", sequential)):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        res[name] = paths * reps / (e0.elapsed_time(e1) / 1000.0) / 1e6
    gpu.close()
    return {"requests": n, "pixels": int(sum(r.settings.width * r.settings.height for r in reqs)), "paths": int(paths),
            "unit": UNIT, **res}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    w = workload(args.workload, args)
    vals = []
    info = None
    for _ in range(args.warmup + args.steps):
        info = cpu_baseline(w, max(2.0, args.cpu_seconds / 2))
        vals.append(info["value"])
    timed = vals[args.warmup:]
    value = statistics.mean(timed)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": info["seconds"] * 1000.0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "impl": "reference", "config": workload_config(w, "n/a (CPU)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"], "kind": "port",
                             "sample": info["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch

    if args.adjoint_only:
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        res = adjoint_bench(int(os.environ.get("LOCAL_RANK", "0")), iters=args.steps, warmup=args.warmup,
                            bvh_width=args.bvh_width, size=args.adjoint_only, form=args.adjoint_form)
        print(json.dumps(res), flush=True)
        return 0
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from shiro_gb300 import GpuBackend
    from shiro_gb300.abi import FrameBuffer

    w = workload(args.workload, args)
    st = w.settings
    spp = st.samples_per_pixel
    gpu = GpuBackend(local)
    gpu.set_bvh_width(args.bvh_width)
    stream = torch.cuda.current_stream()
    gpu.lib.shiro_gpu_set_stream(gpu.handle, stream.cuda_stream)
    t0 = time.perf_counter()
    gpu.upload_scene(w.scene)
    upload_s = time.perf_counter() - t0
    forms = ["plain", "wavefront"] if args.form == "auto" else [args.form]

    npx = st.width * st.height
    dev = {k: torch.empty(npx * c, dtype=torch.float32, device="cuda") for k, c in
           (("beauty", 4), ("albedo", 3), ("normal", 3), ("depth", 1))}
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    import ctypes as C

    from shiro_gb300.abi import Aovs, render_desc

    aov = Aovs(*[C.cast(C.c_void_p(dev[k].data_ptr()), C.POINTER(C.c_float)) for k in ("beauty", "albedo", "normal", "depth")],
               1, 0)
    # weak scaling: every rank traces the full frame at `spp` samples per
    # pixel from its own range of sample indices (the job renders world x spp)
    from shiro_gb300.replicas import combine, sample_range

    start, _ = sample_range(rank, world, 0, world * spp)

    def render_dev(form):
        req = render_desc(w.camera, st, start, spp)
        if form == "plain":
            rc = gpu.lib.shiro_gpu_render(gpu.handle, C.byref(req), None, C.byref(aov))
        else:
            rc = gpu.lib.shiro_gpu_render_batch(gpu.handle, C.byref(req), 1, None, C.byref(aov))
        if rc != 0:
            raise RuntimeError(gpu.lib.shiro_gpu_last_error(gpu.handle).decode())
        return gpu.last_stats()

    tuned = None
    if "wavefront" in forms:
        if args.wf_config:
            gpu.set_wavefront_config(**{k: int(v) for k, v in (kv.split("=") for kv in args.wf_config.split(","))})
        tuned = gpu.wavefront_config() if args.no_autotune else gpu.autotune(w.scene, w.camera, st)

    def timed(form):
        for _ in range(args.warmup):
            render_dev(form)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        launches, path_ms, path_launches = 0, 0.0, 0
        e0.record(stream)
        for _ in range(args.steps):
            flush.zero_()
            s = render_dev(form)
            launches += s["kernel_launches"]
            path_ms += s["path_kernel_ms"]
            path_launches += s["path_kernel_launches"]
        e1.record(stream)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        ms = e0.elapsed_time(e1)
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return {"ms": ms, "launches": launches, "path_ms": path_ms, "path_launches": path_launches}

    results = {}
    with ClockSampler(local) as clocks:
        clocks.wait_first()
        for f in forms:
            results[f] = timed(f)
    total_paths = w.paths * world * args.steps
    for f in forms:
        results[f]["value"] = total_paths / (results[f]["ms"] / 1000.0) / 1e6
    head = max(forms, key=lambda f: results[f]["value"])
    value = results[head]["value"]
    ms = results[head]["ms"]
    launches = results[head]["launches"]
    stats = gpu.last_stats()

    # end to end through the public API with host FrameBuffer planes
    e2e = None
    if not args.no_e2e:
        fb = FrameBuffer(st.width, st.height, pinned=True)  # the caller's frame, page-locked, reused per step

        def api_step():
            if head == "plain":
                gpu.render(w.scene, w.camera, st, start, spp, out=fb)
            else:
                gpu.render_batch(w.scene, [(w.camera, st, start, spp)], outs_fb=[fb])

        api_step()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()
            api_step()
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        if dist:
            t = torch.tensor([el], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            el = float(t.item())
        req_bytes = C.sizeof(render_desc(w.camera, st, 0, 1))
        e2e = {"value": total_paths / el / 1e6, "unit": UNIT, "h2d_bytes_per_step": req_bytes,
               "d2h_bytes_per_step": npx * 44, "form": head, "note": "scene resident (uploaded once, "
               f"{upload_s:.2f} s incl. BVH build); per step: request in, 4 AOV planes out into a page-locked "
               "host FrameBuffer"}

    # replicas: one host-staged combination of the ranks' frames (outside the
    # timed region; the data path has no collective)
    combine_s = None
    if dist:
        gloo = dist.new_group(backend="gloo")
        render_dev(head)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fb = FrameBuffer(st.width, st.height)
        fb.beauty[:] = dev["beauty"].cpu().numpy().reshape(fb.beauty.shape)
        fb.albedo[:] = dev["albedo"].cpu().numpy().reshape(fb.albedo.shape)
        fb.normal[:] = dev["normal"].cpu().numpy().reshape(fb.normal.shape)
        fb.depth[:] = dev["depth"].cpu().numpy().reshape(fb.depth.shape)
        combined = combine(fb, spp, group=gloo)
        combine_s = time.perf_counter() - t0
        if combined is not None:
            assert combined.width == st.width

    # roofline of the headline form's dominant kernel, with the work counted
    # on the BVH that form traverses
    wide = args.bvh_width == 8 or (args.bvh_width == 0 and head == "wavefront")
    BYTES["node"] = 80 if wide else 64
    gpu.set_bvh_width(8 if wide else 2)
    wc = gpu.count_work(w.scene, w.camera, st, stride=64, sample_start=start)
    gpu.set_bvh_width(args.bvh_width)
    npth = max(wc["paths"], 1)
    cn = wc["node_visits"] - wc["occlusion_node_visits"]
    ct = wc["tri_tests"] - wc["occlusion_tri_tests"]
    pk = peaks()
    if head == "plain":
        per_path = (wc["node_visits"] * BYTES["node"] + wc["tri_tests"] * BYTES["tri"] + wc["hits"] * BYTES["hit"]
                    + wc["env_evals"] * BYTES["env_eval"] + wc["env_samples"] * BYTES["env_sample"]) / npth
        per_path += BYTES["record"] / 2  # the megakernel writes its 48-byte record
        kernel, kms, kl = "k_plain_paths", results["plain"]["path_ms"], results["plain"]["path_launches"]
        stage_share = None
    else:
        gpu.set_wavefront_config(use_graph=0)
        diag = render_dev("wavefront")
        gpu.set_wavefront_config(use_graph=1)
        names = ["wf_generate", "wf_extend", "wf_shade", "wf_occlude", "wf_resolve", "wf_shadow+bookkeeping"]
        dom = max(range(6), key=lambda k: diag["stage_ms"][k])
        kernel, kms, kl = names[dom], diag["stage_ms"][dom], diag["stage_launches"][dom]
        stage_share = {names[k]: diag["stage_ms"][k] / max(sum(diag["stage_ms"]), 1e-9) for k in range(6)}
        rays = wc["closest_rays"] / npth
        if dom == 1:     # closest hit: nodes, triangles, ray in (32 B), hit out (20 B), queue (4 B)
            per_path = (cn * BYTES["node"] + ct * BYTES["tri"]) / npth + rays * (32 + 20 + 4)
        elif dom == 3:   # occlusion: nodes, triangles, per path the shadow record
            per_path = (wc["occlusion_node_visits"] * BYTES["node"] + wc["occlusion_tri_tests"] * BYTES["tri"]) / npth
            per_path += wc["occlusion_rays"] / npth * 32 + wc["hits"] / npth * 64
        else:            # shading
            per_path = (wc["hits"] * BYTES["hit"] + wc["env_evals"] * BYTES["env_eval"]
                        + wc["env_samples"] * BYTES["env_sample"]) / npth + rays * 160
    paths_per_launch = w.paths / max(kl, 1)
    avg_launch_ms = kms / max(kl, 1)
    achieved = per_path * paths_per_launch / (avg_launch_ms / 1000.0) / 1e9
    dram_per_path = ncu_traffic(kernel, args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": (dram_per_path * paths_per_launch) if dram_per_path else None,
                "kernel": kernel, "peak_source": pk["source"], "algorithmic_bytes_per_path": per_path,
                "avg_launch_ms": avg_launch_ms, "paths_per_launch": paths_per_launch, "stage_share": stage_share,
                "work_per_path": {k: v / npth for k, v in wc.items() if k != "paths"}}

    adjoint = None
    if rank == 0 and not args.no_adjoint and args.workload == "field" and not (args.width or args.height or args.spp):
        adjoint = adjoint_bench(local, bvh_width=args.bvh_width)

    extra = {}
    full = args.workload == "field" and not (args.width or args.height or args.spp)
    if rank == 0 and not args.no_e2e and full:
        try:
            extra["e2e_adapter"] = adapter_e2e(w, args.steps, max(1, args.warmup))
        except Exception as ex:  # the harness needs a host C++ compiler
            extra["e2e_adapter"] = {"unavailable": str(ex)[:200]}
    if rank == 0 and not args.no_adjoint and full:
        extra["inverse"] = c5_bench(local)
    if rank == 0 and not args.no_rmse and args.workload == "field" and not (args.width or args.height or args.spp):
        extra["rmse"] = rmse_check(local, args.bvh_width, not args.no_cpu_baseline)
    if rank == 0 and not args.no_batch and args.workload == "field" and not (args.width or args.height or args.spp):
        extra["batch"] = batch_bench(local, args.bvh_width)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(w, args.cpu_seconds)
    if rank == 0:
        cfg = workload_config(w, "flushed (512 MiB memset between steps)")
        cfg.update({"form": head, "parallelism": f"replicas x{world}", "scene_upload_s": upload_s, "bvh_width": args.bvh_width,
                    "replica_combine_s": combine_s,
                    "bvh_nodes": int(stats["bvh_nodes"]), "bvh_depth": int(stats["bvh_depth"]),
                    "forms": {f: {"Mpaths_s": results[f]["value"], "ms_per_step": results[f]["ms"] / args.steps}
                              for f in forms}, "wavefront_config": tuned})
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene, random-init HDRI)",
                "config": cfg, "clocks": clocks.summary(), "gpu_launches": launches, "e2e": e2e,
                "roofline": roofline, "cpu_baseline": cpu, "adjoint": adjoint, **extra}
        print(json.dumps(line), flush=True)
    gpu.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
