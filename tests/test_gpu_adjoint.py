"""The differentiable form: adjoint path replay against finite differences.

The adjoint holds sampling decisions, pdfs, MIS weights, Russian-roulette
probabilities (and clamp scales) constant and differentiates the BSDF values
and environment radiance.  shiro_gpu_render_frozen renders exactly that
estimator as a function of a second parameter set, so central finite
differences of it (Richardson-extrapolated central differences; steps of 1e-3,
relative for roughness and environment texels) must match the adjoint to
<= 1e-2 relative error on 64 parameters drawn uniformly among those with a
nonzero gradient, on a small frame and at the full 256-material,
512 x 512 x 32 spp configuration, with the reference's clamps off and on.  Against finite differences of the plain renderer
itself (sampling moves with the parameters) the agreement is statistical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

NO_CLAMP = 2


@pytest.fixture(scope="module")
def setup():
    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import RenderSettings

    scene = scenes.split_sphere_scene(parts=16, env_width=64, env_height=32, seed=4)
    st = RenderSettings(width=48, height=48, samples_per_pixel=8, max_depth=4, diffuse_depth=4, specular_depth=4,
                        backend=1)
    cam = scenes.look_at((0.0, 1.6, 4.5), (0.0, 0.9, 0.0), 45.0, 1.0)
    gpu = GpuBackend(0)
    gpu.upload_scene(scene)
    p = dict(
        base_color=torch.tensor([m.base_color for m in scene.materials], dtype=torch.float32, device="cuda"),
        roughness=torch.tensor([m.roughness for m in scene.materials], dtype=torch.float32, device="cuda"),
        metallic=torch.tensor([m.metallic for m in scene.materials], dtype=torch.float32, device="cuda"),
        env=torch.tensor(scene.dome_lights[0].env, dtype=torch.float32, device="cuda"),
    )
    yield gpu, scene, cam, st, p
    gpu.close()


def test_frozen_render_equals_render(setup):
    gpu, scene, cam, st, p = setup
    gpu.set_params(**p)
    beauty = gpu.render_device(cam, st, flags=NO_CLAMP)
    assert torch.equal(beauty, gpu.render_frozen(cam, st, flags=NO_CLAMP))
    assert torch.equal(beauty, gpu.render_frozen(cam, st, p["base_color"], p["roughness"], p["metallic"], p["env"],
                                                 flags=NO_CLAMP))
    assert torch.equal(beauty, gpu.render_device(cam, st, flags=NO_CLAMP, wavefront=True))


def test_set_params_equals_fresh_upload(setup):
    gpu, scene, cam, st, p = setup
    from shiro_gb300 import GpuBackend

    base = p["base_color"].clone()
    base[3] = torch.tensor([0.9, 0.2, 0.1], device="cuda")
    env = p["env"].clone()
    env[10:14, 20:30] *= 3.0
    gpu.set_params(base_color=base, env=env)
    a = gpu.render_device(cam, st)
    import copy

    sc2 = copy.deepcopy(scene)
    sc2.materials[3].base_color = (0.9, 0.2, 0.1)
    sc2.dome_lights[0].env = env.cpu().numpy()
    with GpuBackend(0) as g2:
        g2.upload_scene(sc2)
        b = g2.render_device(cam, st)
    gpu.set_params(**p)
    assert torch.equal(a, b)


def test_set_params_rewrites_changed_values_only(setup):
    """set_params skips a group whose values equal the last write (a
    multi-view optimisation sets the same parameters before every view) but
    picks up any change, including one made in place without autograd's
    knowledge, and a fresh scene upload restores the scene's values."""
    gpu, scene, cam, st, p = setup
    gpu.set_params(**p)
    ref = gpu.render_device(cam, st)
    q = {k: v.clone() for k, v in p.items()}
    gpu.set_params(**q)  # equal content: nothing is rewritten
    assert torch.equal(gpu.render_device(cam, st), ref)
    q["env"].data[5:9, 12:20] *= 4.0  # an in-place edit of the same tensor
    q["roughness"].data[2] = 0.05
    gpu.set_params(**q)
    edited = gpu.render_device(cam, st)
    assert not torch.equal(edited, ref)
    gpu.set_params(**p)
    assert torch.equal(gpu.render_device(cam, st), ref)
    gpu.set_params(**q)
    assert torch.equal(gpu.render_device(cam, st), edited)
    gpu.upload_scene(scene, force=True)  # the scene's own values again
    gpu.set_params(**q)
    assert torch.equal(gpu.render_device(cam, st), edited)
    gpu.set_params(**p)


def _loss(d, img):
    return float((d.double() * img.double()).sum())


def _step(name, val):
    """Central-difference step: 1e-3 for base colour and metalness; for
    roughness 1e-3 of the value (at least 5e-5), so the GGX width alpha = r^2
    moves by 0.2 % even for the sharpest lobes (a fixed 1e-3 on r = 0.18 is
    1 % of alpha and the difference quotient no longer converged there);
    1e-3 relative for environment texels."""
    if name == "roughness":
        return max(1e-3 * abs(val), 5e-5)
    if name == "env":
        return 1e-3 * max(1.0, abs(val))
    return 1e-3


def _fd_check(gpu, cam, st, p, d, flags, n_mat=32, n_env=32, seed=11, min_roughness=0.0, step_scale=None):
    """Adjoint against finite differences of the frozen estimator on
    parameters drawn uniformly among those with a nonzero gradient: n_mat of
    the material parameters, n_env of the texels.  The difference quotient is
    Richardson-extrapolated from steps h and h/2 ((4 D(h/2) - D(h)) / 3,
    truncation error O(h^4)); `step_scale` (group -> factor) widens a group's
    steps.  A parameter passes when
    |adjoint - fd| <= 1e-2 * max(|fd|, 1e-3 * largest |gradient| of its group).
    Returns the errors, worst first."""
    grads = {k: torch.zeros_like(v) for k, v in p.items()}
    gpu.set_params(**p)
    gpu.adjoint(cam, st, d, grads, flags=flags)
    rng = np.random.default_rng(seed)
    gmax = {k: float(v.abs().max()) for k, v in grads.items()}
    cands = []
    for name in ("base_color", "roughness", "metallic"):
        g = grads[name].flatten().cpu().numpy()
        v = p[name].flatten().cpu().numpy()
        for i in np.nonzero(g != 0.0)[0]:
            if name == "roughness" and abs(v[i] - 0.1414) < 5e-3:  # alpha = max(0.02, r^2) has its kink here
                continue
            if name == "roughness" and v[i] < min_roughness:
                continue
            if name == "metallic" and (v[i] < 0.01 or v[i] > 0.99):
                continue
            cands.append((name, int(i)))
    ge = grads["env"].flatten().cpu().numpy()
    env_c = [("env", int(i)) for i in np.nonzero(ge != 0.0)[0]]
    picks = [cands[i] for i in rng.choice(len(cands), size=min(n_mat, len(cands)), replace=False)]
    picks += [env_c[i] for i in rng.choice(len(env_c), size=min(n_env, len(env_c)), replace=False)]
    assert len(picks) == n_mat + n_env

    def quotient(name, i, h):
        plus = {k: v.clone() for k, v in p.items()}
        minus = {k: v.clone() for k, v in p.items()}
        plus[name].view(-1)[i] += h
        minus[name].view(-1)[i] -= h
        lp = _loss(d, gpu.render_frozen(cam, st, plus["base_color"], plus["roughness"], plus["metallic"],
                                        plus["env"], flags=flags))
        lm = _loss(d, gpu.render_frozen(cam, st, minus["base_color"], minus["roughness"], minus["metallic"],
                                        minus["env"], flags=flags))
        return (lp - lm) / (2.0 * h)

    errs = []
    for name, i in picks:
        val = float(p[name].flatten()[i])
        h = _step(name, val) * (step_scale or {}).get(name, 1.0)
        fd = (4.0 * quotient(name, i, 0.5 * h) - quotient(name, i, h)) / 3.0
        adj = float(grads[name].flatten()[i])
        scale = max(abs(fd), 1e-3 * gmax[name])
        errs.append((abs(adj - fd) / scale, name, i, adj, fd))
    errs.sort(reverse=True)
    return errs


def test_adjoint_matches_frozen_finite_differences(setup):
    gpu, scene, cam, st, p = setup
    gen = torch.Generator(device="cpu").manual_seed(7)
    d = torch.rand((st.height, st.width, 4), generator=gen) - 0.3
    d[..., 3] = 0.0
    errs = _fd_check(gpu, cam, st, p, d.cuda(), NO_CLAMP)
    print("worst relative errors:", errs[:5])
    assert errs[0][0] <= 1e-2, errs[:5]


@pytest.mark.parametrize("flags", [NO_CLAMP, 0])
def test_adjoint_finite_differences_at_full_size(flags):
    """The differentiable configuration at its stated size: 256 materials
    (seeded base colour, roughness, metalness) on the sphere scene cut into
    256 meshes, a 512 x 256 environment, 512 x 512, 32 spp, depth 6, L2 loss
    against a seeded target; 64 parameters drawn uniformly among those with a
    nonzero gradient.  Once with the reference's clamps disabled and once with
    them on (the frozen estimator holds each path's clamp scale constant, as
    the adjoint does)."""
    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import RenderSettings

    scene = scenes.split_sphere_scene(parts=256, env_width=512, env_height=256, seed=4)
    st = RenderSettings(width=512, height=512, samples_per_pixel=32, max_depth=6, diffuse_depth=6, specular_depth=6,
                        backend=1)
    cam = scenes.sphere_camera(1.0)
    with GpuBackend(0) as gpu:
        gpu.upload_scene(scene)
        p = dict(
            base_color=torch.tensor([m.base_color for m in scene.materials], dtype=torch.float32, device="cuda"),
            roughness=torch.tensor([m.roughness for m in scene.materials], dtype=torch.float32, device="cuda"),
            metallic=torch.tensor([m.metallic for m in scene.materials], dtype=torch.float32, device="cuda"),
            env=torch.tensor(scene.dome_lights[0].env, dtype=torch.float32, device="cuda"))
        gpu.set_params(**p)
        target = torch.rand((512, 512, 3), generator=torch.Generator().manual_seed(9)).cuda()
        img = gpu.render_frozen(cam, st, flags=flags)
        d = torch.zeros_like(img)
        d[..., :3] = 2.0 * (img[..., :3] - target) / target.numel()
        errs = _fd_check(gpu, cam, st, p, d, flags, seed=13 + flags)
    print(f"flags {flags}: worst relative errors:", errs[:5])
    assert errs[0][0] <= 1e-2, errs[:5]


def test_adjoint_agrees_with_plain_renderer_fd(setup):
    """Finite differences of the renderer itself (sampling moves with the
    parameters) agree with the adjoint in expectation; checked at high spp on
    parameters with a large image footprint."""
    gpu, scene, cam, st, p = setup
    from shiro_gb300.abi import RenderSettings

    big = RenderSettings(width=48, height=48, samples_per_pixel=256, max_depth=4, diffuse_depth=4, specular_depth=4,
                         backend=1)
    gpu.set_params(**p)
    d = torch.zeros((48, 48, 4), device="cuda")
    d[..., :3] = 1.0 / (48 * 48)
    grads = {k: torch.zeros_like(v) for k, v in p.items()}
    gpu.adjoint(cam, big, d, grads, flags=NO_CLAMP)
    ground = len(scene.materials) - 1
    for name, i in (("base_color", 3 * ground), ("base_color", 3 * ground + 1)):
        h = 2e-2
        plus = {k: v.clone() for k, v in p.items()}
        minus = {k: v.clone() for k, v in p.items()}
        plus[name].view(-1)[i] += h
        minus[name].view(-1)[i] -= h
        gpu.set_params(**plus)
        lp = _loss(d, gpu.render_device(cam, big, flags=NO_CLAMP))
        gpu.set_params(**minus)
        lm = _loss(d, gpu.render_device(cam, big, flags=NO_CLAMP))
        gpu.set_params(**p)
        fd = (lp - lm) / (2 * h)
        adj = float(grads[name].flatten()[i])
        assert abs(adj - fd) <= 0.1 * abs(fd), (name, i, adj, fd)


@pytest.mark.parametrize("adj_start", [None, 8])
def test_autograd_function(setup, adj_start):
    """The autograd binding's gradients equal a direct adjoint of the loss
    gradient, with the backward replaying the forward's samples (its kept
    paths) or an independent sample range (rendered and kept by the forward
    call as a second request)."""
    gpu, scene, cam, st, p = setup
    from shiro_gb300.autograd import render

    params = {k: v.clone().requires_grad_(True) for k, v in p.items()}
    target = torch.rand((st.height, st.width, 3), generator=torch.Generator().manual_seed(3)).cuda()
    img = render(gpu, cam, st, params["base_color"], params["roughness"], params["metallic"], params["env"],
                 flags=NO_CLAMP, adjoint_sample_start=adj_start)
    assert torch.equal(img, gpu.render_device(cam, st, flags=NO_CLAMP))
    loss = ((img[..., :3] - target) ** 2).mean()
    loss.backward()
    assert gpu.last_stats()["kernel_launches"] == 2 + 5 * st.max_depth + 1  # the kept paths replayed
    d = torch.zeros_like(img)
    d[..., :3] = 2.0 * (img[..., :3].detach() - target) / target.numel()
    grads = {k: torch.zeros_like(v) for k, v in p.items()}
    gpu.set_params(**p)
    gpu.adjoint(cam, st, d, grads, sample_start=adj_start or 0, flags=NO_CLAMP)
    for k in p:
        torch.testing.assert_close(params[k].grad, grads[k], rtol=1e-4, atol=1e-7)


def test_adjoint_rejects_extended_lobes():
    """The differentiable form covers reflecting, emitting and cut-out
    materials; a scene with transmission (whose lobe depends on roughness and
    metalness) is refused, not approximated."""
    from shiro_gb300 import GpuBackend, ShiroGpuError, scenes
    from shiro_gb300.abi import RenderSettings

    scene = scenes.split_sphere_scene(parts=4, env_width=32, env_height=16, seed=4)
    scene.materials[1].transmission = 1.0
    st = RenderSettings(width=16, height=16, samples_per_pixel=2, max_depth=3, diffuse_depth=3, specular_depth=3,
                        backend=1)
    cam = scenes.look_at((0.0, 1.6, 4.5), (0.0, 0.9, 0.0), 45.0, 1.0)
    with GpuBackend(0) as gpu:
        gpu.upload_scene(scene)
        gpu.render(scene, cam, st)  # rendering is supported
        d = torch.zeros((16, 16, 4), device="cuda")
        grads = {"base_color": torch.zeros((len(scene.materials), 3), device="cuda")}
        with pytest.raises(ShiroGpuError) as ei:
            gpu.adjoint(cam, st, d, grads)
        assert ei.value.code == -5


@pytest.mark.parametrize("pool", [0, 4096])
@pytest.mark.parametrize("flags", [NO_CLAMP, 0])
def test_wavefront_replay_equals_per_thread_replay(setup, flags, pool):
    """The adjoint's two forms - replay stages in the wavefront pool after
    each wave's forward stages (default), and one thread per path - add the
    same gradients, up to the order of their float atomics; with a pool of
    4096 paths the request spans several waves on two pools."""
    gpu, scene, cam, st, p = setup
    gpu.set_params(**p)
    gen = torch.Generator(device="cpu").manual_seed(5)
    d = (torch.rand((st.height, st.width, 4), generator=gen) - 0.3).cuda()
    d[..., 3] = 0.0
    base = gpu.wavefront_config()
    out = {}
    try:
        if pool:
            gpu.set_wavefront_config(paths_in_flight=pool, concurrent_waves=2, use_graph=1)
        for form in (True, False):
            g = {k: torch.zeros_like(v) for k, v in p.items()}
            gpu.set_adjoint_form(form)
            gpu.adjoint(cam, st, d, g, flags=flags)
            out[form] = g
    finally:
        gpu.set_adjoint_form(True)
        gpu.set_wavefront_config(**base)
    for k in p:
        a, b = out[True][k], out[False][k]
        assert a.abs().max() > 0, k
        torch.testing.assert_close(a, b, rtol=1e-3, atol=1e-5 * float(b.abs().max()), msg=k)


@pytest.mark.parametrize("flags", [NO_CLAMP, 0])
def test_kept_forward_wave_replays_alone(setup, flags):
    """SHIRO_RENDER_KEEP_PATHS: the forward image is unchanged; an adjoint of
    the same request right after it runs the replay stages alone (2 + 5 x
    depth launches, + 1 for the environment gradient) and adds the gradients
    of the full adjoint; so does an adjoint of either request of a kept
    two-request call (an image and an independent sample range, as a
    decorrelated gradient renders them).  A kept wave serves one call;
    another render, another sample range, new parameters or a request of
    several waves in between leave the adjoint on its own forward stages."""
    from shiro_gb300.abi import RENDER_KEEP_PATHS as KEEP

    gpu, scene, cam, st, p = setup
    gpu.set_params(**p)
    gen = torch.Generator(device="cpu").manual_seed(7)
    d = (torch.rand((st.height, st.width, 4), generator=gen) - 0.3).cuda()
    d[..., 3] = 0.0
    replay_only = 2 + 5 * st.max_depth + 1

    def adjoint(start=0):
        g = {k: torch.zeros_like(v) for k, v in p.items()}
        gpu.adjoint(cam, st, d, g, sample_start=start, flags=flags)
        return g, gpu.last_stats()["kernel_launches"]

    def close(a, b):
        for k in p:
            assert b[k].abs().max() > 0, k
            torch.testing.assert_close(a[k], b[k], rtol=1e-3, atol=1e-5 * float(b[k].abs().max()), msg=k)

    img = gpu.render_device(cam, st, flags=flags, wavefront=True)
    full, n_full = adjoint()
    assert n_full > replay_only
    assert torch.equal(gpu.render_device(cam, st, flags=flags | KEEP, wavefront=True), img)
    kept, n = adjoint()
    assert n == replay_only
    close(kept, full)
    assert adjoint()[1] == n_full  # consumed by the first adjoint

    full8, n = adjoint(8)
    assert n == n_full
    for first in (True, False):  # two requests kept: the adjoint of either replays alone
        pair = gpu.render_device(cam, st, flags=flags | KEEP, wavefront=True, also_start=8)
        assert torch.equal(pair, img)
        kept, n = adjoint(0 if first else 8)
        assert n == replay_only
        close(kept, full if first else full8)
        assert adjoint(8)[1] == n_full

    gpu.render_device(cam, st, flags=flags | KEEP, wavefront=True)
    gpu.render_device(cam, st, sample_start=8, flags=flags, wavefront=True)
    assert adjoint()[1] == n_full
    gpu.render_device(cam, st, sample_start=8, flags=flags | KEEP, wavefront=True)
    assert adjoint()[1] == n_full

    base = p["base_color"].clone()
    base[2] = torch.tensor([0.8, 0.3, 0.1], device="cuda")
    try:
        gpu.render_device(cam, st, flags=flags | KEEP, wavefront=True)
        gpu.set_params(base_color=base)
        changed, n = adjoint()
        assert n == n_full
        gpu.render_device(cam, st, flags=flags | KEEP, wavefront=True)
        kept, n = adjoint()
        assert n == replay_only
        close(kept, changed)
    finally:
        gpu.set_params(**p)

    cfg = gpu.wavefront_config()
    try:
        gpu.set_wavefront_config(paths_in_flight=4096)
        assert torch.equal(gpu.render_device(cam, st, flags=flags | KEEP, wavefront=True), img)
        several, n = adjoint()
        assert n > replay_only
        close(several, full)
    finally:
        gpu.set_wavefront_config(**cfg)


@pytest.fixture(scope="module")
def ext_setup():
    """The 16-material sphere scene with two emitting materials (so paths
    also take the emissive-triangle light sample) and two opacity cut-outs,
    under the scene's environment with its radiance clipped at 4 (the 1e3 sun
    of the procedural HDRI in sharp reflections makes finite differences
    ill-conditioned)."""
    from shiro_gb300 import GpuBackend, scenes
    from shiro_gb300.abi import RenderSettings

    scene = scenes.split_sphere_scene(parts=16, env_width=64, env_height=32, seed=4)
    scene.dome_lights[0].env = np.minimum(scene.dome_lights[0].env, np.float32(4.0))
    for k in (2, 9):
        scene.materials[k].emission_strength = 4.0
        scene.materials[k].emission_color = (1.0, 0.8, 0.6)
    for k in (5, 12):
        scene.materials[k].opacity = 0.4
    st = RenderSettings(width=48, height=48, samples_per_pixel=8, max_depth=4, diffuse_depth=4, specular_depth=4,
                        backend=1)
    cam = scenes.look_at((0.0, 1.6, 4.5), (0.0, 0.9, 0.0), 45.0, 1.0)
    gpu = GpuBackend(0)
    gpu.upload_scene(scene)
    p = dict(
        base_color=torch.tensor([m.base_color for m in scene.materials], dtype=torch.float32, device="cuda"),
        roughness=torch.tensor([m.roughness for m in scene.materials], dtype=torch.float32, device="cuda"),
        metallic=torch.tensor([m.metallic for m in scene.materials], dtype=torch.float32, device="cuda"),
        env=torch.tensor(scene.dome_lights[0].env, dtype=torch.float32, device="cuda"),
    )
    yield gpu, scene, cam, st, p
    gpu.close()


def test_emitters_and_cutouts_frozen_render_equals_render(ext_setup):
    """With emitters and cut-outs the frozen estimator still renders the
    forward frame bit for bit (plain and wavefront forms), with the scene's
    own parameters given or not."""
    gpu, scene, cam, st, p = ext_setup
    gpu.set_params(**p)
    beauty = gpu.render_device(cam, st, flags=NO_CLAMP)
    assert torch.equal(beauty, gpu.render_device(cam, st, flags=NO_CLAMP, wavefront=True))
    assert torch.equal(beauty, gpu.render_frozen(cam, st, flags=NO_CLAMP))
    assert torch.equal(beauty, gpu.render_frozen(cam, st, p["base_color"], p["roughness"], p["metallic"], p["env"],
                                                 flags=NO_CLAMP))


@pytest.mark.parametrize("flags", [NO_CLAMP, 0])
def test_emitters_and_cutouts_finite_differences(ext_setup, flags):
    """Adjoint against finite differences of the frozen estimator on a scene
    with emitters (emission at hits, the emissive-triangle light sample) and
    cut-outs (paths passing through), clamps off and on.  Roughness is drawn
    among the lobes of roughness >= 0.3: for the sharpest one (r = 0.18) the
    difference quotient of the clamped frozen frame does not converge in
    float32 - 18.0 / 21.1 / 18.1 at relative steps 5e-4 / 1e-3 / 1e-2 on this
    scene without any emitter or cut-out, against an adjoint of 20.58 that the
    wavefront and one-thread replays give to seven digits.  Base colour and
    metalness enter the frozen BSDF at most quadratically and the texels
    linearly, where central differences are exact at any step: their steps
    are ten times the default, above the float32 rounding of the frames that
    emitters make bright (a metalness read 0.0071 at half the default step,
    0.006867 at the default and 0.006845 at ten times it, adjoint 0.006868)."""
    gpu, scene, cam, st, p = ext_setup
    gen = torch.Generator(device="cpu").manual_seed(21)
    d = torch.rand((st.height, st.width, 4), generator=gen) - 0.3
    d[..., 3] = 0.0
    errs = _fd_check(gpu, cam, st, p, d.cuda(), flags, seed=17 + flags, min_roughness=0.3,
                     step_scale={"base_color": 10.0, "metallic": 10.0, "env": 10.0})
    print("worst relative errors:", errs[:5])
    assert errs[0][0] <= 1e-2, errs[:5]


def test_emitters_and_cutouts_replay_forms_agree(ext_setup):
    """The wavefront replay (logged hits and visibility, emission taken off
    the radiance still to come in its shade stage) and the one-thread replay
    add the same gradients on that scene, and the replay of a kept forward
    wave adds them too."""
    from shiro_gb300.abi import RENDER_KEEP_PATHS as KEEP

    gpu, scene, cam, st, p = ext_setup
    gpu.set_params(**p)
    gen = torch.Generator(device="cpu").manual_seed(5)
    d = (torch.rand((st.height, st.width, 4), generator=gen) - 0.3).cuda()
    d[..., 3] = 0.0
    out = {}
    try:
        for form in (True, False):
            g = {k: torch.zeros_like(v) for k, v in p.items()}
            gpu.set_adjoint_form(form)
            gpu.adjoint(cam, st, d, g, flags=NO_CLAMP)
            out[form] = g
    finally:
        gpu.set_adjoint_form(True)
    gpu.render_device(cam, st, flags=NO_CLAMP | KEEP, wavefront=True)
    kept = {k: torch.zeros_like(v) for k, v in p.items()}
    gpu.adjoint(cam, st, d, kept, flags=NO_CLAMP)
    assert gpu.last_stats()["kernel_launches"] == 2 + 5 * st.max_depth + 1
    for k in p:
        a, b = out[True][k], out[False][k]
        assert a.abs().max() > 0, k
        torch.testing.assert_close(a, b, rtol=1e-3, atol=1e-5 * float(b.abs().max()), msg=k)
        torch.testing.assert_close(kept[k], b, rtol=1e-3, atol=1e-5 * float(b.abs().max()), msg=k)
