"""Inverse rendering through the differentiable form.

A short Adam run with decorrelated adjoint samples on a scene whose materials
are all well observed (sphere + ground), lighting known:

* base colour alone must come within 30 % of its starting error;
* base colour and roughness must both improve when base colour, roughness and
  metalness are unknown together.

The gradient estimate that replays the forward render's own samples is biased
by the derivative of the image variance (with a bright environment it drives
the materials darker), which the correlated run must show: its base-colour
error ends above the decorrelated run's.  The image loss itself is dominated
by sampling noise at these sample counts, so the checks are on the parameters.
"""
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def case():
    from shiro_gb300 import scenes
    from shiro_gb300.abi import RenderSettings
    from shiro_gb300.inverse import orbit_views

    st = RenderSettings(width=40, height=40, samples_per_pixel=4, max_depth=4, diffuse_depth=4, specular_depth=4,
                        backend=1)
    views = orbit_views(3, 4.5, 1.8, target=(0.0, 0.9, 0.0), seed=2)
    return scenes.split_sphere_scene(parts=2, env_width=32, env_height=16, seed=7), st, views


def test_inverse_rendering_recovers_base_colour(case):
    from shiro_gb300 import GpuBackend
    from shiro_gb300.inverse import inverse_render

    scene, st, views = case
    with GpuBackend(0) as gpu:
        r = inverse_render(gpu, scene, views, st, steps=60, lr=0.02, target_spp=32, optimize=("base_color",))
        c = inverse_render(gpu, scene, views, st, steps=60, lr=0.02, target_spp=32, optimize=("base_color",),
                           decorrelate=False)
    assert len(r.loss) == 60
    assert r.rmse_end["base_color"] < 0.3 * r.rmse_start["base_color"], (r.rmse_start, r.rmse_end)
    assert r.rmse_end["roughness"] == 0.0 and r.rmse_end["env_log"] == 0.0
    assert c.rmse_end["base_color"] > r.rmse_end["base_color"], (c.rmse_end, r.rmse_end)


def test_inverse_rendering_materials_jointly(case):
    from shiro_gb300 import GpuBackend
    from shiro_gb300.inverse import inverse_render

    scene, st, views = case
    with GpuBackend(0) as gpu:
        r = inverse_render(gpu, scene, views, st, steps=60, lr=0.02, target_spp=32,
                           optimize=("base_color", "roughness", "metallic"))
    assert r.rmse_end["base_color"] < r.rmse_start["base_color"], (r.rmse_start, r.rmse_end)
    assert r.rmse_end["roughness"] < r.rmse_start["roughness"], (r.rmse_start, r.rmse_end)
