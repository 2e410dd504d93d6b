"""Converged reference and the equal-RMSE rule.

* A high-spp GPU image (plain form, float64 accumulation of batch means,
  sample indices 1024.. disjoint from the ones tested) is checked against the CPU
  oracle at 1 024 spp with per-pixel z-scores: the oracle estimate must lie
  within the statistical spread of the converged image (|z| > 4 for at most
  0.5 % of pixel channels, mean z within +-0.25) and its RMSE must not exceed
  1.5x what plain Monte Carlo would give.
* Plain and wavefront renders at equal spp trace the same paths, so their
  RMSE against the converged image is equal (the images are bit-identical).
* The error falls with the sample count.
"""
import numpy as np
import pytest

import oracle
from oracle import api

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    from shiro_gb300 import GpuBackend

    with GpuBackend(0) as g:
        yield g


@pytest.fixture(scope="module")
def port():
    oracle.build_port()
    return oracle.port_checker()


@pytest.fixture(scope="module")
def case(gpu):
    from shiro_gb300 import scenes
    from shiro_gb300.converge import converged

    w = scenes.sphere_workload(48, 48, 16, 8, env_width=128, env_height=64)
    gpu.upload_scene(w.scene)
    ref = converged(gpu, w.camera, w.settings, total_spp=16384, batch_spp=256, first=1024)
    return w, ref


def test_converged_reference_agrees_with_cpu_oracle(gpu, port, case):
    import torch

    from shiro_gb300.converge import expected_mc_rmse, rmse, z_scores

    w, ref = case
    st = w.settings
    cpu = api.render(port, w.scene, w.camera, st, 0, 1024)
    img = torch.from_numpy(cpu.beauty.reshape(st.height, st.width, 4).copy())
    z = z_scores(img, 1024, ref)
    frac = float((z.abs() > 4.0).double().mean())
    assert frac <= 0.005, frac
    assert abs(float(z.mean())) <= 0.25, float(z.mean())
    assert rmse(img, ref.mean) <= 1.5 * expected_mc_rmse(ref, 1024)


def test_equal_rmse_plain_wavefront(gpu, case):
    from shiro_gb300.converge import rmse

    w, ref = case
    st = w.settings
    plain = gpu.render_device(w.camera, st, 0, st.samples_per_pixel)
    wave = gpu.render_device(w.camera, st, 0, st.samples_per_pixel, wavefront=True)
    assert bool((plain == wave).all())
    a, b = rmse(plain, ref.mean), rmse(wave, ref.mean)
    assert a == b and a > 0.0


def test_error_falls_with_samples(gpu, case):
    from shiro_gb300.converge import rmse

    w, ref = case
    st = w.settings
    errs = [rmse(gpu.render_device(w.camera, st, 0, n), ref.mean) for n in (4, 64, 1024)]
    assert errs[0] > errs[1] > errs[2], errs
    np.testing.assert_array_less(0.0, errs)
