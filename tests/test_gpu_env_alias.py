"""The default (timed) dome sampler: the alias table over the environment's
texels.  The reference samples a texel by binary search over its row and
conditional CDFs (EnvironmentMap::Sample / SampleCdf, EnvironmentMap.cpp:
109-163, 315-330) with the per-texel probability rowMass * columnMass that
BuildImportanceTable (:185-236) defines.  The backend's alias table must give
every texel exactly that probability; these tests check it on the texture
sizes of the benchmark scenes (512 x 256 for the sphere scene, 2048 x 1024
for the field scene):

* the device-built tables (CDFs, masses) equal the reference arithmetic's
  (the oracle port, pinned bit for bit to the reference) exactly, and the
  device-built alias table equals the oracle's sequential sweep exactly;
* each texel's selection probability reconstructed from the uploaded
  thresholds and aliases equals mass / sum(mass) to float rounding;
* a chi-square test of 10^7 device draws against those probabilities;
* the bucket index u.y * n: on every point of the 2^-24 grid each of the
  2^21 (or 2^17) buckets receives exactly 8 (or 128) points, and for a
  texture whose texel count is not a power of two each bucket's count stays
  within one grid point of the exact count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = [(512, 256, 0), (2048, 1024, 101)]


def _scene(w, h, seed):
    from shiro_gb300 import scenes
    from shiro_gb300.abi import DomeLight, Scene

    base = scenes.sphere_scene(env_width=16, env_height=8)
    env = scenes.procedural_hdri(w, h, seed)
    return Scene(materials=base.materials, meshes=base.meshes, dome_lights=[DomeLight(env=env)]), env


@pytest.fixture(scope="module")
def gpu():
    from shiro_gb300 import GpuBackend

    with GpuBackend(0) as g:
        yield g


def _reference_mass(env):
    """rowMass * columnMass in float32 from the oracle port's tables (the
    reference's BuildImportanceTable arithmetic)."""
    import oracle
    from oracle import api

    row, cond = api.env_tables(oracle.port_checker(), env)
    h, w = env.shape[:2]
    cond = cond.reshape(h, w + 1)
    row_mass = (row[1:] - row[:-1]).astype(np.float32)
    col_mass = (cond[:, 1:] - cond[:, :-1]).astype(np.float32)
    return row, cond, (row_mass[:, None] * col_mass).astype(np.float32)


def _alias_probability(thr, alias):
    n = thr.size
    t = thr.astype(np.float64)
    p = t.copy()
    np.add.at(p, alias.astype(np.int64), 1.0 - t)
    # bucket i keeps itself with probability thr[i] and its alias with 1 - thr[i]
    # (an entry whose alias is itself gives 1 either way)
    return p / n


@pytest.mark.parametrize("w,h,seed", SIZES)
def test_alias_table_gives_every_texel_its_reference_mass(gpu, w, h, seed):
    scene, env = _scene(w, h, seed)
    gpu.upload_scene(scene)
    tab = gpu.env_tables(0)
    row, cond, mass = _reference_mass(env)
    assert np.array_equal(tab["row_cdf"].view(np.uint32), row.view(np.uint32))
    assert np.array_equal(tab["cond_cdf"].view(np.uint32), cond.view(np.uint32))
    assert np.array_equal(tab["mass"].view(np.uint32), mass.view(np.uint32))
    thr, alias = tab["alias_threshold"], tab["alias_index"]
    assert np.all((thr >= 0.0) & (thr <= 1.0)) and np.all(alias < w * h)
    p = _alias_probability(thr, alias)
    m = mass.reshape(-1).astype(np.float64)
    target = m / m.sum()
    assert np.all(p[m == 0.0] == 0.0), "a texel of zero mass can be picked"
    live = m > 0.0
    rel = np.abs(p[live] - target[live]) / target[live]
    print(f"{w}x{h}: max relative error of the alias probabilities {rel.max():.3e}, "
          f"sum {p.sum():.12f}")
    assert rel.max() < 2.0e-5, rel.max()
    assert abs(p.sum() - 1.0) < 1.0e-9


@pytest.mark.parametrize("w,h,seed", SIZES + [(1000, 500, 5)])
def test_device_alias_table_equals_the_sequential_sweep(gpu, w, h, seed):
    """The device builds the alias table in parallel (binary searches over
    integer prefix sums); the oracle runs the sequential sweep that defines
    it.  Integer sums make the two equal bit for bit."""
    import oracle
    from oracle import api

    scene, env = _scene(w, h, seed)
    gpu.upload_scene(scene)
    tab = gpu.env_tables(0)
    thr, alias = api.env_alias(oracle.port_checker(), env)
    assert np.array_equal(tab["alias_threshold_bits"], thr)
    assert np.array_equal(tab["alias_index"], alias)


@pytest.mark.parametrize("w,h,seed", SIZES)
def test_chi_square_of_device_draws(gpu, w, h, seed):
    scipy_stats = pytest.importorskip("scipy.stats")
    scene, env = _scene(w, h, seed)
    gpu.upload_scene(scene)
    tab = gpu.env_tables(0)
    p = _alias_probability(tab["alias_threshold"], tab["alias_index"])
    rng = np.random.default_rng(7 + w)
    n_draws = 10_000_000
    counts = np.zeros(w * h, np.int64)
    for _ in range(4):
        u = rng.random((n_draws // 4, 2), dtype=np.float32)
        texel, pdf = gpu.env_sample(u)
        counts += np.bincount(texel.astype(np.int64), minlength=w * h)
        # the pdf reported with a sample is the reference's pdf of its texel
        assert np.all(pdf > 0.0)
    assert counts.sum() == n_draws
    assert counts[p == 0.0].sum() == 0
    # group consecutive texels into bins expecting at least 50 draws
    exp = p * n_draws
    edges = np.searchsorted(np.cumsum(exp), np.arange(50.0, exp.sum(), 50.0))
    grp_obs = np.add.reduceat(counts, np.r_[0, edges[:-1] + 1]) if edges.size > 1 else counts
    grp_exp = np.add.reduceat(exp, np.r_[0, edges[:-1] + 1]) if edges.size > 1 else exp
    keep = grp_exp > 0
    chi2 = float((((grp_obs - grp_exp) ** 2)[keep] / grp_exp[keep]).sum())
    dof = int(keep.sum()) - 1
    pval = float(scipy_stats.chi2.sf(chi2, dof))
    print(f"{w}x{h}: chi2 {chi2:.1f} on {dof} dof, p = {pval:.3f}")
    assert pval > 1.0e-4, (chi2, dof, pval)


@pytest.mark.parametrize("w,h,seed", SIZES + [(1000, 500, 5)])
def test_bucket_index_on_the_float_grid(gpu, w, h, seed):
    """u.y * n on every point k * 2^-24 of [0, 1): for a power-of-two n the
    product only shifts the exponent, so the bucket is exactly k >> (24 -
    log2 n) and every bucket gets 2^24 / n points; otherwise each bucket's
    count stays within one point of the exact count of grid points in
    [i / n, (i + 1) / n)."""
    scene, env = _scene(w, h, seed)
    gpu.upload_scene(scene)
    n = w * h
    k = np.arange(1 << 24, dtype=np.int64)
    u = np.empty((k.size, 2), np.float32)
    u[:, 0] = -1.0  # below every threshold: the bucket keeps itself
    u[:, 1] = (k.astype(np.float64) / float(1 << 24)).astype(np.float32)
    texel, _ = gpu.env_sample(u)
    counts = np.bincount(texel.astype(np.int64), minlength=n)
    exact_idx = (k * n) >> 24  # floor(k n / 2^24) in integers
    exact = np.bincount(exact_idx, minlength=n)
    if n & (n - 1) == 0:
        assert np.array_equal(texel.astype(np.int64), exact_idx)
        assert np.all(counts == (1 << 24) // n)
    else:
        mism = int((texel.astype(np.int64) != exact_idx).sum())
        print(f"{w}x{h}: {mism} of 2^24 grid points land one bucket off floor(u n)")
        assert np.abs(counts - exact).max() <= 1


@pytest.mark.parametrize("kind", ["hdr", "exr"])
def test_tables_of_a_texture_read_from_disk(gpu, tmp_path, kind):
    """A .hdr and an .exr read by the native reader (shiro_hdri_load, the
    C ABI's EnvironmentMap::Load) and uploaded: the device-built CDFs equal the
    reference arithmetic's and the alias table the oracle's sweep, bit for
    bit."""
    import oracle
    from oracle import api
    from shiro_gb300 import scenes
    from shiro_gb300.abi import DomeLight, Scene
    from shiro_gb300.backend import load_environment_file
    from test_hdri import FLOAT, HALF, exr_bytes, float_to_rgbe, hdr_bytes

    src = scenes.procedural_hdri(512, 256, 11)
    path = tmp_path / f"dome.{kind}"
    if kind == "hdr":
        path.write_bytes(hdr_bytes(float_to_rgbe(src), "new"))
    else:
        path.write_bytes(exr_bytes({c: (src[..., i], HALF) for i, c in enumerate("RGB")}, 3))
    env = load_environment_file(str(path))
    assert env.shape == (256, 512, 3)
    base = scenes.sphere_scene(env_width=16, env_height=8)
    gpu.upload_scene(Scene(materials=base.materials, meshes=base.meshes, dome_lights=[DomeLight(env=env)]))
    tab = gpu.env_tables(0)
    ck = oracle.port_checker()
    row, cond = api.env_tables(ck, env)
    assert np.array_equal(tab["row_cdf"].view(np.uint32), row.view(np.uint32))
    assert np.array_equal(tab["cond_cdf"].reshape(-1).view(np.uint32), cond.view(np.uint32))
    thr, alias = api.env_alias(ck, env)
    assert np.array_equal(tab["alias_threshold_bits"], thr)
    assert np.array_equal(tab["alias_index"], alias)
