"""Host-side logic that needs no GPU: the error metric, the denoiser's feature packing and
padding, the scene generators behind the benchmark configurations, the training-view
generators, and the bench's reading of the measured peaks."""
import json
import math
import os

import numpy as np
import pytest


def test_rel_mse_and_reference_noise_correction():
    from salty_gb300 import convergence as cv
    ref = np.full((4, 4, 3), 0.5, np.float32)
    x = ref + 0.1
    want = 0.01 / (0.25 + 0.01)
    assert cv.rel_mse(x, ref) == pytest.approx(want, rel=1e-6)
    assert cv.rel_rmse(x, ref) == pytest.approx(math.sqrt(want), rel=1e-6)
    # the corrected error subtracts the reference's own noise term
    assert cv.corrected_rel_mse(x, {"mean": ref, "noise": 0.001}) == pytest.approx(want - 0.001, rel=1e-6)
    img = np.arange(6 * 8 * 3, dtype=np.float32).reshape(6, 8, 3)
    np.testing.assert_array_equal(cv.crop_of(img, (2, 1, 3, 4)), img[1:5, 2:5])


def test_unet_features_layout_and_noise_level():
    from salty_gb300 import UNET_FEATURES, unet_features
    rng = np.random.default_rng(1)
    mean = rng.uniform(0, 2, (5, 7, 3)).astype(np.float32)
    var = rng.uniform(0, 0.1, (5, 7, 3)).astype(np.float32)
    aov = {"albedo": rng.uniform(0, 1, (5, 7, 3)).astype(np.float32),
           "normal": rng.uniform(-1, 1, (5, 7, 3)).astype(np.float32),
           "depth": rng.uniform(0, 1, (5, 7)).astype(np.float32)}
    f = unet_features(mean, var, aov)
    assert f.shape == (5, 7, UNET_FEATURES) == (5, 7, 11) and f.dtype == np.float32
    np.testing.assert_array_equal(f[..., 0:3], mean)
    np.testing.assert_array_equal(f[..., 3:6], aov["albedo"])
    np.testing.assert_array_equal(f[..., 6:9], aov["normal"])
    np.testing.assert_array_equal(f[..., 9], aov["depth"])
    noise = (np.sqrt(var) / (1.0 + mean)).mean(-1)
    np.testing.assert_allclose(f[..., 10], noise, rtol=1e-6)


def test_pad16_reflects_to_multiples_of_16():
    from salty_gb300.denoiser import _pad16
    a = np.arange(20 * 33 * 2, dtype=np.float32).reshape(20, 33, 2)
    p = _pad16(a)
    assert p.shape == (32, 48, 2)
    np.testing.assert_array_equal(p[:20, :33], a)
    np.testing.assert_array_equal(p[20, :33], a[18])  # reflection without repeating the edge
    np.testing.assert_array_equal(p[:20, 33], a[:, 31])
    b = np.zeros((16, 32, 1), np.float32)
    assert _pad16(b).shape == (16, 32, 1)


def test_training_views_are_seeded_and_sane():
    from salty_gb300 import denoiser as dn
    v1 = dn.random_view(np.random.default_rng(5))
    v2 = dn.random_view(np.random.default_rng(5))
    assert v1 == v2
    for seed in range(50):
        rng = np.random.default_rng(seed)
        v = dn.random_view(rng)
        assert 0.3 <= v["pos"][1] <= 0.55 and v["target"][1] <= 0.1  # above the terrain, looking down
        assert 0.0 < v["fov"] < 2.0 * math.tan(math.radians(33))
        s = np.array(dn.random_sun(rng))
        assert abs(np.linalg.norm(s) - 1.0) < 1e-9 and s[1] > math.sin(math.radians(14.9))


def test_cornell_box_matches_its_configuration():
    from salty_gb300 import scenes
    c = scenes.cornell("baseline")
    assert c["tri_pos"].shape == (34, 9) and c["tri_nrm"].shape == (34, 9)  # + 2 light triangles
    lo, hi = c["tri_pos"].reshape(-1, 3).min(0), c["tri_pos"].reshape(-1, 3).max(0)
    np.testing.assert_allclose(lo, 0.0, atol=1e-6)
    np.testing.assert_allclose(hi, 1.0, atol=1e-6)
    assert tuple(c["camera"]["pos"]) == (0.5, 0.5, -1.4)
    assert c["camera"]["fov"] == pytest.approx(2.0 * math.tan(math.radians(20.0)))
    for v in ("mixed", "glossy", "thinlens", "textured"):
        assert scenes.cornell(v)["tri_pos"].shape[0] >= 34


def test_heightfield_counts_and_materials():
    from salty_gb300 import scenes
    h = scenes.heightfield(grid=64, n_spheres=40, seed=7, subdiv=2)
    n_terrain = 2 * 64 * 64
    assert h["tri_pos"].shape == (n_terrain + 40 * 320, 9)
    assert np.all(h["tri_mat"][:n_terrain] == 0)
    assert len(h["materials"]) == 41
    # the benchmark scene's defaults: a 2048^2 grid and 4096 subdivision-3 icospheres, i.e.
    # 2 x 2048^2 + 4096 x 1280 = 13,631,488 triangles
    import inspect
    d = {k: v.default for k, v in inspect.signature(scenes.heightfield).parameters.items()}
    assert (d["grid"], d["n_spheres"], d["subdiv"], d["seed"]) == (2048, 4096, 3, 2026)
    assert 2 * d["grid"] ** 2 + d["n_spheres"] * 20 * 4 ** d["subdiv"] == 13_631_488
    again = scenes.heightfield(grid=64, n_spheres=40, seed=7, subdiv=2)
    np.testing.assert_array_equal(h["tri_pos"], again["tri_pos"])


def test_batch_scenes_follow_the_configuration():
    from salty_gb300 import scenes
    for seed in range(20260100, 20260110):
        d, o = scenes.batch_scene(seed)
        n = d["tri_pos"].shape[0]
        assert 500 <= n <= 1_100_000, n
        assert o["width"] == o["height"] and o["width"] in (64, 128, 256, 512)
        assert o["spp"] in (4, 16, 64) and o["max_depth"] == 8
        d2, o2 = scenes.batch_scene(seed)
        assert o2 == o and d2["tri_pos"].shape == d["tri_pos"].shape


def test_bench_reads_the_measured_peaks():
    import bench
    p = bench.measured_peaks()
    t = bench.measured_peaks_tensor()
    path = os.path.join(bench.ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        assert p == {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
        assert t["bf16_tflops"] == d["bf16_tflops"]
    else:
        assert p["source"] == "fallback" and t["source"] == "fallback"


def test_clock_sampler_summary_reports_median_max_and_throttle_reasons(tmp_path):
    """The bench's nvidia-smi sampling: median SM clock under the timed region, the maximum
    clock, and every throttle reason seen Active (a run showing hw_slowdown or a thermal
    slowdown is to be taken again; sw_power_cap is kept and noted)."""
    import bench
    rows = [
        "0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1390.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 1980, 2070, 1395.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "garbage line",
    ]
    p = tmp_path / "clocks.csv"
    p.write_text("\n".join(rows) + "\n")
    s = bench.ClockSampler(0)
    s.path = str(p)
    out = s.summary()
    assert out == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    assert not os.path.exists(p)  # the sample file is removed once read
    s2 = bench.ClockSampler(0)
    assert s2.summary() is None  # no nvidia-smi, no samples
