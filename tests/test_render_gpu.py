"""Parity of the wavefront path tracer (salty_render) with the reference and the oracle.

Images at equal spp must agree per pixel within a 3-sigma Monte Carlo bound: with
independent estimates a, b and their variances of the mean, z = (a - b)/sqrt(va + vb);
the count of pixel-channels beyond 3 sigma must stay within the binomial bound of a normal
variable (0.27 % of them, plus four standard deviations of that count), none beyond 6, and
the two image means within 4.5 sigma (conftest.assert_within_3_sigma).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, assert_within_3_sigma

pytestmark = pytest.mark.gpu


def zstats(ma, va, mb, vb):
    # a relative floor of 1e-5 covers pixels with no sampling noise (pixel-centre rays that
    # reach only the environment), where CUDA's and the host's acosf/atan2f may differ in
    # the last bits
    floor = (1e-5 * np.maximum(np.abs(ma), np.abs(mb))) ** 2
    z = (ma - mb) / np.sqrt(np.maximum(va + vb + floor, 1e-30))
    return np.mean(np.abs(z) > 3), np.max(np.abs(z))


def zcheck(ma, va, mb, vb, zmax=6.0):
    """zstats' per pixel-channel z-scores and the image means, against the 3-sigma bounds."""
    ma, va, mb, vb = (np.asarray(x, float) for x in (ma, va, mb, vb))
    floor = (1e-5 * np.maximum(np.abs(ma), np.abs(mb))) ** 2
    v = np.maximum(va + vb + floor, 1e-30)
    assert_within_3_sigma((ma - mb) / np.sqrt(v), zmax, zsum=float((ma - mb).sum() / np.sqrt(v.sum())))


def _gpu_scene(ctx, sc):
    from salty_gb300 import scenes
    s = scenes.upload(ctx, sc)
    s.build()
    return s


def _oracle_scene(sc):
    from oracle.oracle import SceneData
    return SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], sc["sun"],
                     sc["sky"], sc["camera"], tri_uv=sc.get("tri_uv"), textures=sc.get("textures", []),
                     ibl=sc.get("ibl"))


def test_compat_cornell_matches_reference_fixture(ctx):
    """The reference's own estimator (PathTracer::Radiance) vs the GPU compat profile."""
    import salty_gb300
    from salty_gb300 import scenes
    g = np.load(os.path.join(GOLDEN, "cornell_ref_64.npz"))
    s = _gpu_scene(ctx, scenes.cornell("baseline"))
    r = s.render(int(g["width"]), int(g["height"]), int(g["spp"]), int(g["max_bounce"]),
                 profile=salty_gb300.PROFILE_COMPAT, seed=4242)
    zcheck(r["mean"], r["var"], g["mean"], g["var"])
    assert abs(r["mean"].mean() / g["mean"].mean() - 1) < 0.01


@pytest.mark.parametrize("variant,fixture", [("glossy", "cornell_glossy_ref_48.npz"),
                                             ("thinlens", "cornell_thinlens_ref_48.npz"),
                                             ("textured", "cornell_textured_ref_48.npz"),
                                             ("specular", "cornell_specular_ref_48.npz")])
def test_compat_variants_match_reference_fixtures(ctx, variant, fixture):
    """Phong and Plastic, the thin-lens camera, textures, and Mirror and Glass (the latter
    with the reference's 1/0.5 branch weights, src/s3d_glass.cpp:112-126) in the
    reference's estimator vs the GPU compat profile."""
    import salty_gb300
    from salty_gb300 import scenes
    g = np.load(os.path.join(GOLDEN, fixture))
    s = _gpu_scene(ctx, scenes.cornell(variant))
    r = s.render(int(g["width"]), int(g["height"]), int(g["spp"]), int(g["max_bounce"]),
                 profile=salty_gb300.PROFILE_COMPAT, seed=4343)
    zcheck(r["mean"], r["var"], g["mean"], g["var"])
    assert abs(r["mean"].mean() / g["mean"].mean() - 1) < 0.01


@pytest.mark.parametrize("variant", ["baseline", "mixed", "glossy", "thinlens", "textured"])
def test_physical_cornell_matches_oracle(ctx, oracle, variant):
    import salty_gb300
    from oracle.oracle import PROFILE_PHYSICAL
    from salty_gb300 import scenes
    sc = scenes.cornell(variant)
    W = H = 48
    spp = 512
    s = _gpu_scene(ctx, sc)
    r = s.render(W, H, spp, 8, rr_depth=3, profile=salty_gb300.PROFILE_PHYSICAL, seed=99)
    tot, sq = oracle.render(_oracle_scene(sc), W, H, spp, 8, rr_depth=3, profile=PROFILE_PHYSICAL, seed=1234)
    m = tot / spp
    v = np.maximum((sq / spp - m * m) * spp / (spp - 1) / spp, 0)
    zcheck(r["mean"], r["var"], m, v)
    assert r["rays"] > W * H * spp  # primary + extension + shadow rays


@pytest.mark.parametrize("half_angle", [0.0, 0.07])
def test_sun_sky_heightfield_matches_oracle(ctx, oracle, half_angle):
    """Sky + sun (delta, and a disk combined with BSDF sampling by MIS) over a small
    heightfield with spheres of every material."""
    import salty_gb300
    from oracle.oracle import PROFILE_PHYSICAL
    from salty_gb300 import scenes
    sc = scenes.heightfield(grid=48, n_spheres=24, seed=7, subdiv=2, sun_half_angle=half_angle)
    W, H, spp = 40, 24, 256
    s = _gpu_scene(ctx, sc)
    r = s.render(W, H, spp, 6, rr_depth=3, profile=salty_gb300.PROFILE_PHYSICAL, seed=21)
    tot, sq = oracle.render(_oracle_scene(sc), W, H, spp, 6, rr_depth=3, profile=PROFILE_PHYSICAL, seed=22)
    m = tot / spp
    v = np.maximum((sq / spp - m * m) * spp / (spp - 1) / spp, 0)
    zcheck(r["mean"], r["var"], m, v)


def test_crop_window_renders_the_same_samples(ctx):
    """A window keeps its pixels' full-frame rays and random streams: identical values."""
    import salty_gb300
    from salty_gb300 import scenes
    s = _gpu_scene(ctx, scenes.cornell("mixed"))
    full = s.render(64, 48, 8, 8, seed=13, want=("mean",))["mean"]
    win = s.render(64, 48, 8, 8, seed=13, want=("mean",), crop=(10, 7, 30, 20))["mean"]
    assert win.shape == (20, 30, 3)
    np.testing.assert_array_equal(win, full[7:27, 10:40])


def test_first_hit_features(ctx):
    """Albedo, normal and 1/(1+t) of the first hit, averaged over the pixel's samples."""
    from salty_gb300 import scenes
    s = _gpu_scene(ctx, scenes.cornell("baseline"))
    s.render(64, 64, 16, 8, seed=1, want=())
    f = s.aov(64, 64)
    # a pixel well inside the back wall (grey Lambert 0.75, normal -z, t from z=-1.4 to 1)
    al, nr, dp = f["albedo"][20, 32], f["normal"][20, 32], f["depth"][20, 32]
    np.testing.assert_allclose(al, 0.75, rtol=1e-5)
    np.testing.assert_allclose(nr, (0, 0, -1), atol=1e-5)
    assert 1.0 / (1.0 + 2.6) < dp < 1.0 / (1.0 + 2.3)
    # pixels whose samples all escaped past the open front of the box: every feature 0
    esc = f["depth"] == 0
    assert esc.any()
    assert np.all(f["albedo"][esc] == 0) and np.all(f["normal"][esc] == 0)
    n = np.linalg.norm(f["normal"].reshape(-1, 3), axis=1)
    assert np.all(n <= 1.0 + 1e-5)


def test_same_streams_as_oracle_give_nearly_identical_images(ctx, oracle):
    """Same seed => same per-(pixel, sample) PCG streams: most samples follow the same path,
    so the images agree far inside the Monte Carlo bound."""
    import salty_gb300
    from oracle.oracle import PROFILE_PHYSICAL
    from salty_gb300 import scenes
    sc = scenes.cornell("baseline")
    s = _gpu_scene(ctx, sc)
    r = s.render(32, 32, 64, 8, profile=salty_gb300.PROFILE_PHYSICAL, seed=7)
    tot, _ = oracle.render(_oracle_scene(sc), 32, 32, 64, 8, profile=PROFILE_PHYSICAL, seed=7)
    m = tot / 64
    assert np.median(np.abs(r["mean"] - m) / np.maximum(m, 1e-3)) < 1e-3


def test_progressive_accumulation_and_fp64_film(ctx):
    import salty_gb300
    from salty_gb300 import scenes
    s = _gpu_scene(ctx, scenes.cornell("baseline"))
    a = s.render(32, 32, 16, 8, seed=5, want=("mean",))
    b = s.render(32, 32, 16, 8, seed=5, accumulate=True, want=("mean", "var"))
    assert b["samples"] == 32
    s64 = s.render(32, 32, 32, 8, seed=5, fp64=True, want=("mean", "var"))
    assert s64["samples"] == 32
    frac, zmax = zstats(b["mean"], b["var"], s64["mean"], s64["var"])
    assert frac < 0.02
    # the first 16 samples are part of the accumulated film
    assert np.all(np.isfinite(b["mean"])) and not np.array_equal(a["mean"], b["mean"])


def test_srgb8_output_is_tonemapped_film(ctx):
    import salty_gb300
    from salty_gb300 import scenes
    s = _gpu_scene(ctx, scenes.cornell("baseline"))
    r = s.render(40, 30, 16, 8, seed=3, tonemap=salty_gb300.TM_ACES, ref_oetf=True)
    _, s8, _, _ = ctx.tonemap(r["mean"], salty_gb300.TM_ACES, srgb=True, ref_oetf=True)
    assert np.array_equal(r["srgb"], s8)
    assert r["srgb"].max() <= 247  # the reference OETF maps 1.0 to 247


def test_render_rejects_bad_options(ctx):
    import salty_gb300
    from salty_gb300 import scenes
    s = _gpu_scene(ctx, scenes.cornell("baseline"))
    with pytest.raises(salty_gb300.SaltyError):
        s.render(0, 10, 1, 8)
    with pytest.raises(salty_gb300.SaltyError):
        s.render(10, 10, 1, 0)
    with pytest.raises(salty_gb300.SaltyError):
        s.render(10, 10, 1, 8, profile=7)


def test_smd_mesh_instances_match_oracle(ctx, oracle, tmp_path):
    """An SMD mesh (an icosphere with a Plastic material) placed twice by affine transforms
    inside the Cornell box: GPU physical profile vs the oracle."""
    import salty_gb300
    from oracle.oracle import PROFILE_PHYSICAL
    from salty_gb300 import scenes
    from test_smd import write_smd
    unit = scenes._icosphere(2).astype(np.float32).reshape(-1, 9)
    n = unit.shape[0]
    p = str(tmp_path / "ball.smd")
    write_smd(p, unit, unit, np.zeros((n, 6), np.float32), np.zeros(n, np.int32),
              [(4, {"diffuse": (0.7, 0.3, 0.2), "specular": (0.6, 0.6, 0.6), "power": 60.0, "emission": (0, 0, 0)})])
    mesh = salty_gb300.load_smd(p)
    sc = scenes.cornell("baseline")
    pos, nrm, mat = [sc["tri_pos"]], [sc["tri_nrm"]], [sc["tri_mat"]]
    base = len(sc["materials"])
    for M in ([[0.12, 0, 0, 0.3], [0, 0.12, 0, 0.12], [0, 0, 0.12, 0.25]],
              [[0.1, 0.02, 0, 0.72], [0, 0.09, 0, 0.7], [0, 0, 0.11, 0.4]]):
        p2, n2 = salty_gb300.transform_mesh(M, mesh["tri_pos"], mesh["tri_nrm"])
        pos.append(p2)
        nrm.append(n2)
        mat.append(mesh["tri_mat"] + base)
    sc = dict(sc, tri_pos=np.concatenate(pos), tri_nrm=np.concatenate(nrm), tri_mat=np.concatenate(mat),
              materials=sc["materials"] + mesh["materials"])
    W = H = 40
    spp = 256
    s = _gpu_scene(ctx, sc)
    r = s.render(W, H, spp, 8, rr_depth=3, profile=salty_gb300.PROFILE_PHYSICAL, seed=8)
    tot, sq = oracle.render(_oracle_scene(sc), W, H, spp, 8, rr_depth=3, profile=PROFILE_PHYSICAL, seed=9)
    m = tot / spp
    v = np.maximum((sq / spp - m * m) * spp / (spp - 1) / spp, 0)
    zcheck(r["mean"], r["var"], m, v)


@pytest.mark.parametrize("fp64", [False, True])
def test_checkpoint_resume_continues_exactly(ctx, fp64):
    """A film checkpointed after one pass and restored into a fresh scene continues with the
    same random streams and the same sums: identical to never stopping."""
    from salty_gb300 import scenes
    desc = scenes.cornell("mixed")
    a = _gpu_scene(ctx, desc)
    a.render(40, 30, 8, 8, seed=5, fp64=fp64, want=())
    state = a.checkpoint()
    assert state["samples"] == 8 and (state["comp"] is None) == fp64
    a.render(40, 30, 8, 8, seed=5, fp64=fp64, accumulate=True, want=())
    want = a.read(40, 30, fp64=fp64)
    b = _gpu_scene(ctx, desc)
    b.restore(state, 40, 30, fp64=fp64)
    b.render(40, 30, 8, 8, seed=5, fp64=fp64, accumulate=True, want=())
    got = b.read(40, 30, fp64=fp64)
    np.testing.assert_array_equal(got["mean"], want["mean"])
    np.testing.assert_array_equal(got["var"], want["var"])
    np.testing.assert_array_equal(b.aov(40, 30)["albedo"], a.aov(40, 30)["albedo"])


def test_cancel_stops_a_render_and_the_context_recovers(ctx):
    """salty_ctx_cancel from another thread: the render stops between graph launches with
    ERR_CANCELLED (a host-side stop, nothing waits on the device), and the next render works."""
    import threading
    import time
    import salty_gb300
    from salty_gb300 import scenes
    s = _gpu_scene(ctx, scenes.cornell("baseline"))
    default = ctx.tuning
    ctx.tuning = {"wave_paths": 1 << 16}  # 2^16 paths in flight: tens of thousands of iterations
    err = {}

    def run():
        try:
            s.render(512, 512, 4096, 8, seed=1, want=())
        except salty_gb300.SaltyError as e:
            err["status"] = e.status

    th = threading.Thread(target=run)
    th.start()
    time.sleep(0.2)
    ctx.cancel()
    th.join(timeout=120)
    ctx.tuning = default
    assert not th.is_alive()
    assert err.get("status") == salty_gb300.ERR_CANCELLED, err
    r = s.render(32, 32, 4, 8, seed=2, want=("mean",))
    assert np.all(np.isfinite(r["mean"])) and r["samples"] == 4
