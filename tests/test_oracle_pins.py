"""Pins the oracle restatement (oracle/salty_oracle.c) to the reference.

CPU only.  The reference ships no tests or golden vectors, so the pins are (a) the
committed fixtures in tests/golden/, made from the unmodified reference by
tests/golden/make_golden.py, and (b) live comparisons against the reference compiled
from its sources (oracle/_ref), where that build exists.
"""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN, assert_agree

SOUP_SEED, RAY_SEED = 20260001, 20260002


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_generators_reproduce_fixture_inputs(oracle):
    g = np.load(os.path.join(GOLDEN, "trace_soup_1m.npz"))
    assert sha(oracle.gen_soup(SOUP_SEED, 1_000_000)) == str(g["soup_sha"])
    assert sha(oracle.gen_rays(RAY_SEED, 65536)) == str(g["rays_sha"])


def test_library_generators_equal_oracle(oracle):
    import salty_gb300
    from salty_gb300 import build as b
    b.build()
    for n in (0, 1, 1000, 12345):
        assert np.array_equal(salty_gb300.microbench_soup(11, n), oracle.gen_soup(11, n))
        assert np.array_equal(salty_gb300.microbench_rays(12, n, 1e-4), oracle.gen_rays(12, n, 1e-4))


def test_oracle_trace_matches_reference_fixture_small(oracle):
    g = np.load(os.path.join(GOLDEN, "trace_soup_30k.npz"))
    tris = oracle.gen_soup(int(g["soup_seed"]), int(g["n_tris"]))
    rays = oracle.gen_rays(int(g["ray_seed"]), int(g["n_rays"]))
    assert sha(tris) == str(g["soup_sha"]) and sha(rays) == str(g["rays_sha"])
    ids, t, u, v = oracle.trace(tris, rays, mode=0)
    assert np.array_equal(ids, g["ids"])
    hit = ids >= 0
    assert hit.sum() > 50
    assert np.array_equal(t[hit], g["t"][hit])
    assert np.array_equal(u[hit], g["u"][hit]) and np.array_equal(v[hit], g["v"][hit])


def test_oracle_trace_matches_reference_fixture_1m(oracle):
    g = np.load(os.path.join(GOLDEN, "trace_soup_1m.npz"))
    tris = oracle.gen_soup(SOUP_SEED, 1_000_000)
    rays = oracle.gen_rays(RAY_SEED, 65536)
    ids, t, _, _ = oracle.trace(tris, rays, mode=0)
    assert np.array_equal(ids, g["ids"]), f"{(ids != g['ids']).sum()} id mismatches"
    hit = ids >= 0
    assert hit.mean() > 0.95
    assert np.array_equal(t[hit], g["t"][hit])


def test_oracle_trace_matches_live_reference(oracle, reference):
    tris = oracle.gen_soup(31, 20000)
    rays = oracle.gen_rays(32, 4096)
    s = reference.soup(tris)
    rid, rt, ru, rv, _ = s.trace(rays)
    s.close()
    ids, t, u, v = oracle.trace(tris, rays, mode=0)
    assert np.array_equal(ids, rid)
    hit = ids >= 0
    assert np.array_equal(t[hit], rt[hit]) and np.array_equal(u[hit], ru[hit]) and np.array_equal(v[hit], rv[hit])


def test_restated_reference_bvh_matches_reference_fixture_1m(oracle):
    """The restatement of the reference's own BVH8 and walk (the CPU baseline) gives the
    compiled reference's answers on its 1M-triangle fixture, bit for bit."""
    g = np.load(os.path.join(GOLDEN, "trace_soup_1m.npz"))
    tris = oracle.gen_soup(SOUP_SEED, 1_000_000)
    rays = oracle.gen_rays(RAY_SEED, 65536)
    b = oracle.ref_bvh(tris)
    ids, t, _, _, _ = b.trace(rays)
    st = b.stats()
    b.close()
    assert np.array_equal(ids, g["ids"]), f"{(ids != g['ids']).sum()} id mismatches"
    hit = ids >= 0
    assert np.array_equal(t[hit], g["t"][hit])
    assert st["bvh8"] > 0 and st["leaves"] > 0


def test_restated_reference_bvh_matches_live_reference(oracle, reference):
    """Same tree, same walk: equal ids, t and barycentrics with the compiled reference on a
    soup with duplicated triangles, where the first triangle walked keeps a tie."""
    tris = oracle.gen_soup(51, 20000)
    tris[5000:5100] = tris[100:200]          # exact duplicates: ties decided by walk order
    rays = oracle.gen_rays(52, 8192)
    s = reference.soup(tris)
    rid, rt, ru, rv, _ = s.trace(rays)
    s.close()
    b = oracle.ref_bvh(tris)
    ids, t, u, v, _ = b.trace(rays)
    b.close()
    assert np.array_equal(ids, rid)
    hit = ids >= 0
    assert np.array_equal(t[hit], rt[hit]) and np.array_equal(u[hit], ru[hit]) and np.array_equal(v[hit], rv[hit])


def test_watertight_differs_only_at_edges(oracle):
    tris = oracle.gen_soup(41, 200000)
    rays = oracle.gen_rays(42, 20000)
    a, ta, _, _ = oracle.trace(tris, rays, mode=0)
    b, tb, _, _ = oracle.trace(tris, rays, mode=1)
    assert (a != b).mean() < 2e-3
    both = (a == b) & (a >= 0)
    assert np.max(np.abs(ta[both] - tb[both]) / ta[both]) < 1e-5


def test_oracle_compat_render_matches_reference_fixture(oracle):
    from oracle.oracle import PROFILE_COMPAT, SceneData
    from salty_gb300 import scenes
    g = np.load(os.path.join(GOLDEN, "cornell_ref_64.npz"))
    sc = scenes.cornell("baseline")
    sd = SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], None, sc["sky"],
                   sc["camera"])
    spp = int(g["spp"])
    tot, sq = oracle.render(sd, int(g["width"]), int(g["height"]), spp, int(g["max_bounce"]),
                            profile=PROFILE_COMPAT, seed=777)
    m = tot / spp
    v = np.maximum((sq / spp - m * m) * spp / (spp - 1) / spp, 0)
    # 3-sigma per pixel (conftest.assert_within_3_sigma), none beyond 6 sigma
    assert_agree(m, v, g["mean"], g["var"])
    assert abs(m.mean() / g["mean"].mean() - 1) < 0.01


@pytest.mark.parametrize("variant,fixture,seed", [("glossy", "cornell_glossy_ref_48.npz", 31),
                                                  ("thinlens", "cornell_thinlens_ref_48.npz", 32),
                                                  ("textured", "cornell_textured_ref_48.npz", 33),
                                                  ("specular", "cornell_specular_ref_48.npz", 34)])
def test_oracle_compat_variants_match_reference_fixtures(oracle, variant, fixture, seed):
    """Phong and Plastic (src/s3d_phong.cpp:65-88, src/s3d_plastic.cpp:71-142), the
    ThinLensCamera (include/s3d_camera.h:150-267), colour maps with an environment map
    (src/s3d_texturedmaterial.cpp:63-87, src/s3d_texture.cpp:925-972), and Mirror and Glass
    (src/s3d_mirror.cpp:59-71, src/s3d_glass.cpp:60-128), through the reference's
    PathTracer::Radiance, at the fixture's sample count (the caustics of the glass box are
    heavy-tailed: at equal counts both sides miss their rare paths alike)."""
    from oracle.oracle import PROFILE_COMPAT, SceneData
    from salty_gb300 import scenes
    g = np.load(os.path.join(GOLDEN, fixture))
    sc = scenes.cornell(variant)
    sd = SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], None, sc["sky"],
                   sc["camera"], tri_uv=sc.get("tri_uv"), textures=sc.get("textures", []), ibl=sc.get("ibl"))
    spp = int(g["spp"])
    tot, sq = oracle.render(sd, int(g["width"]), int(g["height"]), spp, int(g["max_bounce"]),
                            profile=PROFILE_COMPAT, seed=seed)
    m = tot / spp
    v = np.maximum((sq / spp - m * m) * spp / (spp - 1) / spp, 0)
    assert_agree(m, v, g["mean"], g["var"])
    assert abs(m.mean() / g["mean"].mean() - 1) < 0.01


def test_oracle_physical_glossy_is_consistent(oracle):
    """Physical Phong / Plastic: two independent seeds agree within 3 sigma, and the one-sample
    mixture of the plastic converges (no NaN, finite variance)."""
    from oracle.oracle import PROFILE_PHYSICAL, SceneData
    from salty_gb300 import scenes
    sc = scenes.cornell("glossy")
    sd = SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], None, sc["sky"],
                   sc["camera"])
    res = []
    for seed in (1, 2):
        tot, sq = oracle.render(sd, 32, 32, 256, 8, rr_depth=3, profile=PROFILE_PHYSICAL, seed=seed)
        m = tot / 256
        res.append((m, np.maximum((sq / 256 - m * m) * 256 / 255 / 256, 0)))
    assert all(np.all(np.isfinite(m)) for m, _ in res)
    assert_agree(res[0][0], res[0][1], res[1][0], res[1][1])


def test_oracle_tonemap_matches_reference_fixture(oracle):
    g = np.load(os.path.join(GOLDEN, "tonemap_ref.npz"))
    img = g["img"]
    for k in (0, 1, 2):
        out, ave, mx = oracle.tonemap(k, img)
        assert np.array_equal(out, g[f"tm{k}"]), f"tonemap {k}"


def test_oracle_srgb_matches_reference_capture(oracle):
    g = np.load(os.path.join(GOLDEN, "tonemap_ref.npz"))
    out, _, _ = oracle.tonemap(2, g["img"])
    s8 = oracle.srgb8(out, ref_oetf=True)
    assert np.array_equal(s8, g["srgb_aces_ref"])


def test_oracle_nlm_matches_reference_fixture(oracle):
    g = np.load(os.path.join(GOLDEN, "nlm_ref.npz"))
    out = oracle.nlm_ref(g["rgba"], float(g["coeff"]))
    np.testing.assert_allclose(out, g["out"], rtol=2e-6, atol=1e-7)


def test_oracle_physical_render_is_consistent(oracle):
    """The physical estimator converges to the same image with and without MIS-relevant
    sampling changes: two seeds agree within 3 sigma (self-consistency of the checker)."""
    from oracle.oracle import PROFILE_PHYSICAL, SceneData
    from salty_gb300 import scenes
    sc = scenes.cornell("mixed")
    sd = SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], None, sc["sky"],
                   sc["camera"])
    res = []
    for seed in (1, 2):
        tot, sq = oracle.render(sd, 32, 32, 256, 8, profile=PROFILE_PHYSICAL, seed=seed)
        m = tot / 256
        res.append((m, np.maximum((sq / 256 - m * m) * 256 / 255 / 256, 0)))
    assert_agree(res[0][0], res[0][1], res[1][0], res[1][1])
