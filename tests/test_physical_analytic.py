"""The physical estimator against closed-form images (tests/analytic.py).

The reference cannot express the physical profile, so these scenes pin it from first
principles: white furnaces (energy conservation with and without Russian roulette, for
Lambert, mirror and glass), a Lambert plane under sky and sun (delta and disk, the disk
combined with BSDF sampling by MIS), a Lambert plane under the quad light (next-event
estimation and BSDF hits of the light, MIS), the exact Fresnel reflectance of a glass plane
under a half sky, GGX planes whose BSDF is integrated by quadrature (under the sky, and
under a disk sun through MIS), and a Lambert plane under a light sphere (cone sampling and
BSDF hits combined by MIS), alone and sharing the light list with the quad light.  Every pixel must agree with its expectation within the
3-sigma Monte Carlo bound of tests/analytic.check.

The oracle's physical path is checked here on the CPU at a small size; the CUDA path
(`-m gpu`) at a larger one.
"""
import numpy as np
import pytest

import analytic as A

PHYSICAL = 1

# name -> (builder(width, height) -> (scene, expectation), max_depth, rr_depth)
CASES = {
    "furnace-no-rr": (lambda w, h: A.furnace_box((0.5, 0.7, 0.8), (0.3, 0.2, 0.1), 24), 24, 24),
    "furnace-rr": (lambda w, h: A.furnace_box((0.5, 0.7, 0.8), (0.3, 0.2, 0.1), 24), 24, 3),
    "mirror-furnace": (lambda w, h: A.specular_furnace(A.MIRROR, (0.7, 1.0, 1.3)), 8, 8),
    # a faceted sphere traps some grazing rays in chains of total internal reflection that
    # last hundreds of bounces: the depth limit must not cut them
    "glass-furnace-rr": (lambda w, h: A.specular_furnace(A.GLASS), 2048, 3),
    "lambert-delta-sun": (lambda w, h: A.lambert_plane((0.5, 0.6, 0.7), (0.2, 0.3, 0.4), (0.3, 0.8, 0.2),
                                                       (2.0, 1.5, 1.0), 0.0), 4, 4),
    "lambert-disk-sun": (lambda w, h: A.lambert_plane((0.5, 0.6, 0.7), (0.2, 0.3, 0.4), (0.3, 0.8, 0.2),
                                                      (2.0, 1.5, 1.0), 0.08), 4, 4),
    "lambert-area-light": (lambda w, h: A.area_light_plane((0.6, 0.5, 0.4), (4.0, 3.0, 2.0), w, h), 4, 4),
    "glass-fresnel": (lambda w, h: A.glass_plane(1.5, w, h), 4, 4),
    "lambert-sphere-light": (lambda w, h: A.sphere_light_plane((0.6, 0.5, 0.4), (4.0, 3.0, 2.0), w, h), 4, 4),
    "lambert-sphere-and-quad-lights": (lambda w, h: A.sphere_light_plane((0.6, 0.5, 0.4), (4.0, 3.0, 2.0), w, h,
                                                                         with_quad=True), 4, 4),
    "ggx-sky-r05": (lambda w, h: A.ggx_plane((0.9, 0.7, 0.5), 0.5, w, h), 4, 4),
    "ggx-sky-r035": (lambda w, h: A.ggx_plane((0.95, 0.8, 0.6), 0.35, w, h), 4, 4),
    "ggx-disk-sun": (lambda w, h: A.ggx_plane((0.9, 0.7, 0.5), 0.5, w, h, sky=(0.0, 0.0, 0.0),
                                              sun=((-0.3, 0.9, 0.4), (3.0, 2.0, 1.0), 0.1)), 4, 4),
}


def _oracle_scene(sc):
    from oracle.oracle import SceneData
    return SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], sc["sun"],
                     sc["sky"], sc["camera"], textures=sc["textures"], ibl=sc["ibl"], ibl_scale=sc["ibl_scale"],
                     spheres=sc.get("spheres", []))


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_physical_matches_closed_form(oracle, name):
    build, depth, rr = CASES[name]
    W, H, spp = 24, 16, 256
    sc, expect = build(W, H)
    tot, sq = oracle.render(_oracle_scene(sc), W, H, spp, depth, rr_depth=rr, profile=PHYSICAL, seed=17)
    m = tot / spp
    v = np.maximum((sq / spp - m * m) * spp / (spp - 1) / spp, 0)
    A.check(m, v, expect)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_physical_matches_closed_form(ctx, name):
    from salty_gb300 import scenes
    build, depth, rr = CASES[name]
    W, H, spp = 64, 48, 1024
    sc, expect = build(W, H)
    s = scenes.upload(ctx, sc)
    s.build()
    r = s.render(W, H, spp, depth, rr_depth=rr, profile=PHYSICAL, seed=29)
    s.close()
    A.check(r["mean"], r["var"], expect)


def test_ggx_albedo_is_at_most_one():
    """The quadrature itself: a white (F0 = 1) GGX surface reflects at most what it gets, and
    nearly all of it when smooth (single scattering loses energy only at high roughness)."""
    for rough, lo in ((0.2, 0.97), (0.5, 0.85)):
        th, tab = A.ggx_albedo_table((1.0, 1.0, 1.0), rough * rough, n_o=12)
        assert np.all(tab <= 1.0 + 2e-3), (rough, tab.max())
        assert tab[th < np.radians(60.0)].min() > lo, (rough, tab.min())


def test_fresnel_formula_limits():
    c = np.array([1.0, 0.5, 1e-6])
    f = A.fresnel_unpolarised(c, 1.0, 1.5)
    assert abs(f[0] - 0.04) < 1e-12 and f[2] > 0.999
    assert np.all(A.fresnel_unpolarised(np.array([0.1]), 1.5, 1.0) == 1.0)  # total reflection


@pytest.mark.gpu
@pytest.mark.parametrize("depth,least", [(48, 0.99), (2048, 0.99999)])
def test_gpu_glass_furnace_conserves_energy(ctx, depth, least):
    """A glass object of colour 1 under a uniform sky, without Russian roulette: every
    sample is 1, or 0 when the depth limit cuts a chain of total internal reflections, so no
    pixel exceeds the sky, and with a deep enough limit every pixel equals it."""
    from salty_gb300 import scenes
    sc, sky = A.specular_furnace(A.GLASS)
    s = scenes.upload(ctx, sc)
    s.build()
    r = s.render(64, 48, 512, depth, rr_depth=depth, profile=PHYSICAL, seed=5)
    s.close()
    assert r["mean"].max() <= 1.0 + 1e-6
    assert r["mean"].mean() > least
