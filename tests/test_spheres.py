"""Analytic spheres (Sphere, src/s3d_sphere.cpp:22-115): intersection, shading and sphere
lights.

* Hits: a scene of triangles and spheres against the same triangles traced alone plus a
  float64 ray/sphere test in numpy -- the reference formula (Sphere::IsHit) for the compat
  test, the exact roots for the watertight one.
* Compat renders (PathTracer::Radiance with Sphere::CalcParam and Sphere::Sample, the light
  picked uniformly from the quad light and a light sphere) against the reference's own
  render (tests/golden/cornell_spheres_ref_48.npz, from the unmodified reference).
* Physical renders against the oracle; closed-form sphere-light images are in
  tests/test_physical_analytic.py.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, assert_within_3_sigma


def _oracle_scene(sc):
    from oracle.oracle import SceneData
    return SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], sc["sun"],
                     sc["sky"], sc["camera"], tri_uv=sc.get("tri_uv"), textures=sc.get("textures", []),
                     ibl=sc.get("ibl"), spheres=sc.get("spheres", []))


def _zcheck(ma, va, mb, vb):
    """Per pixel-channel z-scores and the image means against the 3-sigma bounds."""
    ma, va, mb, vb = (np.asarray(x, float) for x in (ma, va, mb, vb))
    floor = (1e-5 * np.maximum(np.abs(ma), np.abs(mb))) ** 2
    v = np.maximum(va + vb + floor, 1e-30)
    assert_within_3_sigma((ma - mb) / np.sqrt(v), zsum=float((ma - mb).sum() / np.sqrt(v.sum())))


def test_oracle_compat_spheres_match_reference_fixture(oracle):
    from oracle.oracle import PROFILE_COMPAT
    from salty_gb300 import scenes
    g = np.load(os.path.join(GOLDEN, "cornell_spheres_ref_48.npz"))
    spp = int(g["spp"])
    tot, sq = oracle.render(_oracle_scene(scenes.cornell("spheres")), int(g["width"]), int(g["height"]), spp,
                            int(g["max_bounce"]), profile=PROFILE_COMPAT, seed=99)
    m = tot / spp
    _zcheck(m, np.maximum((sq / spp - m * m) / (spp - 1), 0), g["mean"], g["var"])


# ---------------------------------------------------------------- GPU
def _sphere_scene_arrays(seed):
    """A floor and 40 random triangles, 60 spheres between them."""
    rng = np.random.default_rng(seed)
    tris = rng.uniform(-2, 2, (40, 3, 3)).astype(np.float32)
    floor = np.array([[[-5, -1, -5], [-5, -1, 5], [5, -1, 5]], [[-5, -1, -5], [5, -1, 5], [5, -1, -5]]], np.float32)
    pos = np.concatenate([tris, floor]).reshape(-1, 9)
    spheres = [{"center": tuple(rng.uniform(-2, 2, 3)), "radius": float(rng.uniform(0.1, 0.7)), "material": 0}
               for _ in range(60)]
    return pos, spheres


def _rays(seed, n):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-3, 3, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = o, 1e-3, d, 1e12
    return r


def _sphere_hits(rays, spheres, reference_formula):
    """float64 closest sphere hit per ray, with the spheres as the library stores them
    (float32 centre and radius): t (inf when none), sphere index and the cosine of the
    angle of incidence (a grazing hit's t is ill-conditioned)."""
    o = rays[:, 0:3].astype(np.float64)
    d = rays[:, 4:7].astype(np.float64)
    tmin = rays[:, 3].astype(np.float64)
    best = np.full(len(rays), np.inf)
    idx = np.full(len(rays), -1)
    cos_in = np.zeros(len(rays))
    for k, s in enumerate(spheres):
        c = np.asarray(s["center"], np.float32).astype(np.float64)
        rad = float(np.float32(s["radius"]))
        po = c - o
        b = np.sum(po * d, 1)
        disc = b * b - np.sum(po * po, 1) + rad * rad
        ok = disc >= 0
        sq = np.sqrt(np.maximum(disc, 0))
        t1, t2 = b - sq, b + sq
        if reference_formula:   # nearer root above tmin, else the farther
            t = np.where(t1 > tmin, t1, t2)
            ok &= ~((t1 < tmin) & (t2 < tmin))
        else:
            t = np.where(t1 >= 0, t1, t2)
            ok &= t >= 0
        better = ok & (t < best)
        best = np.where(better, t, best)
        idx = np.where(better, k, idx)
        cos_in = np.where(better, sq / rad, cos_in)
    return best, idx, cos_in


@pytest.mark.gpu
@pytest.mark.parametrize("watertight", [False, True])
def test_sphere_hits_match_float64(ctx, watertight):
    pos, spheres = _sphere_scene_arrays(3)
    mats = [{"type": 0, "color": (0.5, 0.5, 0.5)}]
    cam = {"pos": (0, 0, -5), "target": (0, 0, 0), "up": (0, 1, 0), "fov": 1.0, "near": 1.0}
    both = ctx.upload_scene(pos, None, np.zeros(len(pos), np.int32), materials=mats, camera=cam)
    both.set_spheres(spheres)
    both.build()
    tri_only = ctx.upload_scene(pos, None, np.zeros(len(pos), np.int32), materials=mats, camera=cam)
    tri_only.build()
    rays = _rays(5, 200_000)
    if watertight:
        rays[:, 3] = 0.0
    hb = both.trace(rays, watertight=watertight)
    ht = tri_only.trace(rays, watertight=watertight)
    ts, ks, cos_in = _sphere_hits(rays, spheres, reference_formula=not watertight)
    n_tris = len(pos)
    tri_t = np.where(ht.ids >= 0, ht.t.astype(np.float64), np.inf)
    want = np.where(ks >= 0, n_tris + ks, -1)
    want = np.where(tri_t <= ts, ht.ids, want)
    # ties within rounding between a triangle and a sphere, or two spheres, are left out
    with np.errstate(invalid="ignore"):  # inf - inf where neither is hit
        near_tie = np.abs(tri_t - ts) <= 1e-4 * np.minimum(tri_t, ts)
    assert (ks >= 0).mean() > 0.2
    ok = ~near_tie
    assert np.mean(hb.ids[ok] == want[ok]) > 0.9999, np.mean(hb.ids[ok] == want[ok])
    # distances of hits that are not grazing (FP32 rounding of t grows as 1 / cos)
    sph = ok & (hb.ids >= n_tris) & (hb.ids == want) & (cos_in > 0.05)
    np.testing.assert_allclose(hb.t[sph], ts[sph], rtol=2e-5, atol=2e-6)
    both.close()
    tri_only.close()


@pytest.mark.gpu
def test_compat_spheres_match_reference_fixture(ctx):
    """The reference's estimator with Sphere shapes and a light sphere, GPU compat profile."""
    import salty_gb300
    from salty_gb300 import scenes
    g = np.load(os.path.join(GOLDEN, "cornell_spheres_ref_48.npz"))
    s = scenes.upload(ctx, scenes.cornell("spheres"))
    s.build()
    r = s.render(int(g["width"]), int(g["height"]), int(g["spp"]), int(g["max_bounce"]),
                 profile=salty_gb300.PROFILE_COMPAT, seed=4545)
    s.close()
    _zcheck(r["mean"], r["var"], g["mean"], g["var"])
    assert abs(r["mean"].mean() / g["mean"].mean() - 1) < 0.01


@pytest.mark.gpu
def test_physical_spheres_match_oracle(ctx, oracle):
    import salty_gb300
    from oracle.oracle import PROFILE_PHYSICAL
    from salty_gb300 import scenes
    sc = scenes.cornell("spheres")
    W = H = 48
    spp = 1024
    s = scenes.upload(ctx, sc)
    s.build()
    r = s.render(W, H, spp, 8, rr_depth=3, profile=salty_gb300.PROFILE_PHYSICAL, seed=98)
    s.close()
    tot, sq = oracle.render(_oracle_scene(sc), W, H, spp, 8, rr_depth=3, profile=PROFILE_PHYSICAL, seed=1235)
    m = tot / spp
    _zcheck(r["mean"], r["var"], m, np.maximum((sq / spp - m * m) / (spp - 1), 0))


@pytest.mark.gpu
def test_sphere_scenes_are_not_batched_or_instanced(ctx):
    import salty_gb300
    from salty_gb300 import scenes
    a = scenes.upload(ctx, scenes.cornell("spheres"))
    a.build()
    b = scenes.upload(ctx, scenes.cornell("baseline"))
    b.build()
    o = {"width": 16, "height": 16, "spp": 1, "max_depth": 2}
    with pytest.raises(salty_gb300.SaltyError):
        ctx.render_batch([a, b], [o, o])
    eye = np.hstack([np.eye(3), np.zeros((3, 1))])
    with pytest.raises(salty_gb300.SaltyError):
        a.set_instances([(0, 10, eye)])
    with pytest.raises(salty_gb300.SaltyError):
        a.set_spheres([{"center": (0, 0, 0), "radius": -1.0}])
    with pytest.raises(salty_gb300.SaltyError):
        a.set_spheres([{"center": (0, 0, 0), "radius": 1.0, "material": 99}])
    a.set_spheres([])          # back to triangles only
    a.build()
    r = a.render(16, 16, 4, 4, want=("mean",))
    assert np.all(np.isfinite(r["mean"]))
    a.close()
    b.close()
