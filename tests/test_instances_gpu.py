"""Two-level instancing (salty_scene_set_instances) against flattened copies.

Instance (src/s3d_instance.cpp:22-101) keeps one copy of a mesh under several transforms;
here a scene's meshes are placed by 3x4 matrices in a two-level BVH and rays enter each
instance transformed to object space.  The same copies placed as transformed triangles in
a flat scene must give the same world: ids (virtual ids number the instances' triangles in
instance order, which is exactly the order of the flattened copies) and distances agree up
to the rounding of transforming rays instead of vertices, and renders agree within the
3-sigma Monte Carlo bound.
"""
import math

import numpy as np
import pytest

from test_render_gpu import zcheck

pytestmark = pytest.mark.gpu


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def _library():
    """Mesh library: an icosphere (320 triangles, smooth normals), a box (12), a ground quad
    (2); materials Lambert, mirror, Lambert."""
    from salty_gb300.scenes import _box, _icosphere, _quad
    ico = _icosphere(2).astype(np.float32)                      # (320, 3, 3), unit sphere
    flat = np.concatenate([np.stack(_box((1.0, 1.0, 1.0), 0.0, (0.0, -0.5, 0.0))),
                           np.stack(_quad((-8, 0, -8), (-8, 0, 8), (8, 0, 8), (8, 0, -8)))]).astype(np.float32)
    g = np.cross(flat[:, 1] - flat[:, 0], flat[:, 2] - flat[:, 0])
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pos = np.concatenate([ico.reshape(-1, 9), flat.reshape(-1, 9)])
    nrm = np.concatenate([ico.reshape(-1, 9), np.tile(g, (1, 3))]).astype(np.float32)
    mat = np.concatenate([np.zeros(320), np.ones(12), np.full(2, 2)]).astype(np.int32)
    mats = [{"type": 0, "color": (0.7, 0.5, 0.3)}, {"type": 1, "color": (0.9, 0.9, 0.9)},
            {"type": 0, "color": (0.6, 0.6, 0.6)}]
    return pos, nrm, mat, mats


def _placements(seed, n):
    rng = np.random.default_rng(seed)
    inst = [(332, 2, np.hstack([np.eye(3), np.zeros((3, 1))]))]  # the ground, untransformed
    for i in range(n):
        first, cnt = ((0, 320), (320, 12))[i % 2]
        lin = _rotation(rng) @ np.diag(rng.uniform(0.15, 0.45, 3))
        t = np.array([rng.uniform(-3, 3), rng.uniform(0.3, 1.5), rng.uniform(-3, 3)])
        inst.append((first, cnt, np.hstack([lin, t[:, None]])))
    return inst


def _flatten(pos, nrm, mat, inst):
    P, N, M = [], [], []
    for first, cnt, m in inst:
        lin, t = m[:, :3].astype(np.float64), m[:, 3].astype(np.float64)
        v = pos[first:first + cnt].reshape(-1, 3, 3).astype(np.float64)
        P.append((v @ lin.T + t).astype(np.float32).reshape(-1, 9))
        n = nrm[first:first + cnt].reshape(-1, 3, 3).astype(np.float64) @ np.linalg.inv(lin)
        n /= np.linalg.norm(n, axis=-1, keepdims=True)
        N.append(n.astype(np.float32).reshape(-1, 9))
        M.append(mat[first:first + cnt])
    return np.concatenate(P), np.concatenate(N), np.concatenate(M)


CAM = {"pos": (0.0, 2.5, -7.0), "target": (0.0, 0.5, 0.0), "up": (0.0, 1.0, 0.0),
       "fov": 2.0 * math.tan(math.radians(28.0)), "near": 1.0}
LIGHT = {"corner": (-1.0, 4.0, -1.0), "edge_a": (2.0, 0.0, 0.0), "edge_b": (0.0, 0.0, 2.0),
         "emission": (6.0, 5.0, 4.0)}


@pytest.fixture(scope="module")
def scenes_pair(ctx):
    pos, nrm, mat, mats = _library()
    inst = _placements(3, 60)
    fp, fn, fm = _flatten(pos, nrm, mat, inst)
    sun = {"dir": (0.3, 0.8, -0.4), "radiance": (2.0, 1.8, 1.5), "half_angle": 0.0}
    common = dict(materials=mats, light=LIGHT, sun=sun, sky=(0.3, 0.35, 0.4), camera=CAM)
    a = ctx.upload_scene(pos, nrm, mat, **common)
    a.set_instances(inst)
    ia = a.build()
    b = ctx.upload_scene(fp, fn, fm, **common)
    ib = b.build()
    yield a, b, ia, ib, fp.shape[0]
    a.close()
    b.close()


def _rays(seed, n):
    rng = np.random.default_rng(seed)
    o = rng.uniform(-4, 4, (n, 3)) * np.array([1.0, 0.5, 1.0]) + np.array([0.0, 2.5, 0.0])
    tgt = rng.uniform(-3, 3, (n, 3)) * np.array([1.0, 0.3, 1.0]) + np.array([0.0, 0.6, 0.0])
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = o, 1e-4, d, np.inf
    return r


@pytest.mark.parametrize("watertight", [True, False])
def test_instanced_hits_match_flattened_copies(scenes_pair, watertight):
    a, b, _, _, n_flat = scenes_pair
    rays = _rays(11, 200_000)
    ha = a.trace(rays, watertight=watertight)
    hb = b.trace(rays, watertight=watertight)
    hit = hb.ids >= 0
    assert hit.mean() > 0.5
    same = ha.ids == hb.ids
    assert same.mean() > 0.999, same.mean()
    both = same & hit
    np.testing.assert_allclose(ha.t[both], hb.t[both], rtol=2e-4, atol=1e-5)
    assert ha.ids.max() < n_flat + 2  # virtual ids: instances' triangles, then the light's two


def test_any_hit_agrees(scenes_pair):
    a, b, _, _, _ = scenes_pair
    rays = _rays(12, 100_000)
    ha = a.trace(rays, any_hit=True, watertight=True)
    hb = b.trace(rays, any_hit=True, watertight=True)
    assert np.mean((ha.ids >= 0) == (hb.ids >= 0)) > 0.999


def test_instances_store_each_mesh_once(scenes_pair):
    """61 placements of three meshes: the instanced scene's BVH holds the meshes once plus
    a small top level, the flattened one every copy."""
    _, _, ia, ib, _ = scenes_pair
    assert ia["n_nodes"] < 0.25 * ib["n_nodes"], (ia["n_nodes"], ib["n_nodes"])


@pytest.mark.parametrize("profile", [0, 1])
def test_instanced_render_matches_flattened(scenes_pair, profile):
    """Sky, sun, quad light (kept in world space), Lambert and mirror instances, both
    estimators: per pixel within 3 sigma of the flattened copies' render."""
    a, b, _, _, _ = scenes_pair
    W, H, spp = 48, 32, 512
    ra = a.render(W, H, spp, 6, rr_depth=3, profile=profile, seed=31)
    rb = b.render(W, H, spp, 6, rr_depth=3, profile=profile, seed=32)
    zcheck(ra["mean"], ra["var"], rb["mean"], rb["var"])
    assert abs(ra["mean"].mean() / rb["mean"].mean() - 1) < 0.01


def test_batch_rejects_instanced_scenes(ctx, scenes_pair):
    import salty_gb300
    a, b, _, _, _ = scenes_pair
    o = {"width": 16, "height": 16, "spp": 1, "max_depth": 2}
    with pytest.raises(salty_gb300.SaltyError):
        ctx.render_batch([a, b], [o, o])


def test_set_instances_validates(ctx):
    import salty_gb300
    pos, nrm, mat, mats = _library()
    s = ctx.upload_scene(pos, nrm, mat, materials=mats, camera=CAM)
    eye = np.hstack([np.eye(3), np.zeros((3, 1))])
    with pytest.raises(salty_gb300.SaltyError):
        s.set_instances([(330, 10, eye)])            # past the scene's triangles
    with pytest.raises(salty_gb300.SaltyError):
        s.set_instances([(0, 320, np.zeros((3, 4)))])  # singular
    s.set_instances([(0, 320, eye)])
    s.build()
    s.set_instances([])                               # back to the flat scene
    s.build()
    assert s.trace(_rays(13, 1000)).ids.max() < pos.shape[0]
    s.close()
