"""Scenes whose images the physical estimator must reproduce in closed form.

The reference cannot express the physical profile (cosine-weighted Lambert, exact-Fresnel
dielectric, GGX, sun and sky, unbiased Russian roulette), so its pins are analytic: each
scene below has a pixel expectation derived here from first principles, independently of
the renderer's sampling code.

  furnace_box       a closed Lambert box of albedo a emitting E on every wall, seen from
                    inside: every pixel = E (1 - a^D) / (1 - a) for D path segments
  specular_furnace  a mirror or glass object of colour 1 under a uniform sky S: every path
                    keeps weight 1 and ends in the sky, so every pixel is S (glass paths
                    cut by the depth limit give a little less, never more)
  lambert_plane     a Lambert plane under a sky S and a sun of irradiance E at angle theta
                    from the normal: a (S + E cos(theta) / pi), for a delta sun and for a
                    disk above the horizon alike
  area_light_plane  a Lambert plane under a one-sided quad light of radiance Le:
                    a Le / pi * (Lambert's polygon formula for the irradiance)
  glass_plane       a glass plane under a half sky (1 above the horizon, 0 below): the
                    pixel is the Fresnel reflectance of an unpolarised ray at its angle
  ggx_plane         a GGX plane under a uniform sky and/or a disk sun: the BSDF
                    f = F D G / (4 |n.o| |n.i|) (Walter et al. 2007; Smith G, Schlick F)
                    integrated by quadrature over incident directions

Pixel expectations average the closed form over the pixel's area (the physical profile
jitters camera rays uniformly in the pixel), using the camera model of PinholeCamera
(include/s3d_camera.h:63-100; fov linear in the screen half-extent).
"""
from __future__ import annotations

import math

import numpy as np

LAMBERT, MIRROR, GLASS, GGX = 0, 1, 2, 3


def _unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


# ---------------------------------------------------------------- camera
def pixel_dirs(cam: dict, width: int, height: int, sub: int = 4):
    """Camera origin and (H, W, sub*sub, 3) ray directions at stratified points of each pixel."""
    pos = np.asarray(cam["pos"], float)
    d = _unit(np.asarray(cam["target"], float) - pos)
    cx = _unit(np.cross(d, np.asarray(cam["up"], float))) * cam["fov"] * (width / height)
    cy = _unit(np.cross(d, cx)) * cam["fov"]
    cz = pos + d * cam.get("near", 1.0)
    j = (np.arange(sub) + 0.5) / sub
    jx, jy = np.meshgrid(j, j)
    fx = (np.arange(width)[None, :, None] + jx.ravel()[None, None, :]) / width - 0.5
    fy = (np.arange(height)[:, None, None] + jy.ravel()[None, None, :]) / height - 0.5
    fx = np.broadcast_to(fx, (height, width, sub * sub))
    fy = np.broadcast_to(fy, (height, width, sub * sub))
    q = cx * fx[..., None] + cy * fy[..., None] + cz
    return pos, _unit(q - pos)


def plane_hits(pos, dirs):
    """Points where the rays meet the plane y = 0 (all rays must point downwards)."""
    assert np.all(dirs[..., 1] < 0), "a camera ray misses the plane"
    t = -pos[1] / dirs[..., 1]
    return pos + dirs * t[..., None]


# ---------------------------------------------------------------- geometry
def quad(p0, p1, p2, p3):
    return [np.array([p0, p1, p2], np.float32), np.array([p0, p2, p3], np.float32)]


def plane_tris(half: float = 60.0):
    return np.stack(quad((-half, 0, -half), (-half, 0, half), (half, 0, half), (half, 0, -half))).reshape(-1, 9)


def cube_tris(h: float = 1.0):
    v = [(-h, -h, -h), (h, -h, -h), (h, h, -h), (-h, h, -h), (-h, -h, h), (h, -h, h), (h, h, h), (-h, h, h)]
    faces = [(0, 1, 2, 3), (5, 4, 7, 6), (4, 0, 3, 7), (1, 5, 6, 2), (3, 2, 6, 7), (4, 5, 1, 0)]
    t = []
    for f in faces:
        t += quad(*[v[k] for k in f])
    return np.stack(t).reshape(-1, 9)


def icosphere_tris(subdiv: int = 3, radius: float = 1.0):
    from salty_gb300.scenes import _icosphere
    return (_icosphere(subdiv) * radius).astype(np.float32).reshape(-1, 9)


def scene(tris, mats, mat_ids=None, *, camera, sky=(0, 0, 0), sun=None, light=None, textures=(), ibl=None,
          spheres=()):
    n = tris.shape[0]
    return {"tri_pos": np.ascontiguousarray(tris, np.float32), "tri_nrm": None,
            "tri_mat": np.zeros(n, np.int32) if mat_ids is None else np.asarray(mat_ids, np.int32),
            "materials": mats, "light": light, "sun": sun, "sky": tuple(sky), "camera": camera,
            "textures": list(textures), "ibl": ibl, "ibl_scale": 1.0, "spheres": list(spheres)}


LOOK_DOWN = {"pos": (0.0, 1.0, -2.0), "target": (0.0, 0.0, 0.0), "up": (0.0, 1.0, 0.0),
             "fov": 2.0 * math.tan(math.radians(10.0)), "near": 1.0}


# ---------------------------------------------------------------- the scenes
def furnace_box(albedo, emission, depth):
    cam = {"pos": (0.1, -0.2, 0.05), "target": (0.4, 0.1, 1.0), "up": (0.0, 1.0, 0.0),
           "fov": 2.0 * math.tan(math.radians(40.0)), "near": 1.0}
    sc = scene(cube_tris(), [{"type": LAMBERT, "color": albedo, "emission": emission}], camera=cam)
    a, e = np.asarray(albedo, float), np.asarray(emission, float)
    return sc, e * (1.0 - a ** depth) / (1.0 - a)


def specular_furnace(kind: int, sky=(1.0, 1.0, 1.0)):
    cam = {"pos": (0.0, 0.3, -4.0), "target": (0.0, 0.0, 0.0), "up": (0.0, 1.0, 0.0),
           "fov": 2.0 * math.tan(math.radians(16.0)), "near": 1.0}
    m = {"type": kind, "color": (1.0, 1.0, 1.0), "ior": 1.5}
    return scene(icosphere_tris(3), [m], camera=cam, sky=sky), np.asarray(sky, float)


def lambert_plane(albedo, sky, sun_dir, sun_e, half_angle):
    sd = _unit(np.asarray(sun_dir, float))
    sun = {"dir": tuple(sd), "radiance": tuple(sun_e), "half_angle": half_angle}
    sc = scene(plane_tris(), [{"type": LAMBERT, "color": albedo}], camera=LOOK_DOWN, sky=sky, sun=sun)
    a = np.asarray(albedo, float)
    return sc, a * (np.asarray(sky, float) + np.asarray(sun_e, float) * sd[1] / math.pi)


def polygon_irradiance(points, verts, normal=(0.0, 1.0, 0.0)):
    """Irradiance per unit radiance at `points` (..., 3) from a polygon (k, 3) fully above
    their tangent plane: Lambert's formula, 1/2 |sum_i angle_i (n . unit(v_i x v_i+1))|."""
    n = np.asarray(normal, float)
    v = _unit(np.asarray(verts, float)[None] - points.reshape(-1, 1, 3))
    w = np.roll(v, -1, axis=1)
    ang = np.arccos(np.clip(np.sum(v * w, -1), -1.0, 1.0))
    g = _unit(np.cross(v, w))
    return (0.5 * np.abs(np.sum(ang * (g @ n), -1))).reshape(points.shape[:-1])


def area_light_plane(albedo, le, width, height, sub=6):
    light = {"corner": (-0.3, 1.0, -0.2), "edge_a": (0.6, 0.0, 0.0), "edge_b": (0.0, 0.0, 0.5),
             "emission": tuple(le)}
    cam = {"pos": (0.0, 0.6, -2.5), "target": (0.0, 0.0, 0.2), "up": (0.0, 1.0, 0.0),
           "fov": 2.0 * math.tan(math.radians(12.0)), "near": 1.0}
    sc = scene(plane_tris(), [{"type": LAMBERT, "color": albedo}], camera=cam, light=light)
    c, ea, eb = (np.asarray(light[k], float) for k in ("corner", "edge_a", "edge_b"))
    verts = np.stack([c, c + ea, c + ea + eb, c + eb])
    pos, dirs = pixel_dirs(cam, width, height, sub)
    # no camera ray may reach the light's plane (y = 1) before the floor
    assert np.all(dirs[..., 1] < 0)
    e = polygon_irradiance(plane_hits(pos, dirs), verts).mean(-1)
    return sc, (np.asarray(albedo, float) * np.asarray(le, float) / math.pi)[None, None, :] * e[..., None]


def sphere_light_plane(albedo, le, width, height, with_quad=False, sub=6):
    """A Lambert plane under a light sphere of radiance le (and, with_quad, also under the
    quad light of area_light_plane, the two sharing the light list).  A sphere of radius R
    whose centre is at distance d and angle theta from the normal, wholly above the horizon,
    gives the irradiance E = pi le (R / d)^2 cos theta; reflected radiance albedo E / pi."""
    c, R = np.array([0.85, 0.9, 0.5]), 0.2  # clear of the quad light and its light paths
    mats = [{"type": LAMBERT, "color": albedo},
            {"type": LAMBERT, "color": (0.0, 0.0, 0.0), "emission": tuple(le)}]
    light = None
    if with_quad:
        light = {"corner": (-0.3, 1.0, -0.2), "edge_a": (0.6, 0.0, 0.0), "edge_b": (0.0, 0.0, 0.5),
                 "emission": tuple(le)}
    cam = {"pos": (0.0, 0.6, -2.5), "target": (0.0, 0.0, 0.2), "up": (0.0, 1.0, 0.0),
           "fov": 2.0 * math.tan(math.radians(12.0)), "near": 1.0}
    sc = scene(plane_tris(), mats, camera=cam, light=light,
               spheres=[{"center": tuple(c), "radius": R, "material": 1, "light": True}])
    pos, dirs = pixel_dirs(cam, width, height, sub)
    assert np.all(dirs[..., 1] < 0) and c[1] - R > cam["pos"][1]  # the camera sees only the floor
    x = plane_hits(pos, dirs)
    w = c - x
    d2 = np.sum(w * w, -1)
    cos_t = w[..., 1] / np.sqrt(d2)
    assert np.all(cos_t > R / np.sqrt(d2))  # the whole sphere above the horizon
    e = (math.pi * R * R / d2 * cos_t).mean(-1)
    if with_quad:
        verts = np.stack([np.asarray(light["corner"]), np.asarray(light["corner"]) + np.asarray(light["edge_a"]),
                          np.asarray(light["corner"]) + np.asarray(light["edge_a"]) + np.asarray(light["edge_b"]),
                          np.asarray(light["corner"]) + np.asarray(light["edge_b"])])
        e = e + polygon_irradiance(x, verts).mean(-1)
    return sc, (np.asarray(albedo, float) * np.asarray(le, float) / math.pi)[None, None, :] * e[..., None]


def fresnel_unpolarised(cos_i, n1, n2):
    """Fresnel reflectance of unpolarised light (Born & Wolf), total reflection -> 1."""
    sin_t = n1 / n2 * np.sqrt(np.maximum(0.0, 1.0 - cos_i ** 2))
    tir = sin_t >= 1.0
    cos_t = np.sqrt(np.maximum(0.0, 1.0 - sin_t ** 2))
    rs = (n1 * cos_i - n2 * cos_t) / (n1 * cos_i + n2 * cos_t)
    rp = (n2 * cos_i - n1 * cos_t) / (n2 * cos_i + n1 * cos_t)
    return np.where(tir, 1.0, 0.5 * (rs ** 2 + rp ** 2))


def half_sky_texture(w: int = 64, h: int = 32):
    """Latitude-longitude map: radiance 1 above the horizon, 0 below (rows are the polar
    angle from +y, Texture::SampleColor(dir))."""
    t = np.zeros((h, w, 3), np.float32)
    t[: h // 2] = 1.0
    return t


def glass_plane(ior, width, height, sub=4):
    sc = scene(plane_tris(), [{"type": GLASS, "color": (1.0, 1.0, 1.0), "ior": ior}], camera=LOOK_DOWN,
               textures=[half_sky_texture()], ibl=0)
    _, dirs = pixel_dirs(LOOK_DOWN, width, height, sub)
    cos_i = -dirs[..., 1]
    # the reflected ray must stay in the texture's lit rows and the refracted one in its dark
    # rows; with 32 rows, polar angles below 87.1 deg read 1 and above 92.9 deg read 0
    assert np.degrees(np.arccos(cos_i)).max() < 87.0
    f = fresnel_unpolarised(cos_i, 1.0, ior).mean(-1)
    return sc, np.repeat(f[..., None], 3, -1)


def _ggx_f(cos_o, wi, f0, alpha):
    """BSDF times cos(theta_i) for outgoing directions at polar angles acos(cos_o) in the
    xy-plane (normal +y) and incident directions wi (..., 3).  Shapes broadcast."""
    wo = np.stack([np.sqrt(np.maximum(0.0, 1.0 - cos_o ** 2)), cos_o, np.zeros_like(cos_o)], -1)
    h = _unit(wo + wi)
    nh, oh, ni = h[..., 1], np.sum(wo * h, -1), wi[..., 1]
    a2 = alpha * alpha
    d = a2 / (math.pi * (nh * nh * (a2 - 1.0) + 1.0) ** 2)

    def g1(c):
        return 2.0 * c / (c + np.sqrt(a2 + (1.0 - a2) * c * c))

    g = g1(cos_o) * g1(ni)
    m5 = (1.0 - oh) ** 5
    f = np.asarray(f0, float) + (1.0 - np.asarray(f0, float)) * m5[..., None]
    val = f * (d * g / (4.0 * cos_o))[..., None]   # f * cos_i: the cos_i cancels
    return np.where((ni > 0)[..., None], val, 0.0)


def ggx_albedo_table(f0, alpha, n_o=96, n_t=384, n_p=768):
    """Directional albedo of the GGX BSDF, per channel, at outgoing polar angles in
    (0, 89) degrees: midpoint quadrature over the incident hemisphere."""
    th_o = np.radians(np.linspace(1.0, 89.0, n_o))
    th = (np.arange(n_t) + 0.5) * (0.5 * math.pi / n_t)
    ph = (np.arange(n_p) + 0.5) * (2.0 * math.pi / n_p)
    T, P = np.meshgrid(th, ph, indexing="ij")
    wi = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1)
    dw = np.sin(T) * (0.5 * math.pi / n_t) * (2.0 * math.pi / n_p)
    out = np.empty((n_o, 3))
    for k, t in enumerate(th_o):
        out[k] = np.sum(_ggx_f(np.full(T.shape, math.cos(t)), wi, f0, alpha) * dw[..., None], axis=(0, 1))
    return th_o, out


def ggx_plane(f0, roughness, width, height, sky=(1.0, 1.0, 1.0), sun=None, sub=3):
    """sun: (dir, irradiance, half_angle) of a disk sun, or None."""
    alpha = roughness * roughness
    s = None
    if sun is not None:
        sd = _unit(np.asarray(sun[0], float))
        s = {"dir": tuple(sd), "radiance": tuple(sun[1]), "half_angle": sun[2]}
    sc = scene(plane_tris(), [{"type": GGX, "color": f0, "roughness": roughness}], camera=LOOK_DOWN, sky=sky,
               sun=s)
    _, dirs = pixel_dirs(LOOK_DOWN, width, height, sub)
    wo = -dirs                                          # towards the camera
    cos_o = wo[..., 1]
    expect = np.zeros((height, width, 3))
    if any(sky):
        th_o, tab = ggx_albedo_table(f0, alpha)
        th = np.arccos(cos_o)
        for c in range(3):
            expect[..., c] += sky[c] * np.interp(th, th_o, tab[:, c]).mean(-1)
    if sun is not None:
        # rotate each wo into the xy-plane about the normal; integrate over the sun's cone
        sd = _unit(np.asarray(sun[0], float))
        half = sun[2]
        n_r, n_c = 16, 64
        psi = (np.arange(n_r) + 0.5) * (half / n_r)
        chi = (np.arange(n_c) + 0.5) * (2.0 * math.pi / n_c)
        Ps, Cs = np.meshgrid(psi, chi, indexing="ij")
        t = _unit(np.cross(sd, [0.0, 0.0, 1.0] if abs(sd[2]) < 0.9 else [1.0, 0.0, 0.0]))
        b = np.cross(sd, t)
        cone = (np.cos(Ps)[..., None] * sd + (np.sin(Ps) * np.cos(Cs))[..., None] * t
                + (np.sin(Ps) * np.sin(Cs))[..., None] * b).reshape(-1, 3)
        dw = (np.sin(Ps) * (half / n_r) * (2.0 * math.pi / n_c)).reshape(-1)
        le = np.asarray(sun[1], float) / (math.pi * math.sin(half) ** 2)   # irradiance facing it
        phi = np.arctan2(wo[..., 2], wo[..., 0])
        cph, sph = np.cos(-phi), np.sin(-phi)
        flat_o, cph, sph = cos_o.reshape(-1), cph.reshape(-1, 1), sph.reshape(-1, 1)
        e = np.empty((flat_o.size, 3))
        for k in range(0, flat_o.size, 512):
            sl = slice(k, k + 512)
            # incident directions in each wo's frame (rotation about +y taking wo to phi = 0)
            cx = cph[sl] * cone[None, :, 0] - sph[sl] * cone[None, :, 2]
            cz = sph[sl] * cone[None, :, 0] + cph[sl] * cone[None, :, 2]
            wi = np.stack([cx, np.broadcast_to(cone[None, :, 1], cx.shape), cz], -1)
            e[sl] = np.sum(_ggx_f(flat_o[sl, None], wi, f0, alpha) * dw[None, :, None], 1) * le
        expect += e.reshape(height, width, -1, 3).mean(2)
    return sc, expect


# ---------------------------------------------------------------- the check
def local_variance(var, r: int = 2):
    """Per pixel, the larger of its own variance of the mean and the mean over its
    (2r+1)^2 neighbourhood.  A pixel whose samples all missed a rare, large contribution
    (a BSDF ray into a small sun disk, a long chain of total internal reflection) has a
    mean below its expectation AND a variance estimate far below its true variance; its
    neighbours' estimates, which include such events, restore a sound bound."""
    v = np.asarray(var, float)
    p = np.pad(v, ((r, r), (r, r)) + ((0, 0),) * (v.ndim - 2), mode="edge")
    acc = np.zeros_like(v)
    for dy in range(2 * r + 1):
        for dx in range(2 * r + 1):
            acc += p[dy:dy + v.shape[0], dx:dx + v.shape[1]]
    return np.maximum(v, acc / (2 * r + 1) ** 2)


def agree(mean, var, expect, rel=2e-4, zmax=6.0):
    """Per pixel-channel z-scores of a render against its expectation (3 sigma bound: the
    fraction beyond 3, the largest |z|) and the image mean's z.  `rel` covers the quadrature
    of the expectation and FP32 accumulation; the variance is the pixel's own or its
    neighbourhood's, whichever is larger (local_variance)."""
    mean, var = np.asarray(mean, float), local_variance(var)
    expect = np.broadcast_to(np.asarray(expect, float), mean.shape)
    floor = (rel * np.abs(expect)) ** 2
    z = (mean - expect) / np.sqrt(var + floor + 1e-30)
    n = mean.size
    zg = (mean.mean() - expect.mean()) / math.sqrt(var.sum() / n / n + (rel * abs(expect.mean())) ** 2 + 1e-30)
    return float(np.mean(np.abs(z) > 3)), float(np.max(np.abs(z))), float(zg)


def check(mean, var, expect, **kw):
    """agree() against the bounds: the count beyond 3 sigma within the binomial bound of a
    normal variable (conftest.beyond3_bound), none beyond zmax, the image mean within 4
    sigma."""
    from conftest import beyond3_bound
    f, zm, zg = agree(mean, var, expect, **kw)
    n = np.asarray(mean).size
    assert f * n <= beyond3_bound(n) and zm < kw.get("zmax", 6.0) and abs(zg) < 4.0, (f, n, zm, zg)
