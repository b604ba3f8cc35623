"""Seeded synthetic scenes of the benchmark configurations (numpy, host side).

Each builder returns a dict with the keyword arguments of Context.upload_scene, plus
"name".  The same arrays feed the GPU library, the oracle restatement and the reference
harness, so all three see identical inputs.
"""
from __future__ import annotations

import math

import numpy as np

from . import GGX, GLASS, LAMBERT, MIRROR, PHONG, PLASTIC, microbench_soup


def _quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3); normal = (p1-p0) x (p2-p0)."""
    return [np.array([p0, p1, p2], np.float32), np.array([p0, p2, p3], np.float32)]


def _box(size, rot_deg, base):
    """Axis box of the given size rotated about y by rot_deg and placed with its base
    centre at `base`; 12 outward-facing triangles."""
    sx, sy, sz = size
    c, s = math.cos(math.radians(rot_deg)), math.sin(math.radians(rot_deg))

    def P(x, y, z):
        x, z = x - sx / 2, z - sz / 2
        return (base[0] + c * x + s * z, base[1] + y, base[2] - s * x + c * z)

    v = {(i, j, k): P(i * sx, j * sy, k * sz) for i in (0, 1) for j in (0, 1) for k in (0, 1)}
    faces = [
        ((0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0)),  # -x
        ((1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1)),  # +x
        ((0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)),  # -y
        ((0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0)),  # +y
        ((0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0)),  # -z
        ((0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)),  # +z
    ]
    tris = []
    for f in faces:
        tris += _quad(*[v[k] for k in f])
    return tris


def cornell(variant: str = "baseline") -> dict:
    """The small Cornell box: 5 wall quads, two rotated boxes, a 0.25 x 0.25 light at
    y = 0.999 emitting (17, 12, 4) downwards; 34 scene triangles + 2 light triangles.
    The camera is the reference's pinhole at (0.5, 0.5, -1.4) looking +z with a 40 degree
    field of view (fov = 2 tan 20 deg), which puts world +x on the image's left, so the
    red "left" wall is the x = 1 plane.

    variant "baseline": all Lambert.  "mixed": tall box mirror, short box glass (IOR 1.5),
    back wall GGX (roughness 0.3) -- exercises every BSDF.  "specular": the same mirror and
    glass boxes with Lambert walls (the materials the reference itself has), the glass box
    2 mm above the floor.  "glossy": tall box Phong
    (specular 0.8, power 40), short box Plastic (diffuse (0.2, 0.4, 0.7), specular 0.6,
    power 120), back wall Phong (power 8).  "thinlens": the baseline box seen through a thin
    lens of radius 0.06 focused on the tall box (target z = 0.6, focal distance 2.0).
    "textured": a checkerboard colour map on the floor and back wall (TexturedMaterial) and
    an environment map in place of the black sky, seen through the open front.  "spheres":
    the room without its boxes, holding analytic spheres (Sphere) instead -- a Lambert, a
    mirror and a glass one and an emitting light sphere that joins the quad light in the
    light list."""
    W, R, G = (0.75, 0.75, 0.75), (0.75, 0.25, 0.25), (0.25, 0.75, 0.25)
    mats = [{"type": LAMBERT, "color": W}, {"type": LAMBERT, "color": R}, {"type": LAMBERT, "color": G}]
    tall_m = short_m = back_m = 0
    if variant == "mixed":
        mats += [{"type": MIRROR, "color": (0.9, 0.9, 0.9)},
                 {"type": GLASS, "color": (1.0, 1.0, 1.0), "ior": 1.5},
                 {"type": GGX, "color": (0.8, 0.6, 0.3), "roughness": 0.3}]
        tall_m, short_m, back_m = 3, 4, 5
    elif variant == "specular":
        mats += [{"type": MIRROR, "color": (0.9, 0.9, 0.9)},
                 {"type": GLASS, "color": (1.0, 1.0, 1.0), "ior": 1.5}]
        tall_m, short_m = 3, 4
    elif variant == "textured":
        mats += [{"type": LAMBERT, "color": (0.9, 0.9, 0.9), "texture": 0}]
        back_m = 3
    elif variant == "spheres":
        mats += [{"type": MIRROR, "color": (0.9, 0.9, 0.9)},
                 {"type": GLASS, "color": (1.0, 1.0, 1.0), "ior": 1.5},
                 {"type": LAMBERT, "color": (0.0, 0.0, 0.0), "emission": (6.0, 7.0, 9.0)}]
    elif variant == "glossy":
        mats += [{"type": PHONG, "color": (0.8, 0.8, 0.8), "power": 40.0},
                 {"type": PLASTIC, "color": (0.2, 0.4, 0.7), "specular": (0.6, 0.6, 0.6), "power": 120.0},
                 {"type": PHONG, "color": (0.7, 0.7, 0.6), "power": 8.0}]
        tall_m, short_m, back_m = 3, 4, 5
    tris, mid = [], []

    def add(ts, m):
        tris.extend(ts)
        mid.extend([m] * len(ts))

    add(_quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)), 3 if variant == "textured" else 0)  # floor, +y
    add(_quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)), 0)      # ceiling, normal -y
    add(_quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)), back_m)  # back wall, normal -z
    add(_quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)), 1)      # x = 1 (image left), red
    add(_quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), 2)      # x = 0 (image right), green
    if variant != "spheres":
        add(_box((0.3, 0.6, 0.3), 15.0, (0.33, 0.0, 0.6)), tall_m)
        # the specular variant lifts the glass box 2 mm off the floor: rays inside it would
        # otherwise meet its bottom face and the floor at the same distance, a tie that
        # floating point rounding decides differently on every machine
        add(_box((0.3, 0.3, 0.3), -18.0, (0.66, 0.002 if variant == "specular" else 0.0, 0.35)), short_m)
    pos = np.stack(tris).reshape(-1, 9).astype(np.float32)
    g = np.cross(pos[:, 3:6] - pos[:, 0:3], pos[:, 6:9] - pos[:, 0:3])
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    nrm = np.tile(g, (1, 3)).astype(np.float32)
    extra = {}
    if variant == "textured":
        # texture coordinates from the floor's (x, z) and the back wall's (x, y); a 64 x 64
        # checkerboard of 8 x 8 blocks, and a 32 x 16 latitude-longitude environment
        uv = np.zeros((pos.shape[0], 6), np.float32)
        for k in range(3):
            p = pos[:, 3 * k:3 * k + 3]
            uv[0:2, 2 * k], uv[0:2, 2 * k + 1] = p[0:2, 0], p[0:2, 2]
            uv[4:6, 2 * k], uv[4:6, 2 * k + 1] = p[4:6, 0], p[4:6, 1]
        yy, xx = np.mgrid[0:64, 0:64]
        chk = ((xx // 8 + yy // 8) % 2).astype(np.float32)
        tex = np.stack([0.2 + 0.7 * chk, 0.25 + 0.5 * chk, 0.9 - 0.6 * chk], -1).astype(np.float32)
        ev, eu = np.mgrid[0:16, 0:32]
        env = np.stack([0.02 + 0.03 * eu / 31, 0.04 * (1 - ev / 15), 0.05 + 0.0 * eu], -1).astype(np.float32)
        extra = {"tri_uv": uv, "textures": [tex, env], "ibl": 1}
    if variant == "spheres":
        extra = {"spheres": [{"center": (0.7, 0.19, 0.62), "radius": 0.18, "material": 0},
                             {"center": (0.28, 0.2, 0.55), "radius": 0.19, "material": 3},
                             {"center": (0.52, 0.16, 0.22), "radius": 0.15, "material": 4},
                             {"center": (0.3, 0.78, 0.35), "radius": 0.07, "material": 5, "light": True}]}
    return {
        "name": f"cornell-{variant}",
        "tri_pos": pos, "tri_nrm": nrm, "tri_mat": np.array(mid, np.int32), "materials": mats,
        "light": {"corner": (0.375, 0.999, 0.375), "edge_a": (0.25, 0.0, 0.0), "edge_b": (0.0, 0.0, 0.25),
                  "emission": (17.0, 12.0, 4.0)},
        "sun": None, "sky": (0.0, 0.0, 0.0),
        "camera": {"pos": (0.5, 0.5, -1.4), "target": (0.5, 0.5, 0.6 if variant == "thinlens" else 0.0),
                   "up": (0.0, 1.0, 0.0), "fov": 2.0 * math.tan(math.radians(20.0)), "near": 1.0,
                   "lens_radius": 0.06 if variant == "thinlens" else 0.0},
        **extra,
    }


def soup(n: int, seed: int = 20260001) -> dict:
    """The traversal microbenchmark's triangle soup (one grey Lambert material)."""
    pos = microbench_soup(seed, n)
    return {"name": f"soup-{n}", "tri_pos": pos, "tri_nrm": None, "tri_mat": None,
            "materials": [{"type": LAMBERT, "color": (0.75, 0.75, 0.75)}], "light": None, "sun": None,
            "sky": (1.0, 1.0, 1.0),
            "camera": {"pos": (0.5, 0.5, -1.5), "target": (0.5, 0.5, 0.5), "up": (0, 1, 0), "fov": 1.0}}


def value_noise(n: int, octaves: int, seed: int, base: int = 4) -> np.ndarray:
    """n x n samples over [0,1]^2 of seeded value noise: sum over octaves k of 0.5^k times a
    smoothstep-interpolated random lattice with base * 2^k cells per side, normalised to [0,1]."""
    rng = np.random.default_rng(seed)
    x = np.linspace(0.0, 1.0, n)
    h = np.zeros((n, n))
    amp_sum = 0.0
    for k in range(octaves):
        f = base * 2 ** k
        lat = rng.random((f + 1, f + 1))
        g = x * f
        i0 = np.minimum(np.floor(g).astype(np.int64), f - 1)
        t = g - i0
        s = t * t * (3.0 - 2.0 * t)
        a = lat[np.ix_(i0, i0)]
        b = lat[np.ix_(i0, i0 + 1)]
        c = lat[np.ix_(i0 + 1, i0)]
        d = lat[np.ix_(i0 + 1, i0 + 1)]
        sy, sx = s[:, None], s[None, :]
        h += (0.5 ** k) * ((a * (1 - sx) + b * sx) * (1 - sy) + (c * (1 - sx) + d * sx) * sy)
        amp_sum += 0.5 ** k
    return h / amp_sum


def _icosphere(subdiv: int) -> np.ndarray:
    """Unit icosphere triangles (20 * 4^subdiv, 3, 3), outward winding."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    tris = np.array([[v[a], v[b], v[c]] for a, b, c in f], np.float64)
    tris /= np.linalg.norm(tris, axis=2, keepdims=True)
    for _ in range(subdiv):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = a + b, b + c, c + a
        ab /= np.linalg.norm(ab, axis=1, keepdims=True)
        bc /= np.linalg.norm(bc, axis=1, keepdims=True)
        ca /= np.linalg.norm(ca, axis=1, keepdims=True)
        tris = np.concatenate([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                               np.stack([ab, bc, ca], 1)])
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    flip = np.einsum("ij,ij->i", n, tris.sum(1)) < 0
    tris[flip] = tris[flip][:, ::-1]
    return tris


def heightfield(grid: int = 2048, n_spheres: int = 4096, seed: int = 2026, height: float = 0.15,
                subdiv: int = 3, sun_half_angle: float = 0.0) -> dict:
    """The 1080p heightfield scene: a grid x grid terrain (2 grid^2 triangles) over [0,1]^2
    with 6-octave value-noise heights (amplitude 0.5^k), n_spheres icospheres (20 * 4^subdiv
    triangles each) with radii log-uniform in [0.005, 0.05] above it; sphere materials 60%
    Lambert (albedo U[0.1,0.9]), 20% mirror, 10% dielectric (IOR 1.5), 10% GGX (roughness
    U[0.05,0.5]); constant sky 1.0 and a directional sun (a delta light, reached by
    next-event estimation only), or, with sun_half_angle > 0, a sun disk of that angular
    radius (sampled together with the BSDF by multiple importance sampling)."""
    rng = np.random.default_rng(seed)
    n = grid + 1
    h = value_noise(n, 6, seed) * height
    xs = np.linspace(0.0, 1.0, n)
    X, Z = np.meshgrid(xs, xs)
    P = np.stack([X, h, Z], -1).astype(np.float32)          # [row(z), col(x), 3]
    dhdx = np.gradient(h, xs, axis=1)
    dhdz = np.gradient(h, xs, axis=0)
    N = np.stack([-dhdx, np.ones_like(h), -dhdz], -1)
    N = (N / np.linalg.norm(N, axis=-1, keepdims=True)).astype(np.float32)
    a, b = P[:-1, :-1], P[:-1, 1:]        # (i,j), (i,j+1)
    c, d = P[1:, 1:], P[1:, :-1]          # (i+1,j+1), (i+1,j)
    na, nb, nc, nd = N[:-1, :-1], N[:-1, 1:], N[1:, 1:], N[1:, :-1]
    t_pos = np.stack([np.stack([a, d, c], 2), np.stack([a, c, b], 2)], 2).reshape(-1, 9)
    t_nrm = np.stack([np.stack([na, nd, nc], 2), np.stack([na, nc, nb], 2)], 2).reshape(-1, 9)
    t_mat = np.zeros(t_pos.shape[0], np.int32)

    mats = [{"type": LAMBERT, "color": (0.45, 0.40, 0.33)}]
    unit = _icosphere(subdiv).astype(np.float32)             # (m, 3, 3)
    m = unit.shape[0]
    cx = rng.uniform(0.05, 0.95, n_spheres)
    cz = rng.uniform(0.05, 0.95, n_spheres)
    r = np.exp(rng.uniform(np.log(0.005), np.log(0.05), n_spheres))
    # terrain height under each centre (bilinear on the grid)
    gx, gz = cx * grid, cz * grid
    i0, j0 = np.minimum(gz.astype(int), grid - 1), np.minimum(gx.astype(int), grid - 1)
    fz, fx = gz - i0, gx - j0
    ground = (h[i0, j0] * (1 - fx) * (1 - fz) + h[i0, j0 + 1] * fx * (1 - fz) + h[i0 + 1, j0] * (1 - fx) * fz
              + h[i0 + 1, j0 + 1] * fx * fz)
    cy = ground + r * (1.0 + rng.uniform(0.0, 1.0, n_spheres))
    kind = rng.random(n_spheres)
    s_mat = np.empty(n_spheres, np.int32)
    for i in range(n_spheres):
        if kind[i] < 0.6:
            mats.append({"type": LAMBERT, "color": tuple(rng.uniform(0.1, 0.9, 3))})
        elif kind[i] < 0.8:
            mats.append({"type": MIRROR, "color": (0.9, 0.9, 0.9)})
        elif kind[i] < 0.9:
            mats.append({"type": GLASS, "color": (1.0, 1.0, 1.0), "ior": 1.5})
        else:
            mats.append({"type": GGX, "color": tuple(rng.uniform(0.5, 0.95, 3)), "roughness": rng.uniform(0.05, 0.5)})
        s_mat[i] = len(mats) - 1
    centers = np.stack([cx, cy, cz], -1).astype(np.float32)
    s_pos = (centers[:, None, None, :] + r.astype(np.float32)[:, None, None, None] * unit[None]).reshape(-1, 9)
    s_nrm = np.broadcast_to(unit[None], (n_spheres, m, 3, 3)).reshape(-1, 9)
    pos = np.concatenate([t_pos, s_pos]).astype(np.float32)
    nrm = np.concatenate([t_nrm, s_nrm]).astype(np.float32)
    mat = np.concatenate([t_mat, np.repeat(s_mat, m)]).astype(np.int32)
    sun = np.array([-0.4, 0.75, -0.55])
    sun /= np.linalg.norm(sun)
    return {
        "name": f"heightfield-{grid}-{n_spheres}",
        "tri_pos": pos, "tri_nrm": nrm, "tri_mat": mat, "materials": mats, "light": None,
        "sun": {"dir": tuple(sun), "radiance": (3.0, 2.9, 2.7), "half_angle": sun_half_angle},
        "sky": (1.0, 1.0, 1.0),
        "camera": {"pos": (0.5, 0.42, -0.3), "target": (0.5, 0.05, 0.6), "up": (0.0, 1.0, 0.0),
                   "fov": 2.0 * math.tan(math.radians(25.0)), "near": 1.0},
    }


def upload(ctx, scene: dict):
    """Context.upload_scene with a scene dict from this module (and its spheres)."""
    kw = {k: v for k, v in scene.items() if k not in ("name", "spheres")}
    s = ctx.upload_scene(**kw)
    if scene.get("spheres"):
        s.set_spheres(scene["spheres"])
    return s


def batch_scene(seed: int) -> tuple[dict, dict]:
    """One scene of the batched-render workload and its render options: a triangle soup or
    a heightfield (even odds) with a triangle count log-uniform in [1e3, 1e6], a square
    resolution from {64, 128, 256, 512} and 4, 16 or 64 samples per pixel, all drawn from
    `seed`.  The heightfield keeps the 1080p scene's make-up at a smaller size: ~60% of the
    triangles in the terrain, the rest in subdivision-2 icospheres (320 triangles each)."""
    rng = np.random.default_rng(seed)
    n = int(round(math.exp(rng.uniform(math.log(1e3), math.log(1e6)))))
    res = int(rng.choice([64, 128, 256, 512]))
    spp = int(rng.choice([4, 16, 64]))
    if rng.random() < 0.5:
        d = soup(n, seed=int(rng.integers(1 << 31)))
    else:
        grid = max(4, int(math.sqrt(0.6 * n / 2)))
        n_sph = max(1, int((n - 2 * grid * grid) / 320))
        d = heightfield(grid=grid, n_spheres=n_sph, seed=int(rng.integers(1 << 31)), subdiv=2)
    opts = {"width": res, "height": res, "spp": spp, "max_depth": 8, "seed": int(rng.integers(1 << 31))}
    return d, opts
