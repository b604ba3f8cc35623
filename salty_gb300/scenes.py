"""Seeded synthetic scenes of the benchmark configurations (numpy, host side).

Each builder returns a dict with the keyword arguments of Context.upload_scene, plus
"name".  The same arrays feed the GPU library, the oracle restatement and the reference
harness, so all three see identical inputs.
"""
from __future__ import annotations

import math

import numpy as np

from . import GGX, GLASS, LAMBERT, MIRROR, microbench_soup


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
    back wall GGX (roughness 0.3) -- exercises every BSDF."""
    W, R, G = (0.75, 0.75, 0.75), (0.75, 0.25, 0.25), (0.25, 0.75, 0.25)
    mats = [{"type": LAMBERT, "color": W}, {"type": LAMBERT, "color": R}, {"type": LAMBERT, "color": G}]
    tall_m = short_m = back_m = 0
    if variant == "mixed":
        mats += [{"type": MIRROR, "color": (0.9, 0.9, 0.9)},
                 {"type": GLASS, "color": (1.0, 1.0, 1.0), "ior": 1.5},
                 {"type": GGX, "color": (0.8, 0.6, 0.3), "roughness": 0.3}]
        tall_m, short_m, back_m = 3, 4, 5
    tris, mid = [], []

    def add(ts, m):
        tris.extend(ts)
        mid.extend([m] * len(ts))

    add(_quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)), 0)      # floor, normal +y
    add(_quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)), 0)      # ceiling, normal -y
    add(_quad((0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)), back_m)  # back wall, normal -z
    add(_quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)), 1)      # x = 1 (image left), red
    add(_quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), 2)      # x = 0 (image right), green
    add(_box((0.3, 0.6, 0.3), 15.0, (0.33, 0.0, 0.6)), tall_m)
    add(_box((0.3, 0.3, 0.3), -18.0, (0.66, 0.0, 0.35)), short_m)
    pos = np.stack(tris).reshape(-1, 9).astype(np.float32)
    g = np.cross(pos[:, 3:6] - pos[:, 0:3], pos[:, 6:9] - pos[:, 0:3])
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    nrm = np.tile(g, (1, 3)).astype(np.float32)
    return {
        "name": f"cornell-{variant}",
        "tri_pos": pos, "tri_nrm": nrm, "tri_mat": np.array(mid, np.int32), "materials": mats,
        "light": {"corner": (0.375, 0.999, 0.375), "edge_a": (0.25, 0.0, 0.0), "edge_b": (0.0, 0.0, 0.25),
                  "emission": (17.0, 12.0, 4.0)},
        "sun": None, "sky": (0.0, 0.0, 0.0),
        "camera": {"pos": (0.5, 0.5, -1.4), "target": (0.5, 0.5, 0.0), "up": (0.0, 1.0, 0.0),
                   "fov": 2.0 * math.tan(math.radians(20.0)), "near": 1.0},
    }


def soup(n: int, seed: int = 20260001) -> dict:
    """The traversal microbenchmark's triangle soup (one grey Lambert material)."""
    pos = microbench_soup(seed, n)
    return {"name": f"soup-{n}", "tri_pos": pos, "tri_nrm": None, "tri_mat": None,
            "materials": [{"type": LAMBERT, "color": (0.75, 0.75, 0.75)}], "light": None, "sun": None,
            "sky": (1.0, 1.0, 1.0),
            "camera": {"pos": (0.5, 0.5, -1.5), "target": (0.5, 0.5, 0.5), "up": (0, 1, 0), "fov": 1.0}}


def upload(ctx, scene: dict):
    """Context.upload_scene with a scene dict from this module."""
    kw = {k: v for k, v in scene.items() if k != "name"}
    return ctx.upload_scene(**kw)
