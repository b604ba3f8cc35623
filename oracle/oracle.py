"""ctypes bindings for the two CPU checkers built by oracle/Makefile.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by __graft_entry__.smoke() and by
the cpu_baseline / reference legs of bench.py -- always as the checker, never as
the thing measured for the GPU path.  The shipped library never loads these.

  Oracle     -- oracle/_build/liboracle.so, the C restatement (salty_oracle.c)
  Reference  -- oracle/_ref/libsalty_ref.so, the unmodified reference sources
                compiled through oracle/ref/shim (present only where it was built)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsalty_ref.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")

LAMBERT, MIRROR, GLASS, GGX, PHONG, PLASTIC = 0, 1, 2, 3, 4, 5
PROFILE_COMPAT, PROFILE_PHYSICAL = 0, 1
TM_REINHARD, TM_UNCHARTED2, TM_ACES = 0, 1, 2


# Where the reference checkout is mounted in the container that builds the fixtures; any
# other checkout is named by $SALTY_REF_SRC.
_REF_MOUNT = "/root/reference/src"


def reference_dir() -> str | None:
    """The reference project's source root ($SALTY_REF_SRC, else the fixture container's
    mount), if its sources are present here."""
    for d in (os.environ.get("SALTY_REF_SRC"), _REF_MOUNT):
        if d and os.path.isfile(os.path.join(d, "src", "s3d_pt.cpp")):
            return d
    return None


def build(with_reference: bool | None = None) -> None:
    """Runs oracle/Makefile (the restatement always; the reference when its sources exist)."""
    target = ["all"] if with_reference is None else (["oracle", "ref"] if with_reference else ["oracle"])
    ref = reference_dir()
    if with_reference and not ref:
        raise RuntimeError("the reference sources are not present (set SALTY_REF_SRC)")
    extra = [f"REF={ref}"] if ref else []
    subprocess.run(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", *extra, *target], check=True)


class _Mat(C.Structure):
    _fields_ = [("type", C.c_int), ("color", C.c_float * 3), ("emission", C.c_float * 3),
                ("ior", C.c_float), ("roughness", C.c_float), ("specular", C.c_float * 3), ("power", C.c_float),
                ("color_map", C.c_int)]


class _Tex(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("rgb", C.c_void_p)]


def _textures(textures, keep):
    """(table, count) of (H, W, 3) float32 images for the C structs."""
    tt = (_Tex * max(1, len(textures)))()
    for i, t in enumerate(textures):
        a = np.ascontiguousarray(t, np.float32)
        keep.append(a)
        tt[i].height, tt[i].width, tt[i].rgb = a.shape[0], a.shape[1], a.ctypes.data
    keep.append(tt)
    return tt, len(textures)


class _Scene(C.Structure):
    _fields_ = [("tri_pos", C.c_void_p), ("tri_nrm", C.c_void_p), ("tri_mat", C.c_void_p),
                ("n_tris", C.c_long), ("mats", C.c_void_p), ("n_mats", C.c_int),
                ("has_light", C.c_int), ("light_corner", C.c_float * 3),
                ("light_edge_a", C.c_float * 3), ("light_edge_b", C.c_float * 3),
                ("light_emission", C.c_float * 3), ("has_sun", C.c_int),
                ("sun_dir", C.c_float * 3), ("sun_radiance", C.c_float * 3), ("sun_half_angle", C.c_float),
                ("sky", C.c_float * 3),
                ("cam_pos", C.c_float * 3), ("cam_target", C.c_float * 3), ("cam_up", C.c_float * 3),
                ("cam_fov", C.c_float), ("cam_near", C.c_float), ("cam_lens", C.c_float), ("cam_focal", C.c_float),
                ("tri_uv", C.c_void_p), ("textures", C.c_void_p), ("n_textures", C.c_int), ("ibl_map", C.c_int),
                ("ibl_scale", C.c_float), ("spheres", C.c_void_p), ("n_spheres", C.c_long)]


class _Opts(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("spp", C.c_int), ("max_depth", C.c_int),
                ("rr_depth", C.c_int), ("profile", C.c_int), ("seed", C.c_uint64),
                ("nthreads", C.c_int), ("row_begin", C.c_int), ("row_end", C.c_int)]


class _RefMat(C.Structure):
    _fields_ = [("type", C.c_int), ("color", C.c_float * 3), ("emission", C.c_float * 3), ("ior", C.c_float),
                ("specular", C.c_float * 3), ("power", C.c_float), ("color_map", C.c_int)]


class _RefScene(C.Structure):
    _fields_ = [("tri_pos", C.c_void_p), ("tri_nrm", C.c_void_p), ("tri_mat", C.c_void_p),
                ("n_tris", C.c_long), ("mats", C.c_void_p), ("n_mats", C.c_int),
                ("has_light", C.c_int), ("light_corner", C.c_float * 3),
                ("light_edge_a", C.c_float * 3), ("light_edge_b", C.c_float * 3),
                ("light_emission", C.c_float * 3), ("cam_pos", C.c_float * 3),
                ("cam_target", C.c_float * 3), ("cam_up", C.c_float * 3),
                ("cam_fov", C.c_float), ("cam_near", C.c_float), ("sky_over_10", C.c_float),
                ("tmp_dir", C.c_char_p), ("cam_lens", C.c_float), ("tri_uv", C.c_void_p), ("textures", C.c_void_p),
                ("n_textures", C.c_int), ("ibl_map", C.c_int), ("spheres", C.c_void_p), ("n_spheres", C.c_int)]


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


@dataclass
class SceneData:
    """A flat scene: the same numbers feed the oracle, the reference and the GPU library."""
    tri_pos: np.ndarray                 # (n, 9) float32
    tri_nrm: np.ndarray | None          # (n, 9) float32 or None
    tri_mat: np.ndarray                 # (n,) int32
    materials: list                     # list of dicts: type, color, emission, ior, roughness
    light: dict | None = None           # corner, edge_a, edge_b, emission
    sun: dict | None = None             # dir, radiance
    sky: tuple = (0.0, 0.0, 0.0)
    camera: dict = field(default_factory=dict)  # pos, target, up, fov, near
    tri_uv: np.ndarray | None = None    # (n, 6) float32 texture coordinates
    textures: list = field(default_factory=list)  # (H, W, 3) float32 images
    ibl: int | None = None              # texture index of the environment map
    ibl_scale: float = 10.0
    spheres: list = field(default_factory=list)  # dicts: center, radius, material, light


def _sphere_array(spheres) -> np.ndarray:
    """(n, 6) float32: centre xyz, radius, material, light (0/1)."""
    a = np.zeros((max(1, len(spheres)), 6), np.float32)
    for i, sp in enumerate(spheres):
        a[i, 0:3] = sp["center"]
        a[i, 3] = sp["radius"]
        a[i, 4] = sp.get("material", 0)
        a[i, 5] = 1.0 if sp.get("light") else 0.0
    return a


class RefBVH:
    """The reference's BVH8 over a triangle soup and its closest-hit walk (BVH8::IsHit,
    src/s3d_bvh8.cpp:191-206), restated in C: trace(rays) -> ids, t, u, v, seconds."""

    def __init__(self, o: "Oracle", tri_pos: np.ndarray):
        self.o = o
        self.pos = np.ascontiguousarray(tri_pos, np.float32).reshape(-1, 9)
        secs = C.c_double()
        self.h = o.L.oracle_refbvh_create(self.pos, self.pos.shape[0], C.byref(secs))
        self.build_seconds = secs.value

    def stats(self) -> dict:
        n8, n4, nl, d = C.c_long(), C.c_long(), C.c_long(), C.c_int()
        self.o.L.oracle_refbvh_stats(self.h, C.byref(n8), C.byref(n4), C.byref(nl), C.byref(d))
        return {"bvh8": n8.value, "bvh4": n4.value, "leaves": nl.value, "depth": d.value}

    def trace(self, rays: np.ndarray, nthreads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        ids = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        secs = self.o.L.oracle_refbvh_trace(self.h, rays, n, nthreads, ids, t, u, v)
        return ids, t, u, v, secs

    def close(self):
        if self.h:
            self.o.L.oracle_refbvh_destroy(self.h)
            self.h = None


class Oracle:
    """The C restatement."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(with_reference=False)
        L = C.CDLL(path)
        self.L = L
        L.oracle_gen_soup.argtypes = [C.c_uint64, C.c_long, _f32p]
        L.oracle_gen_rays.argtypes = [C.c_uint64, C.c_long, C.c_float, _f32p]
        L.oracle_bvh_create.argtypes = [_f32p, C.c_long]
        L.oracle_bvh_create.restype = C.c_void_p
        L.oracle_bvh_destroy.argtypes = [C.c_void_p]
        L.oracle_trace.argtypes = [C.c_void_p, _f32p, C.c_long, C.c_int, C.c_int, C.c_int,
                                   _i32p, _f32p, _f32p, _f32p]
        L.oracle_render.argtypes = [C.POINTER(_Scene), C.POINTER(_Opts), _f64p, _f64p]
        L.oracle_refbvh_create.argtypes = [_f32p, C.c_long, C.POINTER(C.c_double)]
        L.oracle_refbvh_create.restype = C.c_void_p
        L.oracle_refbvh_destroy.argtypes = [C.c_void_p]
        L.oracle_refbvh_stats.argtypes = [C.c_void_p, C.POINTER(C.c_long), C.POINTER(C.c_long),
                                          C.POINTER(C.c_long), C.POINTER(C.c_int)]
        L.oracle_refbvh_trace.argtypes = [C.c_void_p, _f32p, C.c_long, C.c_int, _i32p, _f32p, _f32p, _f32p]
        L.oracle_refbvh_trace.restype = C.c_double
        L.oracle_tonemap.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p,
                                     C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.oracle_srgb8.argtypes = [_f32p, C.c_long, C.c_int, _u8p]
        L.oracle_nlm_ref.argtypes = [C.c_int, C.c_int, C.c_float, _f32p, _f32p]
        L.oracle_nlm_var.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, _f32p, _f32p, _f32p]

    def gen_soup(self, seed: int, n: int) -> np.ndarray:
        out = np.empty((n, 9), np.float32)
        self.L.oracle_gen_soup(seed, n, out)
        return out

    def gen_rays(self, seed: int, n: int, tmin: float = 1e-4) -> np.ndarray:
        out = np.empty((n, 8), np.float32)
        self.L.oracle_gen_rays(seed, n, tmin, out)
        return out

    def trace(self, tri_pos: np.ndarray, rays: np.ndarray, mode: int = 0, any_hit: bool = False,
              nthreads: int = 0):
        tri_pos = np.ascontiguousarray(tri_pos, np.float32).reshape(-1, 9)
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = rays.shape[0]
        ids = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        h = self.L.oracle_bvh_create(tri_pos, tri_pos.shape[0])
        try:
            self.L.oracle_trace(h, rays, n, mode, int(any_hit), nthreads, ids, t, u, v)
        finally:
            self.L.oracle_bvh_destroy(h)
        return ids, t, u, v

    def ref_bvh(self, tri_pos: np.ndarray) -> "RefBVH":
        """The reference's own BVH8 (BVH8::Create, src/s3d_bvh8.cpp:401-479), restated."""
        return RefBVH(self, tri_pos)

    def render(self, sc: SceneData, width: int, height: int, spp: int, max_depth: int,
               rr_depth: int = 3, profile: int = PROFILE_PHYSICAL, seed: int = 1,
               nthreads: int = 0, rows: tuple | None = None):
        keep = []
        pos = np.ascontiguousarray(sc.tri_pos, np.float32)
        keep.append(pos)
        nrm = None if sc.tri_nrm is None else np.ascontiguousarray(sc.tri_nrm, np.float32)
        if nrm is not None:
            keep.append(nrm)
        mat = np.ascontiguousarray(sc.tri_mat, np.int32)
        keep.append(mat)
        mats = (_Mat * max(1, len(sc.materials)))()
        for i, m in enumerate(sc.materials):
            mats[i].type = m.get("type", LAMBERT)
            mats[i].color = _f3(m.get("color", (0.75, 0.75, 0.75)))
            mats[i].emission = _f3(m.get("emission", (0, 0, 0)))
            mats[i].ior = m.get("ior", 1.5)
            mats[i].roughness = m.get("roughness", 0.3)
            mats[i].specular = _f3(m.get("specular", (0.0, 0.0, 0.0)))
            mats[i].power = m.get("power", 32.0)
            mats[i].color_map = 0 if m.get("texture") is None else int(m["texture"]) + 1
        s = _Scene()
        tt, nt = _textures(sc.textures, keep)
        s.textures, s.n_textures = C.addressof(tt), nt
        s.ibl_map = 0 if sc.ibl is None else int(sc.ibl) + 1
        s.ibl_scale = sc.ibl_scale
        if sc.tri_uv is not None:
            uv = np.ascontiguousarray(sc.tri_uv, np.float32)
            keep.append(uv)
            s.tri_uv = uv.ctypes.data
        s.tri_pos = pos.ctypes.data
        s.tri_nrm = nrm.ctypes.data if nrm is not None else None
        s.tri_mat = mat.ctypes.data
        s.n_tris = pos.shape[0]
        s.mats = C.addressof(mats)
        s.n_mats = len(sc.materials)
        if sc.spheres:
            sph = _sphere_array(sc.spheres)
            keep.append(sph)
            s.spheres, s.n_spheres = sph.ctypes.data, len(sc.spheres)
        if sc.light:
            s.has_light = 1
            s.light_corner = _f3(sc.light["corner"])
            s.light_edge_a = _f3(sc.light["edge_a"])
            s.light_edge_b = _f3(sc.light["edge_b"])
            s.light_emission = _f3(sc.light["emission"])
        if sc.sun:
            s.has_sun = 1
            s.sun_dir = _f3(sc.sun["dir"])
            s.sun_radiance = _f3(sc.sun["radiance"])
            s.sun_half_angle = float(sc.sun.get("half_angle", 0.0))
        s.sky = _f3(sc.sky)
        cam = sc.camera
        s.cam_pos = _f3(cam["pos"])
        s.cam_target = _f3(cam["target"])
        s.cam_up = _f3(cam["up"])
        s.cam_fov = cam["fov"]
        s.cam_near = cam.get("near", 1.0)
        s.cam_lens = cam.get("lens_radius", 0.0)
        s.cam_focal = cam.get("focal_distance", 0.0)
        o = _Opts(width, height, spp, max_depth, rr_depth, profile, seed, nthreads,
                  rows[0] if rows else 0, rows[1] if rows else 0)
        total = np.zeros((height, width, 3), np.float64)
        sq = np.zeros((height, width, 3), np.float64)
        self.L.oracle_render(C.byref(s), C.byref(o), total, sq)
        return total, sq

    def tonemap(self, type_: int, img: np.ndarray):
        img = np.ascontiguousarray(img, np.float32)
        h, w = img.shape[:2]
        out = np.empty_like(img)
        ave, mx = C.c_float(), C.c_float()
        self.L.oracle_tonemap(type_, w, h, img, out, C.byref(ave), C.byref(mx))
        return out, ave.value, mx.value

    def srgb8(self, img: np.ndarray, ref_oetf: bool = True) -> np.ndarray:
        img = np.ascontiguousarray(img, np.float32)
        out = np.empty(img.shape, np.uint8)
        self.L.oracle_srgb8(img, img.size // 3, int(ref_oetf), out)
        return out

    def nlm_ref(self, rgba: np.ndarray, coeff: float) -> np.ndarray:
        rgba = np.ascontiguousarray(rgba, np.float32)
        h, w = rgba.shape[:2]
        out = np.empty_like(rgba)
        self.L.oracle_nlm_ref(w, h, coeff, rgba, out)
        return out

    def nlm_var(self, rgb: np.ndarray, var: np.ndarray, search_r: int = 10, patch_r: int = 3,
                k: float = 0.45) -> np.ndarray:
        rgb = np.ascontiguousarray(rgb, np.float32)
        var = np.ascontiguousarray(var, np.float32)
        h, w = rgb.shape[:2]
        out = np.empty_like(rgb)
        self.L.oracle_nlm_var(w, h, search_r, patch_r, k, rgb, var, out)
        return out


class Reference:
    """The unmodified reference, compiled from its own sources (oracle/_ref)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        self.L = L
        L.sref_soup_create.argtypes = [_f32p, C.c_long, C.POINTER(C.c_double)]
        L.sref_soup_create.restype = C.c_void_p
        L.sref_soup_destroy.argtypes = [C.c_void_p]
        L.sref_soup_trace.argtypes = [C.c_void_p, _f32p, C.c_long, C.c_int, _i32p, _f32p, _f32p, _f32p]
        L.sref_soup_trace.restype = C.c_double
        L.sref_scene_create.argtypes = [C.POINTER(_RefScene), C.c_int, C.c_int]
        L.sref_scene_create.restype = C.c_void_p
        L.sref_scene_destroy.argtypes = [C.c_void_p]
        L.sref_render.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int,
                                  _f64p, _f64p]
        L.sref_render.restype = C.c_double
        L.sref_tonemap.argtypes = [C.c_int, C.c_int, C.c_int, _f32p, _f32p]
        L.sref_nlm.argtypes = [C.c_int, C.c_int, C.c_float, _f32p, _f32p]
        L.sref_capture_png.argtypes = [C.c_int, C.c_int, _f32p, C.c_char_p]

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    class Soup:
        def __init__(self, ref: "Reference", tri_pos: np.ndarray):
            self.ref = ref
            self.pos = np.ascontiguousarray(tri_pos, np.float32).reshape(-1, 9)
            secs = C.c_double()
            self.h = ref.L.sref_soup_create(self.pos, self.pos.shape[0], C.byref(secs))
            self.build_seconds = secs.value

        def trace(self, rays: np.ndarray, nthreads: int = 0):
            rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
            n = rays.shape[0]
            ids = np.empty(n, np.int32)
            t = np.empty(n, np.float32)
            u = np.empty(n, np.float32)
            v = np.empty(n, np.float32)
            secs = self.ref.L.sref_soup_trace(self.h, rays, n, nthreads, ids, t, u, v)
            return ids, t, u, v, secs

        def close(self):
            if self.h:
                self.ref.L.sref_soup_destroy(self.h)
                self.h = None

        def __del__(self):
            self.close()

    def soup(self, tri_pos: np.ndarray) -> "Reference.Soup":
        return Reference.Soup(self, tri_pos)

    def render(self, sc: SceneData, width: int, height: int, spp: int, max_bounce: int,
               seed: int = 1, nthreads: int = 0, tmp_dir: str = "/tmp"):
        pos = np.ascontiguousarray(sc.tri_pos, np.float32)
        nrm = np.ascontiguousarray(sc.tri_nrm if sc.tri_nrm is not None else _geom_normals(pos), np.float32)
        mat = np.ascontiguousarray(sc.tri_mat, np.int32)
        mats = (_RefMat * max(1, len(sc.materials)))()
        for i, m in enumerate(sc.materials):
            mats[i].type = LAMBERT if m.get("type", LAMBERT) == GGX else m.get("type", LAMBERT)
            mats[i].color = _f3(m.get("color", (0.75, 0.75, 0.75)))
            mats[i].emission = _f3(m.get("emission", (0, 0, 0)))
            mats[i].ior = m.get("ior", 1.5)
            mats[i].specular = _f3(m.get("specular", (0.0, 0.0, 0.0)))
            mats[i].power = m.get("power", 32.0)
            mats[i].color_map = 0 if m.get("texture") is None else int(m["texture"]) + 1
        s = _RefScene()
        s.tri_pos, s.tri_nrm, s.tri_mat = pos.ctypes.data, nrm.ctypes.data, mat.ctypes.data
        s.n_tris = pos.shape[0]
        s.mats = C.addressof(mats)
        s.n_mats = len(sc.materials)
        if sc.light:
            s.has_light = 1
            s.light_corner = _f3(sc.light["corner"])
            s.light_edge_a = _f3(sc.light["edge_a"])
            s.light_edge_b = _f3(sc.light["edge_b"])
            s.light_emission = _f3(sc.light["emission"])
        cam = sc.camera
        s.cam_pos, s.cam_target, s.cam_up = _f3(cam["pos"]), _f3(cam["target"]), _f3(cam["up"])
        s.cam_fov, s.cam_near = cam["fov"], cam.get("near", 1.0)
        s.cam_lens = cam.get("lens_radius", 0.0)
        s.sky_over_10 = float(sc.sky[0]) / 10.0
        s.tmp_dir = tmp_dir.encode()
        keep = []
        tt, nt = _textures(sc.textures, keep)
        s.textures, s.n_textures = C.addressof(tt), nt
        s.ibl_map = 0 if sc.ibl is None else int(sc.ibl) + 1
        if sc.tri_uv is not None:
            uv = np.ascontiguousarray(sc.tri_uv, np.float32)
            keep.append(uv)
            s.tri_uv = uv.ctypes.data
        if sc.spheres:
            sph = _sphere_array(sc.spheres)
            keep.append(sph)
            s.spheres, s.n_spheres = sph.ctypes.data, len(sc.spheres)
        h = self.L.sref_scene_create(C.byref(s), width, height)
        try:
            total = np.zeros((height, width, 3), np.float64)
            sq = np.zeros((height, width, 3), np.float64)
            secs = self.L.sref_render(h, width, height, spp, max_bounce, seed, nthreads, total, sq)
        finally:
            self.L.sref_scene_destroy(h)
        return total, sq, secs

    def tonemap(self, type_: int, img: np.ndarray) -> np.ndarray:
        img = np.ascontiguousarray(img, np.float32)
        h, w = img.shape[:2]
        out = np.empty_like(img)
        self.L.sref_tonemap(type_, w, h, img, out)
        return out

    def nlm(self, rgba: np.ndarray, coeff: float) -> np.ndarray:
        rgba = np.ascontiguousarray(rgba, np.float32)
        h, w = rgba.shape[:2]
        out = np.empty_like(rgba)
        self.L.sref_nlm(w, h, coeff, rgba, out)
        return out

    def capture_png(self, img: np.ndarray, path: str) -> None:
        img = np.ascontiguousarray(img, np.float32)
        h, w = img.shape[:2]
        self.L.sref_capture_png(w, h, img, path.encode())


def _geom_normals(pos: np.ndarray) -> np.ndarray:
    p = pos.reshape(-1, 3, 3).astype(np.float32)
    n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    n = n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return np.repeat(n[:, None, :], 3, axis=1).reshape(-1, 9).astype(np.float32)
