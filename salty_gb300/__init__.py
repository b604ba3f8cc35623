"""salty_gb300 -- GB300-native path-tracing hot path of ProjectAsura/Salty.

Python host mirror over the C ABI of include/salty_gpu.h (libsalty_gpu.so, built
in-tree by salty_gb300/build.py).  Every call goes to the CUDA library; if the
library is missing or has no GPU the calls raise -- there is no CPU fallback.

Mapping to the reference's API (paths relative to the reference project's src/):
  Context.upload_scene  Scene construction (Mesh::Create, material factories,
                        PinholeCamera::Update; include/s3d_scene.h:22-109)
  Scene.build           BVH8::Create (src/s3d_bvh8.cpp:401-479)
  Scene.trace           Scene::Intersect (include/s3d_scene.h:63-75)
  Scene.render          PathTracer::TracePath / Radiance (src/s3d_pt.cpp:182-353)
  Context.tonemap       ToneMapper::Map + the sRGB8 step of PathTracer::Capture
  Context.nlm_ref       FilterNLM (src/s3d_denoiser.cpp:19-95)
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsalty_gpu.so")

OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_QUEUE_OVERFLOW, ERR_CANCELLED, ERR_NOT_BUILT, ERR_CAPACITY = range(9)
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA_ERROR", 4: "TIMEOUT", 5: "QUEUE_OVERFLOW",
                6: "CANCELLED", 7: "NOT_BUILT", 8: "CAPACITY"}
LAMBERT, MIRROR, GLASS, GGX, PHONG, PLASTIC = 0, 1, 2, 3, 4, 5
TRACE_ANY_HIT, TRACE_WATERTIGHT, TRACE_COUNTERS = 1, 2, 4
PROFILE_COMPAT, PROFILE_PHYSICAL = 0, 1
TM_NONE, TM_REINHARD, TM_UNCHARTED2, TM_ACES = -1, 0, 1, 2
CONV_TCGEN05, CONV_MMA_SYNC, CONV_TCGEN05_CP_ASYNC = 0, 1, 2


class SaltyError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"salty: {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("color", C.c_float * 3), ("emission", C.c_float * 3),
                ("ior", C.c_float), ("roughness", C.c_float), ("specular", C.c_float * 3), ("power", C.c_float),
                ("color_map", C.c_int32)]


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("fov", C.c_float), ("near_clip", C.c_float), ("lens_radius", C.c_float),
                ("focal_distance", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("tri_pos", C.c_void_p), ("tri_nrm", C.c_void_p), ("tri_mat", C.c_void_p),
                ("n_tris", C.c_int64), ("mats", C.c_void_p), ("n_mats", C.c_int32),
                ("has_light", C.c_int32), ("light_corner", C.c_float * 3), ("light_edge_a", C.c_float * 3),
                ("light_edge_b", C.c_float * 3), ("light_emission", C.c_float * 3),
                ("has_sun", C.c_int32), ("sun_dir", C.c_float * 3), ("sun_radiance", C.c_float * 3),
                ("sun_half_angle", C.c_float), ("sky", C.c_float * 3), ("camera", Camera),
                ("tri_uv", C.c_void_p), ("textures", C.c_void_p), ("n_textures", C.c_int32), ("ibl_map", C.c_int32),
                ("ibl_scale", C.c_float)]


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", C.c_void_p)]


class Instance(C.Structure):
    _fields_ = [("first_tri", C.c_int64), ("n_tris", C.c_int64), ("object_to_world", C.c_float * 12)]


class Sphere(C.Structure):
    _fields_ = [("center", C.c_float * 3), ("radius", C.c_float), ("material", C.c_int32), ("light", C.c_int32)]


class BuildOpts(C.Structure):
    _fields_ = [("bins", C.c_int32), ("max_leaf", C.c_int32), ("trav_cost", C.c_float)]


class BvhInfo(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("n_binary", C.c_int64), ("depth", C.c_int32),
                ("binary_depth", C.c_int32), ("sah_cost", C.c_double), ("build_ms", C.c_float)]


class TraceStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("total_ms", C.c_double), ("rays", C.c_int64),
                ("node_fetches", C.c_int64), ("tri_fetches", C.c_int64), ("h2d_bytes", C.c_int64),
                ("d2h_bytes", C.c_int64), ("launches", C.c_int64)]


class RenderOpts(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("rr_depth", C.c_int32), ("profile", C.c_int32), ("seed", C.c_uint64), ("accumulate", C.c_int32),
                ("fp64", C.c_int32), ("tonemap", C.c_int32), ("ref_oetf", C.c_int32), ("crop_x", C.c_int32),
                ("crop_y", C.c_int32), ("crop_w", C.c_int32), ("crop_h", C.c_int32)]


class RenderStats(C.Structure):
    _fields_ = [("ms", C.c_double), ("samples", C.c_int64), ("rays", C.c_int64), ("paths", C.c_int64)]


class Mesh(C.Structure):
    _fields_ = [("n_tris", C.c_int64), ("tri_pos", C.POINTER(C.c_float)), ("tri_nrm", C.POINTER(C.c_float)),
                ("tri_uv", C.POINTER(C.c_float)), ("tri_mat", C.POINTER(C.c_int32)), ("n_mats", C.c_int32),
                ("mats", C.POINTER(Material)), ("mat_texture", C.POINTER(C.c_int32)), ("n_textures", C.c_int32),
                ("texture_names", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("trace_block", C.c_int32), ("trace_pool", C.c_int32), ("trace_postpone", C.c_int32),
                ("shade_block", C.c_int32), ("trace_regs", C.c_int32), ("wave_paths", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every extern "C" symbol declared in include/salty_gpu.h.
EXPORTS = ["salty_ctx_create", "salty_ctx_destroy", "salty_last_error", "salty_abi_version", "salty_ctx_cancel",
           "salty_host_alloc", "salty_host_free", "salty_scene_upload", "salty_scene_destroy", "salty_bvh_build",
           "salty_trace", "salty_last_trace_stats", "salty_render", "salty_film_read", "salty_tonemap",
           "salty_denoise_nlm_ref", "salty_denoise_nlm", "salty_microbench_soup", "salty_microbench_rays",
           "salty_tonemap_noalloc", "salty_film_aov", "salty_unet_create", "salty_unet_destroy",
           "salty_unet_param_count", "salty_unet_get_params", "salty_unet_set_params", "salty_unet_forward",
           "salty_unet_train_step", "salty_scene_set_camera", "salty_denoise_unet", "salty_render_batch",
           "salty_get_tuning", "salty_set_tuning", "salty_autotune", "salty_mesh_load_smd", "salty_mesh_free",
           "salty_mesh_transform", "salty_autotune_trace", "salty_denoise_unet_ensemble", "salty_film_checkpoint",
           "salty_film_restore", "salty_unet_get_adam", "salty_unet_set_adam", "salty_unet_set_conv_kernel",
           "salty_scene_set_instances", "salty_scene_set_spheres"]

_lib = None


def lib() -> C.CDLL:
    """Loads libsalty_gpu.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise SaltyError(ERR_CUDA, f"{LIB_PATH} is missing; run __graft_entry__.build() or salty_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, u32, u64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_uint32, C.c_uint64, C.c_float
    sig = {
        "salty_ctx_create": (i32, [C.POINTER(vp), C.c_int]),
        "salty_ctx_destroy": (None, [vp]),
        "salty_last_error": (C.c_char_p, [vp]),
        "salty_abi_version": (C.c_int, []),
        "salty_ctx_cancel": (None, [vp]),
        "salty_host_alloc": (i32, [vp, C.c_size_t, C.POINTER(vp)]),
        "salty_host_free": (None, [vp, vp]),
        "salty_scene_upload": (i32, [vp, C.POINTER(SceneDesc), C.POINTER(vp)]),
        "salty_scene_destroy": (None, [vp, vp]),
        "salty_scene_set_camera": (i32, [vp, vp, C.POINTER(Camera)]),
        "salty_scene_set_instances": (i32, [vp, vp, vp, C.c_int32]),
        "salty_scene_set_spheres": (i32, [vp, vp, vp, C.c_int32]),
        "salty_bvh_build": (i32, [vp, vp, C.POINTER(BuildOpts), C.POINTER(BvhInfo)]),
        "salty_trace": (i32, [vp, vp, vp, i64, u32, vp]),
        "salty_last_trace_stats": (i32, [vp, C.POINTER(TraceStats)]),
        "salty_render": (i32, [vp, vp, C.POINTER(RenderOpts), vp, vp, vp, C.POINTER(RenderStats)]),
        "salty_film_read": (i32, [vp, vp, vp, vp, C.POINTER(i64)]),
        "salty_film_aov": (i32, [vp, vp, vp, vp, vp]),
        "salty_tonemap": (i32, [vp, i32, i32, i32, vp, vp, vp, i32, C.POINTER(f32), C.POINTER(f32)]),
        "salty_denoise_nlm_ref": (i32, [vp, i32, i32, f32, vp, vp]),
        "salty_tonemap_noalloc": (i32, [vp, vp, i32, i32, i32, vp, vp, vp, i32]),
        "salty_denoise_nlm": (i32, [vp, i32, i32, i32, i32, f32, vp, vp, vp]),
        "salty_microbench_soup": (i32, [u64, i64, vp]),
        "salty_microbench_rays": (i32, [u64, i64, f32, vp]),
        "salty_unet_create": (i32, [vp, u64, C.POINTER(vp)]),
        "salty_unet_destroy": (None, [vp, vp]),
        "salty_unet_param_count": (i64, [vp]),
        "salty_unet_get_params": (i32, [vp, vp, vp, vp]),
        "salty_unet_set_params": (i32, [vp, vp, vp]),
        "salty_unet_forward": (i32, [vp, vp, vp, i32, i32, i32, vp]),
        "salty_unet_train_step": (i32, [vp, vp, vp, vp, i32, i32, i32, f32, C.POINTER(f32)]),
        "salty_denoise_unet": (i32, [vp, vp, vp, vp]),
        "salty_denoise_unet_ensemble": (i32, [vp, vp, vp, i32, vp]),
        "salty_film_checkpoint": (i32, [vp, vp, vp, vp, vp, vp, C.POINTER(i64)]),
        "salty_film_restore": (i32, [vp, vp, C.POINTER(RenderOpts), vp, vp, vp, vp, i64]),
        "salty_unet_get_adam": (i32, [vp, vp, vp, vp, C.POINTER(i64)]),
        "salty_unet_set_adam": (i32, [vp, vp, vp, vp, i64]),
        "salty_unet_set_conv_kernel": (i32, [vp, vp, i32]),
        "salty_render_batch": (i32, [vp, vp, vp, i32, C.POINTER(RenderStats)]),
        "salty_mesh_load_smd": (i32, [vp, C.c_char_p, C.POINTER(C.POINTER(Mesh))]),
        "salty_mesh_free": (None, [C.POINTER(Mesh)]),
        "salty_mesh_transform": (i32, [vp, i64, vp, vp, vp, vp]),
        "salty_get_tuning": (i32, [vp, C.POINTER(Tuning)]),
        "salty_set_tuning": (i32, [vp, C.POINTER(Tuning)]),
        "salty_autotune": (i32, [vp, vp, vp, i32, i32, C.POINTER(Tuning), C.POINTER(f32)]),
        "salty_autotune_trace": (i32, [vp, vp, vp, i64, u32, C.POINTER(Tuning), C.POINTER(f32)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _ptr(a) -> int:
    """Address of a numpy array or a torch tensor (host or CUDA)."""
    if a is None:
        return 0
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported buffer {type(a)}")


def _f3(v) -> C.Array:
    return (C.c_float * 3)(*[float(x) for x in v])


def microbench_soup(seed: int, n: int) -> np.ndarray:
    out = np.empty((n, 9), np.float32)
    st = lib().salty_microbench_soup(seed, n, _ptr(out))
    if st:
        raise SaltyError(st, "microbench_soup")
    return out


def microbench_rays(seed: int, n: int, tmin: float = 1e-4, out: np.ndarray | None = None) -> np.ndarray:
    if out is None:
        out = np.empty((n, 8), np.float32)
    st = lib().salty_microbench_rays(seed, n, tmin, _ptr(out))
    if st:
        raise SaltyError(st, "microbench_rays")
    return out


def render_opts(width: int, height: int, spp: int, max_depth: int, rr_depth: int = 3,
                profile: int = PROFILE_PHYSICAL, seed: int = 1, accumulate: bool = False, fp64: bool = False,
                tonemap: int = TM_REINHARD, ref_oetf: bool = True, crop: tuple | None = None) -> RenderOpts:
    cx, cy, cw, ch = crop if crop else (0, 0, 0, 0)
    return RenderOpts(width, height, spp, max_depth, rr_depth, profile, seed, int(accumulate), int(fp64), tonemap,
                      int(ref_oetf), cx, cy, cw, ch)


def load_smd(path: str, ctx: "Context | None" = None) -> dict:
    """salty_mesh_load_smd: an SMD mesh as a scene dict piece (tri_pos, tri_nrm, tri_uv,
    tri_mat, materials as dicts, textures, mat_texture).  Needs no GPU."""
    m = C.POINTER(Mesh)()
    st = lib().salty_mesh_load_smd(ctx.h if ctx else None, os.fsencode(path), C.byref(m))
    if st:
        msg = lib().salty_last_error(ctx.h).decode() if ctx else f"cannot load {path}"
        raise SaltyError(st, msg)
    try:
        M = m.contents
        n = M.n_tris
        arr = lambda p, k, dt: np.ctypeslib.as_array(p, shape=(n * k,)).astype(dt).reshape(n, k) if k > 1 else \
            np.ctypeslib.as_array(p, shape=(n,)).astype(dt)
        mats = []
        for i in range(M.n_mats):
            x = M.mats[i]
            mats.append({"type": x.type, "color": tuple(x.color), "emission": tuple(x.emission), "ior": x.ior,
                         "roughness": x.roughness, "specular": tuple(x.specular), "power": x.power})
        names = C.string_at(M.texture_names, 256 * M.n_textures) if M.n_textures else b""
        return {"tri_pos": arr(M.tri_pos, 9, np.float32), "tri_nrm": arr(M.tri_nrm, 9, np.float32),
                "tri_uv": arr(M.tri_uv, 6, np.float32), "tri_mat": arr(M.tri_mat, 1, np.int32),
                "materials": mats,
                "textures": [names[256 * t:256 * (t + 1)].split(b"\0", 1)[0].decode("utf-8", "replace")
                             for t in range(M.n_textures)],
                "mat_texture": [M.mat_texture[i] for i in range(M.n_mats)]}
    finally:
        lib().salty_mesh_free(m)


def transform_mesh(matrix, tri_pos, tri_nrm=None):
    """salty_mesh_transform: positions by a 3x4 affine matrix, normals by the inverse
    transpose of its linear part (an instance of the mesh, flattened into the scene)."""
    M = np.ascontiguousarray(np.asarray(matrix, np.float32).reshape(3, 4))
    pos = np.ascontiguousarray(tri_pos, np.float32)
    n = pos.shape[0]
    out_p = np.empty_like(pos)
    nrm = None if tri_nrm is None else np.ascontiguousarray(tri_nrm, np.float32)
    out_n = None if nrm is None else np.empty_like(nrm)
    st = lib().salty_mesh_transform(_ptr(M), n, _ptr(pos), _ptr(nrm), _ptr(out_p), _ptr(out_n))
    if st:
        raise SaltyError(st, "mesh_transform: singular matrix or bad arguments")
    return out_p, out_n


class Context:
    """A device, its stream and scratch (salty_ctx)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        st = lib().salty_ctx_create(C.byref(h), device)
        if st:
            raise SaltyError(st, f"salty_ctx_create(device={device}) failed (is a GPU present?)")
        self.h = h
        self._pinned = []

    def check(self, st: int, what: str) -> None:
        if st:
            raise SaltyError(st, f"{what}: {lib().salty_last_error(self.h).decode(errors='replace')}")

    def close(self) -> None:
        if getattr(self, "h", None):
            for p in self._pinned:
                lib().salty_host_free(self.h, p)
            self._pinned = []
            lib().salty_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pinned(self, shape, dtype=np.float32) -> np.ndarray:
        """A numpy array in page-locked host memory owned by this context."""
        nbytes = int(np.prod(shape)) * np.dtype(dtype).itemsize
        p = C.c_void_p()
        self.check(lib().salty_host_alloc(self.h, nbytes, C.byref(p)), "host_alloc")
        self._pinned.append(p)
        buf = (C.c_char * nbytes).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def upload_scene(self, tri_pos, tri_nrm=None, tri_mat=None, materials=(), light=None, sun=None,
                     sky=(0.0, 0.0, 0.0), camera=None, tri_uv=None, textures=(), ibl=None,
                     ibl_scale: float = 10.0) -> "Scene":
        """textures: (H, W, 3) float arrays; a material's "texture" key names its colour map
        and `ibl` the environment map (indices into textures)."""
        tri_pos = tri_pos if hasattr(tri_pos, "data_ptr") else np.ascontiguousarray(tri_pos, np.float32)
        n = tri_pos.shape[0] if tri_pos.ndim == 2 else tri_pos.size // 9
        if tri_nrm is not None and not hasattr(tri_nrm, "data_ptr"):
            tri_nrm = np.ascontiguousarray(tri_nrm, np.float32)
        if tri_mat is not None and not hasattr(tri_mat, "data_ptr"):
            tri_mat = np.ascontiguousarray(tri_mat, np.int32)
        mats = (Material * max(1, len(materials)))()
        for i, m in enumerate(materials):
            mats[i].type = int(m.get("type", LAMBERT))
            mats[i].color = _f3(m.get("color", (0.75, 0.75, 0.75)))
            mats[i].emission = _f3(m.get("emission", (0, 0, 0)))
            mats[i].ior = float(m.get("ior", 1.5))
            mats[i].roughness = float(m.get("roughness", 0.3))
            mats[i].specular = _f3(m.get("specular", (0.0, 0.0, 0.0)))
            mats[i].power = float(m.get("power", 32.0))
            mats[i].color_map = 0 if m.get("texture") is None else int(m["texture"]) + 1
        texs = [np.ascontiguousarray(t, np.float32) for t in textures]
        ttab = (Texture * max(1, len(texs)))()
        for i, t in enumerate(texs):
            ttab[i].height, ttab[i].width = t.shape[0], t.shape[1]
            ttab[i].rgb = t.ctypes.data
        if tri_uv is not None and not hasattr(tri_uv, "data_ptr"):
            tri_uv = np.ascontiguousarray(tri_uv, np.float32)
        d = SceneDesc()
        d.tri_uv = _ptr(tri_uv)
        d.textures = C.addressof(ttab) if texs else None
        d.n_textures = len(texs)
        d.ibl_map = 0 if ibl is None else int(ibl) + 1
        d.ibl_scale = float(ibl_scale)
        d.tri_pos, d.tri_nrm, d.tri_mat = _ptr(tri_pos), _ptr(tri_nrm), _ptr(tri_mat)
        d.n_tris = n
        d.mats = C.addressof(mats) if materials else None
        d.n_mats = len(materials)
        if light:
            d.has_light = 1
            d.light_corner, d.light_edge_a = _f3(light["corner"]), _f3(light["edge_a"])
            d.light_edge_b, d.light_emission = _f3(light["edge_b"]), _f3(light["emission"])
        if sun:
            d.has_sun = 1
            d.sun_dir, d.sun_radiance = _f3(sun["dir"]), _f3(sun["radiance"])
            d.sun_half_angle = float(sun.get("half_angle", 0.0))
        d.sky = _f3(sky)
        cam = camera or {"pos": (0, 0, -1), "target": (0, 0, 0), "up": (0, 1, 0), "fov": 1.0}
        d.camera.pos, d.camera.target, d.camera.up = _f3(cam["pos"]), _f3(cam["target"]), _f3(cam["up"])
        d.camera.fov = float(cam["fov"])
        d.camera.near_clip = float(cam.get("near", 1.0))
        d.camera.lens_radius = float(cam.get("lens_radius", 0.0))
        d.camera.focal_distance = float(cam.get("focal_distance", 0.0))
        h = C.c_void_p()
        self.check(lib().salty_scene_upload(self.h, C.byref(d), C.byref(h)), "scene_upload")
        return Scene(self, h, n)

    @staticmethod
    def _batch_args(scenes, opts):
        if len(scenes) != len(opts) or not scenes:
            raise ValueError("one options dict per scene")
        arr = (C.c_void_p * len(scenes))(*[sc.h.value for sc in scenes])
        ro = (RenderOpts * len(scenes))(*[render_opts(**o) for o in opts])
        return arr, ro

    def render_batch(self, scenes, opts) -> dict:
        """One salty_render_batch over scenes (Scene objects) with per-scene options (dicts of
        render_opts' arguments).  Each scene's film receives its samples; returns the batch's
        device time, samples, rays and paths."""
        arr, ro = self._batch_args(scenes, opts)
        st = RenderStats()
        self.check(lib().salty_render_batch(self.h, arr, ro, len(scenes), C.byref(st)), "render_batch")
        for sc, o in zip(scenes, opts):
            n = C.c_int64()
            self.check(lib().salty_film_read(self.h, sc.h, None, None, C.byref(n)), "film_read")
            sc.film_samples = n.value
            crop = o.get("crop")
            sc.film_shape = (crop[3], crop[2]) if crop else (o["height"], o["width"])
        return {"ms": st.ms, "samples": st.samples, "rays": st.rays, "paths": st.paths}

    def cancel(self) -> None:
        """salty_ctx_cancel: a render running on this context (in another thread) stops at its
        next wave and returns ERR_CANCELLED; the context stays usable."""
        lib().salty_ctx_cancel(self.h)

    @property
    def tuning(self) -> dict:
        t = Tuning()
        self.check(lib().salty_get_tuning(self.h, C.byref(t)), "get_tuning")
        return t.as_dict()

    @tuning.setter
    def tuning(self, d: dict) -> None:
        t = Tuning()
        lib().salty_get_tuning(self.h, C.byref(t))
        for k, v in d.items():
            setattr(t, k, int(v))
        self.check(lib().salty_set_tuning(self.h, C.byref(t)), "set_tuning")

    def autotune(self, scenes, opts, trial_spp: int = 1) -> tuple[dict, float]:
        """salty_autotune: sets and returns the fastest tuning for this batch and its trial ms."""
        arr, ro = self._batch_args(scenes, opts)
        t, ms = Tuning(), C.c_float()
        self.check(lib().salty_autotune(self.h, arr, ro, len(scenes), trial_spp, C.byref(t), C.byref(ms)), "autotune")
        return t.as_dict(), ms.value

    def tonemap(self, img, type_: int = TM_REINHARD, srgb: bool = True, ref_oetf: bool = True):
        img = img if hasattr(img, "data_ptr") else np.ascontiguousarray(img, np.float32)
        h, w = img.shape[:2]
        out = np.empty((h, w, 3), np.float32)
        s8 = np.empty((h, w, 3), np.uint8) if srgb else None
        ave, mx = C.c_float(), C.c_float()
        self.check(lib().salty_tonemap(self.h, type_, w, h, _ptr(img), _ptr(out), _ptr(s8), int(ref_oetf),
                                       C.byref(ave), C.byref(mx)), "tonemap")
        return out, s8, ave.value, mx.value

    def nlm_ref(self, rgba, coeff: float):
        rgba = np.ascontiguousarray(rgba, np.float32)
        h, w = rgba.shape[:2]
        out = np.empty_like(rgba)
        self.check(lib().salty_denoise_nlm_ref(self.h, w, h, coeff, _ptr(rgba), _ptr(out)), "nlm_ref")
        return out

    def nlm(self, rgb, var, search_r: int = 10, patch_r: int = 3, k: float = 0.45, out=None):
        """Variance-scaled NLM of an (H, W, 3) image; numpy arrays or device tensors."""
        if not hasattr(rgb, "data_ptr"):
            rgb = np.ascontiguousarray(rgb, np.float32)
        if not hasattr(var, "data_ptr"):
            var = np.ascontiguousarray(var, np.float32)
        h, w = rgb.shape[:2]
        if out is None:
            out = rgb.new_empty(rgb.shape) if hasattr(rgb, "data_ptr") else np.empty_like(rgb)
        self.check(lib().salty_denoise_nlm(self.h, w, h, search_r, patch_r, k, _ptr(rgb), _ptr(var), _ptr(out)),
                   "nlm")
        return out


@dataclass
class TraceResult:
    ids: np.ndarray
    t: np.ndarray
    u: np.ndarray
    v: np.ndarray


class Scene:
    """A device scene (salty_scene): triangles, materials, lights, camera, BVH, film."""

    def __init__(self, ctx: Context, h: C.c_void_p, n_tris: int):
        self.ctx, self.h, self.n_tris = ctx, h, n_tris
        self.info = None
        self.film_shape = (0, 0)
        self.film_samples = 0

    def close(self) -> None:
        if getattr(self, "h", None) and self.ctx.h:
            lib().salty_scene_destroy(self.ctx.h, self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def build(self, bins: int = 32, max_leaf: int = 3, trav_cost: float = 0.0) -> dict:
        """salty_bvh_build; trav_cost 0 = the library's default (0.3)."""
        o = BuildOpts(bins, max_leaf, trav_cost)
        info = BvhInfo()
        self.ctx.check(lib().salty_bvh_build(self.ctx.h, self.h, C.byref(o), C.byref(info)), "bvh_build")
        self.info = {k: getattr(info, k) for k, _ in BvhInfo._fields_}
        return self.info

    def trace_raw(self, rays, hits, n: int | None = None, any_hit=False, watertight=False, counters=False) -> dict:
        """rays (n,8) float32 and hits (n,4) 16-byte records; numpy (host) or torch CUDA tensors."""
        flags = (TRACE_ANY_HIT if any_hit else 0) | (TRACE_WATERTIGHT if watertight else 0) | \
                (TRACE_COUNTERS if counters else 0)
        if n is None:
            n = rays.shape[0]
        self.ctx.check(lib().salty_trace(self.ctx.h, self.h, _ptr(rays), n, flags, _ptr(hits)), "trace")
        s = TraceStats()
        lib().salty_last_trace_stats(self.ctx.h, C.byref(s))
        return {k: getattr(s, k) for k, _ in TraceStats._fields_}

    def autotune_trace(self, rays, any_hit=False, watertight=False) -> tuple[dict, float]:
        """salty_autotune_trace: the fastest traversal launch shape for these rays (set on the
        context); returns it and its launch time in ms."""
        n = rays.shape[0]
        flags = (TRACE_ANY_HIT if any_hit else 0) | (TRACE_WATERTIGHT if watertight else 0)
        t, ms = Tuning(), C.c_float()
        self.ctx.check(lib().salty_autotune_trace(self.ctx.h, self.h, _ptr(rays), n, flags, C.byref(t), C.byref(ms)),
                       "autotune_trace")
        return t.as_dict(), ms.value

    def trace(self, rays: np.ndarray, any_hit=False, watertight=False, counters=False) -> TraceResult:
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.empty((rays.shape[0], 4), np.float32)
        self.last_stats = self.trace_raw(rays, hits, any_hit=any_hit, watertight=watertight, counters=counters)
        return TraceResult(hits[:, 1].copy().view(np.int32), hits[:, 0].copy(), hits[:, 2].copy(), hits[:, 3].copy())

    def render(self, width: int, height: int, spp: int, max_depth: int, rr_depth: int = 3,
               profile: int = PROFILE_PHYSICAL, seed: int = 1, accumulate: bool = False, fp64: bool = False,
               tonemap: int = TM_REINHARD, ref_oetf: bool = True, want=("mean", "var", "srgb"),
               crop: tuple | None = None, out: dict | None = None) -> dict:
        """Adds spp samples per pixel to the film and returns its mean / variance of the mean /
        tonemapped sRGB8 (host arrays, or the device tensors given in `out`).  crop = (x, y, w, h)
        renders that window of the width x height frame with the frame's own rays."""
        cx, cy, cw, ch = crop if crop else (0, 0, 0, 0)
        o = render_opts(width, height, spp, max_depth, rr_depth, profile, seed, accumulate, fp64, tonemap, ref_oetf,
                        crop)
        fh, fw = (ch, cw) if crop else (height, width)
        self.film_shape = (fh, fw)
        out = out or {}
        mean = out.get("mean", np.empty((fh, fw, 3), np.float32) if "mean" in want else None)
        var = out.get("var", np.empty((fh, fw, 3), np.float32) if "var" in want else None)
        s8 = out.get("srgb", np.empty((fh, fw, 3), np.uint8) if "srgb" in want else None)
        st = RenderStats()
        self.ctx.check(lib().salty_render(self.ctx.h, self.h, C.byref(o), _ptr(mean), _ptr(var), _ptr(s8),
                                          C.byref(st)), "render")
        self.film_samples = int(st.samples)
        return {"mean": mean, "var": var, "srgb": s8, "ms": st.ms, "samples": st.samples, "rays": st.rays,
                "paths": st.paths}

    def read(self, width: int, height: int, crop: tuple | None = None, fp64: bool = False,
             want=("mean", "var"), out: dict | None = None, **kw) -> dict:
        """The film's mean / variance / sRGB8 without adding samples (salty_render with spp 0);
        width, height, crop and fp64 must be those the film was rendered with."""
        return self.render(width, height, 0, kw.pop("max_depth", 1), accumulate=True, fp64=fp64, crop=crop,
                           want=want, out=out, **kw)

    def set_camera(self, pos, target, up=(0.0, 1.0, 0.0), fov: float = 1.0, near: float = 1.0,
                   lens_radius: float = 0.0, focal_distance: float = 0.0) -> None:
        c = Camera()
        c.pos, c.target, c.up = _f3(pos), _f3(target), _f3(up)
        c.fov, c.near_clip = float(fov), float(near)
        c.lens_radius, c.focal_distance = float(lens_radius), float(focal_distance)
        self.ctx.check(lib().salty_scene_set_camera(self.ctx.h, self.h, C.byref(c)), "scene_set_camera")

    def set_instances(self, instances) -> None:
        """salty_scene_set_instances: the world becomes placed copies of the scene's meshes,
        each an (first_tri, n_tris, 3x4 object-to-world matrix) triple; build afterwards."""
        arr = (Instance * max(1, len(instances)))()
        for i, (first, n, m) in enumerate(instances):
            arr[i].first_tri, arr[i].n_tris = int(first), int(n)
            arr[i].object_to_world = (C.c_float * 12)(*np.asarray(m, np.float32).reshape(12).tolist())
        self.ctx.check(lib().salty_scene_set_instances(self.ctx.h, self.h, C.byref(arr), len(instances)),
                       "scene_set_instances")

    def set_spheres(self, spheres) -> None:
        """salty_scene_set_spheres: sphere shapes, each a dict with center, radius, material
        and optionally light (a light of the scene); build afterwards."""
        arr = (Sphere * max(1, len(spheres)))()
        for i, sp in enumerate(spheres):
            arr[i].center = _f3(sp["center"])
            arr[i].radius = float(sp["radius"])
            arr[i].material = int(sp.get("material", 0))
            arr[i].light = int(bool(sp.get("light", False)))
        self.ctx.check(lib().salty_scene_set_spheres(self.ctx.h, self.h, C.byref(arr), len(spheres)),
                       "scene_set_spheres")

    def aov(self, width: int, height: int) -> dict:
        """Mean first-hit features of the film: albedo, normal (H, W, 3), depth = 1/(1+t) (H, W)."""
        al = np.empty((height, width, 3), np.float32)
        nr = np.empty((height, width, 3), np.float32)
        dp = np.empty((height, width), np.float32)
        self.ctx.check(lib().salty_film_aov(self.ctx.h, self.h, _ptr(al), _ptr(nr), _ptr(dp)), "film_aov")
        return {"albedo": al, "normal": nr, "depth": dp}

    def checkpoint(self) -> dict:
        """salty_film_checkpoint: the film's raw state (numpy arrays) and sample count."""
        h, w = self.film_shape
        sum_ = np.empty((h, w, 3), np.float64)
        sq = np.empty((h, w, 3), np.float64)
        aov = np.empty((h, w, 7), np.float32)
        n = C.c_int64()
        self.ctx.check(lib().salty_film_read(self.ctx.h, self.h, None, None, C.byref(n)), "film_read")
        # FP32 films also keep their Kahan terms; try with them first
        comp = np.empty((h, w, 3), np.float32)
        st = lib().salty_film_checkpoint(self.ctx.h, self.h, _ptr(sum_), _ptr(sq), _ptr(comp), _ptr(aov), C.byref(n))
        if st:
            comp = None
            self.ctx.check(lib().salty_film_checkpoint(self.ctx.h, self.h, _ptr(sum_), _ptr(sq), None, _ptr(aov),
                                                       C.byref(n)), "film_checkpoint")
        return {"sum": sum_, "sumsq": sq, "comp": comp, "aov": aov, "samples": n.value, "shape": (h, w)}

    def restore(self, state: dict, width: int, height: int, crop: tuple | None = None, fp64: bool = False,
                **kw) -> None:
        """salty_film_restore: the film takes a checkpoint's state for this frame / window."""
        o = render_opts(width, height, 0, kw.pop("max_depth", 1), fp64=fp64, crop=crop, **kw)
        self.ctx.check(lib().salty_film_restore(self.ctx.h, self.h, C.byref(o), _ptr(state["sum"]),
                                                _ptr(state["sumsq"]), _ptr(state.get("comp")), _ptr(state.get("aov")),
                                                int(state["samples"])), "film_restore")
        self.film_shape = (crop[3], crop[2]) if crop else (height, width)
        self.film_samples = int(state["samples"])

    def film(self, width: int, height: int):
        s = np.empty((height, width, 3), np.float64)
        q = np.empty((height, width, 3), np.float64)
        n = C.c_int64()
        self.ctx.check(lib().salty_film_read(self.ctx.h, self.h, _ptr(s), _ptr(q), C.byref(n)), "film_read")
        return s, q, n.value


UNET_FEATURES = 11  # input floats per pixel

# The learned denoiser's layers (cin, cout, relu) in parameter order; every layer is a 3x3
# convolution with weights [9][cout][cin] followed by biases [cout].
UNET_LAYERS = [(16, 32, 1), (32, 32, 1), (32, 48, 1), (48, 48, 1), (48, 64, 1), (64, 64, 1), (64, 80, 1),
               (80, 80, 1), (80, 96, 1), (176, 80, 1), (144, 64, 1), (112, 48, 1), (80, 32, 1), (32, 8, 0)]


def unet_features(mean, var, aov: dict) -> np.ndarray:
    """(H, W, 11) denoiser input: noisy colour, first-hit albedo, normal, 1/(1 + distance) and
    the colour's noise level in log space, mean_c sqrt(var_c) / (1 + colour_c), from the mean
    and the variance of the mean of a film."""
    mean = np.asarray(mean, np.float32)
    noise = (np.sqrt(np.maximum(np.asarray(var, np.float32), 0.0)) / (1.0 + np.maximum(mean, 0.0))).mean(-1)
    return np.concatenate([mean, aov["albedo"], aov["normal"], aov["depth"][..., None], noise[..., None]],
                          axis=-1).astype(np.float32)


class Unet:
    """The learned denoiser (salty_unet): BF16 tensor-core convolutions, FP32 master weights."""

    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(lib().salty_unet_create(ctx.h, seed, C.byref(h)), "unet_create")
        self.h = h
        self.n_params = int(lib().salty_unet_param_count(h))

    def close(self) -> None:
        if getattr(self, "h", None) and self.ctx.h:
            lib().salty_unet_destroy(self.ctx.h, self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_conv_kernel(self, kind: int) -> None:
        """CONV_TCGEN05 (default), CONV_TCGEN05_CP_ASYNC or CONV_MMA_SYNC for the forward /
        backward-data convolutions."""
        self.ctx.check(lib().salty_unet_set_conv_kernel(self.ctx.h, self.h, int(kind)), "unet_set_conv_kernel")

    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        self.ctx.check(lib().salty_unet_get_params(self.ctx.h, self.h, _ptr(p), None), "unet_get_params")
        return p

    def grads(self) -> np.ndarray:
        g = np.empty(self.n_params, np.float32)
        self.ctx.check(lib().salty_unet_get_params(self.ctx.h, self.h, None, _ptr(g)), "unet_get_params")
        return g

    def adam_state(self) -> dict:
        m = np.empty(self.n_params, np.float32)
        v = np.empty(self.n_params, np.float32)
        step = C.c_int64()
        self.ctx.check(lib().salty_unet_get_adam(self.ctx.h, self.h, _ptr(m), _ptr(v), C.byref(step)), "unet_get_adam")
        return {"m": m, "v": v, "step": step.value}

    def set_adam_state(self, st: dict) -> None:
        m = np.ascontiguousarray(st["m"], np.float32)
        v = np.ascontiguousarray(st["v"], np.float32)
        self.ctx.check(lib().salty_unet_set_adam(self.ctx.h, self.h, _ptr(m), _ptr(v), int(st["step"])),
                       "unet_set_adam")

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        self.ctx.check(lib().salty_unet_set_params(self.ctx.h, self.h, _ptr(p)), "unet_set_params")

    @staticmethod
    def _batch(a, ch):
        if not hasattr(a, "data_ptr"):
            a = np.ascontiguousarray(a, np.float32)
        if a.ndim == 3:
            a = a[None]
        if a.ndim != 4 or a.shape[-1] != ch:
            raise ValueError(f"expected (N, H, W, {ch}) or (H, W, {ch}), got {tuple(a.shape)}")
        return a

    def forward(self, features, out=None):
        f = self._batch(features, UNET_FEATURES)
        n, h, w = f.shape[:3]
        if out is None:
            out = np.empty((n, h, w, 3), np.float32)
        self.ctx.check(lib().salty_unet_forward(self.ctx.h, self.h, _ptr(f), n, h, w, _ptr(out)), "unet_forward")
        return out[0] if features.ndim == 3 and isinstance(out, np.ndarray) else out

    def denoise_film(self, scene: "Scene", out=None, mirrors: int = 1):
        """Denoised image of the scene's film (H, W, 3), computed on the device; mirrors > 1
        averages the network over mirror images of the frame (salty_denoise_unet_ensemble)."""
        h, w = scene.film_shape
        if out is None:
            out = np.empty((h, w, 3), np.float32)
        self.ctx.check(lib().salty_denoise_unet_ensemble(self.ctx.h, self.h, scene.h, mirrors, _ptr(out)),
                       "denoise_unet")
        return out

    def train_step(self, features, target, lr: float) -> float:
        f = self._batch(features, UNET_FEATURES)
        t = self._batch(target, 3)
        n, h, w = f.shape[:3]
        if tuple(t.shape[:3]) != (n, h, w):
            raise ValueError("features and target differ in shape")
        loss = C.c_float()
        self.ctx.check(lib().salty_unet_train_step(self.ctx.h, self.h, _ptr(f), _ptr(t), n, h, w, lr,
                                                   C.byref(loss)), "unet_train_step")
        return loss.value
