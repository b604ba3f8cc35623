"""Generates the committed golden fixtures from the UNMODIFIED reference.

Run in a checkout where the reference sources exist (oracle/Makefile builds
oracle/_ref/libsalty_ref.so from them):

    python tests/golden/make_golden.py

The reference has no tests, golden vectors or known-answer files of its own, so these
fixtures are its outputs on seeded inputs, produced through the harness in
oracle/ref/sref_harness.cpp.  Inputs are regenerated from their seeds by the tests
(sha256 digests below detect any drift of the generators between hosts).
"""
from __future__ import annotations

import hashlib
import os
import struct
import sys
import tempfile
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Oracle, Reference, SceneData, build  # noqa: E402

SOUP_SEED, RAY_SEED = 20260001, 20260002


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def decode_png(path: str) -> np.ndarray:
    """Minimal PNG reader for 8-bit RGB, non-interlaced (what stb_image_write emits)."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        ln, = struct.unpack(">I", data[pos:pos + 4])
        typ = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + ln]
        if typ == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert depth == 8 and ctype == 2
        elif typ == b"IDAT":
            idat += body
        pos += 12 + ln
    raw = zlib.decompress(idat)
    stride = w * 3
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        line = np.frombuffer(raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)], np.uint8).astype(np.int32)
        cur = np.zeros(stride, np.int32)
        for x in range(stride):
            a = cur[x - 3] if x >= 3 else 0
            b = prev[x]
            c = prev[x - 3] if x >= 3 else 0
            if f == 0:
                p = 0
            elif f == 1:
                p = a
            elif f == 2:
                p = b
            elif f == 3:
                p = (a + b) // 2
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            cur[x] = (line[x] + p) & 0xFF
        out[y] = cur
        prev = cur
    return out.reshape(h, w, 3)


def cornell_scene(variant: str = "baseline") -> SceneData:
    from salty_gb300 import scenes  # noqa: E402  (numpy-only module)
    sc = scenes.cornell(variant)
    return SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], None,
                     sc["sky"], sc["camera"], tri_uv=sc.get("tri_uv"), textures=sc.get("textures", []),
                     ibl=sc.get("ibl"), spheres=sc.get("spheres", []))


def hdr_image(seed: int, w: int, h: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    img = np.exp(rng.normal(-1.0, 1.5, size=(h, w, 3))).astype(np.float32)
    img[0, 0] = 0.0            # exercises the epsilon floor of the log-average
    img[1, 1] = (40.0, 35.0, 30.0)
    return img


def glossy_fixture(r) -> None:
    """The Cornell box with Phong and Plastic surfaces through PathTracer::Radiance."""
    sc = cornell_scene("glossy")
    W = H = 48
    spp, depth = 1024, 8
    total, sq, secs = r.render(sc, W, H, spp, depth, seed=777)
    mean = total / spp
    var = (sq / spp - mean * mean) * spp / (spp - 1) / spp
    np.savez_compressed(os.path.join(HERE, "cornell_glossy_ref_48.npz"), mean=mean.astype(np.float32),
                        var=np.maximum(var, 0).astype(np.float32), spp=spp, max_bounce=depth, width=W, height=H)
    print(f"glossy cornell reference render: {secs:.2f} s")


def thinlens_fixture(r) -> None:
    """The Cornell box through ThinLensCamera (include/s3d_camera.h:150-267)."""
    sc = cornell_scene("thinlens")
    W = H = 48
    spp, depth = 1024, 8
    total, sq, secs = r.render(sc, W, H, spp, depth, seed=4242)
    mean = total / spp
    var = (sq / spp - mean * mean) * spp / (spp - 1) / spp
    np.savez_compressed(os.path.join(HERE, "cornell_thinlens_ref_48.npz"), mean=mean.astype(np.float32),
                        var=np.maximum(var, 0).astype(np.float32), spp=spp, max_bounce=depth, width=W, height=H)
    print(f"thin-lens cornell reference render: {secs:.2f} s")


def textured_fixture(r) -> None:
    """The Cornell box with colour maps and an environment map (TexturedMaterial, the IBL)."""
    sc = cornell_scene("textured")
    W = H = 48
    spp, depth = 1024, 8
    total, sq, secs = r.render(sc, W, H, spp, depth, seed=5151)
    mean = total / spp
    var = (sq / spp - mean * mean) * spp / (spp - 1) / spp
    np.savez_compressed(os.path.join(HERE, "cornell_textured_ref_48.npz"), mean=mean.astype(np.float32),
                        var=np.maximum(var, 0).astype(np.float32), spp=spp, max_bounce=depth, width=W, height=H)
    print(f"textured cornell reference render: {secs:.2f} s")


def specular_fixture(r) -> None:
    """The Cornell box with a mirror tall box and a glass short box through
    PathTracer::Radiance: Mirror::Shade (src/s3d_mirror.cpp:59-71) and Glass::Shade with its
    1/0.5 branch weights (src/s3d_glass.cpp:60-128)."""
    sc = cornell_scene("specular")
    W = H = 48
    spp, depth = 16384, 8
    total, sq, secs = r.render(sc, W, H, spp, depth, seed=6161)
    mean = total / spp
    var = (sq / spp - mean * mean) * spp / (spp - 1) / spp
    np.savez_compressed(os.path.join(HERE, "cornell_specular_ref_48.npz"), mean=mean.astype(np.float32),
                        var=np.maximum(var, 0).astype(np.float32), spp=spp, max_bounce=depth, width=W, height=H)
    print(f"specular cornell reference render: {secs:.2f} s")


def spheres_fixture(r) -> None:
    """Analytic spheres (Sphere::IsHit/CalcParam/Sample): Lambert, mirror and glass spheres
    and a light sphere sharing the light list with the quad light."""
    sc = cornell_scene("spheres")
    W = H = 48
    spp, depth = 4096, 8
    total, sq, secs = r.render(sc, W, H, spp, depth, seed=7171)
    mean = total / spp
    var = (sq / spp - mean * mean) * spp / (spp - 1) / spp
    np.savez_compressed(os.path.join(HERE, "cornell_spheres_ref_48.npz"), mean=mean.astype(np.float32),
                        var=np.maximum(var, 0).astype(np.float32), spp=spp, max_bounce=depth, width=W, height=H)
    print(f"sphere cornell reference render: {secs:.2f} s")


def c1_fixture(r) -> None:
    """The Cornell frame as configured for the CPU-runnable benchmark case: 256x256, max
    depth 8, the reference's estimator; 1024 samples per pixel (64 of the configured 16-spp
    frames) so that a per-pixel comparison has power.  Mean and standard error of the mean
    stored as float16 (relative precision 5e-4, far below the noise)."""
    sc = cornell_scene()
    W = H = 256
    spp, depth = 1024, 8
    total, sq, secs = r.render(sc, W, H, spp, depth, seed=16016)
    mean = total / spp
    var = (sq / spp - mean * mean) * spp / (spp - 1) / spp
    np.savez_compressed(os.path.join(HERE, "cornell_c1_ref_256.npz"), mean=mean.astype(np.float16),
                        sem=np.sqrt(np.maximum(var, 0)).astype(np.float16), spp=spp, max_bounce=depth,
                        width=W, height=H)
    print(f"configured cornell frame: {secs:.2f} s")


def main() -> None:
    build(with_reference=True)
    o, r = Oracle(), Reference()
    only = {"glossy": glossy_fixture, "thinlens": thinlens_fixture, "textured": textured_fixture,
            "specular": specular_fixture, "c1": c1_fixture, "spheres": spheres_fixture}
    if sys.argv[1:] and all(a in only for a in sys.argv[1:]):
        for a in sys.argv[1:]:
            only[a](r)
        return

    # 1. traversal: 1M-triangle soup, first 65536 rays of the microbenchmark stream
    tris = o.gen_soup(SOUP_SEED, 1_000_000)
    rays = o.gen_rays(RAY_SEED, 65536)
    s = r.soup(tris)
    ids, t, u, v, _ = s.trace(rays)
    s.close()
    np.savez_compressed(os.path.join(HERE, "trace_soup_1m.npz"), ids=ids, t=t,
                        soup_sha=sha(tris), rays_sha=sha(rays), n_tris=1_000_000, n_rays=65536,
                        soup_seed=SOUP_SEED, ray_seed=RAY_SEED)

    # 2. traversal, small soup, with barycentrics
    tris_s = o.gen_soup(7, 30000)
    rays_s = o.gen_rays(8, 8192)
    s = r.soup(tris_s)
    ids, t, u, v, _ = s.trace(rays_s)
    s.close()
    np.savez_compressed(os.path.join(HERE, "trace_soup_30k.npz"), ids=ids, t=t, u=u, v=v,
                        soup_sha=sha(tris_s), rays_sha=sha(rays_s), soup_seed=7, ray_seed=8,
                        n_tris=30000, n_rays=8192)

    # 3. Cornell box through PathTracer::Radiance (reference estimator)
    sc = cornell_scene()
    W = H = 64
    spp, depth = 1024, 8
    total, sq, secs = r.render(sc, W, H, spp, depth, seed=12345)
    mean = total / spp
    var = (sq / spp - mean * mean) * spp / (spp - 1) / spp
    np.savez_compressed(os.path.join(HERE, "cornell_ref_64.npz"), mean=mean.astype(np.float32),
                        var=np.maximum(var, 0).astype(np.float32), spp=spp, max_bounce=depth, width=W, height=H)
    print(f"cornell reference render: {secs:.2f} s")
    glossy_fixture(r)
    thinlens_fixture(r)
    textured_fixture(r)
    specular_fixture(r)
    c1_fixture(r)
    spheres_fixture(r)

    # 4. tonemapping and the sRGB8 capture
    img = hdr_image(99, 48, 32)
    out = {f"tm{k}": r.tonemap(k, img) for k in (0, 1, 2)}
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "cap.png")
        r.capture_png(img, p)
        png = decode_png(p)
    np.savez_compressed(os.path.join(HERE, "tonemap_ref.npz"), img=img, srgb_aces_ref=png, **out)

    # 5. NLM
    rng = np.random.default_rng(5)
    rgba = rng.random((20, 24, 4), dtype=np.float32)
    rgba[..., 3] = 1.0
    nl = r.nlm(rgba, 0.2)
    np.savez_compressed(os.path.join(HERE, "nlm_ref.npz"), rgba=rgba, coeff=0.2, out=nl)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
