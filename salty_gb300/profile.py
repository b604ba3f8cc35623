"""Small fixed workloads for profiling the kernels (run them under ncu or alone).

    python -m salty_gb300.profile render [--spp 1] [--frames 2] [--width 1920 --height 1080]
                                                                     heightfield frames
    python -m salty_gb300.profile unet [--n 1 --h 1088 --w 1920] [--conv tcgen05|tcgen05_cp_async|mma_sync|all]
                                                                     denoiser forward passes
    python -m salty_gb300.profile trace-sweep                        traversal launch shapes
    python -m salty_gb300.profile cornell                            the 256^2 Cornell box, 16 spp
    python -m salty_gb300.profile wave-sweep [--spp 64]              1080p heightfield per wave size
    python -m salty_gb300.profile nlm --h 1080                       1080p NLM vs the FP32 peak
    python -m salty_gb300.profile tonemap                            tonemap + sRGB8 vs the copy peak

`render` and `unet` print one line of timings; `trace-sweep` times every traversal launch
shape (block size x register budget x pool x postpone) on the 1M-triangle microbenchmark
soup with 16,777,216 rays and checks that all give the same hits.
"""
from __future__ import annotations

import argparse
import itertools
import json
import time

import numpy as np

from . import Context, Unet, UNET_FEATURES, microbench_rays, microbench_soup
from . import scenes


def render(spp: int, frames: int, width: int = 1920, height: int = 1080) -> dict:
    ctx = Context(0)
    s = scenes.upload(ctx, scenes.heightfield())
    info = s.build()
    out = []
    for i in range(frames):
        r = s.render(width, height, spp, 12, seed=3 + i, want=())
        out.append({"ms": r["ms"], "rays": r["rays"], "paths": r["paths"], "Mrays_s": r["rays"] / r["ms"] / 1e3})
    return {"workload": f"{width}x{height} heightfield, {spp} spp x {frames} frames", "bvh_build_ms": info["build_ms"],
            "frames": out}


def cornell() -> dict:
    """The small Cornell box at 256 x 256, 16 spp, depth 8, Russian roulette from depth 3, in
    the reference-compatible estimator: device time per frame (best of 5 after a warm-up)."""
    from . import PROFILE_COMPAT, TM_REINHARD
    ctx = Context(0)
    s = scenes.upload(ctx, scenes.cornell("baseline"))
    s.build()
    s.render(256, 256, 16, 8, profile=PROFILE_COMPAT, seed=1, want=())
    runs = [s.render(256, 256, 16, 8, profile=PROFILE_COMPAT, seed=2 + i, tonemap=TM_REINHARD, want=())
            for i in range(5)]
    best = min(runs, key=lambda r: r["ms"])
    return {"workload": "Cornell box 256x256, 16 spp, depth 8, compat profile", "ms": best["ms"],
            "Mrays_s": best["rays"] / best["ms"] / 1e3, "Mpaths_s": best["paths"] / best["ms"] / 1e3}


def wave_sweep(spp: int) -> dict:
    """The 1080p heightfield at `spp` samples, depth 12, default launch shapes, for waves of
    2^22 .. 2^27 paths: best of two renders each after an 8-spp warm-up."""
    ctx = Context(0)
    s = scenes.upload(ctx, scenes.heightfield())
    s.build()
    base = ctx.tuning
    res = []
    for e in range(22, 28):
        t = dict(base)
        t["wave_paths"] = 1 << e
        ctx.tuning = t
        s.render(1920, 1080, 8, 12, seed=1, want=())
        best = min((s.render(1920, 1080, spp, 12, seed=2 + i, want=()) for i in range(2)), key=lambda r: r["ms"])
        res.append({"wave_paths": 1 << e, "ms": best["ms"], "Mrays_s": best["rays"] / best["ms"] / 1e3,
                    "Mpaths_s": best["paths"] / best["ms"] / 1e3})
    return {"workload": f"1920x1080 heightfield, {spp} spp, depth 12, default launch shapes", "waves": res}


def tonemap() -> dict:
    """salty_tonemap_noalloc (Reinhard, linear + sRGB8 outputs) on device-resident images,
    timed with CUDA events on the caller's stream, a torch stream of its own (a NULL stream
    would mean the library's stream, which torch's events do not see); mean of 20 calls after
    3 warm-ups.
    Algorithmic bytes per pixel: 12 read for the log-average, 12 read + 12 written + 3
    written for the map = 39."""
    import ctypes as C
    import torch
    from . import lib, TM_REINHARD
    ctx = Context(0)
    st = torch.cuda.Stream()
    res = []
    for w, h in ((1920, 1080), (4096, 4096)):
        rgb = torch.rand((h, w, 3), device="cuda") * 4.0
        out = torch.empty_like(rgb)
        s8 = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")

        def call():
            ctx.check(lib().salty_tonemap_noalloc(ctx.h, C.c_void_p(st.cuda_stream), TM_REINHARD, w, h,
                                                  C.c_void_p(rgb.data_ptr()), C.c_void_p(out.data_ptr()),
                                                  C.c_void_p(s8.data_ptr()), 1), "tonemap_noalloc")
        torch.cuda.synchronize()
        with torch.cuda.stream(st):
            for _ in range(3):
                call()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(20):
                call()
            e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 20
        gbs = 39.0 * w * h / (ms * 1e-3) / 1e9
        res.append({"width": w, "height": h, "ms": ms, "GB_s": gbs})
    return {"workload": "tonemap (Reinhard) + sRGB8, device arrays", "sizes": res}


def nlm(h: int, w: int) -> dict:
    """salty_denoise_nlm (21x21 search, 7x7 patch) on a w x h device-resident image: the
    best of 5 host-timed synchronous calls, against the measured FP32 peak.  Algorithmic
    work of the filter: 441 offsets x 49 taps x 3 channels x 3 flops (difference, square,
    sum) = 194,481 FP32 flops per pixel."""
    import torch
    ctx = Context(0)
    peak = ctx.fp32_peak()
    g = torch.Generator(device="cuda").manual_seed(1)
    rgb = torch.rand((h, w, 3), device="cuda", generator=g)
    var = torch.rand((h, w, 3), device="cuda", generator=g) * 0.01
    out = torch.empty_like(rgb)
    ctx.nlm(rgb, var, 10, 3, 0.45, out=out)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(5):
        t0 = time.perf_counter()
        ctx.nlm(rgb, var, 10, 3, 0.45, out=out)
        torch.cuda.synchronize()
        best = min(best, (time.perf_counter() - t0) * 1e3)
    flops = 194481.0 * w * h
    ach = flops / (best * 1e-3) / 1e12
    return {"workload": f"NLM 21x21 search, 7x7 patch, {w}x{h}", "ms": best, "algorithmic_tflops": ach,
            "fp32_peak_tflops": peak, "frac": ach / peak}


def unet(n: int, h: int, w: int, conv: str = "tcgen05", train: bool = False) -> dict:
    """Forward passes (and, with train, training steps at lr 0) on random features: the
    best of 5 wall-clock times after a warm-up, per convolution kernel."""
    import torch
    from . import CONV_MMA_SYNC, CONV_TCGEN05, CONV_TCGEN05_CP_ASYNC
    ctx = Context(0)
    net = Unet(ctx, seed=1)
    f = torch.rand((n, h, w, UNET_FEATURES), device="cuda")
    o = torch.empty((n, h, w, 3), device="cuda")
    tgt = torch.rand((n, h, w, 3), device="cuda")
    names = {CONV_TCGEN05: "tcgen05", CONV_TCGEN05_CP_ASYNC: "tcgen05_cp_async", CONV_MMA_SYNC: "mma_sync"}
    kinds = {"tcgen05": [CONV_TCGEN05], "tcgen05_cp_async": [CONV_TCGEN05_CP_ASYNC], "mma_sync": [CONV_MMA_SYNC],
             "all": [CONV_TCGEN05, CONV_TCGEN05_CP_ASYNC, CONV_MMA_SYNC]}[conv]
    res = {"workload": f"U-Net {n}x{h}x{w}"}
    for k in kinds:
        net.set_conv_kernel(k)
        name = names[k]
        steps = [("forward_ms", lambda: net.forward(f, out=o))]
        if train:
            steps.append(("train_step_ms", lambda: net.train_step(f, tgt, lr=0.0)))
        for key, fn in steps:
            fn()
            torch.cuda.synchronize()
            best = float("inf")
            for _ in range(5):
                t0 = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                best = min(best, (time.perf_counter() - t0) * 1e3)
            res[f"{name}_{key}"] = best
    net.close()
    return res


def trace_sweep() -> dict:
    import torch
    ctx = Context(0)
    sc = ctx.upload_scene(microbench_soup(20260001, 1_000_000))
    sc.build()
    n = 16_777_216
    rays = torch.from_numpy(microbench_rays(20260002, n, 1e-4)).cuda()
    hits = torch.empty((n, 4), device="cuda")
    ref, res = None, []
    for blk, regs, pool, post in itertools.product((64, 128, 256), (64, 48), (64, 128, 256), (1, 4, 7, 10)):
        ctx.tuning = {"trace_block": blk, "trace_regs": regs, "trace_pool": pool, "trace_postpone": post}
        for _ in range(2):
            sc.trace_raw(rays, hits)
        ms = min(sc.trace_raw(rays, hits)["kernel_ms"] for _ in range(4))
        ids = hits.cpu().numpy().view(np.int32)[:, 1]
        if ref is None:
            ref = ids.copy()
        res.append({"ms": ms, "Mrays_s": n / ms / 1e3, "trace_block": blk, "trace_regs": regs, "trace_pool": pool,
                    "trace_postpone": post, "same_hits": bool(np.array_equal(ids, ref))})
    res.sort(key=lambda r: r["ms"])
    return {"workload": "traversal microbenchmark, 1M triangles, 16,777,216 rays, closest hit", "shapes": res}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("what", choices=["render", "unet", "trace-sweep", "cornell", "wave-sweep", "nlm", "tonemap"])
    ap.add_argument("--spp", type=int, default=None, help="render: 1, wave-sweep: 64")
    ap.add_argument("--frames", type=int, default=2)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--n", type=int, default=1)
    ap.add_argument("--h", type=int, default=1088)
    ap.add_argument("--w", type=int, default=1920)
    ap.add_argument("--conv", default="tcgen05", choices=["tcgen05", "tcgen05_cp_async", "mma_sync", "all"])
    ap.add_argument("--train", action="store_true", help="unet: also time training steps")
    a = ap.parse_args(argv)
    if a.what == "render":
        r = render(a.spp or 1, a.frames, a.width, a.height)
    elif a.what == "unet":
        r = unet(a.n, a.h, a.w, a.conv, a.train)
    elif a.what == "cornell":
        r = cornell()
    elif a.what == "tonemap":
        r = tonemap()
    elif a.what == "nlm":
        r = nlm(a.h, a.w)
    elif a.what == "wave-sweep":
        r = wave_sweep(a.spp or 64)
    else:
        r = trace_sweep()
    print(json.dumps(r))


if __name__ == "__main__":
    main()
