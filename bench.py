"""Traversal microbenchmark of the Salty hot path on GB300.

Workload (one step): closest-hit queries for 16,777,216 seeded rays against a
1,000,000-triangle soup (centroids uniform in [0,1]^3, vertices within +-0.005), BVH
built on the device with 32-bin SAH and collapsed to 8-wide quantised nodes.  Rays start
on a radius-2 sphere about (0.5,0.5,0.5) and aim at uniform points of the cube; tmin
1e-4, tmax inf.  Metric: Mrays/s (rays traced per second), whole job.

  value  device-resident rays and hits (torch CUDA tensors), one salty_trace per step
  e2e    the same call with rays in pinned host memory and hits written back to it:
         host->device and device->host copies inside every step
  any_hit  the same rays as occlusion queries (first hit ends the walk)
Rays (512 MiB) and hits (256 MiB) are larger than L2, so no flush is needed between steps;
the BVH (nodes + leaf triangles) stays resident, as in any traversal.

The default run then measures the 1080p heightfield scene as configured (measure_c3:
directional sun, depth 12): one 64-spp frame (render_c3) and the time to relRMSE 0.01 of
plain rendering and of the chosen path (autotuned launch shapes + U-Net), against FP64
references of four windows at 2^20 spp (time_to_rmse); --no-c3 skips it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Other workloads (--workload), one JSON line each:
  time-to-rmse  1080p heightfield: seconds to relRMSE 0.01, plain vs autotuned + U-Net
  batch         256 uneven scenes in one salty_render_batch vs one call per scene
  cornell       the 256x256 Cornell box at 16 spp, with the CPU port beside it
  denoise       U-Net vs NLM on the held-out 4-spp 1080p film (relMSE, time, tensor roofline)
Profiling workloads (fixed small cases to time alone or under ncu):
  render        1080p heightfield frames (--spp, --frames, --width, --height)
  wave-sweep    1080p heightfield at --spp for waves of 2^22..2^27 paths
  trace-sweep   every traversal launch shape on the microbenchmark
  unet          U-Net forward passes / training steps (--unet-n/-h/-w, --conv, --train)
  nlm           variance-scaled NLM on a --width x --height image vs the nominal FP32 peak
  tonemap       salty_tonemap_noalloc at 1080p and 4096^2 vs the copy peak
"""
from __future__ import annotations

import argparse
import itertools
import json
import math
import os
import shutil
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_TRIS = 1_000_000
N_RAYS = 16_777_216
SOUP_SEED, RAY_SEED = 20260001, 20260002
TMIN = 1e-4
METRIC = "Mrays/s"
CPU_SAMPLE = 2_097_152      # rays of the same stream timed on the host cores (~10 s of CPU work)
# DRAM bytes (read + write) per ray of the closest-hit k_trace launch, from one ncu capture
# of that kernel at the default launch shape (128 threads, 56 registers, pool 64, no
# triangle postponing) on the same soup at 4,194,304 rays; the traffic (rays in, hits out,
# L2 misses) scales with the ray count, so traffic per launch is this figure times the rays
# of the launch.
NCU_DRAM_BYTES_PER_RAY = (388.030208e6 + 69.070336e6) / 4_194_304


def measured_peaks_tensor() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"bf16_tflops": d.get("bf16_tflops", 1900.0), "source": "measured (burst)"}
    return {"bf16_tflops": 1900.0, "source": "fallback"}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.out,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.out.close()

    def summary(self) -> dict | None:
        if not self.path or not os.path.exists(self.path):
            return None
        rows = [l.strip().split(", ") for l in open(self.path) if l.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("SALTY_BENCH_GLOO") is None else "gloo")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x: float, device) -> float:
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_reference_rays_per_s(tris: np.ndarray, rays: np.ndarray) -> tuple[float, int, float, float]:
    """The reference's own traversal on all host cores: BVH8::Create and BVH8::IsHit
    (src/s3d_bvh8.cpp:191-206,401-479) with Triangle::IsHit, as restated in the oracle (same
    tree, walk order and answers as the compiled reference; it cannot travel, being built
    from the reference's sources).  Returns (rays/s, threads, trace seconds, build seconds)."""
    from oracle.oracle import Oracle, build
    build(with_reference=False)
    o = Oracle()
    threads = os.cpu_count() or 1
    b = o.ref_bvh(tris)
    try:
        _, _, _, _, secs = b.trace(rays, nthreads=threads)
    finally:
        b.close()
    return rays.shape[0] / secs, threads, secs, b.build_seconds


REFERENCE_NOTE = ("the reference's BVH8::Create + BVH8::IsHit + Triangle::IsHit (16-bucket SAH, 8-wide "
                  "boxes without clipping to the best hit, child order 0..7), restated in C (oracle/) "
                  "with the compiled reference's tree, walk order and hit ids; its speed equals the "
                  "compiled reference's within 10 % on an x86 host (0.0137 vs 0.0128 Mrays/s per thread)")


def run_reference(args, ws, rank, local, pg):
    """The reference's CPU implementation of the path, timed on the host cores."""
    if rank != 0:
        return
    import salty_gb300
    tris = salty_gb300.microbench_soup(SOUP_SEED, N_TRIS)
    sample = 262_144  # ~1.3 s per step on 16 host threads: the default run stays within a minute
    rays = salty_gb300.microbench_rays(RAY_SEED, sample, TMIN)
    from oracle.oracle import Oracle, build
    build(with_reference=False)
    o = Oracle()
    threads = os.cpu_count() or 1
    b = o.ref_bvh(tris)
    for _ in range(args.warmup):
        b.trace(rays, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        b.trace(rays, nthreads=threads)
    dt = time.perf_counter() - t0
    build_s = b.build_seconds
    b.close()
    value = sample * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded PCG soup and rays)",
        "config": {"workload": "traversal microbenchmark: 1M-triangle soup, closest hit", "n_tris": N_TRIS,
                   "rays_per_step": sample, "full_rays": N_RAYS, "bvh_build_seconds": build_s},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"first {sample} rays of the 16,777,216-ray stream per step, 1M triangles",
                         "implementation": REFERENCE_NOTE},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


C3_WINDOWS = ((448, 560, 128, 128), (1344, 560, 128, 128), (704, 860, 128, 128), (1088, 860, 128, 128))


def measure_c3(args) -> dict:
    """The 1080p heightfield scene as configured (2048^2 terrain + 4096 icospheres, 13.6M
    triangles, sky 1.0 + a directional sun, max depth 12, physical profile):
      render_c3     one 64-spp frame with the default launch shapes (Mrays/s, Mpaths/s)
      time_to_rmse  seconds until each method's image reaches relRMSE <= target on four
                    128x128 windows of the frame against FP64 renders of them at
                    --ref-spp samples (their own noise subtracted): plain progressive
                    rendering with the default launch shapes, and the chosen path (launch
                    shapes from salty_autotune, untimed; the film denoised by the U-Net)."""
    import torch
    import salty_gb300
    from salty_gb300 import build as b
    from salty_gb300 import convergence as cv
    from salty_gb300 import denoiser as dn
    from salty_gb300 import scenes
    b.build()
    W, H, D = 1920, 1080, 12
    ctx = salty_gb300.Context(0)
    t0 = time.perf_counter()
    sc = scenes.heightfield(sun_half_angle=args.sun_half_angle)
    s = scenes.upload(ctx, sc)
    info = s.build()
    setup_s = time.perf_counter() - t0
    ref = cv.reference_image(s, W, H, list(C3_WINDOWS), D, spp=args.ref_spp)
    den = dn.Denoiser(ctx)
    for _ in range(3):
        s.render(W, H, 4, D, seed=3, want=())
    torch.cuda.synchronize()
    r = s.render(W, H, 64, D, seed=5, want=())
    render = {"spp": 64, "ms": r["ms"], "Mrays_s": r["rays"] / r["ms"] / 1e3, "Mpaths_s": r["paths"] / r["ms"] / 1e3,
              "rays_per_path": r["rays"] / max(r["paths"], 1)}
    # the plain path renders with the default launch shapes; the denoised path with the
    # shapes salty_autotune picks for this frame (trial renders at 64 spp -- 132.7M samples,
    # enough to tell wave sizes up to 2^27 apart -- untimed, reported as autotune_seconds)
    default = ctx.tuning
    t0 = time.perf_counter()
    tuned, trial_ms = ctx.autotune([s], [{"width": W, "height": H, "spp": 64, "max_depth": D,
                                          "profile": salty_gb300.PROFILE_PHYSICAL}], trial_spp=64)
    tune_s = time.perf_counter() - t0
    res = {}
    with ClockSampler(0) as clk:
        for m in args.methods.split(","):
            ctx.tuning = default if m == "plain" else tuned
            res[m] = cv.converge(s, W, H, ref, D, args.target, method=m, ctx=ctx, denoiser=den,
                                 max_spp=args.max_spp)
    ctx.tuning = default
    plain = res.get("plain", {}).get("seconds_to_target")
    best = res.get("unet", {}).get("seconds_to_target")
    out = {
        "workload": "1920x1080 heightfield: 2048^2 terrain + 4096 icospheres (13.6M triangles), sky 1.0 + "
                    + ("a directional sun" if args.sun_half_angle == 0 else
                       f"a sun disk of {math.degrees(args.sun_half_angle):.1f} deg") + ", max depth 12, physical profile",
        "n_tris": int(sc["tri_pos"].shape[0]), "bvh_nodes": info["n_nodes"], "bvh_build_ms": info["build_ms"],
        "target_rel_rmse": args.target, "windows": [list(c) for c in C3_WINDOWS], "ref_spp": args.ref_spp,
        "ref_noise_rel_mse": ref["noise"], "ref_noise_of_target": ref["noise"] / args.target ** 2,
        "ref_seconds": ref["seconds"], "setup_seconds": setup_s,
        "plain_seconds": plain, "chosen_seconds": best,
        "speedup_vs_plain": (plain / best) if plain and best else None,
        "denoiser": {"method": den.method, "hq_from_spp": den.hq_from_spp, "mirrors": den.mirrors,
                     "weights": {k: v for k, v in den.meta.items() if k != "scenes"},
                     "hq_weights": {k: v for k, v in den.hq_meta.items() if k != "scenes"}},
        "tuning_plain": default, "tuning_chosen": tuned, "autotune_seconds": tune_s, "autotune_trial_ms": trial_ms,
        "methods": {m: {"seconds_to_target": v["seconds_to_target"], "curve": v["curve"]} for m, v in res.items()},
        "render_c3": render, "clocks": clk.summary(),
    }
    den.close()
    s.close()
    ctx.close()
    return out


def run_time_to_rmse(args):
    """measure_c3 as its own JSON line (value: the chosen path's seconds to the target)."""
    r = measure_c3(args)
    line = {
        "metric": f"seconds to relRMSE <= {args.target} (1080p heightfield, four 128x128 windows vs FP64 "
                  f"{args.ref_spp}-spp)",
        "value": r["chosen_seconds"], "unit": "s", "n_gpus": 1, "higher_is_better": False, "dtype": "f32",
        "data": "synthetic (seeded heightfield scene generated on the host)",
        "config": {"workload": r["workload"]}, "time_to_rmse": r, "clocks": r["clocks"],
    }
    print(json.dumps(line), flush=True)


def run_batch(args):
    """256 seeded scenes of uneven size (soups and heightfields, 1e3..1e6 triangles,
    64^2..512^2 pixels, 4/16/64 spp, depth 8, physical profile): one salty_render_batch per
    step (tuning from salty_autotune) against one salty_render call per scene per step."""
    import torch
    import salty_gb300
    from salty_gb300 import build as b
    from salty_gb300 import scenes
    b.build()
    ctx = salty_gb300.Context(0)
    t0 = time.perf_counter()
    ss, opts, tris = [], [], 0
    build_ms = 0.0
    for i in range(args.scenes):
        d, o = scenes.batch_scene(20260100 + i)
        o["profile"] = salty_gb300.PROFILE_PHYSICAL
        s = scenes.upload(ctx, d)
        build_ms += s.build()["build_ms"]
        tris += int(d["tri_pos"].shape[0])
        ss.append(s)
        opts.append(o)
    setup_s = time.perf_counter() - t0
    samples = sum(o["width"] * o["height"] * o["spp"] for o in opts)
    default = ctx.tuning
    t0 = time.perf_counter()
    tuned, trial_ms = ctx.autotune(ss, opts, trial_spp=1)
    tune_s = time.perf_counter() - t0

    def batched():
        return ctx.render_batch(ss, opts)

    def per_scene():
        tot = {"ms": 0.0, "rays": 0, "paths": 0}
        for s, o in zip(ss, opts):
            o2 = dict(o)
            r = s.render(o2.pop("width"), o2.pop("height"), o2.pop("spp"), o2.pop("max_depth"), want=(), **o2)
            for k in tot:
                tot[k] += r[k]
        return tot

    res = {}
    with ClockSampler(0) as clk:
        for name, fn in (("batched", batched), ("per_scene", per_scene)):
            for _ in range(args.warmup):
                fn()
            torch.cuda.synchronize()
            rays = 0
            t0 = time.perf_counter()
            dev_ms = 0.0
            for _ in range(args.steps):
                r = fn()
                rays += r["rays"]
                dev_ms += r["ms"]
            wall = time.perf_counter() - t0
            res[name] = {"Mrays_s": rays / wall / 1e6, "wall_ms_per_step": wall * 1e3 / args.steps,
                         "device_ms_per_step": dev_ms / args.steps, "rays_per_step": rays // args.steps,
                         "wall_ms_per_scene": wall * 1e3 / args.steps / len(ss)}
    clocks = clk.summary()
    line = {
        "metric": "Mrays/s (batched uneven renders)", "value": res["batched"]["Mrays_s"], "unit": "Mrays/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f32",
        "ms_per_step": res["batched"]["wall_ms_per_step"],
        "data": "synthetic (seeded soups and heightfields generated on the host)",
        "config": {"workload": f"{len(ss)} scenes, soup or heightfield, 1e3..1e6 triangles, 64^2..512^2 px, "
                               "4/16/64 spp, depth 8, physical profile, one salty_render_batch per step",
                   "scenes": len(ss), "triangles": tris, "samples_per_step": samples,
                   "bvh_build_ms_total": build_ms, "setup_seconds": setup_s,
                   "tuning": tuned, "default_tuning": default, "autotune_seconds": tune_s,
                   "autotune_trial_ms": trial_ms},
        "batched": res["batched"], "per_scene": res["per_scene"],
        "speedup_vs_per_scene": res["batched"]["Mrays_s"] / res["per_scene"]["Mrays_s"],
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    for s in ss:
        s.close()
    ctx.close()


UNET_FWD_GFLOP_1080P = 305.0  # sum over the 14 convolutions of 2*9*cin*cout*pixels, 1 x 1088 x 1920


def run_denoise(args):
    """The learned denoiser against NLM (the C5 comparison): the held-out 1080p heightfield
    rendered at 4 spp; the film denoised whole by the U-Net (averaged over the 8 grid
    symmetries) and by NLM (21x21 search, 7x7 patch, variance-scaled); relMSE on the four
    128x128 windows of the time-to-RMSE measurement against FP64 65,536-spp renders of them,
    the reference's own noise subtracted.  value: the U-Net's relMSE (lower is better); timings are the
    synchronous calls on device-resident films (best of 3)."""
    import torch
    import salty_gb300
    from salty_gb300 import build as b
    from salty_gb300 import convergence as cv
    from salty_gb300 import denoiser as dn
    from salty_gb300 import scenes
    b.build()
    W, H, D, SPP = 1920, 1080, 12, 4
    ctx = salty_gb300.Context(0)
    s = scenes.upload(ctx, scenes.heightfield())
    s.build()
    ref = cv.reference_image(s, W, H, list(C3_WINDOWS), D, spp=65536)
    s.render(W, H, SPP, D, seed=4242, want=())
    film = s.read(W, H)
    # the network trained as configured (512 crops of 512^2 at 4 vs 4096 spp), and the
    # multi-level one the time-to-RMSE path uses below 1024 spp
    den = dn.Denoiser(ctx, weights=dn.C5_WEIGHTS, hq_weights=None)
    den_multi = dn.Denoiser(ctx, hq_weights=None)

    def best_of(fn, k=3):
        fn()
        torch.cuda.synchronize()
        t = float("inf")
        for _ in range(k):
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            t = min(t, time.perf_counter() - t0)
        return out, t * 1e3

    dev = torch.empty((H, W, 3), device="cuda")
    with ClockSampler(0) as clk:
        _, unet_ms = best_of(lambda: den.film(s, out=dev))
        unet = dev.cpu().numpy()
        den_multi.film(s, out=dev)
        torch.cuda.synchronize()
        unet_multi = dev.cpu().numpy()
        mean_d = torch.from_numpy(film["mean"]).cuda()
        var_d = torch.from_numpy(film["var"]).cuda()
        nlm_d = torch.empty_like(mean_d)
        _, nlm_ms = best_of(lambda: ctx.nlm(mean_d, var_d, 10, 3, 0.45, out=nlm_d))
        nlm = nlm_d.cpu().numpy()
    clocks = clk.summary()
    e = {"noisy": cv.corrected_rel_mse(film["mean"], ref),
         "nlm": cv.corrected_rel_mse(nlm, ref),
         "unet": cv.corrected_rel_mse(unet, ref),
         "unet_multilevel": cv.corrected_rel_mse(unet_multi, ref)}
    peaks = measured_peaks_tensor()
    mirrors = den.mirrors
    achieved = mirrors * UNET_FWD_GFLOP_1080P / unet_ms  # GFLOP/ms = TFLOP/s
    line = {
        "metric": "relMSE of the denoised 4-spp film (four 128x128 windows vs FP64 65,536 spp, reference noise "
                  "subtracted)",
        "value": e["unet"], "unit": "relMSE", "n_gpus": 1, "higher_is_better": False, "dtype": "bf16",
        "data": "synthetic (the held-out heightfield scene generated on the host; weights trained on "
                "renderer-generated pairs of other seeds)",
        "config": {"workload": "1920x1080 heightfield (seed 2026, held out), 4 spp, depth 12; U-Net over "
                               f"{mirrors} grid symmetries vs NLM 21x21/7x7", "windows": [list(c) for c in C3_WINDOWS],
                   "ref_spp": 65536, "ref_noise_rel_mse": ref["noise"]},
        "rel_mse": e, "unet_vs_nlm": e["nlm"] / e["unet"],
        "training": {k: v for k, v in den.meta.items() if k != "scenes"},
        "unet_ms_per_frame": unet_ms, "nlm_ms_per_frame": nlm_ms,
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": achieved / peaks["bf16_tflops"], "traffic": None,
                     "note": f"{mirrors} forward passes of {UNET_FWD_GFLOP_1080P} GFLOP each, over the whole "
                             "film denoise call (feature packing and output included)",
                     "peak_source": peaks["source"]},
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    den.close()
    den_multi.close()
    s.close()
    ctx.close()


def run_cornell(args):
    """The small Cornell box (36 triangles, area light) at 256 x 256, 16 spp, depth 8, Russian
    roulette from depth 3, the reference-compatible estimator, Reinhard to sRGB8 -- the
    configuration the reference renders on its CPU.  value: device time of the render calls
    (film already resident); e2e: the same call writing the sRGB8 image and the linear mean
    to host memory every step.  cpu_baseline: the oracle's compat renderer on the host cores,
    same scene, size and samples."""
    import torch
    import salty_gb300
    from salty_gb300 import build as b
    from salty_gb300 import scenes
    b.build()
    W, H, SPP, D = 256, 256, 16, 8
    ctx = salty_gb300.Context(0)
    c = scenes.cornell("baseline")
    s = scenes.upload(ctx, c)
    s.build()
    kw = dict(profile=salty_gb300.PROFILE_COMPAT, tonemap=salty_gb300.TM_REINHARD)
    for i in range(args.warmup):
        s.render(W, H, SPP, D, seed=1 + i, want=(), **kw)
    torch.cuda.synchronize()
    dev_ms, rays, paths = 0.0, 0, 0
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            r = s.render(W, H, SPP, D, seed=100 + i, want=(), **kw)
            dev_ms += r["ms"]
            rays += r["rays"]
            paths += r["paths"]
        wall = time.perf_counter() - t0
        t0 = time.perf_counter()
        e2e_rays = 0
        for i in range(args.steps):
            r = s.render(W, H, SPP, D, seed=200 + i, want=("mean", "srgb"), **kw)
            e2e_rays += r["rays"]
        e2e_wall = time.perf_counter() - t0
    clocks = clk.summary()
    line = {
        "metric": METRIC, "value": rays / dev_ms / 1e3, "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (the Cornell box scene generated on the host)",
        "config": {"workload": "Cornell box (36 triangles), 256x256, 16 spp, depth 8, RR from 3, compat profile, "
                               "Reinhard sRGB8", "rays_per_step": rays // args.steps,
                   "paths_per_step": paths // args.steps, "wall_ms_per_step": wall * 1e3 / args.steps,
                   "l2": "scene and film fit in L2 (the workload is this small)"},
        "e2e": {"value": e2e_rays / e2e_wall / 1e6, "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": W * H * (3 + 12)},
        "clocks": clocks,
    }
    if not args.no_cpu:
        from oracle.oracle import PROFILE_COMPAT, Oracle, SceneData, build
        build(with_reference=False)
        o = Oracle()
        sd = SceneData(c["tri_pos"], c["tri_nrm"], c["tri_mat"], c["materials"], c["light"], None, c["sky"],
                       c["camera"])
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        o.render(sd, W, H, SPP, D, profile=PROFILE_COMPAT, seed=1, nthreads=cores)
        secs = time.perf_counter() - t0
        # the port traces the same number of rays per path on average as the device renderer
        line["cpu_baseline"] = {"value": rays / args.steps / secs / 1e6, "unit": "Mrays/s", "cores": cores,
                                "kind": "port", "sample": f"the whole workload, one frame ({secs:.2f} s); rays "
                                                          "counted as the device renderer's per frame"}
    print(json.dumps(line), flush=True)
    s.close()
    ctx.close()


# ---------------------------------------------------------------- profiling workloads
# Small fixed workloads to time alone or to run under ncu: `bench.py --workload NAME`
# prints one JSON line of timings (render, unet, trace-sweep, wave-sweep, nlm, tonemap,
# prof-cornell).


def fp32_nominal_tflops() -> float:
    """SMs x 128 FP32 lanes x 2 flops (a fused multiply-add) x the maximum SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = 2070.0
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    return sms * 128 * 2 * mhz * 1e6 / 1e12


def prof_render(spp: int, frames: int, width: int = 1920, height: int = 1080) -> dict:
    """The 1080p heightfield: `frames` renders of `spp` samples, depth 12, default launch
    shapes; device time and rays per frame."""
    from salty_gb300 import Context, scenes
    ctx = Context(0)
    s = scenes.upload(ctx, scenes.heightfield())
    info = s.build()
    out = []
    for i in range(frames):
        r = s.render(width, height, spp, 12, seed=3 + i, want=())
        out.append({"ms": r["ms"], "rays": r["rays"], "paths": r["paths"], "Mrays_s": r["rays"] / r["ms"] / 1e3})
    return {"workload": f"{width}x{height} heightfield, {spp} spp x {frames} frames", "bvh_build_ms": info["build_ms"],
            "frames": out}


def prof_wave_sweep(spp: int) -> dict:
    """The 1080p heightfield at `spp` samples, depth 12, default launch shapes, for queues of
    2^20 .. 2^27 paths in flight: best of two renders each after an 8-spp warm-up."""
    from salty_gb300 import Context, scenes
    ctx = Context(0)
    s = scenes.upload(ctx, scenes.heightfield())
    s.build()
    base = ctx.tuning
    res = []
    for e in range(20, 28):
        t = dict(base)
        t["wave_paths"] = 1 << e
        ctx.tuning = t
        s.render(1920, 1080, 8, 12, seed=1, want=())
        best = min((s.render(1920, 1080, spp, 12, seed=2 + i, want=()) for i in range(2)), key=lambda r: r["ms"])
        res.append({"wave_paths": 1 << e, "ms": best["ms"], "Mrays_s": best["rays"] / best["ms"] / 1e3,
                    "Mpaths_s": best["paths"] / best["ms"] / 1e3})
    return {"workload": f"1920x1080 heightfield, {spp} spp, depth 12, default launch shapes", "waves": res}


def prof_tonemap() -> dict:
    """salty_tonemap_noalloc (Reinhard, linear + sRGB8 outputs) on device-resident images,
    timed with CUDA events on the caller's stream, a torch stream of its own (a NULL stream
    would mean the library's stream, which torch's events do not see); mean of 20 calls after
    3 warm-ups.
    Algorithmic bytes per pixel: 12 read for the log-average, 12 read + 12 written + 3
    written for the map = 39."""
    import ctypes as C
    import torch
    from salty_gb300 import lib, TM_REINHARD
    from salty_gb300 import Context
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


def prof_nlm(h: int, w: int) -> dict:
    """salty_denoise_nlm (21x21 search, 7x7 patch) on a w x h device-resident image: the
    best of 5 host-timed synchronous calls, against the nominal FP32 peak (SMs x 128 lanes x
    2 flops x the maximum SM clock).  Algorithmic work of the filter: 441 offsets x 49 taps
    x 3 channels x 3 flops (difference, square, sum) = 194,481 FP32 flops per pixel."""
    import torch
    from salty_gb300 import Context
    ctx = Context(0)
    peak = fp32_nominal_tflops()
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
            "fp32_peak_tflops": peak, "peak_source": "nominal", "frac": ach / peak}


def prof_unet(n: int, h: int, w: int, conv: str = "tcgen05", train: bool = False) -> dict:
    """Forward passes (and, with train, training steps at lr 0) on random features: the
    best of 5 wall-clock times after a warm-up, per convolution kernel."""
    import torch
    from salty_gb300 import CONV_MMA_SYNC, CONV_TCGEN05, CONV_TCGEN05_CP_ASYNC, UNET_FEATURES, Unet
    from salty_gb300 import Context
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


def prof_trace_sweep() -> dict:
    """Every traversal launch shape (block x registers x pool x postpone) on the microbenchmark
    (1M triangles, 16,777,216 rays, closest hit): kernel time, and whether the hits are the
    same as the first shape's."""
    import torch
    from salty_gb300 import Context
    ctx = Context(0)
    from salty_gb300 import microbench_rays, microbench_soup
    sc = ctx.upload_scene(microbench_soup(20260001, 1_000_000))
    sc.build()
    n = 16_777_216
    rays = torch.from_numpy(microbench_rays(20260002, n, 1e-4)).cuda()
    hits = torch.empty((n, 4), device="cuda")
    ref, res = None, []
    for blk, regs, pool, post in itertools.product((64, 128, 256), (64, 56), (64, 128, 256), (1, 4, 7, 10)):
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


PROFILING = ("render", "unet", "trace-sweep", "wave-sweep", "nlm", "tonemap")


def run_profiling(args) -> None:
    from salty_gb300 import build as b
    b.build()
    w = args.workload
    if w == "render":
        r = prof_render(args.spp or 1, args.frames, args.width, args.height)
    elif w == "unet":
        r = prof_unet(args.unet_n, args.unet_h, args.unet_w, args.conv, args.train)
    elif w == "trace-sweep":
        r = prof_trace_sweep()
    elif w == "wave-sweep":
        r = prof_wave_sweep(args.spp or 64)
    elif w == "nlm":
        r = prof_nlm(args.height, args.width)
    else:
        r = prof_tonemap()
    print(json.dumps(r), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--any-hit", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="rays per step (smaller cases for profiling)")
    ap.add_argument("--trace-shape", default="", help="block,regs,pool,postpone instead of salty_autotune_trace")
    ap.add_argument("--workload", default="traversal",
                    choices=["traversal", "time-to-rmse", "batch", "cornell", "denoise", *PROFILING])
    ap.add_argument("--scenes", type=int, default=256, help="batch: number of scenes")
    ap.add_argument("--target", type=float, default=0.01, help="time-to-rmse: relRMSE target")
    ap.add_argument("--ref-spp", type=int, default=1 << 20, help="time-to-rmse: samples of the FP64 reference")
    ap.add_argument("--sun-half-angle", type=float, default=0.0,
                    help="time-to-rmse: the sun's angular radius in radians (0: directional, as configured)")
    ap.add_argument("--no-c3", action="store_true", help="skip the 1080p heightfield measurement of the "
                                                        "default run")
    ap.add_argument("--max-spp", type=int, default=1 << 17, help="time-to-rmse: give up beyond this")
    ap.add_argument("--methods", default="plain,unet", help="time-to-rmse: plain,unet (U-Net: the chosen path),nlm")
    ap.add_argument("--spp", type=int, default=None, help="render: 1, wave-sweep: 64")
    ap.add_argument("--frames", type=int, default=2, help="render: frames")
    ap.add_argument("--width", type=int, default=1920, help="render, nlm: image width")
    ap.add_argument("--height", type=int, default=1080, help="render, nlm: image height")
    ap.add_argument("--unet-n", type=int, default=1, help="unet: images per batch")
    ap.add_argument("--unet-h", type=int, default=1088, help="unet: image height (multiple of 16)")
    ap.add_argument("--unet-w", type=int, default=1920, help="unet: image width (multiple of 16)")
    ap.add_argument("--conv", default="tcgen05", choices=["tcgen05", "tcgen05_cp_async", "mma_sync", "all"])
    ap.add_argument("--train", action="store_true", help="unet: also time training steps")
    args = ap.parse_args()
    if args.workload in PROFILING:
        run_profiling(args)
        return
    if args.workload == "time-to-rmse":
        run_time_to_rmse(args)
        return
    if args.workload == "batch":
        run_batch(args)
        return
    if args.workload == "cornell":
        run_cornell(args)
        return
    if args.workload == "denoise":
        run_denoise(args)
        return
    n_rays = args.rays
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    ws, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank, local, pg)
        return

    import torch
    import salty_gb300
    from salty_gb300 import build as b
    b.build()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = salty_gb300.Context(local)
    tris = salty_gb300.microbench_soup(SOUP_SEED, N_TRIS)
    scene = ctx.upload_scene(tris)
    info = scene.build()
    rays_h = ctx.pinned((n_rays, 8), np.float32)
    salty_gb300.microbench_rays(RAY_SEED, n_rays, TMIN, out=rays_h)
    hits_h = ctx.pinned((n_rays, 4), np.float32)
    d_rays = torch.from_numpy(rays_h).to(dev)
    d_hits = torch.empty((n_rays, 4), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()  # the library runs on its own stream
    any_hit = args.any_hit

    # launch shape for this workload: salty_autotune_trace (untimed), or given
    default_tuning = ctx.tuning
    if args.trace_shape:
        b_, r_, p_, q_ = (int(x) for x in args.trace_shape.split(","))
        ctx.tuning = {"trace_block": b_, "trace_regs": r_, "trace_pool": p_, "trace_postpone": q_}
        tuning = ctx.tuning
    else:
        tuning, tune_ms = scene.autotune_trace(d_rays, any_hit=any_hit)

    # fetch counts (untimed): algorithmic bytes per ray
    st = scene.trace_raw(d_rays, d_hits, any_hit=any_hit, counters=True)
    n_node = st["node_fetches"] / n_rays
    n_tri = st["tri_fetches"] / n_rays
    bytes_per_ray = 32 + 16 + 80 * n_node + 48 * n_tri

    # ---- device-resident steps
    for _ in range(args.warmup):
        scene.trace_raw(d_rays, d_hits, any_hit=any_hit)
    barrier(pg)
    torch.cuda.synchronize()
    kernel_ms = 0.0
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            s = scene.trace_raw(d_rays, d_hits, any_hit=any_hit)
            kernel_ms += s["kernel_ms"]
        e1.record()
        torch.cuda.synchronize()
    barrier(pg)
    region_ms = e0.elapsed_time(e1)
    region_ms = max_over_ranks(pg, region_ms, dev)
    clocks = clk.summary()
    value = ws * n_rays * args.steps / (region_ms / 1e3) / 1e6
    launch_ms = kernel_ms / args.steps

    # ---- end to end: pinned host rays in, host hits out, every step
    for _ in range(args.warmup):
        scene.trace_raw(rays_h, hits_h, any_hit=any_hit)
    barrier(pg)
    torch.cuda.synchronize()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record()
    h2d = d2h = 0
    e2e_kernels = 0
    for _ in range(args.steps):
        s = scene.trace_raw(rays_h, hits_h, any_hit=any_hit)
        h2d, d2h = s["h2d_bytes"], s["d2h_bytes"]
        e2e_kernels += s["launches"]
    e3.record()
    torch.cuda.synchronize()
    barrier(pg)
    e2e_ms = max_over_ranks(pg, e2.elapsed_time(e3), dev)
    e2e_value = ws * n_rays * args.steps / (e2e_ms / 1e3) / 1e6

    # check: the last device step's hits equal the host path's, bit for bit (a miss stores
    # id -1, whose float bit pattern is a NaN, so compare the raw words)
    same = bool(np.array_equal(d_hits.cpu().numpy().view(np.int32), hits_h.view(np.int32)))

    # ---- any-hit (occlusion) queries of the same rays, device-resident, same launch shape
    anyhit = None
    if not any_hit:
        for _ in range(args.warmup):
            scene.trace_raw(d_rays, d_hits, any_hit=True)
        barrier(pg)
        torch.cuda.synchronize()
        a_kernel = 0.0
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record()
        for _ in range(args.steps):
            a_kernel += scene.trace_raw(d_rays, d_hits, any_hit=True)["kernel_ms"]
        e5.record()
        torch.cuda.synchronize()
        barrier(pg)
        a_ms = max_over_ranks(pg, e4.elapsed_time(e5), dev)
        occluded = int((d_hits[:, 1].view(torch.int32) >= 0).sum().item())
        anyhit = {"value": ws * n_rays * args.steps / (a_ms / 1e3) / 1e6, "unit": "Mrays/s",
                  "ms_per_step": a_ms / args.steps, "kernel_ms": a_kernel / args.steps,
                  "occluded_fraction": occluded / n_rays}

    peaks = measured_peaks()
    achieved = bytes_per_ray * n_rays / (launch_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": region_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded PCG soup and rays, generated on the host)",
        "config": {"workload": f"traversal microbenchmark: 1M-triangle soup, {n_rays:,} rays, "
                               + ("any hit" if any_hit else "closest hit"),
                   "n_tris": N_TRIS, "rays_per_step": n_rays, "bvh": "device 32-bin SAH -> 8-wide, 8-bit planes",
                   "bvh_nodes": info["n_nodes"], "bvh_depth": info["depth"], "bvh_build_ms": info["build_ms"],
                   "sah_cost": info["sah_cost"], "triangle_test": "reference-compatible (bit-exact ids)",
                   "l2": "inputs larger than L2 (rays 512 MiB, hits 256 MiB); BVH resident",
                   "tuning": tuning, "default_tuning": default_tuning,
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": args.steps + e2e_kernels,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"],
                     "traffic": None if any_hit else NCU_DRAM_BYTES_PER_RAY * n_rays,
                     "traffic_source": "ncu dram bytes per ray at 4,194,304 rays, scaled to the launch",
                     "peak_source": peaks["source"], "kernel_ms": launch_ms,
                     "bytes_per_ray": bytes_per_ray, "node_fetches_per_ray": n_node, "tri_fetches_per_ray": n_tri},
        "clocks": clocks,
        "host_device_hits_equal": same,
        "any_hit": anyhit,
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        sample = CPU_SAMPLE
        cps, cores, secs, build_s = cpu_reference_rays_per_s(tris, rays_h[:sample].copy())
        line["cpu_baseline"] = {"value": cps / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
                                "sample": f"first {sample} rays of the same stream, same 1M triangles "
                                          f"({secs:.1f} s on {cores} threads; BVH build {build_s:.1f} s)",
                                "implementation": REFERENCE_NOTE}
    scene.close()
    ctx.close()
    del d_rays, d_hits
    if rank == 0 and ws == 1 and not args.no_c3 and not any_hit:
        c3 = measure_c3(args)
        line["render_c3"] = c3["render_c3"]
        line["time_to_rmse"] = {k: v for k, v in c3.items() if k != "render_c3"}
        line["gpu_launches_note"] = "gpu_launches counts the traversal steps only (the C3 keys run after them)"
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
