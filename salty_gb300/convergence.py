"""Time-to-RMSE measurement: plain progressive rendering vs denoised paths.

Error metric (relative MSE, used throughout the denoising literature):
    relMSE = mean over pixels and channels of (x - r)^2 / (r^2 + 0.01),  relRMSE = sqrt(relMSE)
where r is the converged image: an FP64-accumulated render at many samples per pixel
(65,536 or more).  At 1080p that reference would cost ~1.4e11 camera paths or more, so it
is rendered for a few windows (crops) of the frame; the windows' pixels keep their
full-frame rays, so the methods render the whole frame and are scored on the windows.

The reference is itself a Monte Carlo estimate: against it, an image's measured relMSE is
its true relMSE plus the reference's own, E = mean(var_r / (r^2 + 0.01)) with var_r the
variance of the reference's mean (independent samples).  Every error reported here is the
measured relMSE minus E (an unbiased estimate of the error against the exact image), and E
is reported beside it; with 2^20 reference samples E is a few percent of the 1e-4 target.

A method's time to reach a target relRMSE is measured with a doubling sample schedule:
the frame is rendered progressively (each pass doubles the samples), after each pass the
method's image is formed on the device and scored, and the time at which the curve crosses
the target is interpolated in log(error) against time between the two passes that bracket
it.  Times are host wall-clock around the synchronous library calls of each pass (render
plus the method's own post-processing), excluding the scoring read-back.
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import PROFILE_PHYSICAL


def rel_mse(x: np.ndarray, ref: np.ndarray) -> float:
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.mean((x - ref) ** 2 / (ref * ref + 1e-2)))


def rel_rmse(x: np.ndarray, ref: np.ndarray) -> float:
    return math.sqrt(rel_mse(x, ref))


def reference_image(scene, width: int, height: int, crops, max_depth: int, spp: int = 65536,
                    chunk: int = 4096, seed: int = 987654321, rr_depth: int = 3) -> dict:
    """FP64-accumulated windows of the frame at `spp` samples each: {"mean", "var" (of the
    mean), lists with one array per window, "noise" (the relMSE its own noise adds, E above,
    over all windows' pixels), "spp", "seconds", "crops"}.  `crops` is one (x, y, w, h)
    window or a list of them."""
    crops = [tuple(crops)] if isinstance(crops[0], int) else [tuple(c) for c in crops]
    t0 = time.perf_counter()
    means, vars_ = [], []
    for crop in crops:
        done = 0
        out = None
        while done < spp:
            k = min(chunk, spp - done)
            out = scene.render(width, height, k, max_depth, rr_depth=rr_depth, profile=PROFILE_PHYSICAL, seed=seed,
                               accumulate=done > 0, fp64=True, want=("mean", "var"), crop=crop)
            done += k
        means.append(out["mean"])
        vars_.append(out["var"])
    m = np.concatenate([a.reshape(-1, 3) for a in means]).astype(np.float64)
    v = np.concatenate([a.reshape(-1, 3) for a in vars_]).astype(np.float64)
    return {"mean": means, "var": vars_, "noise": float(np.mean(v / (m * m + 1e-2))), "spp": spp,
            "seconds": time.perf_counter() - t0, "crops": crops}


def corrected_rel_mse(x, ref: dict) -> float:
    """relMSE against the exact image, estimated as measured minus the reference's noise.
    x: a list of window images, one window image, or the full frame (its windows are then
    cut out here)."""
    means = ref["mean"] if isinstance(ref["mean"], (list, tuple)) else [ref["mean"]]
    crops = ref.get("crops")
    if not isinstance(x, (list, tuple)):
        whole_window = len(means) == 1 and np.shape(x)[:2] == np.shape(means[0])[:2]
        x = [crop_of(x, c) for c in crops] if crops and not whole_window else [x]
    xs = np.concatenate([np.asarray(a, np.float64).reshape(-1, 3) for a in x])
    rs = np.concatenate([np.asarray(a, np.float64).reshape(-1, 3) for a in means])
    return rel_mse(xs, rs) - ref["noise"]


def crop_of(img, crop: tuple):
    x, y, w, h = crop
    return img[y:y + h, x:x + w]


def converge(scene, width: int, height: int, ref: dict, max_depth: int, target: float,
             method: str = "plain", ctx=None, denoiser=None, spp0: int = 4, max_spp: int = 1 << 16, seed: int = 1,
             rr_depth: int = 3, nlm_k: float = 0.45) -> dict:
    """Progressive full-frame rendering with doubling spp until the method's image reaches
    relRMSE <= target on the reference's windows.  method: "plain" (the film mean), "nlm" (salty_denoise_nlm
    of mean and variance) or "unet" (salty_denoise_unet of the film through `denoiser`, a
    salty_gb300.denoiser.Denoiser, which picks its network by the film's samples)."""
    import torch
    dev = torch.device("cuda")
    mean = torch.empty((height, width, 3), dtype=torch.float32, device=dev)
    var = torch.empty_like(mean)
    img = torch.empty_like(mean)
    curve = []
    spent = 0.0
    total = 0
    step = spp0
    target_mse = target * target
    while total < max_spp:
        step = min(step, max_spp - total)
        t0 = time.perf_counter()
        if method == "plain":
            scene.render(width, height, step, max_depth, rr_depth=rr_depth, profile=PROFILE_PHYSICAL, seed=seed,
                         accumulate=total > 0, want=("mean",), out={"mean": mean})
            out = mean
        elif method == "nlm":
            scene.render(width, height, step, max_depth, rr_depth=rr_depth, profile=PROFILE_PHYSICAL, seed=seed,
                         accumulate=total > 0, want=("mean", "var"), out={"mean": mean, "var": var})
            ctx.nlm(mean, var, 10, 3, nlm_k, out=img)
            out = img
        elif method == "unet":
            scene.render(width, height, step, max_depth, rr_depth=rr_depth, profile=PROFILE_PHYSICAL, seed=seed,
                         accumulate=total > 0, want=())
            denoiser.film(scene, out=img)
            out = img
        else:
            raise ValueError(f"unknown method {method}")
        torch.cuda.synchronize()
        spent += time.perf_counter() - t0
        total += step
        err = corrected_rel_mse([crop_of(out, c).cpu().numpy() for c in ref["crops"]], ref)
        curve.append({"spp": total, "seconds": spent, "rel_mse": err})
        if err <= target_mse:
            break
        step = total  # doubles the film each pass
    hit = next((i for i, c in enumerate(curve) if c["rel_mse"] <= target_mse), None)
    if hit is None:
        t_target = None
    elif hit == 0:
        t_target = curve[0]["seconds"]
    else:
        a, b = curve[hit - 1], curve[hit]
        la = math.log(max(a["rel_mse"], 1e-30))
        lb = math.log(max(b["rel_mse"], 1e-30))
        lt = math.log(target_mse)
        f = (la - lt) / (la - lb) if la != lb else 1.0
        t_target = a["seconds"] + f * (b["seconds"] - a["seconds"])
    return {"method": method, "curve": curve, "seconds_to_target": t_target, "target": target,
            "ref_noise": ref["noise"]}
