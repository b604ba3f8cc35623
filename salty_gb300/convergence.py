"""Time-to-RMSE measurement: plain progressive rendering vs a denoised path.

Error metric (relative MSE, used throughout the denoising literature):
    relMSE = mean over pixels and channels of (x - r)^2 / (r^2 + 0.01),  relRMSE = sqrt(relMSE)
where r is the converged image: an FP64-accumulated render at 65,536 samples per pixel.
At 1080p that reference would cost ~1.4e11 camera paths, so it is rendered for a window
(crop) of the frame; the window's pixels keep their full-frame rays, so the methods render
the whole frame and are scored on the window.

A method's time to reach a target relRMSE is measured with a doubling sample schedule:
the frame is rendered progressively (each pass doubles the samples), after each pass the
method's image is scored, and the time at which the curve crosses the target is
interpolated in log(error) against time between the two passes that bracket it.  Times are
host wall-clock around the library calls (which are synchronous), excluding scoring.
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


def reference_image(scene, width: int, height: int, crop: tuple, max_depth: int, spp: int = 65536,
                    chunk: int = 2048, seed: int = 987654321, rr_depth: int = 3) -> tuple[np.ndarray, float]:
    """FP64-accumulated mean of the crop window at `spp` samples; returns (image, seconds)."""
    t0 = time.perf_counter()
    done = 0
    out = None
    while done < spp:
        k = min(chunk, spp - done)
        out = scene.render(width, height, k, max_depth, rr_depth=rr_depth, profile=PROFILE_PHYSICAL, seed=seed,
                           accumulate=done > 0, fp64=True, want=("mean",), crop=crop)
        done += k
    return out["mean"], time.perf_counter() - t0


def crop_of(img: np.ndarray, crop: tuple) -> np.ndarray:
    x, y, w, h = crop
    return img[y:y + h, x:x + w]


def converge(scene, width: int, height: int, crop: tuple, ref: np.ndarray, max_depth: int, target: float,
             denoise=None, spp0: int = 4, max_spp: int = 1 << 16, seed: int = 1, rr_depth: int = 3) -> dict:
    """Progressive full-frame rendering with doubling spp; denoise(mean, var) -> image (or None
    for the plain path).  Returns the error curve and the interpolated time to `target`."""
    curve = []
    spent = 0.0
    total = 0
    step = spp0
    while total < max_spp:
        t0 = time.perf_counter()
        r = scene.render(width, height, step, max_depth, rr_depth=rr_depth, profile=PROFILE_PHYSICAL, seed=seed,
                         accumulate=total > 0, want=("mean", "var") if denoise else ("mean",))
        img = denoise(r["mean"], r["var"]) if denoise else r["mean"]
        spent += time.perf_counter() - t0
        total += step
        err = rel_rmse(crop_of(img, crop), ref)
        curve.append({"spp": total, "seconds": spent, "rel_rmse": err})
        if err <= target:
            break
        step = total  # doubles the film each pass
    hit = next((i for i, c in enumerate(curve) if c["rel_rmse"] <= target), None)
    if hit is None:
        t_target = None
    elif hit == 0:
        t_target = curve[0]["seconds"]
    else:
        a, b = curve[hit - 1], curve[hit]
        la, lb, lt = math.log(a["rel_rmse"]), math.log(b["rel_rmse"]), math.log(target)
        f = (la - lt) / (la - lb) if la != lb else 1.0
        t_target = a["seconds"] + f * (b["seconds"] - a["seconds"])
    return {"curve": curve, "seconds_to_target": t_target, "target": target}
