"""The trained U-Net against NLM (its fallback) on a scene it has not seen.

The committed weights (salty_gb300/weights/unet_heightfield.npz) were trained by
`python -m salty_gb300.denoiser train` on renderer-generated pairs of heightfield scenes
with seeds 1..16; the held-out scene is the 1080p benchmark heightfield (seed 2026).
Errors are relMSE against a 4096-spp FP64 render of a 256x256 window, minus the
reference's own noise (salty_gb300.convergence)."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H, DEPTH = 1920, 1080, 12
CROP = (832, 412, 256, 256)


@pytest.fixture(scope="module")
def held_out(ctx):
    from salty_gb300 import scenes
    s = scenes.upload(ctx, scenes.heightfield())
    s.build()
    yield s
    s.close()


@pytest.fixture(scope="module")
def ref(held_out):
    from salty_gb300 import convergence as cv
    return cv.reference_image(held_out, W, H, CROP, DEPTH, spp=4096)


@pytest.fixture(scope="module")
def denoiser(ctx):
    from salty_gb300 import denoiser as dn
    d = dn.Denoiser(ctx)
    yield d
    d.close()


def test_weights_are_trained_and_exclude_the_held_out_scene(denoiser):
    assert denoiser.method == "unet"
    assert 2026 not in denoiser.meta["scenes"] and denoiser.meta["steps"] > 0


@pytest.mark.parametrize("spp", [4, 256])
def test_unet_beats_nlm_on_held_out_scene(ctx, held_out, ref, denoiser, spp):
    from salty_gb300 import convergence as cv
    r = held_out.render(W, H, spp, DEPTH, seed=4242 + spp, want=("mean", "var"), crop=CROP)
    aov = held_out.aov(CROP[2], CROP[3])
    e_noisy = cv.corrected_rel_mse(r["mean"], ref)
    e_nlm = cv.corrected_rel_mse(ctx.nlm(r["mean"], r["var"], 10, 3, 0.45), ref)
    e_unet = cv.corrected_rel_mse(denoiser(r["mean"], r["var"], aov), ref)
    print(json.dumps({"spp": spp, "noisy": e_noisy, "nlm": e_nlm, "unet": e_unet}))
    assert e_nlm < e_noisy
    assert e_unet < 0.5 * e_nlm, (e_unet, e_nlm)


def test_film_denoise_matches_host_features(ctx, held_out, denoiser):
    r = held_out.render(W, H, 16, DEPTH, seed=5, want=("mean", "var"), crop=(100, 40, 200, 120))
    aov = held_out.aov(200, 120)
    host = denoiser(r["mean"], r["var"], aov)       # features packed on the host, borders reflected
    film = denoiser.net.denoise_film(held_out)       # the same, packed on the device
    assert film.shape == (120, 200, 3)
    np.testing.assert_allclose(film, host, rtol=2e-2, atol=1e-3)
    assert np.mean(np.abs(film - host) > 1e-6) < 0.01


def test_nlm_is_the_fallback(ctx, held_out):
    from salty_gb300 import denoiser as dn
    d = dn.Denoiser(ctx, weights=None)
    assert d.method == "nlm"
    r = held_out.render(W, H, 8, DEPTH, seed=6, want=("mean", "var"), crop=(0, 0, 64, 48))
    np.testing.assert_array_equal(d(r["mean"], r["var"]), ctx.nlm(r["mean"], r["var"], 10, 3, 0.45))


def test_self_ensemble(ctx, held_out, ref, denoiser):
    """Averaging the network over the frame's mirror images: one mirror is the plain film
    denoise, four lower the error on the held-out window."""
    from salty_gb300 import convergence as cv
    held_out.render(W, H, 256, DEPTH, seed=99, want=(), crop=CROP)
    one = denoiser.net.denoise_film(held_out)
    np.testing.assert_array_equal(denoiser.net.denoise_film(held_out, mirrors=1), one)
    four = denoiser.net.denoise_film(held_out, mirrors=4)
    eight = denoiser.net.denoise_film(held_out, mirrors=8)
    assert np.all(np.isfinite(four)) and np.all(np.isfinite(eight))
    e1, e4, e8 = (cv.corrected_rel_mse(x, ref) for x in (one, four, eight))
    print(json.dumps({"single": e1, "ensemble4": e4, "ensemble8": e8}))
    assert e4 < e1 and e8 < e1


def test_ensemble_over_all_grid_symmetries(ctx, held_out, denoiser):
    """mirrors=8 averages the network over the 8 symmetries of the pixel grid (the four
    mirror images and their transposes).  On a non-square 200 x 120 window (padded to
    208 x 128, transposed 128 x 208) it equals the same average computed from host-packed
    features, up to the host/device feature rounding the single-pass test allows."""
    from salty_gb300 import unet_features
    from salty_gb300.denoiser import _pad16
    r = held_out.render(W, H, 16, DEPTH, seed=7, want=("mean", "var"), crop=(100, 40, 200, 120))
    aov = held_out.aov(200, 120)
    net = denoiser.pick(16)
    feat = unet_features(r["mean"], r["var"], aov)
    host = np.zeros((120, 200, 3), np.float32)
    for k in range(8):
        g = feat[:, ::-1] if k & 1 else feat
        g = g[::-1] if k & 2 else g
        g = _pad16(np.ascontiguousarray(g))
        if k & 4:
            g = np.ascontiguousarray(g.transpose(1, 0, 2))
        o = net.forward(g)
        if k & 4:
            o = o.transpose(1, 0, 2)
        o = o[:120, :200]
        o = o[::-1] if k & 2 else o
        o = o[:, ::-1] if k & 1 else o
        host += o / 8
    film = net.denoise_film(held_out, mirrors=8)
    assert film.shape == (120, 200, 3)
    np.testing.assert_allclose(film, host, rtol=2e-2, atol=1e-3)
    assert np.mean(np.abs(film - host) > 1e-5) < 0.02
    with pytest.raises(Exception):
        net.denoise_film(held_out, mirrors=3)
