"""Parity of the tonemapping and NLM kernels with the reference and the oracle."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_tonemap_matches_reference(ctx, kind):
    """Same per-pixel arithmetic; the log-average is summed in double on the GPU where the
    reference adds floats one by one, so outputs agree to a few ulps of the key."""
    g = np.load(os.path.join(GOLDEN, "tonemap_ref.npz"))
    out, _, _, _ = ctx.tonemap(g["img"], kind, srgb=False)
    np.testing.assert_allclose(out, g[f"tm{kind}"], rtol=2e-5, atol=1e-7)


def test_srgb8_matches_reference_capture_png(ctx):
    """PathTracer::Capture: ACES, clamp, the reference OETF, x*255+0.5 -- within 1 LSB."""
    g = np.load(os.path.join(GOLDEN, "tonemap_ref.npz"))
    _, s8, _, _ = ctx.tonemap(g["img"], 2, srgb=True, ref_oetf=True)
    d = np.abs(s8.astype(int) - g["srgb_aces_ref"].astype(int))
    assert d.max() <= 1 and (d > 0).mean() < 0.01


def test_tonemap_large_image_matches_oracle(ctx, oracle):
    rng = np.random.default_rng(8)
    img = np.exp(rng.normal(0.0, 2.0, size=(540, 960, 3))).astype(np.float32)
    for kind in (0, 1, 2):
        out, _, ave, mx = ctx.tonemap(img, kind, srgb=False)
        o, oave, omx = oracle.tonemap(kind, img)
        assert mx == omx
        assert abs(ave / oave - 1) < 1e-4
        np.testing.assert_allclose(out, o, rtol=2e-4, atol=1e-6)


def test_nlm_ref_matches_reference(ctx):
    g = np.load(os.path.join(GOLDEN, "nlm_ref.npz"))
    out = ctx.nlm_ref(g["rgba"], float(g["coeff"]))
    np.testing.assert_allclose(out, g["out"], rtol=1e-5, atol=1e-6)


def test_nlm_ref_larger_image_matches_oracle(ctx, oracle):
    rng = np.random.default_rng(9)
    rgba = rng.random((70, 90, 4), dtype=np.float32)
    out = ctx.nlm_ref(rgba, 0.15)
    np.testing.assert_allclose(out, oracle.nlm_ref(rgba, 0.15), rtol=1e-5, atol=1e-6)


def test_variance_nlm_matches_oracle(ctx, oracle):
    rng = np.random.default_rng(10)
    clean = np.tile(np.linspace(0.1, 1.0, 64, dtype=np.float32)[None, :, None], (48, 1, 3))
    var = np.full_like(clean, 0.01)
    noisy = clean + rng.normal(0, 0.1, clean.shape).astype(np.float32)
    out = ctx.nlm(noisy, var, search_r=10, patch_r=3, k=0.45)
    ref = oracle.nlm_var(noisy, var, 10, 3, 0.45)
    np.testing.assert_allclose(out, ref, rtol=1e-4, atol=1e-5)
    assert np.mean((out - clean) ** 2) < 0.5 * np.mean((noisy - clean) ** 2)


@pytest.mark.parametrize("ref_oetf", [True, False])
def test_srgb8_equals_the_exact_oetf_of_the_linear_output(ctx, ref_oetf):
    """The sRGB8 encode takes the power from the hardware approximation and falls back to
    powf only near a code boundary: every code must equal the all-powf formula applied to
    the linear output (torch's CUDA pow is powf; the same IEEE operations in the same
    order), here on 12.6M values covering every code the curve reaches (the reference's OETF
    tops out at 1.055^(1/2.4) - 0.055, code 247)."""
    import torch
    rng = np.random.default_rng(21)
    img = np.exp(rng.normal(0.0, 2.0, size=(1024, 4096, 3))).astype(np.float32)
    out, s8, _, _ = ctx.tonemap(img, 0, srgb=True, ref_oetf=ref_oetf)
    y = torch.from_numpy(out).cuda().clamp(0.0, 1.0)
    e = torch.tensor(np.float32(1.0) / np.float32(2.4), device="cuda")
    lin = y <= np.float32(0.0031308)
    if ref_oetf:
        v = torch.pow(y * np.float32(1.055), e) - np.float32(0.055)
    else:
        v = torch.pow(y, e) * np.float32(1.055) - np.float32(0.055)
    v = torch.where(lin, y * np.float32(12.92), v)
    want = (v * np.float32(255.0) + np.float32(0.5)).to(torch.uint8).cpu().numpy()
    assert len(np.unique(want)) == (248 if ref_oetf else 256)
    np.testing.assert_array_equal(s8, want)
