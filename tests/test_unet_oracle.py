"""Pins of the learned denoiser's oracle (oracle/unet_oracle.py) on the CPU.

The reference has no learned denoiser, so the oracle is pinned by (1) its BF16 rounding
against torch's, (2) its convolution pieces against torch's conv2d and autograd in float64,
and (3) its hand-written backward pass against central finite differences of its own loss.
"""
import numpy as np
import pytest
import torch

from oracle.unet_oracle import LAYERS, UnetOracle, bf16_round, param_count, split_params


def _init(seed):
    rng = np.random.default_rng(seed)
    ps = []
    for ci, co, relu in LAYERS:
        bound = np.sqrt(6.0 / (9 * ci))
        ps.append(rng.uniform(-bound, bound, 9 * co * ci))
        ps.append(rng.uniform(-0.05, 0.05, co))
    return np.concatenate(ps)


def _features(rng, n, h, w):
    f = np.empty((n, h, w, 11), np.float32)
    f[..., :3] = rng.lognormal(-1.0, 1.0, (n, h, w, 3))
    f[..., 3:6] = rng.uniform(0, 1, (n, h, w, 3))
    nr = rng.normal(size=(n, h, w, 3))
    f[..., 6:9] = nr / np.linalg.norm(nr, axis=-1, keepdims=True)
    f[..., 9] = rng.uniform(0.2, 1, (n, h, w))
    f[..., 10] = rng.uniform(0.0, 0.5, (n, h, w))
    return f


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(1)
    a = np.concatenate([rng.normal(size=4096) * 10.0 ** rng.integers(-6, 6, 4096),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, 65504.0]]).astype(np.float32)
    want = torch.from_numpy(a).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(bf16_round(a), want)


def test_param_layout():
    p = np.arange(param_count(), dtype=np.float64)
    parts = split_params(p)
    assert len(parts) == len(LAYERS)
    assert parts[0][0].shape == (9, 32, 16) and parts[-1][0].shape == (9, 8, 32)
    assert parts[-1][1][-1] == param_count() - 1
    assert 560_000 < param_count() < 570_000


def test_conv_pieces_match_torch():
    rng = np.random.default_rng(2)
    x = rng.normal(size=(2, 8, 12, 16))
    w = rng.normal(size=(9, 24, 16))
    b = rng.normal(size=24)
    g = rng.normal(size=(2, 8, 12, 24))
    xt = torch.tensor(x.transpose(0, 3, 1, 2), requires_grad=True)
    # torch weight [cout][cin][ky][kx]; tap = 3 ky + kx
    wt = torch.tensor(w.reshape(3, 3, 24, 16).transpose(2, 3, 0, 1).copy(), requires_grad=True)
    yt = torch.nn.functional.conv2d(xt, wt, torch.tensor(b), padding=1)
    yt.backward(torch.tensor(g.transpose(0, 3, 1, 2)))
    np.testing.assert_allclose(UnetOracle._conv(x, w, b), yt.detach().numpy().transpose(0, 2, 3, 1), rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(UnetOracle._conv_dgrad(g, w), xt.grad.numpy().transpose(0, 2, 3, 1), rtol=1e-10, atol=1e-10)
    dw = wt.grad.numpy().transpose(2, 3, 0, 1).reshape(9, 24, 16)
    np.testing.assert_allclose(UnetOracle._conv_wgrad(g, x), dw, rtol=1e-10, atol=1e-10)


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = _init(4)
    feat = _features(rng, 1, 16, 16)
    target = feat[..., :3] * rng.uniform(0.5, 1.5, feat[..., :3].shape)
    orc = UnetOracle(p, bf16=False)
    loss, g = orc.loss_and_grads(feat, target)
    assert abs(loss - orc.loss(feat, target)) < 1e-12
    # the largest gradients of every layer plus random entries
    idx, o = [], 0
    for ci, co, _ in LAYERS:
        n = 9 * ci * co + co
        seg = np.abs(g[o:o + n])
        idx += list(o + np.argsort(seg)[-2:]) + list(o + rng.integers(0, n, 1))
        o += n
    eps = 1e-6
    for i in idx:
        q = p.copy(); q[i] += eps
        lp = UnetOracle(q, bf16=False).loss(feat, target)
        q[i] -= 2 * eps
        lm = UnetOracle(q, bf16=False).loss(feat, target)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-7 + 1e-4 * abs(g[i]), (i, fd, g[i])
