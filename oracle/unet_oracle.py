"""NumPy float64 restatement of the learned denoiser (forward, loss, backward).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of salty_unet_forward and
salty_unet_train_step, never by the shipped library.

The reference has no learned denoiser (its only one is FilterNLM, src/s3d_denoiser.cpp:19-95),
so this oracle is pinned by central finite differences of its own loss instead of by
reference outputs.  With bf16=True it rounds to BF16 at the points the CUDA kernels store
BF16 (input features, weights, every layer output, every backward operand), so the GPU's
result differs from it only by FP32-vs-FP64 accumulation order.

Layout (shared with the CUDA path): NHWC activations; per layer, weights [9][cout][cin]
(tap = 3*ky + kx reads input pixel (y + ky - 1, x + kx - 1)) followed by biases [cout].
"""
from __future__ import annotations

import numpy as np

LAYERS = [(16, 32, 1), (32, 32, 1), (32, 48, 1), (48, 48, 1), (48, 64, 1), (64, 64, 1), (64, 80, 1),
          (80, 80, 1), (80, 96, 1), (176, 80, 1), (144, 64, 1), (112, 48, 1), (80, 32, 1), (32, 8, 0)]


def param_count() -> int:
    return sum(9 * ci * co + co for ci, co, _ in LAYERS)


def split_params(p: np.ndarray):
    """[(w (9, cout, cin), b (cout,))] views of the flat parameter vector."""
    out, o = [], 0
    for ci, co, _ in LAYERS:
        w = p[o:o + 9 * co * ci].reshape(9, co, ci)
        o += 9 * co * ci
        out.append((w, p[o:o + co]))
        o += co
    return out


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


class UnetOracle:
    def __init__(self, params: np.ndarray, bf16: bool = True):
        self.bf16 = bf16
        self.params = np.asarray(params, np.float64)
        self.layers = []
        for (w, b), (_, _, relu) in zip(split_params(self.params), LAYERS):
            self.layers.append((self.r(w), b.copy(), relu))

    def r(self, a):
        return bf16_round(a) if self.bf16 else np.asarray(a, np.float64)

    # ---------------------------------------------------------------- pieces
    @staticmethod
    def _conv(x, w, b):
        n, h, wd, _ = x.shape
        xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
        y = np.zeros((n, h, wd, w.shape[1]))
        for tap in range(9):
            ky, kx = divmod(tap, 3)
            y += xp[:, ky:ky + h, kx:kx + wd, :] @ w[tap].T
        return y + b if b is not None else y

    @staticmethod
    def _conv_wgrad(g, x):
        n, h, wd, _ = x.shape
        xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
        g2 = g.reshape(-1, g.shape[-1])
        return np.stack([g2.T @ xp[:, ky:ky + h, kx:kx + wd, :].reshape(-1, x.shape[-1])
                         for ky in range(3) for kx in range(3)])

    @staticmethod
    def _conv_dgrad(g, w):
        # dx[q] = sum_tap W[tap]^T g[q - off(tap)]
        n, h, wd, _ = g.shape
        gp = np.pad(g, ((0, 0), (1, 1), (1, 1), (0, 0)))
        dx = np.zeros((n, h, wd, w.shape[2]))
        for tap in range(9):
            ky, kx = divmod(tap, 3)
            # off = (ky-1, kx-1): g at q - off = padded index q + 1 - (ky - 1) = q + 2 - ky
            dx += gp[:, 2 - ky:2 - ky + h, 2 - kx:2 - kx + wd, :] @ w[tap]
        return dx

    @staticmethod
    def _pool(x):
        n, h, w, c = x.shape
        q = np.stack([x[:, 0::2, 0::2], x[:, 0::2, 1::2], x[:, 1::2, 0::2], x[:, 1::2, 1::2]])
        return q.max(axis=0), q.argmax(axis=0)  # argmax: first of equal maxima

    @staticmethod
    def _pool_bwd(arg, d, shape):
        out = np.zeros(shape)
        for k, (dy, dx) in enumerate(((0, 0), (0, 1), (1, 0), (1, 1))):
            out[:, dy::2, dx::2] += np.where(arg == k, d, 0.0)
        return out

    @staticmethod
    def _up(x):
        return x.repeat(2, axis=1).repeat(2, axis=2)

    @staticmethod
    def _up_bwd(d):
        return d[:, 0::2, 0::2] + d[:, 0::2, 1::2] + d[:, 1::2, 0::2] + d[:, 1::2, 1::2]

    def prep(self, feat):
        feat = np.asarray(feat, np.float32)
        x = np.zeros(feat.shape[:3] + (16,))
        x[..., :3] = np.log1p(np.maximum(feat[..., :3], 0.0)).astype(np.float32)
        x[..., 3:11] = feat[..., 3:11]
        return self.r(x)

    # ---------------------------------------------------------------- passes
    def forward(self, feat):
        """Returns (linear RGB (N, H, W, 3), saved activations)."""
        S = {"x": self.prep(feat)}
        L = self.layers

        def conv(i, x):
            w, b, relu = L[i]
            y = self._conv(x, w, b)
            return self.r(np.maximum(y, 0.0) if relu else y)

        S["a0"] = conv(0, S["x"]); S["e0"] = conv(1, S["a0"])
        S["p0"], S["i0"] = self._pool(S["e0"])
        S["a1"] = conv(2, S["p0"]); S["e1"] = conv(3, S["a1"])
        S["p1"], S["i1"] = self._pool(S["e1"])
        S["a2"] = conv(4, S["p1"]); S["e2"] = conv(5, S["a2"])
        S["p2"], S["i2"] = self._pool(S["e2"])
        S["a3"] = conv(6, S["p2"]); S["e3"] = conv(7, S["a3"])
        S["p3"], S["i3"] = self._pool(S["e3"])
        S["b"] = conv(8, S["p3"])
        S["c3"] = np.concatenate([self._up(S["b"]), S["e3"]], -1); S["d3"] = conv(9, S["c3"])
        S["c2"] = np.concatenate([self._up(S["d3"]), S["e2"]], -1); S["d2"] = conv(10, S["c2"])
        S["c1"] = np.concatenate([self._up(S["d2"]), S["e1"]], -1); S["d1"] = conv(11, S["c1"])
        S["c0"] = np.concatenate([self._up(S["d1"]), S["e0"]], -1); S["d0"] = conv(12, S["c0"])
        S["out"] = conv(13, S["d0"])
        S["pred"] = S["out"][..., :3] + S["x"][..., :3]  # correction of the input's log colour
        return np.maximum(np.expm1(S["pred"]), 0.0), S

    def loss_and_grads(self, feat, target):
        """Mean |out - log(1 + target)| and the gradient of every parameter (flat vector)."""
        _, S = self.forward(feat)
        t = np.log1p(np.maximum(np.asarray(target, np.float32 if self.bf16 else np.float64), 0.0)).astype(np.float64)
        npx = t.shape[0] * t.shape[1] * t.shape[2]
        d = S["pred"] - t
        loss = np.abs(d).sum() / (3.0 * npx)
        scale = float(np.float32(1.0) / np.float32(3.0 * npx)) if self.bf16 else 1.0 / (3.0 * npx)
        dout = np.zeros(S["out"].shape)
        dout[..., :3] = np.sign(d) * scale
        grads = [None] * len(self.layers)
        f32 = (lambda a: a.astype(np.float32).astype(np.float64)) if self.bf16 else (lambda a: a)

        def back(i, x, y, dy, want_dx=True):
            w, _, relu = self.layers[i]
            g = self.r(dy * (y > 0) if relu else dy)
            grads[i] = (self._conv_wgrad(g, x), g.reshape(-1, g.shape[-1]).sum(0))
            return self.r(self._conv_dgrad(g, w)) if want_dx else None

        def split(dc, cc):
            return f32(self._up_bwd(dc[..., :cc])), dc[..., cc:]

        dd0 = back(13, S["d0"], S["out"], dout)
        dc0 = back(12, S["c0"], S["d0"], dd0)
        dd1, de0 = split(dc0, 48)
        dc1 = back(11, S["c1"], S["d1"], dd1)
        dd2, de1 = split(dc1, 64)
        dc2 = back(10, S["c2"], S["d2"], dd2)
        dd3, de2 = split(dc2, 80)
        dc3 = back(9, S["c3"], S["d3"], dd3)
        db, de3 = split(dc3, 96)
        dp3 = back(8, S["p3"], S["b"], db)
        de3 = de3 + self._pool_bwd(S["i3"], dp3, de3.shape)
        da3 = back(7, S["a3"], S["e3"], de3)
        dp2 = back(6, S["p2"], S["a3"], da3)
        de2 = de2 + self._pool_bwd(S["i2"], dp2, de2.shape)
        da2 = back(5, S["a2"], S["e2"], de2)
        dp1 = back(4, S["p1"], S["a2"], da2)
        de1 = de1 + self._pool_bwd(S["i1"], dp1, de1.shape)
        da1 = back(3, S["a1"], S["e1"], de1)
        dp0 = back(2, S["p0"], S["a1"], da1)
        de0 = de0 + self._pool_bwd(S["i0"], dp0, de0.shape)
        da0 = back(1, S["a0"], S["e0"], de0)
        back(0, S["x"], S["a0"], da0, want_dx=False)
        flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
        return loss, flat

    def loss(self, feat, target):
        out, S = self.forward(feat)
        t = np.log1p(np.maximum(np.asarray(target, np.float64), 0.0))
        return np.abs(S["pred"] - t).mean()
