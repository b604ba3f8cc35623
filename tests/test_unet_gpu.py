"""The learned denoiser's CUDA path (salty_unet_*) against the float64 oracle with BF16
rounding at the same points (oracle/unet_oracle.py).

Tolerances: the two differ only by FP32 (tensor-core) vs FP64 accumulation order, which
now and then moves a BF16 rounding by one step (2^-8 relative); those differences
propagate.  Outputs are compared at 0.5 % relative L2 (measured on the GB300: at most
0.09 %); per-layer gradients of a 1 x 48 x 272 batch at 2.5 % relative L2 with a cosine
similarity above 0.9995 (measured: at most 1.7 %, at least 0.99986), and of the tiny
2 x 32 x 32 batch, whose small gradients carry relatively more rounding, at 5 % and 0.999
(measured: at most 3.4 %, at least 0.99945).
"""
import numpy as np
import pytest

from test_unet_oracle import _features

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def net(ctx):
    import salty_gb300
    n = salty_gb300.Unet(ctx, seed=11)
    yield n
    n.close()


def _batch(seed, n=2, h=32, w=32):
    rng = np.random.default_rng(seed)
    f = _features(rng, n, h, w)
    t = (f[..., :3] * rng.uniform(0.6, 1.4, f[..., :3].shape)).astype(np.float32)
    return f, t


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def test_parameter_count_and_init(net):
    from oracle.unet_oracle import param_count, split_params
    assert net.n_params == param_count()
    p = net.params()
    assert np.all(np.isfinite(p))
    w0, b0 = split_params(p)[0]
    assert np.all(w0[..., 11:] == 0) and np.all(b0 == 0)  # padded input channels unused


def test_forward_matches_oracle(net):
    from oracle.unet_oracle import UnetOracle
    f, _ = _batch(1)
    out = net.forward(f)
    want, _ = UnetOracle(net.params()).forward(f)
    assert out.shape == (2, 32, 32, 3)
    assert _rel(out, want) < 0.005, _rel(out, want)


def test_gradients_match_oracle(net):
    from oracle.unet_oracle import LAYERS, UnetOracle
    f, t = _batch(2)
    p0 = net.params()
    loss = net.train_step(f, t, lr=0.0)
    np.testing.assert_array_equal(net.params(), p0)  # lr = 0: no update
    g = net.grads()
    lo, go = UnetOracle(p0).loss_and_grads(f, t)
    assert abs(loss / lo - 1) < 1e-2, (loss, lo)
    o = 0
    for i, (ci, co, _) in enumerate(LAYERS):
        n = 9 * ci * co + co
        a, b = g[o:o + n], go[o:o + n]
        cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert _rel(a, b) < 0.05 and cos > 0.999, (i, _rel(a, b), cos)
        o += n


@pytest.mark.parametrize("kind", ["tcgen05", "tcgen05_cp_async", "mma_sync"])
def test_an_image_gives_the_same_output_in_any_batch(ctx, kind):
    """Each image of a batch goes through its own strips, borders and pooling windows, so
    its output is the same bit for bit alone or in a batch -- the film ensemble runs its
    mirror images as one batch on that ground."""
    import salty_gb300
    net = salty_gb300.Unet(ctx, seed=15)
    net.set_conv_kernel({"tcgen05": salty_gb300.CONV_TCGEN05, "tcgen05_cp_async": salty_gb300.CONV_TCGEN05_CP_ASYNC,
                         "mma_sync": salty_gb300.CONV_MMA_SYNC}[kind])
    f, _ = _batch(16, n=3, h=48, w=272)
    both = net.forward(f)
    for i in range(3):
        np.testing.assert_array_equal(net.forward(f[i:i + 1])[0], both[i])
    net.close()


def test_weight_gradient_kernels_agree(ctx):
    """The tensor-core weight gradient (tcgen05, partial sums per CTA added in a fixed
    order) against the mma.sync one, layer by layer: the two differ only by FP32 summation
    order, in the weight gradients and in the BF16 roundings of the backward pass."""
    import salty_gb300
    from oracle.unet_oracle import LAYERS
    f, t = _batch(21, n=2, h=64, w=96)
    grads = {}
    for kind in (salty_gb300.CONV_MMA_SYNC, salty_gb300.CONV_TCGEN05):
        net = salty_gb300.Unet(ctx, seed=13)
        net.set_conv_kernel(kind)
        net.train_step(f, t, lr=0.0)
        grads[kind] = net.grads()
        net.close()
    a, b = grads[salty_gb300.CONV_TCGEN05], grads[salty_gb300.CONV_MMA_SYNC]
    o = 0
    for i, (ci, co, _) in enumerate(LAYERS):
        n = 9 * ci * co
        wa, wb = a[o:o + n], b[o:o + n]
        cos = wa @ wb / max(np.linalg.norm(wa) * np.linalg.norm(wb), 1e-30)
        assert _rel(wa, wb) < 0.02 and cos > 0.9998, (i, _rel(wa, wb), cos)
        o += n + co


def test_tensor_core_training_is_deterministic(ctx):
    """Two identical training steps give bit-identical gradients: no atomics in the
    tensor-core backward pass."""
    import salty_gb300
    f, t = _batch(22, n=2, h=48, w=64)
    g = []
    for _ in range(2):
        net = salty_gb300.Unet(ctx, seed=14)
        net.set_conv_kernel(salty_gb300.CONV_TCGEN05)
        net.train_step(f, t, lr=0.0)
        g.append(net.grads())
        net.close()
    np.testing.assert_array_equal(g[0], g[1])


def test_adam_first_step(ctx):
    """First Adam step moves every parameter with a clear gradient by lr against its sign."""
    import salty_gb300
    net = salty_gb300.Unet(ctx, seed=5)
    f, t = _batch(3, n=1, h=16, w=16)
    p0 = net.params()
    net.train_step(f, t, lr=0.0)
    g = net.grads()
    net.train_step(f, t, lr=1e-3)
    d = net.params() - p0
    big = np.abs(g) > 1e-5
    np.testing.assert_allclose(d[big], -1e-3 * np.sign(g[big]), rtol=1e-3, atol=1e-7)
    net.close()


def test_training_reduces_loss(ctx):
    import salty_gb300
    net = salty_gb300.Unet(ctx, seed=6)
    f, _ = _batch(4, n=4, h=64, w=64)
    t = np.ascontiguousarray(2.0 * f[..., 3:6])  # a function of the features the net can learn
    l0 = net.train_step(f, t, lr=0.0)
    for _ in range(400):
        l = net.train_step(f, t, lr=2e-3)
    assert l < 0.6 * l0, (l0, l)
    net.close()


def test_device_arrays_and_batching(ctx, net):
    import torch
    f, _ = _batch(5, n=3, h=16, w=48)
    host = net.forward(f)
    dev = torch.empty((3, 16, 48, 3), dtype=torch.float32, device="cuda")
    net.forward(torch.from_numpy(f).cuda(), out=dev)
    np.testing.assert_array_equal(dev.cpu().numpy(), host)
    # images of a batch are independent
    np.testing.assert_array_equal(net.forward(f[1]), host[1])


def test_rejects_bad_shapes(net):
    import salty_gb300
    f, t = _batch(6, n=1, h=16, w=16)
    with pytest.raises(salty_gb300.SaltyError):
        net.forward(np.zeros((1, 20, 16, 11), np.float32))
    with pytest.raises(ValueError):
        net.train_step(f, t[:, :8], lr=0.0)


def test_training_checkpoint_resumes_exactly(ctx, tmp_path):
    """Parameters + Adam state saved mid-training and loaded into a new network: the next
    steps give the parameters of an uninterrupted run."""
    import salty_gb300
    from salty_gb300 import denoiser as dn
    f, t = _batch(7, n=2, h=32, w=32)
    a = salty_gb300.Unet(ctx, seed=8)
    for _ in range(3):
        a.train_step(f, t, lr=1e-3)
    p = str(tmp_path / "ckpt.npz")
    dn.save_weights(a, p, optimizer=True)
    for _ in range(2):
        a.train_step(f, t, lr=1e-3)
    b = salty_gb300.Unet(ctx, seed=99)
    dn.load_weights(b, p)
    assert b.adam_state()["step"] == 3
    for _ in range(2):
        b.train_step(f, t, lr=1e-3)
    # weight gradients are summed with FP32 atomics, so runs agree to rounding, not bits;
    # a resume without the optimiser state lands far further away
    c = salty_gb300.Unet(ctx, seed=99)
    c.set_params(np.load(p)["params"])
    for _ in range(2):
        c.train_step(f, t, lr=1e-3)
    d_state = np.abs(b.params() - a.params()).max()
    d_fresh = np.abs(c.params() - a.params()).max()
    assert d_state < 2e-5 and d_fresh > 10 * d_state, (d_state, d_fresh)
    for n in (a, b, c):
        n.close()


@pytest.mark.parametrize("kind", ["tcgen05", "tcgen05_cp_async", "mma_sync"])
def test_conv_kernels_match_oracle_on_ragged_strips(ctx, kind):
    """1 x 48 x 272 pixels: the tensor-core kernel's 128-pixel strips end ragged (272 =
    2 x 128 + 16) and its row groups (8, 5, 4, 3 or 2 rows by channel count) do not divide
    the level heights 48, 24, 12, 6, 3; forward output and every layer's gradients against
    the oracle, for every convolution kernel."""
    import salty_gb300
    from oracle.unet_oracle import LAYERS, UnetOracle
    net = salty_gb300.Unet(ctx, seed=12)
    net.set_conv_kernel({"tcgen05": salty_gb300.CONV_TCGEN05, "tcgen05_cp_async": salty_gb300.CONV_TCGEN05_CP_ASYNC,
                         "mma_sync": salty_gb300.CONV_MMA_SYNC}[kind])
    f, t = _batch(8, n=1, h=48, w=272)
    p0 = net.params()
    orc = UnetOracle(p0)
    out = net.forward(f)
    want, _ = orc.forward(f)
    assert _rel(out, want) < 0.005, _rel(out, want)
    loss = net.train_step(f, t, lr=0.0)
    lo, go = orc.loss_and_grads(f, t)
    assert abs(loss / lo - 1) < 1e-2, (loss, lo)
    g = net.grads()
    o = 0
    for i, (ci, co, _) in enumerate(LAYERS):
        n = 9 * ci * co + co
        a, b = g[o:o + n], go[o:o + n]
        cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert _rel(a, b) < 0.025 and cos > 0.9995, (i, _rel(a, b), cos)
        o += n
    net.close()


def test_tcgen05_and_mma_sync_agree(ctx):
    """The convolution kernels on a 2 x 144 x 400 batch: same outputs and gradients up to the
    order of the FP32 sums (a BF16 rounding step now and then); the two tcgen05 variants run
    the same MMAs in the same order, so they agree bit for bit."""
    import salty_gb300
    net = salty_gb300.Unet(ctx, seed=13)
    f, t = _batch(9, n=2, h=144, w=400)
    res = {}
    for kind in (salty_gb300.CONV_MMA_SYNC, salty_gb300.CONV_TCGEN05, salty_gb300.CONV_TCGEN05_CP_ASYNC):
        net.set_conv_kernel(kind)
        out = net.forward(f)
        loss = net.train_step(f, t, lr=0.0)
        res[kind] = (out, loss, net.grads())
    (o1, l1, g1), (o2, l2, g2) = res[salty_gb300.CONV_MMA_SYNC], res[salty_gb300.CONV_TCGEN05]
    assert _rel(o2, o1) < 0.01, _rel(o2, o1)
    assert abs(l2 / l1 - 1) < 1e-3, (l1, l2)
    cos = g1 @ g2 / (np.linalg.norm(g1) * np.linalg.norm(g2))
    assert _rel(g2, g1) < 0.02 and cos > 0.9995, (_rel(g2, g1), cos)
    np.testing.assert_array_equal(res[salty_gb300.CONV_TCGEN05_CP_ASYNC][0], o2)
    with pytest.raises(salty_gb300.SaltyError):
        net.set_conv_kernel(7)
    net.close()


@pytest.mark.parametrize("shape", [(1, 1088, 1920), (3, 16, 16)])
def test_tcgen05_full_frame_and_tiny_batch(ctx, shape):
    """The tensor-core kernels at the denoiser's working size (a 1080p frame padded to 1088
    rows: 15 strips of 128 pixels, 136 row groups, the persistent TMA kernel looping over
    many strips per CTA) and at the smallest legal size (16 x 16, one ragged strip at every
    level, 1 x 1 at the bottleneck): outputs equal the mma.sync kernel's up to FP32
    summation order, and the input gradients of a training step as well."""
    import torch
    import salty_gb300
    n, h, w = shape
    net = salty_gb300.Unet(ctx, seed=14)
    g = torch.Generator(device="cuda").manual_seed(3)
    f = torch.rand((n, h, w, salty_gb300.UNET_FEATURES), device="cuda", generator=g)
    t = f[..., :3] * (0.6 + 0.8 * torch.rand((n, h, w, 3), device="cuda", generator=g))
    res = {}
    for kind in (salty_gb300.CONV_MMA_SYNC, salty_gb300.CONV_TCGEN05):
        net.set_conv_kernel(kind)
        o = torch.empty((n, h, w, 3), device="cuda")
        net.forward(f, out=o)
        loss = net.train_step(f, t.contiguous(), lr=0.0)
        res[kind] = (o.cpu().numpy(), loss, net.grads())
    (o1, l1, g1), (o2, l2, g2) = res[salty_gb300.CONV_MMA_SYNC], res[salty_gb300.CONV_TCGEN05]
    assert np.all(np.isfinite(o2))
    assert _rel(o2, o1) < 0.01, _rel(o2, o1)
    assert abs(l2 / l1 - 1) < 1e-3, (l1, l2)
    cos = g1 @ g2 / (np.linalg.norm(g1) * np.linalg.norm(g2))
    assert cos > 0.999, cos
    net.close()
