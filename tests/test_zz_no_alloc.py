"""salty_tonemap_noalloc: the tonemap entry point for callers that cannot allocate.

A render loop that tonemaps every frame for display (where cudaMalloc would synchronise
the device) or an engine that owns all GPU memory cannot call cudaMalloc at that point;
this entry point works only on device arrays the caller already owns and on a fixed
scratch array inside the library.  Its output must match salty_tonemap's (same tolerance as the tonemap tests),
call after call.  This file is collected last, so a run that stops at the first failure
has already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PIXELS = 4096 * 4096


@pytest.fixture(scope="module")
def noalloc_ctx():
    import salty_gb300
    from salty_gb300 import build as b
    b.build()
    c = salty_gb300.Context(0)
    yield c
    c.close()


def _image(seed, h, w):
    rng = np.random.default_rng(seed)
    img = np.exp(rng.normal(-0.5, 1.7, size=(h, w, 3))).astype(np.float32)
    img[0, 0] = 0.0
    return img


def _noalloc(ctx, d_img, kind, h, w, ref_oetf=1):
    import torch
    import salty_gb300
    d_out = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    d_s8 = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    st = salty_gb300.lib().salty_tonemap_noalloc(ctx.h, None, kind, w, h, d_img.data_ptr(), d_out.data_ptr(),
                                                 d_s8.data_ptr(), ref_oetf)
    ctx.check(st, "tonemap_noalloc")
    # the call only enqueues on the context's stream: wait for the whole device
    torch.cuda.synchronize()
    return d_out, d_s8


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_noalloc_matches_tonemap_on_two_calls_in_a_row(noalloc_ctx, kind):
    import torch
    import salty_gb300
    ctx = noalloc_ctx
    for call, (h, w) in enumerate([(270, 480), (333, 517)]):
        img = _image(100 * kind + call, h, w)
        d_img = torch.from_numpy(img).cuda()
        d_out, d_s8 = _noalloc(ctx, d_img, kind, h, w)
        # the context's stream may still run: the existing entry point syncs it
        ref_out, ref_s8, _, _ = ctx.tonemap(img, kind, srgb=True, ref_oetf=True)
        out = d_out.cpu().numpy()
        s8 = d_s8.cpu().numpy()
        np.testing.assert_allclose(out, ref_out, rtol=2e-5, atol=1e-7)
        d = np.abs(s8.astype(int) - ref_s8.astype(int))
        assert d.max() <= 1 and (d > 0).mean() < 0.01


def test_noalloc_rejects_images_beyond_its_scratch(noalloc_ctx):
    import torch
    import salty_gb300
    ctx = noalloc_ctx
    d_img = torch.zeros((4, 4, 3), dtype=torch.float32, device="cuda")
    d_out = torch.empty_like(d_img)
    # 4097 x 4096 pixels: more than the fixed scratch holds; rejected before any launch
    st = salty_gb300.lib().salty_tonemap_noalloc(ctx.h, None, 0, 4097, 4096, d_img.data_ptr(), d_out.data_ptr(),
                                                 None, 1)
    assert st == salty_gb300.ERR_CAPACITY
    assert b"scratch" in salty_gb300.lib().salty_last_error(ctx.h)


def test_noalloc_rejects_host_arrays(noalloc_ctx):
    import salty_gb300
    ctx = noalloc_ctx
    img = _image(1, 8, 8)
    out = np.empty_like(img)
    st = salty_gb300.lib().salty_tonemap_noalloc(ctx.h, None, 0, 8, 8, img.ctypes.data, out.ctypes.data, None, 1)
    assert st == salty_gb300.ERR_INVALID_ARG


def test_noalloc_on_the_callers_stream_allocates_nothing(noalloc_ctx):
    """The pattern such a caller uses: the image produced on its own stream, the call
    enqueued on that same stream (no extra synchronisation), and device memory unchanged
    across the calls once the first call has looked up the scratch array."""
    import torch
    import salty_gb300
    ctx = noalloc_ctx
    h, w = 540, 960
    img = _image(7, h, w)
    ref_out, ref_s8, _, _ = ctx.tonemap(img, 0, srgb=True, ref_oetf=True)
    s = torch.cuda.Stream()
    host = torch.from_numpy(img).pin_memory()
    with torch.cuda.stream(s):
        d_img = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
        d_out = torch.empty_like(d_img)
        d_s8 = torch.empty((h, w, 3), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    L = salty_gb300.lib()
    ctx.check(L.salty_tonemap_noalloc(ctx.h, s.cuda_stream, 0, w, h, d_img.data_ptr(), d_out.data_ptr(),
                                      d_s8.data_ptr(), 1), "tonemap_noalloc")  # warm call
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        with torch.cuda.stream(s):
            d_out.zero_()
            d_img.copy_(host, non_blocking=True)
        ctx.check(L.salty_tonemap_noalloc(ctx.h, s.cuda_stream, 0, w, h, d_img.data_ptr(), d_out.data_ptr(),
                                          d_s8.data_ptr(), 1), "tonemap_noalloc")
        s.synchronize()
        np.testing.assert_allclose(d_out.cpu().numpy(), ref_out, rtol=2e-5, atol=1e-7)
        d = np.abs(d_s8.cpu().numpy().astype(int) - ref_s8.astype(int))
        assert d.max() <= 1 and (d > 0).mean() < 0.01
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
