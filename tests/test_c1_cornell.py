"""The Cornell frame at its configured size (256x256, max depth 8, the reference's
estimator) against the reference's own render of it (tests/golden/cornell_c1_ref_256.npz,
1024 spp through PathTracer::Radiance, src/s3d_pt.cpp:182-246).

Bar: the frame is cut into 8x8-pixel blocks; a block's mean has a near-normal error
(64 pixels' worth of samples), so its z-score z = (a - b) / sqrt(va + vb) follows the
normal law closely, unlike a single pixel's at a few hundred samples (a pixel's variance
estimate is itself noisy and its error heavy-tailed).  Required: the count of block
channels beyond 3 sigma within the binomial bound of a normal variable (0.27 %, plus four
standard deviations of that count: conftest.beyond3_bound), none beyond 5.5 sigma, and
the whole frame's mean within 4 standard errors.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, beyond3_bound

BLOCK = 8


def _fixture():
    g = np.load(os.path.join(GOLDEN, "cornell_c1_ref_256.npz"))
    mean = g["mean"].astype(np.float64)
    var = g["sem"].astype(np.float64) ** 2
    return g, mean, var


def _blocks(a):
    h, w, c = a.shape
    return a.reshape(h // BLOCK, BLOCK, w // BLOCK, BLOCK, c).mean(axis=(1, 3))


def check_against_reference(mean, var):
    g, gm, gv = _fixture()
    n = BLOCK * BLOCK
    zb = (_blocks(mean) - _blocks(gm)) / np.sqrt((_blocks(var) + _blocks(gv)) / n + 1e-30)
    k, zmax = int(np.count_nonzero(np.abs(zb) > 3)), float(np.max(np.abs(zb)))
    assert k <= beyond3_bound(zb.size) and zmax < 5.5, (k, zb.size, zmax)
    se = np.sqrt(var.sum() + gv.sum()) / mean.size
    assert abs(mean.mean() - gm.mean()) < 4 * se, (mean.mean(), gm.mean(), se)


def test_oracle_matches_reference_at_configured_size(oracle):
    """The oracle's compat path (the checker of the GPU tests) on the configured frame."""
    from oracle.oracle import PROFILE_COMPAT, SceneData
    from salty_gb300 import scenes
    g, _, _ = _fixture()
    sc = scenes.cornell("baseline")
    sd = SceneData(sc["tri_pos"], sc["tri_nrm"], sc["tri_mat"], sc["materials"], sc["light"], None, sc["sky"],
                   sc["camera"])
    spp = 256
    tot, sq = oracle.render(sd, int(g["width"]), int(g["height"]), spp, int(g["max_bounce"]),
                            profile=PROFILE_COMPAT, seed=77)
    m = tot / spp
    check_against_reference(m, np.maximum((sq / spp - m * m) / (spp - 1), 0))


@pytest.mark.gpu
def test_gpu_matches_reference_at_configured_size(ctx):
    """salty_render's compat profile on the configured frame, same spp as the fixture."""
    import salty_gb300
    from salty_gb300 import scenes
    g, _, _ = _fixture()
    s = scenes.upload(ctx, scenes.cornell("baseline"))
    s.build()
    r = s.render(int(g["width"]), int(g["height"]), int(g["spp"]), int(g["max_bounce"]),
                 profile=salty_gb300.PROFILE_COMPAT, seed=16161)
    s.close()
    check_against_reference(r["mean"].astype(np.float64), r["var"].astype(np.float64))
