"""Parity of the CUDA traversal (salty_trace) with the reference and the oracle.

The bar (closest hit): triangle ids bit-exact, ties to the lowest id; hit t within
1e-5 relative (the reference-compatible test in fact reproduces t bit for bit, which
is also asserted).  Any hit: occluded exactly when a closest hit exists.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

T_RTOL = 1e-5


def _scene(ctx, tris, **kw):
    import salty_gb300
    sc = ctx.upload_scene(tris, **kw)
    sc.build()
    return sc


def _check_closest(res, ids, t, exact_t=True):
    assert np.array_equal(res.ids, ids), f"{np.count_nonzero(res.ids != ids)} id mismatches of {ids.size}"
    hit = ids >= 0
    if hit.any():
        rel = np.abs(res.t[hit] - t[hit]) / np.abs(t[hit])
        assert rel.max() <= T_RTOL
        if exact_t:
            assert np.array_equal(res.t[hit], t[hit])
    assert np.all(np.isinf(res.t[~hit]))


def test_closest_hit_matches_reference_fixture_1m(gpu_soup_1m):
    import salty_gb300
    g = np.load(os.path.join(GOLDEN, "trace_soup_1m.npz"))
    rays = salty_gb300.microbench_rays(20260002, 65536, 1e-4)
    res = gpu_soup_1m.trace(rays)
    _check_closest(res, g["ids"], g["t"])


def test_closest_hit_matches_reference_fixture_30k(ctx):
    import salty_gb300
    g = np.load(os.path.join(GOLDEN, "trace_soup_30k.npz"))
    tris = salty_gb300.microbench_soup(int(g["soup_seed"]), int(g["n_tris"]))
    rays = salty_gb300.microbench_rays(int(g["ray_seed"]), int(g["n_rays"]), 1e-4)
    sc = _scene(ctx, tris)
    res = sc.trace(rays)
    _check_closest(res, g["ids"], g["t"])
    hit = g["ids"] >= 0
    assert np.array_equal(res.u[hit], g["u"][hit]) and np.array_equal(res.v[hit], g["v"][hit])


def test_full_workload_subset_matches_oracle(gpu_soup_1m, soup_1m, oracle, ctx):
    """All 16,777,216 microbenchmark rays on the device; a seeded random subset checked
    against the oracle, plus size-independent properties on every ray."""
    import torch
    import salty_gb300
    n = 16_777_216
    rays = salty_gb300.microbench_rays(20260002, n, 1e-4)
    d_rays = torch.from_numpy(rays).cuda()
    d_hits = torch.empty((n, 4), dtype=torch.float32, device="cuda")
    gpu_soup_1m.trace_raw(d_rays, d_hits)
    hits = d_hits.cpu().numpy()
    ids = hits[:, 1].view(np.int32)
    sub = np.random.default_rng(3).choice(n, 32768, replace=False)
    oid, ot, _, _ = oracle.trace(soup_1m, rays[sub], mode=0)
    assert np.array_equal(ids[sub], oid)
    h = oid >= 0
    assert np.array_equal(hits[sub, 0][h], ot[h])
    assert (ids >= 0).mean() > 0.97
    assert np.all((ids >= -1) & (ids < 1_000_000))
    # any hit: occluded iff a closest hit exists (every ray)
    d_any = torch.empty_like(d_hits)
    gpu_soup_1m.trace_raw(d_rays, d_any, any_hit=True)
    any_ids = d_any[:, 1].cpu().numpy().view(np.int32)
    assert np.array_equal(any_ids >= 0, ids >= 0)
    # the any-hit t is a real hit no nearer than the closest
    a_t = d_any[:, 0].cpu().numpy()
    hit = ids >= 0
    assert np.all(a_t[hit] >= hits[hit, 0])


def test_host_and_device_buffers_agree(gpu_soup_1m):
    import torch
    import salty_gb300
    rays = salty_gb300.microbench_rays(5, 3_000_001, 1e-4)  # spans two host chunks, ragged tail
    host = gpu_soup_1m.trace(rays)
    d_hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    gpu_soup_1m.trace_raw(torch.from_numpy(rays).cuda(), d_hits)
    dev = d_hits.cpu().numpy()
    assert np.array_equal(host.ids, dev[:, 1].view(np.int32))
    assert np.array_equal(host.t, dev[:, 0])


@pytest.mark.parametrize("n", [0, 1, 31, 33, 1000])
def test_ragged_and_empty_ray_counts(ctx, oracle, n):
    import salty_gb300
    tris = salty_gb300.microbench_soup(21, 5000)
    sc = _scene(ctx, tris)
    rays = salty_gb300.microbench_rays(22, n, 1e-4)
    res = sc.trace(rays)
    assert res.ids.shape == (n,)
    if n:
        oid, ot, _, _ = oracle.trace(tris, rays, mode=0)
        _check_closest(res, oid, ot)


def test_single_triangle_and_axis_aligned_rays(ctx, oracle):
    tris = np.array([[0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0, 0.0]], np.float32)
    sc = _scene(ctx, tris)
    rays = np.array([
        [0.25, 0.25, -1.0, 1e-4, 0.0, 0.0, 1.0, np.inf],   # straight +z: hit at t = 1
        [0.25, 0.25, 1.0, 1e-4, 0.0, 0.0, -1.0, np.inf],   # straight -z: hit (two-sided)
        [0.25, 0.25, -1.0, 1e-4, 0.0, 0.0, -1.0, np.inf],  # away: miss
        [2.0, 2.0, -1.0, 1e-4, 0.0, 0.0, 1.0, np.inf],     # outside: miss
        [0.25, 0.25, -1.0, 1e-4, 0.0, 0.0, 1.0, 0.5],      # tmax before the triangle: miss
        [0.25, 0.25, -1.0, 2.0, 0.0, 0.0, 1.0, np.inf],    # tmin after the triangle: miss
        [-1.0, 0.25, 0.0, 1e-4, 1.0, 0.0, 0.0, np.inf],    # in the triangle's plane: miss
    ], np.float32)
    res = sc.trace(rays)
    oid, ot, _, _ = oracle.trace(tris, rays, mode=0)
    assert list(res.ids) == [0, 0, -1, -1, -1, -1, -1]
    _check_closest(res, oid, ot)
    assert res.t[0] == 1.0


def test_duplicate_triangles_tie_to_lowest_id(ctx, oracle):
    import salty_gb300
    base = salty_gb300.microbench_soup(51, 2000)
    tris = np.concatenate([base, base[::-1]])  # triangle i duplicated at 3999 - i
    sc = _scene(ctx, tris)
    rays = salty_gb300.microbench_rays(52, 20000, 1e-4)
    res = sc.trace(rays)
    oid, ot, _, _ = oracle.trace(tris, rays, mode=0)
    _check_closest(res, oid, ot)
    hit = res.ids >= 0
    assert hit.sum() > 100 and np.all(res.ids[hit] < 2000)


def test_degenerate_triangles_never_hit(ctx, oracle):
    import salty_gb300
    tris = salty_gb300.microbench_soup(61, 3000)
    tris[::3, 3:6] = tris[::3, 0:3]          # zero-area (repeated vertex)
    tris[1::7, 6:9] = 2 * tris[1::7, 3:6] - tris[1::7, 0:3]  # collinear
    sc = _scene(ctx, tris)
    rays = salty_gb300.microbench_rays(62, 20000, 1e-4)
    res = sc.trace(rays)
    oid, ot, _, _ = oracle.trace(tris, rays, mode=0)
    _check_closest(res, oid, ot)
    assert not np.any(np.isin(res.ids[res.ids >= 0], np.arange(0, 3000, 3)))


def test_watertight_mode_matches_oracle(ctx, oracle):
    import salty_gb300
    tris = salty_gb300.microbench_soup(71, 100000)
    sc = _scene(ctx, tris)
    rays = salty_gb300.microbench_rays(72, 20000, 1e-4)
    res = sc.trace(rays, watertight=True)
    oid, ot, _, _ = oracle.trace(tris, rays, mode=1)
    _check_closest(res, oid, ot, exact_t=False)


def test_watertight_closes_shared_edges(ctx):
    """A quad split along its diagonal: rays aimed at the diagonal hit in watertight mode;
    the reference test (strict inequalities) misses some of them."""
    quad = np.array([[0, 0, 0, 1, 0, 0, 1, 1, 0], [0, 0, 0, 1, 1, 0, 0, 1, 0]], np.float32)
    sc = _scene(ctx, quad)
    s = np.linspace(0.01, 0.99, 999, dtype=np.float32)
    rays = np.zeros((s.size, 8), np.float32)
    rays[:, 0] = s; rays[:, 1] = s; rays[:, 2] = -1.0; rays[:, 3] = 1e-4
    rays[:, 6] = 1.0; rays[:, 7] = np.inf
    wt = sc.trace(rays, watertight=True)
    assert np.all(wt.ids >= 0)


@pytest.mark.parametrize("bins,max_leaf", [(8, 1), (16, 2), (32, 3)])
def test_build_options_do_not_change_results(ctx, oracle, bins, max_leaf):
    import salty_gb300
    tris = salty_gb300.microbench_soup(81, 50000)
    sc = ctx.upload_scene(tris)
    info = sc.build(bins=bins, max_leaf=max_leaf)
    assert info["n_nodes"] > 0 and 0 < info["depth"] <= 40 and np.isfinite(info["sah_cost"])
    rays = salty_gb300.microbench_rays(82, 8192, 1e-4)
    res = sc.trace(rays)
    oid, ot, _, _ = oracle.trace(tris, rays, mode=0)
    _check_closest(res, oid, ot)


def test_counters_report_fetches(gpu_soup_1m):
    import salty_gb300
    rays = salty_gb300.microbench_rays(20260002, 100000, 1e-4)
    gpu_soup_1m.trace(rays, counters=True)
    st = gpu_soup_1m.last_stats
    assert st["node_fetches"] > st["rays"] and st["tri_fetches"] > 0


def test_errors_are_reported_not_crashing(ctx):
    import salty_gb300
    tris = salty_gb300.microbench_soup(91, 100)
    sc = ctx.upload_scene(tris)
    with pytest.raises(salty_gb300.SaltyError) as e:
        sc.trace(salty_gb300.microbench_rays(1, 10))
    assert e.value.status == salty_gb300.ERR_NOT_BUILT
    with pytest.raises(salty_gb300.SaltyError) as e:
        sc.build(bins=64)
    assert e.value.status == salty_gb300.ERR_INVALID_ARG
    with pytest.raises(salty_gb300.SaltyError):
        ctx.upload_scene(np.zeros((0, 9), np.float32))


def test_autotune_trace_keeps_results(ctx, gpu_soup_1m):
    """Every traversal launch shape gives the same hits; the autotuner picks one of them."""
    import torch
    import salty_gb300
    rays = torch.from_numpy(salty_gb300.microbench_rays(20260002, 1 << 20, 1e-4)).cuda()
    hits = torch.empty((1 << 20, 4), device="cuda")
    default = ctx.tuning
    gpu_soup_1m.trace_raw(rays, hits)
    ref = hits.cpu().numpy().view(np.int32).copy()
    t, ms = gpu_soup_1m.autotune_trace(rays)
    assert ms > 0 and t == ctx.tuning and t["trace_block"] in (64, 128, 256) and t["trace_regs"] in (56, 64)
    gpu_soup_1m.trace_raw(rays, hits)
    np.testing.assert_array_equal(hits.cpu().numpy().view(np.int32), ref)
    ctx.tuning = default
