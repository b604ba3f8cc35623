"""Batched rendering (salty_render_batch) and the autotuner (salty_autotune).

A batch concatenates its scenes' BVHs into one arena and renders all their samples in
shared waves; every scene's film must come out bit-identical to rendering that scene alone
with the same options, and no launch shape the autotuner may pick changes a result.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch(ctx):
    import salty_gb300
    from salty_gb300 import scenes
    descs = [scenes.cornell("baseline"), scenes.cornell("mixed"),
             scenes.heightfield(grid=64, n_spheres=40, seed=3, subdiv=2),
             dict(scenes.soup(20000, seed=5), sky=(1.0, 1.0, 1.0)),
             scenes.cornell("textured"), scenes.cornell("thinlens")]
    ss = []
    for d in descs:
        s = scenes.upload(ctx, d)
        s.build()
        ss.append(s)
    P = salty_gb300.PROFILE_PHYSICAL
    opts = [dict(width=48, height=40, spp=8, max_depth=8, seed=1, profile=P),
            dict(width=64, height=64, spp=4, max_depth=6, seed=2, profile=P, crop=(8, 16, 40, 24)),
            dict(width=96, height=54, spp=5, max_depth=12, seed=3, profile=P),
            dict(width=32, height=32, spp=16, max_depth=4, seed=4, profile=P),
            dict(width=40, height=40, spp=6, max_depth=8, seed=5, profile=P),
            dict(width=36, height=28, spp=7, max_depth=8, seed=6, profile=P)]
    yield ss, opts
    for s in ss:
        s.close()


def _films(ss, opts):
    out = []
    for s, o in zip(ss, opts):
        r = s.read(o["width"], o["height"], crop=o.get("crop"), want=("mean", "var"))
        h, w = r["mean"].shape[:2]
        out.append((r["mean"], r["var"], s.aov(w, h)))
    return out


def _alone(ss, opts):
    for s, o in zip(ss, opts):
        o = dict(o)
        s.render(o.pop("width"), o.pop("height"), o.pop("spp"), o.pop("max_depth"), want=(), **o)
    return _films(ss, opts)


def _same(a, b):
    for (m1, v1, f1), (m2, v2, f2) in zip(a, b):
        np.testing.assert_array_equal(m1, m2)
        np.testing.assert_array_equal(v1, v2)
        for k in f1:
            np.testing.assert_array_equal(f1[k], f2[k])


def test_batch_equals_scenes_rendered_alone(ctx, batch):
    ss, opts = batch
    alone = _alone(ss, opts)
    st = ctx.render_batch(ss, opts)
    assert st["paths"] == sum(o["spp"] * (o["crop"][2] * o["crop"][3] if "crop" in o else o["width"] * o["height"])
                              for o in opts)
    assert st["rays"] > st["paths"]
    _same(_films(ss, opts), alone)
    assert all(s.film_samples == o["spp"] for s, o in zip(ss, opts))


def test_batch_accumulates_progressively(ctx, batch):
    ss, opts = batch
    more = [dict(o, accumulate=True) for o in opts]
    _alone(ss, opts)
    alone = _alone(ss, more)
    assert all(s.film_samples == 2 * o["spp"] for s, o in zip(ss, opts))
    ctx.render_batch(ss, opts)
    ctx.render_batch(ss, more)
    assert all(s.film_samples == 2 * o["spp"] for s, o in zip(ss, opts))
    _same(_films(ss, opts), alone)


def test_tuning_does_not_change_results(ctx, batch):
    ss, opts = batch
    default = ctx.tuning
    ctx.render_batch(ss, opts)
    ref = _films(ss, opts)
    for t in ({"trace_block": 64, "trace_pool": 32, "trace_postpone": 1, "shade_block": 128, "trace_regs": 56,
               "wave_paths": 1 << 16},
              {"trace_block": 256, "trace_pool": 256, "trace_postpone": 10, "shade_block": 512, "trace_regs": 64,
               "wave_paths": 1 << 20}):
        ctx.tuning = t
        assert ctx.tuning == t
        ctx.render_batch(ss, opts)
        _same(_films(ss, opts), ref)
    ctx.tuning = default


def test_autotune_picks_a_valid_tuning(ctx, batch):
    ss, opts = batch
    default = ctx.tuning
    t, ms = ctx.autotune(ss, opts, trial_spp=2)
    assert ms > 0 and t == ctx.tuning
    assert t["trace_block"] in (64, 128, 256) and t["shade_block"] in (128, 256, 512)
    ctx.render_batch(ss, opts)
    tuned = _films(ss, opts)
    ctx.tuning = default
    ctx.render_batch(ss, opts)
    _same(tuned, _films(ss, opts))


def test_batch_rejects_bad_input(ctx, batch):
    import salty_gb300
    ss, opts = batch
    with pytest.raises(salty_gb300.SaltyError):
        ctx.render_batch([ss[0], ss[0]], [opts[0], opts[0]])
    with pytest.raises(salty_gb300.SaltyError):
        ctx.render_batch(ss[:2], [opts[0], dict(opts[1], profile=salty_gb300.PROFILE_COMPAT)])
    with pytest.raises(salty_gb300.SaltyError):
        ctx.tuning = {"trace_block": 100}


def test_host_loop_renders_the_same_films(ctx, batch, monkeypatch):
    """SALTY_RENDER_HOST_LOOP=1 launches the path loop's iterations from the host instead of
    one conditional CUDA graph (for profilers that cannot see into graph bodies): the same
    kernels in the same order, so the films are identical."""
    ss, opts = batch
    ctx.render_batch(ss, opts)
    ref = _films(ss, opts)
    monkeypatch.setenv("SALTY_RENDER_HOST_LOOP", "1")
    ctx.render_batch(ss, opts)
    _same(_films(ss, opts), ref)
