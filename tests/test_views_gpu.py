"""Batched views: many cameras of uneven size and spp rendered in shared wavefront batches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VIEWS = [dict(frm=(0, 0, 3.5), at=(0, 0, 0), up=(0, 1, 0), vfov=40, focus=3.5, width=96, height=80, spp=8, seed=3),
         dict(frm=(2, 1, 3), at=(0, 0, 0), vfov=50, focus=3, width=64, height=48, spp=4, seed=9),
         dict(frm=(-1, 0.5, 3), at=(0, -0.2, 0), vfov=35, focus=3, width=128, height=128, spp=16, seed=11)]


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


def test_view_equal_to_scene_camera_equals_lts_render(ctx, scene_dirs):
    """A view with the scene file's camera, film size, spp and seed renders the film lts_render
    renders (same samples, same fixed-order gather)."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["box_sphere"]
    s = lts.Scene.parse(ctx, d, sc, sub, 96, 80)
    single = lts.PathTracingIntegrator(5, 3, s, integrator=1).render(8, 3)["film"]
    films, ms = lts.render_views(s, VIEWS, 5, 3)
    print(f"3 views: {ms:.2f} ms")
    assert np.allclose(films[0], single, rtol=1e-6, atol=1e-7)
    for f in films:
        assert np.isfinite(f).all() and f.mean() > 0


def test_batching_does_not_change_a_view(ctx, scene_dirs):
    """Each view renders the same alone, in a batch, and split into sample slices across batches."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["materials"]
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    together, _ = lts.render_views(s, VIEWS, 6, 3)
    for k, v in enumerate(VIEWS):
        alone, _ = lts.render_views(s, [v], 6, 3)
        assert np.allclose(alone[0], together[k], rtol=1e-6, atol=1e-7)
    ctx.set_option("wavefront_sample_chunk", 128 * 128 * 3)  # forces slices of 3 spp and several batches
    try:
        sliced, _ = lts.render_views(s, VIEWS, 6, 3)
    finally:
        ctx.set_option("wavefront_sample_chunk", 0)
    for a, b in zip(sliced, together):
        assert np.allclose(a, b, rtol=1e-5, atol=1e-7)


def test_autotuner_picks_a_setting_and_keeps_results(ctx, scene_dirs):
    """The autotuner returns one of its candidates, no slower than the defaults it started from,
    and rendering after it gives the same images (the knobs change speed, not samples)."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["box_sphere"]
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    before, _ = lts.render_views(s, VIEWS, 5, 3)
    res = lts.autotune_views(s, VIEWS, 5, 3)
    print(res)
    assert (res["pool_log2"] == 0 or 18 <= res["pool_log2"] <= 26) and res["trace_blocks_per_sm"] in (0, 2, 4) \
        and res["graph"] in (0, 1)
    assert res["ms_best"] <= res["ms_default"]
    after, _ = lts.render_views(s, VIEWS, 5, 3)
    for a, b in zip(before, after):
        assert np.allclose(a, b, rtol=1e-5, atol=1e-7)
    for k, v in (("wavefront_pool", 0), ("trace_blocks_per_sm", 0), ("wavefront_graph", 1)):
        ctx.set_option(k, v)


def test_batched_view_matches_the_fp64_renderer(ctx, scene_dirs):
    """A view rendered in a batch (wavefront, FP32) against the FP64 renderer drawing the same
    samples (a scene file with that view's camera, the view's spp and seed): the films agree to a
    relative RMSE below 5e-3, the film tolerance of the reference parity tests."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    d, sc, sub = scene_dirs["materials"]
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    films, _ = lts.render_views(s, VIEWS, 6, 3)
    for k in (1, 2):
        v = VIEWS[k]
        name = scenes.with_camera(d, sc, v, f"view{k}")
        sv = lts.Scene.parse(ctx, d, name, sub, v["width"], v["height"])
        ref = lts.PathTracingIntegrator(6, 3, sv, integrator=lts.INTEGRATOR_FP64).render(v["spp"], v["seed"])["film"]
        ref = ref.reshape(v["height"], v["width"], 3)
        err = np.sqrt(np.mean((films[k] - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
        print(f"view {k}: {v['width']}x{v['height']} {v['spp']} spp, rel-RMSE against FP64 {err:.3g}")
        assert err < 5e-3
