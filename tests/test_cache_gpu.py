"""The radiance cache inside the wavefront renderer: paths end in the MLP after their first rough
vertex, 3 % (here more) are traced in full and train it online; the cache has to pay for itself
in image error at equal samples."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


def _rmse(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)))


def test_cache_off_is_the_plain_renderer(ctx, scene_dirs):
    """With the option off the wavefront renders exactly what it rendered before (bit-identical
    film), even after an MLP exists."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["box_sphere"]
    s = lts.Scene.parse(ctx, d, sc, sub, 96, 96)
    integ = lts.PathTracingIntegrator(5, 3, s, integrator=1)
    f0 = integ.render(8, 3)["film"]
    lts.RadianceCacheMLP(ctx, seed=1)
    ctx.set_option("radiance_cache", 0)
    f1 = integ.render(8, 3)["film"]
    assert np.array_equal(f0.view(np.uint32), f1.view(np.uint32))


def test_cache_trains_online_and_beats_plain_at_equal_spp(ctx, scene_dirs):
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["box_sphere"]
    W = H = 128
    s = lts.Scene.parse(ctx, d, sc, sub, W, H)
    integ = lts.PathTracingIntegrator(5, 3, s, integrator=1)
    ref = integ.render(2048, 101)["film"]               # plain, high spp
    plain = integ.render(4, 7)["film"]
    lts.RadianceCacheMLP(ctx, seed=5)
    ctx.set_option("radiance_cache", 1)
    ctx.set_option("radiance_cache_unbiased_permille", 200)
    ctx.set_option("radiance_cache_lr_micro", 3000)
    try:
        losses, biases = [], []
        for frame in range(60):
            r = integ.render(4, 1000 + frame)
            m = ctx.metrics()
            assert m.cache_queries > 0 and m.cache_train_samples > 0
            losses.append(m.cache_train_loss)
            biases.append(m.cache_bias)
        cached = r["film"]
    finally:
        ctx.set_option("radiance_cache", 0)
    e_plain, e_cached = _rmse(plain, ref), _rmse(cached, ref)
    print(f"loss {losses[0]:.4f} -> {losses[-1]:.4f}; bias {biases[0]:+.3f} -> {biases[-1]:+.3f}; "
          f"RMSE at 4 spp: plain {e_plain:.4f}, cached {e_cached:.4f}")
    assert np.isfinite(cached).all()
    assert np.mean(losses[-10:]) < np.mean(losses[:5])
    assert abs(np.mean(biases[-10:])) < 0.1
    assert e_cached < e_plain
