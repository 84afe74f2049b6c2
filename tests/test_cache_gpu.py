"""The radiance cache inside the wavefront renderer: paths end in the MLP at the first rough vertex
after their first rough one, 3 % (here more) are traced in full and train it online; the cache
has to pay for itself in image error at equal samples and at equal device time."""
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
    assert e_cached < 0.9 * e_plain


def test_cache_at_config3_settings_beats_plain_wavefront_at_equal_time(ctx, scene_dirs):
    """The stress scene (glass, rough conductors, marble floor, area + infinite light) at the
    cached workload's settings: 3 % of paths traced in full, Adam at lr 1e-3, 65,536 training
    records per frame, 16 bounces, roulette from 4, on a 960 x 540 film (~30,000 records per
    frame).  Against a 4096-spp plain render: the cached renderer's image bias stays within 5 %
    and its full-frame RMSE is at least 10 % below the plain wavefront's after the same device
    time (both accumulate frames; the cached time includes its warm-up frames, the bias check and
    the Adam steps; measured: 0.0130 against 0.0173 after 600 ms).  The floor's caustic under the
    glass sphere is in the frame: it holds only because paths are traced through specular
    vertices to the next rough one before they end in the cache."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["stress_small"]
    W, H = 960, 540
    s = lts.Scene.parse(ctx, d, sc, sub, W, H)
    integ = lts.PathTracingIntegrator(16, 4, s, integrator=1)
    ref = None
    for k in range(4):
        ctx.set_option("film_accumulate", 0 if k == 0 else 1)
        ref = integ.render(1024, 500 + k)["film"].astype(np.float64)

    def accumulate(budget_ms, spp, cached):
        t, frame, img = 0.0, 0, None
        if cached:
            for k in range(8):  # warm-up frames: training only
                ctx.set_option("film_accumulate", 0)
                t += integ.render(1, 9000 + k, film=False)["render_ms"]
        while t < budget_ms:
            ctx.set_option("film_accumulate", 0 if frame == 0 else 1)
            r = integ.render(spp, 100 + frame)
            t += r["render_ms"]
            frame += 1
            img = r["film"].astype(np.float64)
        return img, t, frame

    try:
        lts.RadianceCacheMLP(ctx, seed=7)
        ctx.set_option("radiance_cache", 1)
        for k, v in (("radiance_cache_unbiased_permille", 30), ("radiance_cache_lr_micro", 1000),
                     ("radiance_cache_train_samples", 65536)):
            ctx.set_option(k, v)
        cached, t_cached, n_cached = accumulate(600.0, 4, True)
        m = ctx.metrics()
        ctx.set_option("radiance_cache", 0)
        plain, t_plain, n_plain = accumulate(t_cached, 4, False)
    finally:
        ctx.set_option("radiance_cache", 0)
        ctx.set_option("film_accumulate", 0)
    bias = (cached.mean() - ref.mean()) / ref.mean()
    e_plain, e_cached = _rmse(plain, ref), _rmse(cached, ref)
    print(f"{n_cached} cached frames in {t_cached:.0f} ms, {n_plain} plain frames in {t_plain:.0f} ms; "
          f"RMSE plain {e_plain:.4f}, cached {e_cached:.4f}; image bias {bias:+.4f}; "
          f"record bias {m.cache_bias:+.3f}, records {m.cache_train_samples}")
    assert np.isfinite(cached).all() and m.cache_train_samples > 0
    assert abs(bias) < 0.05
    assert e_cached < 0.9 * e_plain
