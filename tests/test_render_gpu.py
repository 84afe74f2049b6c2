"""GPU parity of the path tracer (through the C-ABI) against the reference integrator's own
per-(pixel, sample) radiance, with the shared project sampler.  The stress scene's rough
conductors cannot be loaded by the reference, so its fixtures come from the oracle port, which
is bit-exact to the reference on every scene the reference can load.

Rule (float renderers; the library is built without FMA contraction, as the reference's host
build rounds):
  * divergent: the sample's event hash (hit primitive per bounce, shadow visibility, MIS-ray hit,
    texture branch decisions, the BSDF's reflect / same-hemisphere tests) differs from the
    reference's, or the FP64 renderer's hash for the same sample does: a decision taken at a
    grazing hit or an epsilon boundary, where exact arithmetic goes the other way.  At most 1 %
    of the samples may be divergent.
  * every other sample: |L - L_ref| <= 1e-4 |L_ref| + 1e-6 + 4 |L_fp64 - L_ref| per channel, and no
    sample may fail (MAX_MISMATCH = 0).  |L_fp64 - L_ref| is the reference's own rounding error on
    that path, measured against the same path evaluated in double: where the reference's float
    value is itself that far from the exact value (long mirror, glass and glossy chains amplify the
    last-bit differences of single operations, including the transcendentals of two libms), a
    second correct float evaluation differs from it by that much as well.  On paths the reference
    evaluates accurately the bound is the FP32 parity tolerance, 1e-4.

The FP64 renderer itself is held to 1e-2 per sample (it does not round like the reference's
float code); on the stress scene at most 0.1 % of its samples may leave the 5e-2 bound.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-4, 1e-6
MAX_DIVERGENT = 0.01   # fraction of samples flagged divergent
MAX_MISMATCH = 0       # non-divergent samples outside the bound
ERR_SCALE = 4.0        # multiple of the reference's own rounding error added to the bound
DRIFT_RTOL = 5e-2      # bound on every non-divergent sample of the FP64 renderer


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def fp64_samples(ctx, scene_dirs):
    """Per-sample radiance and event hashes of the FP64 renderer on each fixture's crop."""
    import lighttransportsimulation_gb300 as lts
    cache = {}

    def get(kind):
        if kind not in cache:
            d, sc, sub = scene_dirs[kind]
            fx = np.load(os.path.join(GOLDEN, f"render_{kind}.npz"))
            w, h, spp, maxb, rr, seed, x0, y0, x1, y1 = (int(v) for v in fx["meta"])
            s = lts.Scene.parse(ctx, d, sc, sub, w, h)
            r = lts.PathTracingIntegrator(maxb, rr, s, integrator=lts.INTEGRATOR_FP64).render(
                spp, seed, crop=(x0, y0, x1, y1), record=True, film=False)
            cache[kind] = (r["L"].reshape(-1, 3).copy(), r["sig"].reshape(-1).copy())
        return cache[kind]
    return get


def check_samples(L, sig, Lr, sr, L64, s64, label):
    """The parity rule of this module over one crop; returns (divergent share, worst excess)."""
    same = (sig == sr) & (s64 == sr)
    bound = RTOL * np.abs(Lr) + ATOL + ERR_SCALE * np.abs(L64 - Lr)
    ok = np.all(np.abs(L - Lr) <= bound, axis=1)
    bad = np.where(same & ~ok)[0]
    within = np.all(np.abs(L - Lr) <= RTOL * np.abs(Lr) + ATOL, axis=1)
    print(f"{label}: samples={len(sig)} divergent={1 - same.mean():.5f} (renderer {np.mean(sig != sr):.5f}, "
          f"fp64 {np.mean(s64 != sr):.5f}); within 1e-4 {within[same].mean():.6f}; outside the bound {len(bad)}; "
          f"bit-exact {np.mean(np.all(L.view(np.uint32) == Lr.view(np.uint32), axis=1)):.4f}")
    for k in bad[:5]:
        print(f"  sample {k}: L={L[k]} ref={Lr[k]} fp64={L64[k]}")
    assert np.isfinite(L).all()
    assert 1.0 - same.mean() <= MAX_DIVERGENT
    assert len(bad) <= MAX_MISMATCH


KINDS = ["box_sphere", "materials", "stress_small", "closeup_diamond", "closeup_moai", "bigbox_diamond"]


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("bvh_mode,integrator,width", [(0, 0, 2), (0, 1, 8), (1, 0, 8), (1, 1, 8), (1, 1, 2), (1, 2, 2)])
def test_per_sample_radiance(ctx, scene_dirs, fp64_samples, kind, bvh_mode, integrator, width):
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs[kind]
    fx = np.load(os.path.join(GOLDEN, f"render_{kind}.npz"))
    w, h, spp, maxb, rr, seed, x0, y0, x1, y1 = (int(v) for v in fx["meta"])
    L64, s64 = fp64_samples(kind) if integrator != 2 else (None, None)
    s = lts.Scene.parse(ctx, d, sc, sub, w, h)
    integ = lts.PathTracingIntegrator(maxb, rr, s, integrator=integrator, bvh_mode=bvh_mode)
    ctx.set_option("bvh_width", width)
    try:
        r = integ.render(spp, seed, crop=(x0, y0, x1, y1), record=True, film=False)
    finally:
        ctx.set_option("bvh_width", 8)
    L = r["L"].reshape(-1, 3)
    sig = r["sig"].reshape(-1)
    Lr = fx["L"].reshape(-1, 3)
    sr = fx["sig"].reshape(-1)
    label = f"{kind} bvh={bvh_mode} integrator={integrator} width={width}"
    if integrator != 2:
        check_samples(L, sig, Lr, sr, L64, s64, label)
        return
    # the FP64 renderer: same decisions as the reference (<= 1 % divergent), values to 1e-2
    same = sig == sr
    ok = np.all(np.abs(L - Lr) <= 1e-2 * np.abs(Lr) + ATOL, axis=1)
    print(f"{label}: samples={len(sig)} divergent={1 - same.mean():.5f} outside 1e-2 {1 - ok[same].mean():.6f}")
    assert np.isfinite(L).all()
    assert 1.0 - same.mean() <= MAX_DIVERGENT
    assert 1.0 - ok[same].mean() <= (0.005 if kind != "stress_small" else 0.01)
    drift = np.all(np.abs(L - Lr) <= DRIFT_RTOL * np.abs(Lr) + 1e-5, axis=1)
    bad = np.where(same & ~drift)[0]
    if kind == "stress_small":
        assert len(bad) <= 0.001 * same.sum()
    else:
        assert drift[same].all()


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("integrator", [0, 1, 2])
def test_film_matches_reference(ctx, scene_dirs, kind, integrator):
    """Full-frame film (Kahan FP32 + FP64 resolve) against the reference's single-thread film."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs[kind]
    fx = np.load(os.path.join(GOLDEN, f"film_{kind}.npz"))
    w, h, spp, maxb, rr, seed = (int(v) for v in fx["meta"])
    s = lts.Scene.parse(ctx, d, sc, sub, w, h)
    r = lts.PathTracingIntegrator(maxb, rr, s, integrator=integrator).render(spp, seed)
    film = r["film"].reshape(-1)
    ref = fx["film"].reshape(-1)
    err = np.abs(film - ref)
    rel_rmse = np.sqrt(np.mean(err ** 2)) / np.sqrt(np.mean(ref ** 2))
    print(f"{kind} integrator={integrator}: film rel-RMSE vs reference {rel_rmse:.3g}, pixels off by >1e-3 rel: "
          f"{np.mean(err > 1e-3 * np.abs(ref) + 1e-5):.4f}")
    # the FP64 renderer takes other decisions at grazing and epsilon boundaries than the float
    # reference (its per-sample bound is 1e-2), so its films are held to 1e-2
    assert rel_rmse < (5e-3 if integrator != 2 else 1e-2)


def test_wavefront_equals_megakernel_bit_for_bit(ctx, scene_dirs):
    """Same device functions, different schedule: every sample takes the same decisions (identical
    event hashes) and, with no multiply-add contracted, the same radiance bit for bit."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["materials"]
    s = lts.Scene.parse(ctx, d, sc, sub, 96, 96)
    a = lts.PathTracingIntegrator(8, 3, s, integrator=0).render(4, 11, crop=(0, 0, 96, 96), record=True, film=False)
    b = lts.PathTracingIntegrator(8, 3, s, integrator=1).render(4, 11, crop=(0, 0, 96, 96), record=True, film=False)
    assert np.array_equal(a["sig"], b["sig"])
    La, Lb = a["L"].reshape(-1, 3), b["L"].reshape(-1, 3)
    ok = np.all(np.abs(La - Lb) <= RTOL * np.abs(La) + ATOL, axis=1)
    print(f"wavefront vs megakernel: bit-equal {np.mean(np.all(La == Lb, axis=1)):.4f}, within 1e-4 {ok.mean():.5f}")
    assert np.array_equal(La.view(np.uint32), Lb.view(np.uint32))


def test_wavefront_chunked_small_pool(ctx, scene_dirs):
    """A 1,000-path pool and 3-sample chunks (several drains and film gathers) give the same
    decisions, radiance and film as one chunk with the default pool."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["materials"]
    w = h = 64
    s = lts.Scene.parse(ctx, d, sc, sub, w, h)
    a = lts.PathTracingIntegrator(8, 3, s, integrator=1).render(8, 5, record=True)
    ctx.set_option("wavefront_pool", 1000)
    ctx.set_option("wavefront_sample_chunk", w * h * 3)
    try:
        b = lts.PathTracingIntegrator(8, 3, s, integrator=1).render(8, 5, record=True)
    finally:
        ctx.set_option("wavefront_pool", 0)
        ctx.set_option("wavefront_sample_chunk", 0)
    assert np.array_equal(a["sig"], b["sig"])
    La, Lb = a["L"].reshape(-1, 3), b["L"].reshape(-1, 3)
    assert np.all(np.abs(La - Lb) <= DRIFT_RTOL * np.abs(La) + 1e-5)
    fa, fb = a["film"].reshape(-1), b["film"].reshape(-1)
    assert np.all(np.abs(fa - fb) <= 1e-5 * np.abs(fa) + 1e-7)


def test_wavefront_film_reproducible(ctx, scene_dirs):
    """The gathered film has no atomics on its main path: two renders are bit-identical."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["box_sphere"]
    s = lts.Scene.parse(ctx, d, sc, sub, 96, 80)
    integ = lts.PathTracingIntegrator(5, 3, s, integrator=1)
    f1 = integ.render(16, 3)["film"]
    f2 = integ.render(16, 3)["film"]
    assert np.array_equal(f1.view(np.uint32), f2.view(np.uint32))


@pytest.mark.parametrize("kind", ["materials", "soup"])
def test_wide_bvh_same_hits_as_binary(ctx, scene_dirs, tmp_path, kind):
    """The 8-wide compressed BVH (conservative quantised boxes) finds the binary LBVH's closest
    hits: identical event hashes and bit-identical radiance wherever no exact tie between two
    triangles decided the hit."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    if kind == "soup":
        d = str(tmp_path)
        sc, sub = scenes.write_random_tris(d, 20000, seed=7)
    else:
        d, sc, sub = scene_dirs[kind]
    s = lts.Scene.parse(ctx, d, sc, sub, 128, 96)
    integ = lts.PathTracingIntegrator(6, 3, s, integrator=1)
    out = {}
    for width in (2, 8):
        ctx.set_option("bvh_width", width)
        out[width] = integ.render(4, 9, record=True, film=False)
    ctx.set_option("bvh_width", 8)
    a, b = out[2], out[8]
    same = a["sig"].reshape(-1) == b["sig"].reshape(-1)
    print(f"{kind}: hash-equal {same.mean():.6f}")
    assert same.mean() >= 0.999
    La, Lb = a["L"].reshape(-1, 3)[same], b["L"].reshape(-1, 3)[same]
    assert np.array_equal(La.view(np.uint32), Lb.view(np.uint32))


def test_fp64_oracle_converges_to_fp32_estimator(ctx, scene_dirs):
    """The FP64 renderer computes the same estimator: a 256-spp FP64 film and a 256-spp FP32
    wavefront film of the same seed agree far below their Monte Carlo noise, and the RMSE of 16-spp
    FP32 films against the FP64 film falls as more samples are taken."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["box_sphere"]
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    ref = lts.PathTracingIntegrator(5, 3, s, integrator=lts.INTEGRATOR_FP64).render(256, 1)["film"]
    same = lts.PathTracingIntegrator(5, 3, s, integrator=1).render(256, 1)["film"]
    rel = np.sqrt(np.mean((same - ref) ** 2)) / np.sqrt(np.mean(ref ** 2))
    print(f"fp32 vs fp64, same samples: rel-RMSE {rel:.2e}")
    assert rel < 1e-3
    errs = []
    for spp in (4, 16, 64):
        f = lts.PathTracingIntegrator(5, 3, s, integrator=1).render(spp, 7)["film"]
        errs.append(np.sqrt(np.mean((f - ref) ** 2)))
    print("RMSE vs FP64 at 4/16/64 spp:", errs)
    assert errs[0] > errs[1] > errs[2]


def test_graph_and_kernel_by_kernel_iterations_agree(ctx, scene_dirs):
    """The wavefront iteration launched as captured CUDA graphs (grids for the largest lists,
    control on the device) renders exactly what the kernel-by-kernel loop renders."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs["materials"]
    s = lts.Scene.parse(ctx, d, sc, sub, 80, 64)
    integ = lts.PathTracingIntegrator(8, 3, s, integrator=1)
    out = {}
    for g in (1, 0):
        ctx.set_option("wavefront_graph", g)
        out[g] = integ.render(8, 21, record=True)
    ctx.set_option("wavefront_graph", 1)
    assert np.array_equal(out[0]["sig"], out[1]["sig"])
    assert np.array_equal(out[0]["L"].view(np.uint32), out[1]["L"].view(np.uint32))
    assert np.array_equal(out[0]["film"].view(np.uint32), out[1]["film"].view(np.uint32))


@pytest.mark.parametrize("kind", ["box_sphere", "materials"])
def test_render_bvh_choice_finds_the_same_hits(ctx, scene_dirs, kind):
    """The 8-wide BVH collapsed from the PLOC tree (render_bvh 1: SAH-optimal collapse, 2:
    greedy) and from the LBVH itself (render_bvh 0) traverse the same triangles: the per-sample
    hit and visibility signatures agree except where a ray meets an edge shared by two triangles
    at the same distance (the test order then picks one of them), and the radiance agrees to
    1e-4."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs[kind]
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    integ = lts.PathTracingIntegrator(8, 3, s, integrator=1)
    out = {}
    for rb in (0, 1, 2):
        ctx.set_option("render_bvh", rb)
        out[rb] = integ.render(8, 5, record=True)
    ctx.set_option("render_bvh", 1)
    for rb in (1, 2):
        same = (out[0]["sig"] == out[rb]["sig"]).reshape(-1)
        assert same.mean() >= 0.999
        a, b = out[0]["L"].reshape(-1, 3)[same], out[rb]["L"].reshape(-1, 3)[same]
        assert np.all(np.abs(a - b) <= 1e-4 * np.maximum(1.0, np.abs(a)))


@pytest.mark.parametrize("integrator", ["megakernel", "wavefront"])
def test_host_program_writes_the_render(ctx, tmp_path, integrator):
    """The C host program (host/render_app.c) renders app.params' scene and writes the image the
    Python API writes for the same render (same film bytes)."""
    import subprocess

    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import build, scenes
    d = str(tmp_path)
    sc, sub = scenes.write_box_sphere(d)
    scenes.write_app_params(os.path.join(d, "app.params"), 64, 48, 4, 5, 3, 1, "out", sc, sub)
    r = subprocess.run([build.APP, d, "--seed", "9", "--integrator", integrator], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 48)
    res = lts.PathTracingIntegrator(5, 3, s, integrator={"megakernel": 0, "wavefront": 1}[integrator]).render(4, 9)
    lts.write_image(os.path.join(d, "py.pfm"), res["film"].reshape(48, 64, 3), 1)
    a = open(os.path.join(d, "out.pfm"), "rb").read()
    b = open(os.path.join(d, "py.pfm"), "rb").read()
    assert a == b
