"""The two-level render BVH of scenes with instanced meshes (the loader's `instances` record, no
counterpart in the reference, whose scenes list one mesh file per placement): one 8-wide tree per
instanced mesh file under a top-level tree over the other triangles, each instance entered with
the ray moved to its object space.  The scene's triangle table stays the flattened one, so the
oracle's CPU port renders the same scene through its own flat BVH.

  * ray queries: the two-level tree finds the flat trees' closest hits and any-hit answers;
  * renders: per-sample parity against the port, with the event-hash rule of
    tests/test_render_gpu.py and a tolerance for the instances' own rounding;
  * memory: the two-level tree holds each prototype's triangles once."""
import os
import subprocess

import numpy as np
import pytest

from test_render_gpu import ATOL, ERR_SCALE, MAX_DIVERGENT, RTOL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def inst_scene(tmp_path_factory):
    """The stress scene with 64 x 128 conductor spheres (16,128 triangles each) as eight
    instances of one unit-sphere file."""
    from lighttransportsimulation_gb300 import scenes
    d = str(tmp_path_factory.mktemp("inst"))
    sc, sub = scenes.write_stress_scene(d, rings=64, segs=128, instanced=True)
    return d, sc, sub


def _rays(n, seed, centres):
    """Half the rays from random points of the box in random directions, half aimed at random
    points of random conductor spheres (so that most of those reach an instance)."""
    rng = np.random.default_rng(seed)
    o = rng.uniform(-0.95, 0.95, (n, 3)).astype(np.float32)
    d = rng.standard_normal((n, 3))
    m = n // 2
    tgt = centres[rng.integers(0, len(centres), m)] + 0.14 * rng.uniform(-1, 1, (m, 3))
    d[:m] = tgt - o[:m]
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def _centres(d, sc):
    """The instances' translations, read back from the scene file's `instances` record."""
    txt = open(os.path.join(d, sc + ".scene")).read().split("instances")[1].split("\n")[1:]
    return np.array([[float(x) for x in line.split("\t")[1].split()] for line in txt if line.strip()])


@pytest.mark.parametrize("watertight", [0, 1])
def test_ray_queries_match_the_flat_trees(ctx, inst_scene, watertight):
    """Closest hits and any-hit answers of 400,000 rays through the two-level tree against the flat
    8-wide tree and the binary LBVH over the flattened triangles.  The instance's triangles are
    tested in object space, so a hit's distance and barycentrics round differently: a ray that
    meets an edge shared by two triangles may take the other one (same distance), and a ray
    grazing a silhouette may hit in one and miss in the other; both stay below 0.1 %."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    d, sc, sub = inst_scene
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    assert s.info["instances"] == 8 and s.info["prototypes"] == 1
    per = len(scenes.uv_sphere(64, 128)[1])  # triangles per sphere; the glass sphere is mesh 0
    o, dr = _rays(400_000, 11 + watertight, _centres(d, sc))
    tmax = np.random.default_rng(5).uniform(0.05, 2.5, len(o)).astype(np.float32)
    ctx.set_option("watertight", watertight)
    out = {}
    try:
        for name, opts in (("two", dict(two_level_bvh=1, bvh_width=8)), ("flat", dict(two_level_bvh=0, bvh_width=8)),
                           ("binary", dict(two_level_bvh=1, bvh_width=2))):
            for k, v in opts.items():
                ctx.set_option(k, v)
            prim, t = s.intersect(o, dr)
            anyh = s.simple_intersect(o, dr, tmax)
            m = ctx.metrics()
            out[name] = (prim, t, anyh, m.render_two_level, m.render_bvh_bytes)
    finally:
        for k, v in (("two_level_bvh", 1), ("bvh_width", 8), ("watertight", 0)):
            ctx.set_option(k, v)
    p2, t2, a2, tl2, b2 = out["two"]
    pf, tf, af, tlf, bf = out["flat"]
    pb, tb, ab, _, _ = out["binary"]
    assert tl2 == 1 and tlf == 0
    ninst = (p2 >= per) & (p2 < 9 * per)
    diff = p2 != pf
    both = diff & (p2 >= 0) & (pf >= 0)
    hitmiss = (p2 >= 0) != (pf >= 0)
    rel = np.abs(t2[both] - tf[both]) / np.maximum(tf[both], 1e-3)
    same = ~diff & (p2 >= 0)
    rs = np.abs(t2[same] - tf[same]) / np.maximum(tf[same], 1e-3)
    print(f"watertight={watertight}: hits {np.mean(p2 >= 0):.4f}, on instances {ninst.mean():.4f}; "
          f"prim differs {diff.mean():.6f} (both hit {both.mean():.6f}, max rel dt {rel.max() if both.any() else 0:.2e}; "
          f"hit/miss {hitmiss.mean():.6f}); same prim: rel dt 99.99 % {np.quantile(rs, 0.9999):.2e}, max {rs.max():.2e}; "
          f"any-hit differs {np.mean(a2 != af):.6f}; flat vs binary differs {np.mean(pf != pb):.6f}; "
          f"BVH bytes two-level {b2}, flat {bf} ({b2 / bf:.3f})")
    assert ninst.mean() > 0.3
    assert diff.mean() <= 1e-3 and hitmiss.mean() <= 1e-3
    if watertight:  # no ray leaks: a different triangle is a neighbour at the same distance
        assert both.sum() == 0 or rel.max() <= 1e-4
    # the same triangle: the distance rounds differently in object space, most within a few ulps;
    # grazing hits (small determinant) amplify it
    assert np.quantile(rs, 0.9999) <= 5e-5 and rs.max() <= 1e-3
    assert np.mean(a2 != af) <= 1e-3
    assert b2 < 0.3 * bf


def test_two_level_render_matches_the_port(ctx, inst_scene, port_exe, tmp_path):
    """The whole 160 x 90 frame at 2 spp, 16 bounces, roulette from 4, through the megakernel and
    the wavefront integrators on the two-level tree, against the port's samples of the flattened
    scene: divergent event hash at most 1 % (as tests/test_render_gpu.py), and the other samples
    within that module's bound (1e-4 relative plus 1e-6 plus four times the port's own distance
    from the FP64 renderer's value) up to 0.1 % of them, all within 1e-2 relative."""
    import lighttransportsimulation_gb300 as lts
    from oracle import ltsd
    d, sc, sub = inst_scene
    w, h, spp, maxb, rr, seed = 160, 90, 2, 16, 4, 3
    out = str(tmp_path / "port.ltsd")
    args = (port_exe, "render", d + "/", sc, sub, out, w, h, spp, maxb, rr, seed, 0, 0, w, h, os.cpu_count(), 0, 0)
    subprocess.run([str(a) for a in args], check=True)
    ref = ltsd.read(out)
    Lr, sr = ref["L"].reshape(-1, 3), ref["sig"].reshape(-1)
    s = lts.Scene.parse(ctx, d, sc, sub, w, h)
    res = {}
    for integ in (lts.INTEGRATOR_FP64, lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
        r = lts.PathTracingIntegrator(maxb, rr, s, integrator=integ).render(spp, seed, record=True, film=False)
        res[integ] = (r["L"].reshape(-1, 3).copy(), r["sig"].reshape(-1).copy(), ctx.metrics().render_two_level)
    L64, s64, _ = res[lts.INTEGRATOR_FP64]
    assert Lr.mean() > 0
    worst = {}
    for integ in (lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
        L, sig, two = res[integ]
        assert two == 1
        same = (sig == sr) & (s64 == sr)
        bound = RTOL * np.abs(Lr) + ATOL + ERR_SCALE * np.abs(L64 - Lr)
        inside = np.all(np.abs(L - Lr) <= bound, axis=1)
        rel = np.max(np.abs(L - Lr) / (np.abs(Lr) + 1e-5), axis=1)
        worst[integ] = (1 - same.mean(), 1 - inside[same].mean(), rel[same].max())
        print(f"instanced stress integrator={integ}: divergent {1 - same.mean():.5f}, outside the flat path's bound "
              f"{np.sum(same & ~inside)} of {same.sum()}, worst relative difference {rel[same].max():.2e}")
        assert np.isfinite(L).all()
    # the flat path's rule (zero samples outside the bound) assumes the reference's rounding of
    # every hit; the instances' hits round in object space, so a few samples of long glossy or
    # glass paths drift a little further: at most 0.1 % of them, and none beyond 1e-2 relative
    for div, out, rel in worst.values():
        assert div <= MAX_DIVERGENT and out <= 1e-3 and rel <= 1e-2


def test_two_level_and_flat_films_agree(ctx, inst_scene):
    """The wavefront film through the two-level tree and through the flat tree, same samples: the
    same paths up to the hits that round differently, so the two films differ by far less than
    two films of different seeds do."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = inst_scene
    s = lts.Scene.parse(ctx, d, sc, sub, 192, 108)
    integ = lts.PathTracingIntegrator(16, 4, s, integrator=1)
    films = {}
    try:
        for tl, seed in ((1, 77), (0, 77), (0, 78)):
            ctx.set_option("two_level_bvh", tl)
            films[tl, seed] = integ.render(16, seed)["film"].astype(np.float64)
            assert ctx.metrics().render_two_level == tl
    finally:
        ctx.set_option("two_level_bvh", 1)
    same = np.sqrt(np.mean((films[1, 77] - films[0, 77]) ** 2))
    noise = np.sqrt(np.mean((films[0, 78] - films[0, 77]) ** 2))
    print(f"two-level vs flat film RMSE {same:.3e}; seed-to-seed RMSE {noise:.3e}")
    assert same < 0.1 * noise
