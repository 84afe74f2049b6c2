"""The watertight triangle test (option "watertight", the fixed mode of the reference's
epsilon-shrunk Moller-Trumbore test) through the ray-query entry point lts_intersect.

Edge leaks: rays from a point near the centre of the closed icosphere (inside the box) aimed
exactly at its vertices and at the midpoints of its edges.  The reference's test rejects
barycentrics within 1e-4 of a triangle's border, so such rays slip between the triangles and
reach the box; the watertight test lets none through.  Away from edges both tests hit the same
triangle at the same distance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def box_scene(built_lib, tmp_path_factory):
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    d = str(tmp_path_factory.mktemp("wt"))
    sc, sub = scenes.write_box_sphere(d, level=4)
    ctx = lts.Context(0)
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    v, f = scenes.icosphere(4)
    yield ctx, s, (v * 0.5).astype(np.float32), f
    ctx.close()


def _edge_and_vertex_dirs(v, f):
    edges = set()
    for a, b, c in f:
        for x, y in ((a, b), (b, c), (c, a)):
            edges.add((min(x, y), max(x, y)))
    e = np.array(sorted(edges))
    mids = 0.5 * (v[e[:, 0]].astype(np.float64) + v[e[:, 1]])
    return np.concatenate([v.astype(np.float64), mids]).astype(np.float32)


@pytest.mark.parametrize("width", [8, 2])
def test_no_ray_leaks_through_edges_or_vertices(box_scene, width):
    ctx, s, v, f = box_scene
    nsphere = len(f)  # subject meshes come first in scene order
    # from a point near the centre (not on it: from the centre, rays with a zero direction
    # component start on the planes of boxes that touch the coordinate planes, where the slab
    # test's (plane - origin) / d is 0 / 0; that is the box test's degenerate case, not the
    # triangle test's), through the mesh's vertices and edge midpoints
    org = np.broadcast_to(np.array([1e-3, 2e-3, -1.5e-3], np.float32), (1, 3))
    dirs = (_edge_and_vertex_dirs(v, f) - org).astype(np.float32)
    org = np.repeat(org, len(dirs), axis=0)
    ctx.set_option("bvh_width", width)
    try:
        ctx.set_option("watertight", 0)
        p0, _ = s.intersect(org, dirs)
        ctx.set_option("watertight", 1)
        p1, t1 = s.intersect(org, dirs)
    finally:
        ctx.set_option("watertight", 0)
        ctx.set_option("bvh_width", 8)
    leak0 = np.mean((p0 < 0) | (p0 >= nsphere))
    leak1 = np.mean((p1 < 0) | (p1 >= nsphere))
    print(f"width {width}: {len(dirs)} rays through vertices and edge midpoints; leaked {leak0:.3f} with the "
          f"reference's test, {leak1:.3f} watertight")
    assert leak0 > 0.5      # the reference's test misses most of them
    assert leak1 == 0.0     # the watertight test none
    assert np.allclose(t1, 1.0, rtol=1e-4)  # d runs from the origin to the vertex / midpoint: t = 1


def test_watertight_equals_reference_away_from_edges(box_scene):
    ctx, s, v, f = box_scene
    rng = np.random.default_rng(12)
    n = 20000
    org = rng.uniform(-0.9, 0.9, (n, 3)).astype(np.float32)
    org[:, 2] = rng.uniform(0.6, 0.9, n)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ctx.set_option("watertight", 0)
    p0, t0 = s.intersect(org, d)
    occ0 = s.simple_intersect(org, d, 0.5)
    ctx.set_option("watertight", 1)
    try:
        p1, t1 = s.intersect(org, d)
        occ1 = s.simple_intersect(org, d, 0.5)
    finally:
        ctx.set_option("watertight", 0)
    same = p0 == p1
    print(f"same closest primitive {same.mean():.5f}; same occlusion {np.mean(occ0 == occ1):.5f}")
    assert same.mean() > 0.998 and np.mean(occ0 == occ1) > 0.998
    hit = same & (p0 >= 0)
    assert np.allclose(t1[hit], t0[hit], rtol=1e-5, atol=1e-6)
