"""GPU parity of the LBVH build (through the C-ABI) against the reference's own builds and the
numpy statement of its arithmetic."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


def _u32(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("kind", ["box_sphere", "materials", "closeup_diamond", "closeup_moai", "bigbox_diamond"])
def test_reference_mode_bit_exact(ctx, scene_dirs, kind):
    """Codes, stable order, children and every node's AABB bit pattern equal the reference's."""
    import lighttransportsimulation_gb300 as lts
    d, sc, sub = scene_dirs[kind]
    fx = np.load(os.path.join(GOLDEN, f"lbvh_{kind}.npz"))
    meta = np.load(os.path.join(GOLDEN, f"render_{kind}.npz"))["meta"]
    s = lts.Scene.parse(ctx, d, sc, sub, int(meta[0]), int(meta[1]))
    out = s.create_bvh_tree(lts.BVH_REFERENCE)
    assert np.array_equal(out["sorted_codes"], fx["sorted_codes"])
    assert np.array_equal(out["sorted_ids"], fx["sorted_ids"])
    assert np.array_equal(out["node_left"], fx["node_left"])
    assert np.array_equal(out["node_right"], fx["node_right"])
    assert np.array_equal(out["node_key"], fx["node_key"])
    assert np.array_equal(_u32(out["node_bounds"]), _u32(fx["node_bounds"]))


@pytest.mark.parametrize("kind", ["box_sphere", "materials"])
def test_sorted_mode_is_the_textbook_lbvh(ctx, scene_dirs, kind):
    """Every primitive coded; leaf l holds ids[l]; same topology rules; boxes consistent."""
    import lighttransportsimulation_gb300 as lts
    from oracle import lbvh_np
    d, sc, sub = scene_dirs[kind]
    s = lts.Scene.parse(ctx, d, sc, sub, 64, 64)
    out = s.create_bvh_tree(lts.BVH_SORTED)
    tris = s.triangles()
    codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris))
    assert np.array_equal(out["sorted_codes"], codes) and np.array_equal(out["sorted_ids"], ids)
    left, right = lbvh_np.karras_topology(codes)
    n = len(tris)
    assert np.array_equal(out["node_left"][: n - 1], left) and np.array_equal(out["node_right"][: n - 1], right)
    mn, mx = lbvh_np.tri_bounds(tris)
    lbvh_np.check_tree(out["node_left"], out["node_right"], out["node_bounds"], np.concatenate([mn, mx], 1)[ids])


@pytest.mark.parametrize("n", [1, 2, 3, 17, 511, 512, 513, 1025, 3841, 100_003])
def test_edge_sizes(ctx, n):
    """Single primitive, tiny trees, sizes at the tree kernel's 512-leaf blocks and straddling the
    sort tile (3840 keys)."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from oracle import lbvh_np
    tris = scenes.random_triangles(n, seed=n)
    out = lts.build_bvh_triangles(ctx, tris, lts.BVH_SORTED)
    codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris))
    assert np.array_equal(out["sorted_codes"], codes) and np.array_equal(out["sorted_ids"], ids)
    mn, mx = lbvh_np.tri_bounds(tris)
    if n == 1:
        assert np.array_equal(_u32(out["node_bounds"]), _u32(np.concatenate([mn, mx], 1).reshape(-1)))
        return
    left, right = lbvh_np.karras_topology(codes)
    assert np.array_equal(out["node_left"][: n - 1], left) and np.array_equal(out["node_right"][: n - 1], right)
    lbvh_np.check_tree(out["node_left"], out["node_right"], out["node_bounds"], np.concatenate([mn, mx], 1)[ids])


def test_duplicate_codes_keep_stable_order(ctx):
    """Many equal centroids: equal codes keep input order; delta's index tie-break shapes the tree."""
    import lighttransportsimulation_gb300 as lts
    from oracle import lbvh_np
    rng = np.random.default_rng(3)
    base = rng.random((50, 1, 3), dtype=np.float32)
    tris = np.repeat(base, 200, axis=0) + np.zeros((1, 3, 3), np.float32)
    tris = tris[rng.permutation(len(tris))]
    out = lts.build_bvh_triangles(ctx, tris, lts.BVH_SORTED)
    codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris))
    assert np.array_equal(out["sorted_codes"], codes) and np.array_equal(out["sorted_ids"], ids)
    left, right = lbvh_np.karras_topology(codes)
    n = len(tris)
    assert np.array_equal(out["node_left"][: n - 1], left) and np.array_equal(out["node_right"][: n - 1], right)


def test_rebuilds_reuse_the_arrival_words(ctx):
    """Builds of different sizes in one context (the tree's arrival words are reused across builds
    without clearing): every build's topology and boxes are those of a fresh build."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from oracle import lbvh_np
    for n, seed in ((70_001, 4), (4_097, 5), (70_001, 6), (70_001, 4)):
        tris = scenes.random_triangles(n, seed=seed)
        out = lts.build_bvh_triangles(ctx, tris, lts.BVH_SORTED)
        codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris))
        left, right = lbvh_np.karras_topology(codes)
        assert np.array_equal(out["node_left"][: n - 1], left) and np.array_equal(out["node_right"][: n - 1], right)
        mn, mx = lbvh_np.tri_bounds(tris)
        lbvh_np.check_tree(out["node_left"], out["node_right"], out["node_bounds"], np.concatenate([mn, mx], 1)[ids])


def test_rebuilds_across_epoch_wraps(built_lib):
    """The tree's arrival words carry the build's epoch (127 epochs) instead of being cleared per
    build; they are cleared when the epoch wraps.  Build 0 sizes the buffers (60,001 triangles);
    build 2 (60,001) has epoch 3; build 33 (30,001) rewrites the first half of the words; the wrap
    falls on a 3,001-triangle build (127); build 129 (60,001, other triangles) has epoch 3 again
    over words past 30,000 that still hold build 2's.  Every build must equal a fresh build."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from oracle import lbvh_np
    cases = {}
    for key, n, seed in (("big_x", 60_001, 10), ("big_a", 60_001, 11), ("mid", 30_001, 12), ("big_c", 60_001, 13),
                         ("small", 3_001, 14)):
        tris = scenes.random_triangles(n, seed=seed)
        codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris))
        cases[key] = (tris, codes, ids, *lbvh_np.karras_topology(codes))
    c = lts.Context(0)  # a fresh context: its builds start at epoch 1
    try:
        for k in range(130):
            key = {0: "big_x", 2: "big_a", 33: "mid", 129: "big_c"}.get(k, "small")
            tris, codes, ids, left, right = cases[key]
            out = lts.build_bvh_triangles(c, tris, lts.BVH_SORTED)
            n = len(tris)
            assert np.array_equal(out["sorted_codes"], codes) and np.array_equal(out["sorted_ids"], ids), (k, key)
            assert np.array_equal(out["node_left"][: n - 1], left), (k, key)
            assert np.array_equal(out["node_right"][: n - 1], right), (k, key)
    finally:
        c.close()


@pytest.mark.parametrize("n", [1_000_000, 16_000_000])
def test_benchmark_sizes_both_modes(ctx, n):
    """The build benchmark's random triangles (seed 1) at 1M and 16M, in the reference's mode
    (leaf l holds primitive l) and the sorted-leaf mode: codes, stable order and topology
    bit-exact against the numpy statement; every interior box the union of its children and
    every leaf box its primitive's, bit for bit."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from oracle import lbvh_np
    tris = scenes.random_triangles(n, seed=1)
    codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris))
    left, right = lbvh_np.karras_topology(codes)
    mn, mx = lbvh_np.tri_bounds(tris)
    boxes = np.concatenate([mn, mx], 1)
    for mode in (lts.BVH_REFERENCE, lts.BVH_SORTED):
        out = lts.build_bvh_triangles(ctx, tris, mode)
        assert np.array_equal(out["sorted_codes"], codes) and np.array_equal(out["sorted_ids"], ids)
        assert np.array_equal(out["node_left"][: n - 1], left) and np.array_equal(out["node_right"][: n - 1], right)
        lbvh_np.check_tree(out["node_left"], out["node_right"], out["node_bounds"],
                           boxes if mode == lts.BVH_REFERENCE else boxes[ids])
        del out


def test_reference_mode_code_limit(ctx):
    """Primitives past the reference's Morton launch extent keep code 0 and id 0."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from oracle import lbvh_np
    tris = scenes.random_triangles(5000, seed=9)
    out = lts.build_bvh_triangles(ctx, tris, lts.BVH_REFERENCE, code_limit=4096)
    codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris, code_limit=4096))
    assert np.array_equal(out["sorted_codes"], codes) and np.array_equal(out["sorted_ids"], ids)
    mn, mx = lbvh_np.tri_bounds(tris)
    lbvh_np.check_tree(out["node_left"], out["node_right"], out["node_bounds"], np.concatenate([mn, mx], 1))


def test_reference_mode_on_the_bench_scene(ctx, tmp_path):
    """The displaced-icosphere bench scene (1,310,732 triangles) in the reference's mode: codes,
    order, children and every node box have the sha256 digests of the reference's own build
    (tests/golden/digest_displaced.npz)."""
    import hashlib

    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    z = np.load(os.path.join(GOLDEN, "digest_displaced.npz"))
    d = str(tmp_path)
    scenes.write_displaced(d, level=8)
    s = lts.Scene.parse(ctx, d, "box", "displaced", 1024, 1024)
    out = s.create_bvh_tree(lts.BVH_REFERENCE)
    for k in ("sorted_codes", "sorted_ids", "node_key", "node_left", "node_right", "node_bounds"):
        assert hashlib.sha256(np.ascontiguousarray(out[k]).tobytes()).hexdigest() == str(z[k]), k


def test_reference_mode_on_the_dragon_scene(ctx, tmp_path):
    """The reference's res/blackDragon subject on res/platforms/closeupPlane (37,986 triangles) in
    the reference's mode: codes, order, children and every node box have the sha256 digests of
    the reference's own build (tests/golden/digest_dragon.npz)."""
    import hashlib

    import lighttransportsimulation_gb300 as lts
    from conftest import write_dragon
    z = np.load(os.path.join(GOLDEN, "digest_dragon.npz"))
    root, sc, sub = write_dragon(str(tmp_path))
    s = lts.Scene.parse(ctx, root, sc, sub, 480, 270)
    out = s.create_bvh_tree(lts.BVH_REFERENCE)
    for k in ("sorted_codes", "sorted_ids", "node_key", "node_left", "node_right", "node_bounds"):
        assert hashlib.sha256(np.ascontiguousarray(out[k]).tobytes()).hexdigest() == str(z[k]), k
