"""CPU tests: the oracle's C++ port reproduces the reference's own outputs bit for bit (LBVH,
per-sample radiance and event hashes, resolved film) on the committed fixtures."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def _run(exe, *args):
    subprocess.run([exe] + [str(a) for a in args], check=True)


@pytest.mark.parametrize("kind", ["box_sphere", "materials"])
def test_port_lbvh_bit_exact(port_exe, scene_dirs, kind, tmp_path):
    from oracle import ltsd
    d, sc, sub = scene_dirs[kind]
    fx = np.load(os.path.join(GOLDEN, f"lbvh_{kind}.npz"))
    meta = np.load(os.path.join(GOLDEN, f"render_{kind}.npz"))["meta"]
    out = tmp_path / "b.ltsd"
    _run(port_exe, "bvh", d + "/", sc, sub, out, int(meta[0]), int(meta[1]), 0)
    b = ltsd.read(out)
    for k in ("sorted_codes", "sorted_ids", "node_key", "node_left", "node_right", "node_bounds"):
        assert np.array_equal(b[k].view(np.uint32), fx[k].view(np.uint32)), k


@pytest.mark.parametrize("kind", ["box_sphere", "materials", "stress_small"])
def test_port_per_sample_radiance_bit_exact(port_exe, scene_dirs, kind, tmp_path):
    from oracle import ltsd
    d, sc, sub = scene_dirs[kind]
    fx = np.load(os.path.join(GOLDEN, f"render_{kind}.npz"))
    out = tmp_path / "r.ltsd"
    _run(port_exe, "render", d + "/", sc, sub, out, *[int(v) for v in fx["meta"]], 0, 0)
    r = ltsd.read(out)
    assert np.array_equal(r["L"].view(np.uint32), fx["L"].reshape(-1).view(np.uint32))
    assert np.array_equal(r["sig"], fx["sig"].reshape(-1))


@pytest.mark.parametrize("kind", ["box_sphere", "materials", "stress_small"])
def test_port_film_bit_exact(port_exe, scene_dirs, kind, tmp_path):
    from oracle import ltsd
    d, sc, sub = scene_dirs[kind]
    fx = np.load(os.path.join(GOLDEN, f"film_{kind}.npz"))
    w, h, spp, maxb, rr, seed = (int(v) for v in fx["meta"])
    out = tmp_path / "f.ltsd"
    _run(port_exe, "render", d + "/", sc, sub, out, w, h, spp, maxb, rr, seed, 0, 0, w, h, 1, 1)
    assert np.array_equal(ltsd.read(out)["film"].view(np.uint32), fx["film"].view(np.uint32))


def test_port_sorted_mode_matches_numpy(port_exe, tmp_path):
    """The port's textbook-LBVH mode against the numpy statement on a random soup."""
    from lighttransportsimulation_gb300 import scenes
    from oracle import lbvh_np, ltsd
    tris = scenes.random_triangles(20000, seed=4)
    src = tmp_path / "soup.f32"
    tris.reshape(-1).tofile(src)
    out = tmp_path / "b.ltsd"
    _run(port_exe, "bvhsoup", src, out, 1)
    b = ltsd.read(out)
    codes, ids = lbvh_np.stable_sort(*lbvh_np.morton_codes(tris))
    assert np.array_equal(b["sorted_codes"], codes) and np.array_equal(b["sorted_ids"], ids)
    left, right = lbvh_np.karras_topology(codes)
    n = len(tris)
    assert np.array_equal(b["node_left"][: n - 1], left) and np.array_equal(b["node_right"][: n - 1], right)
    mn, mx = lbvh_np.tri_bounds(tris)
    lbvh_np.check_tree(b["node_left"], b["node_right"], b["node_bounds"], np.concatenate([mn, mx], 1)[ids])
