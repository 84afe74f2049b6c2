"""Regenerates the host I/O golden fixtures from the reference itself.

Runs oracle/_ref/lts_ref -- tierChampion/LightTransportSimulation's own sources compiled for the
host by oracle/ref/build_ref.sh -- and stores under tests/golden/io/:

  sphere_a.obj, sphere_b.obj   seeded OBJ inputs written here (icosphere level 2).  sphere_a has
                               statements the reader skips, a trailing comment whose tokens the
                               reader takes as a normal, faces before the first "vt" (uv index 0)
                               and "p//n" corners after it (the uv field keeps the value read
                               last); sphere_b has no "vt" at all.
  sphere_a.bin, sphere_b.bin   what the reference's parseMesh wrote for them (parseMeshFile +
                               binMeshWrite, core/FileIO.cuh:20-45, 73-164, 213-232) while loading
                               a scene whose subject meshes are these OBJ files.
  obj_scene.npz                world-space triangles of that scene (the box of the box_sphere
                               scene plus both spheres under a subject transform), in primitive
                               order, from the same run (lts_ref bvh).
  film_in.f32, film.ppm, film.pfm   a seeded 7 x 5 film (negative, > 1 and exact 0 / 1 values)
                               and the reference's writeToPPM / writeToPFM output for it
                               (core/ImageO.cuh:16-78).

Usage (from the repository root):  oracle/ref/build_ref.sh && python tests/golden/make_golden_io.py
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from lighttransportsimulation_gb300 import scenes  # noqa: E402
from oracle import ltsd  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "lts_ref")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "io")

SUBJECT_XFORM = "0.1 -0.2 0.05\t0.3 1 0.2\t25\t0.6\n"  # translation, axis, angle (deg), scale


def _fmt(x):
    return np.format_float_positional(np.float32(x), unique=True, trim="-")


def obj_text(level, with_uv, seed):
    """An icosphere as OBJ text, per the docstring's coverage."""
    rng = np.random.default_rng(seed)
    v, f = scenes.icosphere(level)
    v = (v * 0.5).astype(np.float32)
    nrm = scenes.icosphere(level)[0].astype(np.float32)
    lines = ["# seeded test mesh", "mtllib none.mtl", "o sphere", "g part", "s 1", "usemtl white"]
    for p in v:
        lines.append("v " + " ".join(_fmt(c) for c in p))
    for n in nrm:
        lines.append("vn " + " ".join(_fmt(c) for c in n))
    first = 20 if with_uv else len(f)
    for t in f[:first]:  # before any "vt": the reader stores uv index 0
        lines.append("f " + " ".join(f"{i + 1}//{i + 1}" for i in t))
    if with_uv:
        uv = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi), 0.5 - np.arcsin(v[:, 1] / 0.5) / np.pi],
                      1).astype(np.float32)
        for q in uv:
            lines.append("vt " + " ".join(_fmt(c) for c in q))
        for t in f[first:]:
            corners = []
            for i in t:
                # one corner in five as p//n: the uv field keeps the position index just read
                corners.append(f"{i + 1}//{i + 1}" if rng.random() < 0.2 else f"{i + 1}/{i + 1}/{i + 1}")
            lines.append("f " + " ".join(corners))
    lines.append("# trailing comment vn 0 0 1")  # read as one more normal, unreferenced
    return "\n".join(lines) + "\n"


def main():
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/lts_ref missing: run oracle/ref/build_ref.sh first")
    os.makedirs(OUT, exist_ok=True)
    with tempfile.TemporaryDirectory() as d:
        scenes._box_meshes(d)
        with open(os.path.join(d, "box.scene"), "w") as fh:  # camera, then the subject transform
            fh.write(scenes._box_scene_text().replace(scenes.IDENTITY_SUBJECT, SUBJECT_XFORM, 1))
        for name, uv, seed in (("sphere_a", True, 3), ("sphere_b", False, 4)):
            text = obj_text(2, uv, seed)
            for path in (os.path.join(d, name + ".obj"), os.path.join(OUT, name + ".obj")):
                with open(path, "w") as fh:
                    fh.write(text)
        with open(os.path.join(d, "spheres.subject"), "w") as fh:
            fh.write("0\n2\tsphere_a\tsphere_b\n2\nL\tc\t0.8 0.8 0.8\t0\nL\tc\t0.5 0.6 0.7\t0\n")
        dump = os.path.join(d, "dump.ltsd")
        subprocess.run([REF, "bvh", d + "/", "box", "spheres", dump, "64", "64"], check=True)
        for name in ("sphere_a", "sphere_b"):
            shutil.copy(os.path.join(d, name + ".bin"), os.path.join(OUT, name + ".bin"))
        r = ltsd.read(dump)
        np.savez_compressed(os.path.join(OUT, "obj_scene.npz"), tri_p=r["tri_p"], subject=np.array(SUBJECT_XFORM))

        rng = np.random.default_rng(9)
        film = rng.uniform(-0.5, 2.0, (5, 7, 3)).astype(np.float32)
        film[0, 0] = [0.0, 1.0, 0.5]
        film[1, 1] = [1.0, 0.0, 2.0]
        film_in = os.path.join(OUT, "film_in.f32")
        film.tofile(film_in)
        for fmt, ext in ((0, "ppm"), (1, "pfm")):
            subprocess.run([REF, "image", film_in, "7", "5", str(fmt), os.path.join(OUT, "film." + ext)], check=True)
    print("wrote", sorted(os.listdir(OUT)))


if __name__ == "__main__":
    main()
