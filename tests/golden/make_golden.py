"""Regenerates the committed golden fixtures from the reference itself.

Runs oracle/_ref/lts_ref -- tierChampion/LightTransportSimulation's own sources compiled for
the host by oracle/ref/build_ref.sh -- on seeded synthetic scenes written by
lighttransportsimulation_gb300.scenes, and stores what the parity tests compare against:

  lbvh_<scene>.npz     sorted Morton codes and ids, the flattened LBVH (children + AABB bit
                       patterns of all 2N-1 nodes) of the reference's own build (BVH.cuh:411-452),
                       plus the loader outputs (world triangles, camera, light distribution).
  render_<scene>.npz   per-(pixel, sample) radiance L before the film splat and a hash of each
                       sample's hit/visibility events for a pixel crop
                       (PathTracingIntegrator.cuh:26-109), with the project sampler.
  film_<scene>.npz     the resolved film (Camera::getRender) of a small full render on one
                       thread (the reference's filter-weight update is not atomic).

Each fixture records sha256 digests of the scene files it was made from, so a test can tell a
changed generator from a changed renderer.  Usage (from the repository root):
    oracle/ref/build_ref.sh && python tests/golden/make_golden.py
"""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from lighttransportsimulation_gb300 import scenes  # noqa: E402
from oracle import ltsd  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "lts_ref")
OUT = os.path.dirname(os.path.abspath(__file__))

# name -> (writer, width, height, render settings, crop)
CASES = {
    "box_sphere": dict(write=scenes.write_box_sphere, w=256, h=256, spp=4, maxb=5, rr=3, seed=7,
                       crop=(112, 112, 144, 144), film=dict(w=64, h=64, spp=16)),
    "materials": dict(write=scenes.write_materials_scene, w=128, h=128, spp=4, maxb=8, rr=3, seed=5,
                      crop=(40, 10, 88, 58), film=dict(w=64, h=64, spp=16)),
}


def scene_digest(d):
    h = {}
    for f in sorted(os.listdir(d)):
        with open(os.path.join(d, f), "rb") as fh:
            h[f] = hashlib.sha256(fh.read()).hexdigest()
    return h


def run(args):
    subprocess.run([REF] + [str(a) for a in args], check=True)


def main():
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/lts_ref is missing: run oracle/ref/build_ref.sh first")
    for name, c in CASES.items():
        with tempfile.TemporaryDirectory() as td:
            sc, sub = c["write"](td)
            dig = scene_digest(td)
            digest = np.array([f"{k}:{v}" for k, v in dig.items()])
            root = td + "/"
            b = os.path.join(td, "bvh.ltsd")
            run(["bvh", root, sc, sub, b, c["w"], c["h"]])
            d = ltsd.read(b)
            np.savez_compressed(os.path.join(OUT, f"lbvh_{name}.npz"), scene_digest=digest, **d)
            r = os.path.join(td, "render.ltsd")
            x0, y0, x1, y1 = c["crop"]
            run(["render", root, sc, sub, r, c["w"], c["h"], c["spp"], c["maxb"], c["rr"], c["seed"],
                 x0, y0, x1, y1, 8, 0])
            d = ltsd.read(r)
            meta = np.array([c["w"], c["h"], c["spp"], c["maxb"], c["rr"], c["seed"], x0, y0, x1, y1], np.int64)
            np.savez_compressed(os.path.join(OUT, f"render_{name}.npz"), scene_digest=digest, meta=meta,
                                L=d["L"], sig=d["sig"])
            f = c["film"]
            r2 = os.path.join(td, "film.ltsd")
            run(["render", root, sc, sub, r2, f["w"], f["h"], f["spp"], c["maxb"], c["rr"], c["seed"],
                 0, 0, f["w"], f["h"], 1, 1])
            d = ltsd.read(r2)
            meta = np.array([f["w"], f["h"], f["spp"], c["maxb"], c["rr"], c["seed"]], np.int64)
            np.savez_compressed(os.path.join(OUT, f"film_{name}.npz"), scene_digest=digest, meta=meta,
                                film=d["film"])
            print(name, "ok")


if __name__ == "__main__":
    main()
