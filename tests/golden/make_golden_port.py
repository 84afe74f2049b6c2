"""Golden fixtures for the conductor (Trowbridge-Reitz MetalMaterial) stress scene, made with the
oracle port (oracle/_build/lts_port).

The reference cannot load a conductor from its files (its loader parses 'M' and skips it,
core/SceneLoader_kernels.cu:16,47-48), so the stress scene -- which needs the documented 'C'
grammar extension -- is pinned to the port, the scalar restatement of the reference integrator
that tests/test_port.py holds bit-exact to the reference's own build on every scene the
reference can load.  The port restates MetalMaterial (materials/Material.cuh:97-130),
TrowbridgeReitzMicrofacetDistribution and MicrofacetReflection (models/Microfacet.cuh:53-229) and
FresnelConductor (models/BxDF.cuh:44-90) from the reference's sources.

  render_stress_small.npz  per-(pixel, sample) radiance and event hashes for a crop
  film_stress_small.npz    the port's resolved single-thread film

Usage (from the repository root): python oracle/port/build_port.py && python tests/golden/make_golden_port.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from lighttransportsimulation_gb300 import scenes  # noqa: E402
from make_golden import scene_digest  # noqa: E402
from oracle import ltsd  # noqa: E402

PORT = os.path.join(ROOT, "oracle", "_build", "lts_port")
OUT = os.path.dirname(os.path.abspath(__file__))

# the stress scene with 16 x 32 spheres (960 triangles each)
STRESS_SMALL = dict(rings=16, segs=32, w=160, h=90, spp=4, maxb=16, rr=4, seed=3, crop=(40, 20, 120, 70),
                    film=dict(w=80, h=45, spp=16))


def main():
    if not os.path.exists(PORT):
        sys.exit("oracle/_build/lts_port is missing: run oracle/port/build_port.py first")
    c = STRESS_SMALL
    with tempfile.TemporaryDirectory() as td:
        sc, sub = scenes.write_stress_scene(td, rings=c["rings"], segs=c["segs"])
        digest = np.array([f"{k}:{v}" for k, v in scene_digest(td).items()])
        root = td + "/"
        x0, y0, x1, y1 = c["crop"]
        r = os.path.join(td, "render.ltsd")
        subprocess.run([PORT, "render", root, sc, sub, r] + [str(a) for a in (
            c["w"], c["h"], c["spp"], c["maxb"], c["rr"], c["seed"], x0, y0, x1, y1, 8, 0)], check=True)
        d = ltsd.read(r)
        meta = np.array([c["w"], c["h"], c["spp"], c["maxb"], c["rr"], c["seed"], x0, y0, x1, y1], np.int64)
        np.savez_compressed(os.path.join(OUT, "render_stress_small.npz"), scene_digest=digest, meta=meta,
                            L=d["L"], sig=d["sig"])
        f = c["film"]
        r2 = os.path.join(td, "film.ltsd")
        subprocess.run([PORT, "render", root, sc, sub, r2] + [str(a) for a in (
            f["w"], f["h"], f["spp"], c["maxb"], c["rr"], c["seed"], 0, 0, f["w"], f["h"], 1, 1)], check=True)
        d = ltsd.read(r2)
        meta = np.array([f["w"], f["h"], f["spp"], c["maxb"], c["rr"], c["seed"]], np.int64)
        np.savez_compressed(os.path.join(OUT, "film_stress_small.npz"), scene_digest=digest, meta=meta,
                            film=d["film"])
    print("stress_small ok")


if __name__ == "__main__":
    main()
