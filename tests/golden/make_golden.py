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
    python tests/golden/make_golden.py shipped /path/to/reference   # the shipped scenes (SHIPPED)
    python tests/golden/make_golden.py digests                      # the bench scene's digests
    python tests/golden/make_golden.py kernel_box /path/to/reference  # the image-texture scene's inputs
    python tests/golden/make_golden.py dragon /path/to/reference  # res/blackDragon on closeupPlane

kernel_box_inputs.npz holds the input files of the reference's own image-texture scene
(res/kernel_box_scene: a 64 x 64 PNG on a box); the reference cannot render it reproducibly (its
texel storage is undefined), so only its inputs are stored, and the tests compare the renderer
with the oracle's port and numpy restatement of the fixed mode.
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


# The reference's own shipped scenes (res/ of the reference tree) that need no image texture:
# the scene of the published 1080p times with two of its subjects (app.params:20-23), and the
# big box with an area and an infinite light.  Their input files are stored in
# shipped_inputs.npz, so that the tests can rebuild the scene directory without the reference.
SHIPPED_FILES = ["res/platforms/closeupPlane.scene", "res/platforms/triPlane.bin", "res/platforms/bigBox.scene",
                 "res/platforms/bigBox.bin", "res/platforms/bigBox_light.bin", "res/diamond.subject",
                 "res/diamond.bin", "res/moai.subject", "res/moai.bin"]
SHIPPED = {
    "closeup_diamond": dict(scene="res/platforms/closeupPlane", subject="res/diamond", w=480, h=270, spp=4, maxb=5,
                            rr=2, seed=3, crop=(220, 95, 260, 135), film=dict(w=96, h=54, spp=16)),
    "closeup_moai": dict(scene="res/platforms/closeupPlane", subject="res/moai", w=480, h=270, spp=4, maxb=5,
                         rr=2, seed=3, crop=(220, 80, 260, 120), film=dict(w=96, h=54, spp=16)),
    "bigbox_diamond": dict(scene="res/platforms/bigBox", subject="res/diamond", w=480, h=270, spp=4, maxb=5,
                           rr=2, seed=3, crop=(220, 115, 260, 155), film=dict(w=96, h=54, spp=16)),
}


def shipped_key(rel):
    return "in__" + rel.replace("/", "__")


def write_shipped_inputs(npz_path, d):
    """Recreates the shipped scenes' input files under directory d (paths as in the reference
    tree, relative to its root, which the .scene files name their meshes by)."""
    z = np.load(npz_path)
    for k in z.files:
        if not k.startswith("in__"):
            continue
        rel = k[4:].replace("__", "/")
        os.makedirs(os.path.join(d, os.path.dirname(rel)), exist_ok=True)
        with open(os.path.join(d, rel), "wb") as fh:
            fh.write(z[k].tobytes())


def scene_digest(d):
    h = {}
    for f in sorted(os.listdir(d)):
        with open(os.path.join(d, f), "rb") as fh:
            h[f] = hashlib.sha256(fh.read()).hexdigest()
    return h


def run(args):
    subprocess.run([REF] + [str(a) for a in args], check=True)


def make_case(name, c, root, sc, sub, digest):
    b = os.path.join(root, "bvh.ltsd")
    run(["bvh", root, sc, sub, b, c["w"], c["h"]])
    d = ltsd.read(b)
    os.remove(b)
    if d["tri_p"].size > 9 * 20000:  # large meshes: the loader's triangles are pinned by their digest
        d["tri_p_sha256"] = np.array(hashlib.sha256(np.ascontiguousarray(d.pop("tri_p")).tobytes()).hexdigest())
    np.savez_compressed(os.path.join(OUT, f"lbvh_{name}.npz"), scene_digest=digest, **d)
    r = os.path.join(root, "render.ltsd")
    x0, y0, x1, y1 = c["crop"]
    run(["render", root, sc, sub, r, c["w"], c["h"], c["spp"], c["maxb"], c["rr"], c["seed"], x0, y0, x1, y1, 8, 0])
    d = ltsd.read(r)
    os.remove(r)
    meta = np.array([c["w"], c["h"], c["spp"], c["maxb"], c["rr"], c["seed"], x0, y0, x1, y1], np.int64)
    np.savez_compressed(os.path.join(OUT, f"render_{name}.npz"), scene_digest=digest, meta=meta, L=d["L"], sig=d["sig"])
    f = c["film"]
    r2 = os.path.join(root, "film.ltsd")
    run(["render", root, sc, sub, r2, f["w"], f["h"], f["spp"], c["maxb"], c["rr"], c["seed"], 0, 0, f["w"], f["h"], 1, 1])
    d = ltsd.read(r2)
    os.remove(r2)
    meta = np.array([f["w"], f["h"], f["spp"], c["maxb"], c["rr"], c["seed"]], np.int64)
    np.savez_compressed(os.path.join(OUT, f"film_{name}.npz"), scene_digest=digest, meta=meta, film=d["film"])
    print(name, "ok")


def make_shipped(reference_root):
    """Fixtures of the reference's shipped scenes; `reference_root` is the reference checkout."""
    files = {}
    for rel in SHIPPED_FILES:
        with open(os.path.join(reference_root, rel), "rb") as fh:
            files[shipped_key(rel)] = np.frombuffer(fh.read(), np.uint8)
    inputs = os.path.join(OUT, "shipped_inputs.npz")
    np.savez_compressed(inputs, **files)
    with tempfile.TemporaryDirectory() as td:
        write_shipped_inputs(inputs, td)
        digest = np.array([f"{k}:{v}" for k, v in shipped_digest(td).items()])
        for name, c in SHIPPED.items():
            make_case(name, c, td + "/", c["scene"], c["subject"], digest)


def shipped_digest(d):
    h = {}
    for rel in SHIPPED_FILES:
        with open(os.path.join(d, rel), "rb") as fh:
            h[rel] = hashlib.sha256(fh.read()).hexdigest()
    return h


def make_digests():
    """digest_displaced.npz: sha256 of every array the reference's loader and LBVH build produce
    for the displaced-icosphere bench scene (1,310,732 triangles, 1024 x 1024), far too large to
    store: the world triangles, camera, light distribution, sorted codes / ids, children and node
    boxes of the reference's own build."""
    with tempfile.TemporaryDirectory() as td:
        scenes.write_displaced(td, level=8)
        digest = np.array([f"{k}:{v}" for k, v in scene_digest(td).items()])
        b = os.path.join(td, "bvh.ltsd")
        run(["bvh", td + "/", "box", "displaced", b, 1024, 1024])
        d = ltsd.read(b)
        sums = {k: np.array(hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()) for k, v in d.items()}
        np.savez_compressed(os.path.join(OUT, "digest_displaced.npz"), scene_digest=digest,
                            n=np.array(len(d["sorted_codes"])), **sums)
    print("digest_displaced ok")


KERNEL_BOX_FILES = ["res/kernel_box_scene/kernel.scene", "res/kernel_box_scene/kernel.png",
                    "res/kernel_box_scene/kernelBox_box.bin", "res/kernel_box_scene/kernelBox_light.bin"]


def make_kernel_box(reference_root):
    files = {}
    for rel in KERNEL_BOX_FILES:
        with open(os.path.join(reference_root, rel), "rb") as fh:
            files[shipped_key(rel)] = np.frombuffer(fh.read(), np.uint8)
    np.savez_compressed(os.path.join(OUT, "kernel_box_inputs.npz"), **files)
    print("kernel_box_inputs ok")


DRAGON_FILES = ["res/platforms/closeupPlane.scene", "res/platforms/triPlane.bin", "res/blackDragon.subject",
                "res/blackDragon.bin", "res/blackDragon.jpg"]


DRAGON_CONSTANT_SUBJECT = "0\n1\tres/blackDragon\n1\nL\tc\t0.5 0.5 0.5\t0.5"


def make_dragon(reference_root):
    """dragon_inputs.npz: the reference's JPEG-textured subject (res/blackDragon.subject, .bin,
    .jpg) on res/platforms/closeupPlane; digest_dragon.npz: sha256 of every array the reference's
    loader and LBVH build produce for it at 480 x 270.  The reference's loader crashes (SIGSEGV) in
    its image-texture set-up on this subject in the host build (its BlockedArray writes past its
    allocation for images taller than 16 texels), so the digests are taken on the same subject
    with its texture replaced by a constant (DRAGON_CONSTANT_SUBJECT): triangles, camera, light
    distribution and the LBVH do not depend on the subject's material."""
    files = {}
    for rel in DRAGON_FILES:
        with open(os.path.join(reference_root, rel), "rb") as fh:
            files[shipped_key(rel)] = np.frombuffer(fh.read(), np.uint8)
    inputs = os.path.join(OUT, "dragon_inputs.npz")
    np.savez_compressed(inputs, **files)
    with tempfile.TemporaryDirectory() as td:
        write_shipped_inputs(inputs, td)
        with open(os.path.join(td, "res", "blackDragon_constant.subject"), "w") as fh:
            fh.write(DRAGON_CONSTANT_SUBJECT)
        b = os.path.join(td, "bvh.ltsd")
        run(["bvh", td + "/", "res/platforms/closeupPlane", "res/blackDragon_constant", b, 480, 270])
        d = ltsd.read(b)
        sums = {k: np.array(hashlib.sha256(np.ascontiguousarray(v).tobytes()).hexdigest()) for k, v in d.items()}
        np.savez_compressed(os.path.join(OUT, "digest_dragon.npz"), n=np.array(len(d["sorted_codes"])), **sums)
    print("dragon ok")


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "dragon":
        if not os.path.exists(REF):
            sys.exit("oracle/_ref/lts_ref is missing: run oracle/ref/build_ref.sh first")
        make_dragon(sys.argv[2] if len(sys.argv) > 2 else "/root/reference")
        return
    if len(sys.argv) > 1 and sys.argv[1] == "kernel_box":
        make_kernel_box(sys.argv[2] if len(sys.argv) > 2 else "/root/reference")
        return
    if not os.path.exists(REF):
        sys.exit("oracle/_ref/lts_ref is missing: run oracle/ref/build_ref.sh first")
    if len(sys.argv) > 1 and sys.argv[1] == "digests":
        make_digests()
        return
    if len(sys.argv) > 1 and sys.argv[1] == "shipped":
        make_shipped(sys.argv[2] if len(sys.argv) > 2 else "/root/reference")
        return
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
