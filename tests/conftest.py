import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """The compiled renderer library (built in-tree on first use)."""
    from lighttransportsimulation_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def port_exe():
    """The oracle's CPU port (oracle/_build/lts_port), built on first use."""
    sys.path.insert(0, os.path.join(ROOT, "oracle", "port"))
    import build_port
    return build_port.build()


def write_scene(kind, d):
    from lighttransportsimulation_gb300 import scenes
    if kind == "stress_small":  # the stress scene with 16 x 32 spheres (tests/golden/make_golden_port.py)
        return scenes.write_stress_scene(d, rings=16, segs=32)
    return {"box_sphere": scenes.write_box_sphere, "materials": scenes.write_materials_scene}[kind](d)


def scene_digest(d):
    import hashlib
    out = []
    for f in sorted(os.listdir(d)):
        with open(os.path.join(d, f), "rb") as fh:
            out.append(f"{f}:{hashlib.sha256(fh.read()).hexdigest()}")
    return out


# The reference's own shipped scenes (tests/golden/shipped_inputs.npz holds their input files,
# tests/golden/make_golden.py made the fixtures from the reference): kind -> (scene, subject).
SHIPPED = {"closeup_diamond": ("res/platforms/closeupPlane", "res/diamond"),
           "closeup_moai": ("res/platforms/closeupPlane", "res/moai"),
           "bigbox_diamond": ("res/platforms/bigBox", "res/diamond")}


def write_shipped(d):
    """Recreates the shipped scenes' input files under d, at their paths in the reference tree."""
    import hashlib
    z = np.load(os.path.join(GOLDEN, "shipped_inputs.npz"))
    digest = []
    for k in z.files:
        rel = k[4:].replace("__", "/")
        os.makedirs(os.path.join(d, os.path.dirname(rel)), exist_ok=True)
        data = z[k].tobytes()
        with open(os.path.join(d, rel), "wb") as fh:
            fh.write(data)
        digest.append(f"{rel}:{hashlib.sha256(data).hexdigest()}")
    return digest


def write_kernel_box(d):
    """Recreates the reference's image-texture scene (res/kernel_box_scene) under d from
    tests/golden/kernel_box_inputs.npz; returns (root, scene, subject) as lts_load_scene takes them."""
    z = np.load(os.path.join(GOLDEN, "kernel_box_inputs.npz"))
    for k in z.files:
        rel = k[4:].replace("__", "/")
        os.makedirs(os.path.join(d, os.path.dirname(rel)), exist_ok=True)
        with open(os.path.join(d, rel), "wb") as fh:
            fh.write(z[k].tobytes())
    return d, "res/kernel_box_scene/kernel", ""


def write_dragon(d):
    """Recreates the reference's JPEG-textured subject on its closeupPlane platform
    (res/blackDragon.subject / .bin / .jpg, res/platforms/closeupPlane.scene / triPlane.bin) under d
    from tests/golden/dragon_inputs.npz; returns (root, scene, subject)."""
    z = np.load(os.path.join(GOLDEN, "dragon_inputs.npz"))
    for k in z.files:
        rel = k[4:].replace("__", "/")
        os.makedirs(os.path.join(d, os.path.dirname(rel)), exist_ok=True)
        with open(os.path.join(d, rel), "wb") as fh:
            fh.write(z[k].tobytes())
    return d, "res/platforms/closeupPlane", "res/blackDragon"


@pytest.fixture(scope="session")
def scene_dirs(tmp_path_factory):
    """Generated parity scenes and the reference's shipped scenes, checked against the digests
    recorded in the fixtures."""
    out = {}
    for kind in ("box_sphere", "materials", "stress_small"):
        d = str(tmp_path_factory.mktemp(kind))
        sc, sub = write_scene(kind, d)
        fx = np.load(os.path.join(GOLDEN, f"lbvh_{kind}.npz" if kind != "stress_small" else f"render_{kind}.npz"))
        assert list(fx["scene_digest"]) == scene_digest(d), f"scene generator drifted for {kind}"
        out[kind] = (d, sc, sub)
    d = str(tmp_path_factory.mktemp("shipped"))
    digest = write_shipped(d)
    for kind, (sc, sub) in SHIPPED.items():
        fx = np.load(os.path.join(GOLDEN, f"lbvh_{kind}.npz"))
        assert sorted(fx["scene_digest"]) == sorted(digest), f"shipped inputs differ from the fixture's for {kind}"
        out[kind] = (d, sc, sub)
    return out


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
