"""Image textures on the GPU (the fixed mode of the reference's ImageTexture / Mipmap): the device
lookup against the oracle's numpy restatement bit for bit, for every wrap mode, on pyramids read
at level 0 only and between two levels; and the reference's own image-texture scene
(res/kernel_box_scene) rendered per sample against the oracle's CPU port, by the parity rule of
tests/test_render_gpu.py."""
import os
import subprocess

import numpy as np
import pytest

from conftest import write_dragon, write_kernel_box
from test_render_gpu import check_samples

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built_lib):
    import lighttransportsimulation_gb300 as lts
    c = lts.Context(0)
    yield c
    c.close()


def test_device_lookup_matches_the_oracle(ctx, tmp_path):
    """64 x 64 (level coordinate < 0: bilinear on level 0), 256 x 128 (between levels 0 and 1) and
    1000 x 600 (levels 1 and 2), each in repeat, black and clamp mode, at 20,000 texture
    coordinates in [-1.5, 2.5]^2 plus the corners of [0, 1]^2."""
    import lighttransportsimulation_gb300 as lts
    from lighttransportsimulation_gb300 import scenes
    from oracle import image_np
    d = str(tmp_path)
    rng = np.random.default_rng(9)
    pngs, want = [], []
    for k, (h, w) in enumerate([(64, 64), (128, 256), (600, 1000)]):
        rgb = rng.integers(0, 256, (h, w, 3))
        data = image_np.encode_png(rgb, 2, 8)
        name = f"t{k}.png"
        open(os.path.join(d, name), "wb").write(data)
        for wrap in (0, 1, 2):
            pngs.append((name, wrap))
            want.append(image_np.pyramid(w, h, rgb.astype(np.uint8), wrap))
    sc, sub = scenes.write_box_sphere(d)
    txt = open(os.path.join(d, sc + ".scene")).read().split("\n")
    txt[2] = "%d\t" % len(pngs) + "\t".join("%d\t%s" % (wrap, name) for name, wrap in pngs)
    open(os.path.join(d, "img.scene"), "w").write("\n".join(txt))
    s = lts.Scene.parse(ctx, d, "img", sub, 32, 32)
    st = rng.uniform(-1.5, 2.5, (20000, 2)).astype(np.float32)
    st = np.concatenate([st, np.array([[0, 0], [1, 0], [0, 1], [1, 1], [0.5, 0.5]], np.float32)])
    for i, img in enumerate(want):
        got = s.image_lookup(i, st)
        ref = image_np.lookup(img, st)
        diff = np.any(got.view(np.uint32) != ref.view(np.uint32), axis=1)
        print(f"image {i}: levels {img['levels']}, lod {float(img['lod']):.3f}, wrap {img['wrap']}: "
              f"differing {diff.sum()} of {len(st)}")
        assert not diff.any()


def test_reference_image_scene_matches_the_port(ctx, port_exe, tmp_path):
    """res/kernel_box_scene (a 64 x 64 PNG on a box lit by one area light), 96 x 96, 4 spp,
    5 bounces: the megakernel and the wavefront integrator against the port's samples."""
    import lighttransportsimulation_gb300 as lts
    from oracle import ltsd
    root, sc, sub = write_kernel_box(str(tmp_path))
    w, h, spp, maxb, rr, seed = 96, 96, 4, 5, 3, 1
    out = str(tmp_path / "port.ltsd")
    args = (port_exe, "render", root + "/", sc, sub or "-", out, w, h, spp, maxb, rr, seed, 0, 0, w, h,
            os.cpu_count(), 0, 0)
    subprocess.run([str(a) for a in args], check=True)
    ref = ltsd.read(out)
    Lr, sr = ref["L"].reshape(-1, 3), ref["sig"].reshape(-1)
    s = lts.Scene.parse(ctx, root, sc, sub, w, h)
    assert s.info["images"] == 1
    res = {}
    for integ in (lts.INTEGRATOR_FP64, lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
        r = lts.PathTracingIntegrator(maxb, rr, s, integrator=integ).render(spp, seed, record=True, film=False)
        res[integ] = (r["L"].reshape(-1, 3).copy(), r["sig"].reshape(-1).copy())
    L64, s64 = res[lts.INTEGRATOR_FP64]
    assert Lr.mean() > 0
    for integ in (lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
        L, sig = res[integ]
        check_samples(L, sig, Lr, sr, L64, s64, f"kernel_box integrator={integ}")


def test_reference_jpeg_scene_matches_the_port(ctx, port_exe, tmp_path):
    """The reference's JPEG-textured subject res/blackDragon on res/platforms/closeupPlane,
    480 x 270, a 48 x 48 crop on the dragon, 4 spp, 5 bounces: the megakernel and the wavefront
    integrator against the port's samples."""
    import lighttransportsimulation_gb300 as lts
    from oracle import ltsd
    root, sc, sub = write_dragon(str(tmp_path))
    w, h, spp, maxb, rr, seed = 480, 270, 4, 5, 3, 2
    x0, y0, x1, y1 = 216, 111, 264, 159
    out = str(tmp_path / "port.ltsd")
    args = (port_exe, "render", root + "/", sc, sub, out, w, h, spp, maxb, rr, seed, x0, y0, x1, y1,
            os.cpu_count(), 0, 0)
    subprocess.run([str(a) for a in args], check=True)
    ref = ltsd.read(out)
    Lr, sr = ref["L"].reshape(-1, 3), ref["sig"].reshape(-1)
    s = lts.Scene.parse(ctx, root, sc, sub, w, h)
    assert s.info["images"] == 1
    res = {}
    for integ in (lts.INTEGRATOR_FP64, lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
        r = lts.PathTracingIntegrator(maxb, rr, s, integrator=integ).render(spp, seed, crop=(x0, y0, x1, y1),
                                                                            record=True, film=False)
        res[integ] = (r["L"].reshape(-1, 3).copy(), r["sig"].reshape(-1).copy())
    L64, s64 = res[lts.INTEGRATOR_FP64]
    assert Lr.mean() > 0
    for integ in (lts.INTEGRATOR_MEGAKERNEL, lts.INTEGRATOR_WAVEFRONT):
        L, sig = res[integ]
        check_samples(L, sig, Lr, sr, L64, s64, f"blackDragon integrator={integ}")
