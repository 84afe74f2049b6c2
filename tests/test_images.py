"""Image textures on the CPU: the oracle's PNG reader against its own writer for every colour type,
bit depth and filter, then the renderer's loader (its own inflate, filters and pyramid) against
the oracle's numpy restatement, bit for bit, on generated images and on the reference's own
image-texture scene (res/kernel_box_scene/kernel.png)."""
import os

import numpy as np
import pytest

from conftest import write_kernel_box

# (colour type, bit depth) of every PNG kind
KINDS = [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2), (3, 4), (3, 8),
         (4, 8), (4, 16), (6, 8), (6, 16)]


def _samples(rng, h, w, ctype, depth):
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    top = (1 << depth) - 1
    if ctype == 3:
        top = min(top, 12)
    return rng.integers(0, top + 1, (h, w, chans))


def _expected_rgb(s, ctype, depth, palette):
    if depth == 16:
        s = s >> 8
    if ctype == 3:
        return palette[s[:, :, 0]]
    if ctype in (0, 4):
        g = s[:, :, :1] * ({1: 255, 2: 85, 4: 17}.get(depth, 1) if ctype == 0 else 1)
        return np.repeat(g, 3, axis=2)
    return s[:, :, :3]


@pytest.mark.parametrize("ctype,depth", KINDS)
def test_oracle_png_reader_inverts_its_writer(ctype, depth):
    from oracle import image_np
    rng = np.random.default_rng(ctype * 100 + depth)
    h, w = 13, 29
    s = _samples(rng, h, w, ctype, depth)
    pal = rng.integers(0, 256, (13, 3))
    data = image_np.encode_png(s, ctype, depth, palette=pal if ctype == 3 else None)
    ww, hh, rgb = image_np.decode_png(data)
    assert (ww, hh) == (w, h)
    assert np.array_equal(rgb, _expected_rgb(s, ctype, depth, pal).astype(np.uint8))


def _scene_with_images(d, pngs):
    """A box scene whose back wall is textured by the first image; every image is listed."""
    from lighttransportsimulation_gb300 import scenes
    sc, sub = scenes.write_box_sphere(d)
    txt = open(os.path.join(d, sc + ".scene")).read().split("\n")
    imgs = "%d\t" % len(pngs) + "\t".join("%d\t%s" % (wrap, name) for name, wrap in pngs)
    assert txt[2] == "0"
    txt[2] = imgs
    body = "\n".join(txt).replace("L\tc\t0.7 0.7 0.7\t0", "L\ti\t0\t0", 1)
    open(os.path.join(d, "img.scene"), "w").write(body)
    return "img", sub


def test_loader_pyramids_match_the_oracle(built_lib, tmp_path):
    """Every PNG kind (odd sizes, stored / fixed / dynamic deflate blocks, all five filters)
    through the loader: each pyramid level equals the oracle's bit for bit."""
    import lighttransportsimulation_gb300 as lts
    from oracle import image_np
    d = str(tmp_path)
    rng = np.random.default_rng(3)
    pngs, made = [], []
    sizes = [(23, 37), (64, 64), (5, 300), (129, 70)]
    for k, (ctype, depth) in enumerate(KINDS):
        h, w = sizes[k % len(sizes)]
        s = _samples(rng, h, w, ctype, depth)
        pal = rng.integers(0, 256, (13, 3))
        data = image_np.encode_png(s, ctype, depth, palette=pal if ctype == 3 else None, level=(0, 1, 9)[k % 3])
        name = f"img{k}.png"
        open(os.path.join(d, name), "wb").write(data)
        pngs.append((name, k % 3))
        made.append(data)
    sc, sub = _scene_with_images(d, pngs)
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d, sc, sub, 32, 32)
    assert s.info["images"] == len(pngs)
    for k, data in enumerate(made):
        w, h, rgb = image_np.decode_png(data)
        want = image_np.pyramid(w, h, rgb, k % 3)
        for level in range(want["levels"]):
            got, levels = s.image(k, level)
            assert levels == want["levels"]
            assert np.array_equal(got.view(np.uint32), want["rgb"][level].view(np.uint32)), (k, level)
    ctx.close()


def test_reference_image_scene_loads(built_lib, tmp_path):
    """The reference's res/kernel_box_scene: its 64 x 64 RGB PNG decodes to the oracle's pyramid
    (6 levels) and the scene's materials and lights load."""
    import lighttransportsimulation_gb300 as lts
    from oracle import image_np
    root, sc, sub = write_kernel_box(str(tmp_path))
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, root, sc, sub, 64, 64)
    assert s.info["images"] == 1 and s.info["lights"] >= 1
    w, h, rgb = image_np.decode_png(open(os.path.join(root, "res/kernel_box_scene/kernel.png"), "rb").read())
    want = image_np.pyramid(w, h, rgb, 1)
    assert (w, h, want["levels"]) == (64, 64, 6)
    for level in range(6):
        got, _ = s.image(0, level)
        assert np.array_equal(got.view(np.uint32), want["rgb"][level].view(np.uint32))
    ctx.close()


def test_malformed_png_is_a_parse_error(built_lib, tmp_path):
    import lighttransportsimulation_gb300 as lts
    from oracle import image_np
    d = str(tmp_path)
    good = image_np.encode_png(np.zeros((8, 8, 3), np.int64), 2, 8)
    for name, data in (("trunc.png", good[:40]), ("chunk.png", good[:33] + b"\x00" * 8 + good[41:])):
        open(os.path.join(d, name), "wb").write(data)
        sc, sub = _scene_with_images(d, [(name, 1)])
        ctx = lts.Context(-1)
        with pytest.raises(lts.LtsError) as e:
            lts.Scene.parse(ctx, d, sc, sub, 32, 32)
        assert e.value.code == 3, name
        ctx.close()
