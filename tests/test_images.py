"""Image textures on the CPU: the oracle's PNG reader against its own writer for every colour type,
bit depth and filter, then the renderer's loader (its own inflate, filters and pyramid) against
the oracle's numpy restatement, bit for bit, on generated images and on the reference's own
image-texture scene (res/kernel_box_scene/kernel.png); its JPEG decoder against the reference's
own reader (stb_image through loadImageFile_s: tests/golden/jpeg_golden.npz, made by
tests/golden/make_golden_jpeg.py), bit for bit, on 22 JPEG forms and on res/blackDragon.jpg."""
import hashlib
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


def _jpeg_golden():
    from conftest import GOLDEN
    g = np.load(os.path.join(GOLDEN, "jpeg_golden.npz"))
    cases = []
    for k, name in enumerate(g["names"]):
        data = g["jpeg"][g["jpeg_off"][k]:g["jpeg_off"][k + 1]].tobytes()
        w, h = (int(x) for x in g["dims"][k])
        rgb = g["rgb"][g["rgb_off"][k]:g["rgb_off"][k + 1]].reshape(h, w, 3)
        cases.append((str(name), data, rgb))
    return g, cases


def test_jpeg_decoder_matches_the_reference_reader(built_lib, tmp_path):
    """Every JPEG form of the golden set (stb's own writer at 4:2:0 / 4:4:4; greyscale, 4:2:2,
    4:4:0, 4:1:1, 1 x 4 and mixed sampling, one scan per component, restart intervals, 16-bit
    tables, SOF1, Adobe RGB / CMYK / YCCK, RGB component ids, widths 1 and 2): the loader's level 0
    equals the reference's decoded, row-flipped texels bit for bit."""
    import lighttransportsimulation_gb300 as lts
    d = str(tmp_path)
    _, cases = _jpeg_golden()
    for name, data, _ in cases:
        open(os.path.join(d, name + ".jpg"), "wb").write(data)
    sc, sub = _scene_with_images(d, [(name + ".jpg", 1) for name, _, _ in cases])
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d, sc, sub, 32, 32)
    for k, (name, _, rgb) in enumerate(cases):
        got, _ = s.image(k, 0)
        got = got.reshape(rgb.shape)
        assert np.array_equal(got.view(np.uint32), rgb.view(np.uint32)), name
    ctx.close()


def test_black_dragon_jpeg(built_lib, tmp_path):
    """The reference's res/blackDragon.jpg (512 x 512, 4:2:0, JFIF + Exif): texels hash-equal to
    the reference reader's, and the pyramid of a JPEG is built like a PNG's."""
    import lighttransportsimulation_gb300 as lts
    from oracle import image_np
    d = str(tmp_path)
    g, _ = _jpeg_golden()
    open(os.path.join(d, "blackDragon.jpg"), "wb").write(g["dragon_jpeg"].tobytes())
    sc, sub = _scene_with_images(d, [("blackDragon.jpg", 1)])
    ctx = lts.Context(-1)
    s = lts.Scene.parse(ctx, d, sc, sub, 32, 32)
    w, h = (int(x) for x in g["dragon_dims"])
    got, levels = s.image(0, 0)
    got = got.reshape(h, w, 3)
    assert np.array_equal(got[224:288, 224:288].view(np.uint32), g["dragon_crop"].view(np.uint32))
    assert hashlib.sha256(got.tobytes()).hexdigest() == str(g["dragon_sha256"])
    # the pyramid over the decoded 8-bit texels: invert the float conversion of level 0
    lut = np.array([np.float32(np.power(np.float64(np.float32(c) / np.float32(255)), np.float64(np.float32(2.2))))
                    for c in range(256)], np.float32)
    rgb8 = np.searchsorted(lut, got[::-1].reshape(-1)).astype(np.uint8).reshape(h, w, 3)
    assert np.array_equal(lut[rgb8][::-1].view(np.uint32), got.view(np.uint32))
    want = image_np.pyramid(w, h, rgb8, 1)
    assert levels == want["levels"] == 9
    for level in range(levels):
        lv, _ = s.image(0, level)
        assert np.array_equal(lv.view(np.uint32), want["rgb"][level].view(np.uint32)), level
    ctx.close()


def test_malformed_and_unsupported_jpeg(built_lib, tmp_path):
    """Progressive and 12-bit JPEGs are refused as unsupported (code 6); a truncated stream, a
    coefficient run past its block and a missing restart marker are parse errors (code 3)."""
    import lighttransportsimulation_gb300 as lts
    from oracle import jpeg_np
    d = str(tmp_path)
    rng = np.random.default_rng(5)
    q = [jpeg_np.quant_table(2.0), jpeg_np.quant_table(3.0)]
    good = jpeg_np.encode(jpeg_np.test_planes(rng, 24, 16, [(2, 2), (1, 1), (1, 1)]), [(2, 2), (1, 1), (1, 1)], q,
                          width=24, height=16, restart=1)
    sof = good.index(b"\xff\xc0")
    rst = good.index(b"\xff\xd0")
    cases = [("prog.jpg", good[:sof + 1] + b"\xc2" + good[sof + 2:], 6),
             ("p12.jpg", good[:sof + 4] + b"\x0c" + good[sof + 5:], 6),
             ("trunc.jpg", good[:len(good) // 2], 3),
             ("norst.jpg", good[:rst] + good[rst + 2:], 3)]
    for name, data, code in cases:
        open(os.path.join(d, name), "wb").write(data)
        sc, sub = _scene_with_images(d, [(name, 1)])
        ctx = lts.Context(-1)
        with pytest.raises(lts.LtsError) as e:
            lts.Scene.parse(ctx, d, sc, sub, 32, 32)
        assert e.value.code == code, (name, str(e.value))
        ctx.close()


def _corrupt(rng, data, keep):
    """One random corruption of `data`: flipped bytes, truncation, inserted or deleted bytes
    (the first `keep` bytes kept)."""
    b = bytearray(data)
    kind = rng.integers(4)
    if kind == 0:
        for _ in range(rng.integers(1, 8)):
            b[rng.integers(keep, len(b))] = rng.integers(256)
    elif kind == 1:
        b = b[:rng.integers(keep, len(b))]
    elif kind == 2:
        i = rng.integers(keep, len(b))
        b[i:i] = bytes(rng.integers(0, 256, rng.integers(1, 20)).astype(np.uint8))
    else:
        i = rng.integers(keep, len(b))
        del b[i:i + rng.integers(1, 50)]
    return bytes(b)


def test_corrupt_images_fail_cleanly(built_lib, tmp_path):
    """300 corrupted JPEGs (from the golden set) and 300 corrupted PNGs through the loader: each
    either decodes or is refused with LTS_ERR_PARSE / LTS_ERR_UNSUPPORTED, in this process (a
    read past a buffer would end it).  The decoders were also run on 4,800 and 2,400 such inputs
    under AddressSanitizer and UndefinedBehaviorSanitizer without a report."""
    import lighttransportsimulation_gb300 as lts
    from oracle import image_np
    d = str(tmp_path)
    rng = np.random.default_rng(11)
    _, cases = _jpeg_golden()
    jpegs = [data for _, data, _ in cases]
    pngs = [image_np.encode_png(rng.integers(0, 256, (int(rng.integers(1, 30)), int(rng.integers(1, 30)), c)), t, 8,
                                level=int(rng.integers(0, 10)))
            for t, c in ((0, 1), (2, 3), (4, 2), (6, 4))]
    ctx = lts.Context(-1)
    seen = {}
    for k in range(600):
        src = jpegs[k % len(jpegs)] if k < 300 else pngs[k % len(pngs)]
        name = f"c{k}." + ("jpg" if k < 300 else "png")
        open(os.path.join(d, name), "wb").write(_corrupt(rng, src, 2 if k < 300 else 8))
        sc, sub = _scene_with_images(d, [(name, 1)])
        try:
            lts.Scene.parse(ctx, d, sc, sub, 8, 8)
            code = 0
        except lts.LtsError as e:
            code = e.code
        assert code in (0, 3, 6), (name, code)
        seen[code] = seen.get(code, 0) + 1
    ctx.close()
    assert seen.get(3, 0) > 100 and seen.get(0, 0) > 10
