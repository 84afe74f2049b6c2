"""Writes tests/golden/jpeg_golden.npz: JPEG inputs and the reference's own decoding of each.

The expected texels come from the reference's image reader, loadImageFile_s (core/ImageI.cuh:11-34:
stbi_loadf of the vendored stb_image v2.27 with three channels, rows flipped), compiled from the
reference checkout into oracle/_ref/lts_ref by oracle/ref/build_ref.sh ("lts_ref imread").
Inputs:
  * stb_*: written by the reference's own JPEG writer (stbi_write_jpg of its vendored
    stb_image_write, "lts_ref jpgwrite"): 4:2:0 at quality <= 90, 4:4:4 above;
  * own_*: written by oracle/jpeg_np.py in the forms stb's writer never makes (greyscale, 4:2:2,
    4:4:0, 4:1:1, 1 x 4, mixed factors, one scan per component, restart intervals, 16-bit tables,
    SOF1, Adobe RGB / CMYK / YCCK, 'R' 'G' 'B' ids, widths of one and two);
  * dragon: the reference's res/blackDragon.jpg (512 x 512 4:2:0, JFIF + Exif), stored whole; its
    expected texels are stored as a SHA-256 of the float32 bytes and a 64 x 64 crop.

Usage: python tests/golden/make_golden_jpeg.py [REFERENCE_ROOT]  (needs oracle/_ref/lts_ref)."""
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import jpeg_np  # noqa: E402

LTS_REF = os.path.join(ROOT, "oracle", "_ref", "lts_ref")


def ref_read(path):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "img.f32")
        subprocess.run([LTS_REF, "imread", path, out], check=True)
        b = open(out, "rb").read()
    w, h = (int(x) for x in np.frombuffer(b[:8], np.int32))
    return np.frombuffer(b[8:], np.float32).reshape(h, w, 3).copy()


def stb_write(pixels, quality):
    h, w, c = pixels.shape
    with tempfile.TemporaryDirectory() as d:
        raw, jpg = os.path.join(d, "px.raw"), os.path.join(d, "img.jpg")
        open(raw, "wb").write(np.ascontiguousarray(pixels, np.uint8).tobytes())
        subprocess.run([LTS_REF, "jpgwrite", raw, str(w), str(h), str(c), str(quality), jpg], check=True)
        return open(jpg, "rb").read()


def own_cases(rng):
    q = [jpeg_np.quant_table(2.0), jpeg_np.quant_table(3.0)]
    Y2, C1 = (2, 2), (1, 1)
    cases = []

    def add(name, w, h, factors, **kw):
        planes = jpeg_np.test_planes(rng, w, h, factors)
        cases.append((name, jpeg_np.encode(planes, factors, q, width=w, height=h, **kw)))

    add("own_grey", 35, 19, [C1], restart=3)
    add("own_grey_2x2", 33, 17, [Y2])
    add("own_422_restart", 41, 26, [(2, 1), C1, C1], restart=5)
    add("own_440", 30, 45, [(1, 2), C1, C1])
    add("own_411", 70, 20, [(4, 1), C1, C1])
    add("own_mixed", 27, 31, [Y2, (1, 2), (2, 1)])
    add("own_1x4", 19, 37, [(1, 4), C1, C1])
    add("own_scans_16bit_sof1", 40, 40, [Y2, C1, C1], interleaved=False, restart=2, sixteen_bit=True, sof=0xC1)
    add("own_adobe_rgb", 20, 18, [C1, C1, C1], jfif=False, adobe=0)
    add("own_rgb_ids", 21, 13, [C1, C1, C1], ids=[ord("R"), ord("G"), ord("B")])
    add("own_cmyk", 16, 12, [C1, C1, C1, C1], jfif=False, adobe=0, tq=[0, 1, 1, 0])
    add("own_ycck", 23, 21, [Y2, C1, C1, Y2], jfif=False, adobe=2, tq=[0, 1, 1, 0])
    add("own_ycbcrk", 17, 9, [C1, C1, C1, C1], jfif=False, adobe=1, tq=[0, 1, 1, 0])
    add("own_w1_420", 1, 9, [Y2, C1, C1])
    add("own_w2_422", 2, 11, [(2, 1), C1, C1], restart=1)
    add("own_big_restart", 130, 66, [Y2, C1, C1], restart=7)
    return cases


def stb_cases(rng):
    cases = []
    for name, (h, w, quality, comp) in (("stb_420_q90", (23, 37, 90, 3)), ("stb_444_q95", (64, 48, 95, 3)),
                                        ("stb_q50", (17, 9, 50, 3)), ("stb_1x1", (1, 1, 80, 3)),
                                        ("stb_grey_q100", (40, 33, 100, 1)), ("stb_rgba_q20", (129, 70, 20, 4))):
        yy, xx = np.mgrid[0:h, 0:w]
        px = np.stack([(xx * 7 + yy * 3) % 256, (xx * yy) % 256, rng.integers(0, 256, (h, w)),
                       np.full((h, w), 255)], -1)[..., :comp]
        cases.append((name, stb_write(px, quality)))
    return cases


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    if not os.path.exists(LTS_REF):
        sys.exit("build oracle/_ref/lts_ref first (oracle/ref/build_ref.sh)")
    rng = np.random.default_rng(2024)
    cases = stb_cases(rng) + own_cases(rng)
    names, blobs, rgbs, dims = [], [], [], []
    with tempfile.TemporaryDirectory() as d:
        for name, data in cases:
            path = os.path.join(d, name + ".jpg")
            open(path, "wb").write(data)
            rgb = ref_read(path)
            names.append(name)
            blobs.append(np.frombuffer(data, np.uint8))
            rgbs.append(rgb.reshape(-1))
            dims.append(rgb.shape[:2][::-1])
    dragon_path = os.path.join(ref_root, "res", "blackDragon.jpg")
    dragon = ref_read(dragon_path)
    np.savez_compressed(
        os.path.join(HERE, "jpeg_golden.npz"),
        names=np.array(names), dims=np.array(dims, np.int32),
        jpeg_off=np.cumsum([0] + [len(b) for b in blobs]).astype(np.int64), jpeg=np.concatenate(blobs),
        rgb_off=np.cumsum([0] + [len(r) for r in rgbs]).astype(np.int64), rgb=np.concatenate(rgbs),
        dragon_jpeg=np.frombuffer(open(dragon_path, "rb").read(), np.uint8),
        dragon_dims=np.array(dragon.shape[:2][::-1], np.int32),
        dragon_sha256=np.array(hashlib.sha256(dragon.tobytes()).hexdigest()),
        dragon_crop=dragon[224:288, 224:288].copy())
    print(f"wrote {len(names)} JPEG cases + blackDragon.jpg")


if __name__ == "__main__":
    main()
