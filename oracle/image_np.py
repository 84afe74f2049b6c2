"""Oracle (test infrastructure only: imported by tests/, never by the package): image textures in
the fixed mode, restated in numpy from the file formats and the reference's texture code.

* PNG (RFC 2083) decoding to 8-bit RGB as stb_image documents it for three requested channels
  (grey replicated, alpha dropped, palette expanded, 1/2/4-bit grey scaled by 255 / (2^d - 1),
  16-bit samples reduced to the high byte); inflate is Python's zlib, independent of the
  renderer's own inflate.  A PNG writer (every colour type, bit depth and filter) makes the test
  images.
* The pyramid: stbi_loadf's LDR-to-linear conversion (c / 255)^2.2 in float32, rows flipped
  (core/ImageI.cuh:11-34); floor(log2(max(w, h))) levels (Mipmap_kernel.cu:45), each the 2 x 2
  box mean of the level below with black outside (pyramidInitKernel, Mipmap_kernel.cu:23-37),
  over the whole level (the reference's kernel fills only 16 >> l texels per axis).
* The lookup: Mipmap::lookUp / triangle / texel (materials/textures/Mipmap.cuh:14-73) at the fixed
  width 0.01 (ImageTexture.cuh:7-8), in the reference's float32 operation order; repeat wraps into
  the level and the coarsest-level read is texel (0, 0) of that level (the two fixes of the mode).

Parity for image textures cannot be pinned to the reference (its storage is undefined,
core/MemoryHelper.cuh:86-100); this restatement is the specification the renderer is held to."""
import struct
import zlib

import numpy as np

_SIG = b"\x89PNG\r\n\x1a\n"


def _chunk(kind, data):
    return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xffffffff)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _filter_row(f, row, prev, bpp):
    out = bytearray(len(row))
    for i, x in enumerate(row):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i] if prev is not None else 0
        c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
        pred = (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]
        out[i] = (x - pred) & 0xff
    return bytes(out)


def encode_png(samples, ctype, depth, filters=None, palette=None, level=6):
    """PNG bytes of an (h, w, channels) integer array of samples (channels by colour type: 0 grey,
    2 RGB, 3 palette index, 4 grey + alpha, 6 RGBA) at the given bit depth; filters: one filter
    type per row (default cycles 0..4)."""
    samples = np.asarray(samples)
    h, w = samples.shape[:2]
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    samples = samples.reshape(h, w, chans).astype(np.int64)
    bpp_bits = depth * chans
    bpp = max(1, bpp_bits // 8)
    raw = bytearray()
    prev = None
    for y in range(h):
        if depth == 16:
            row = b"".join(struct.pack(">H", int(v)) for v in samples[y].reshape(-1))
        elif depth == 8:
            row = bytes(int(v) for v in samples[y].reshape(-1))
        else:
            bits = "".join(format(int(v), "0%db" % depth) for v in samples[y].reshape(-1))
            bits += "0" * (-len(bits) % 8)
            row = bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))
        f = (filters[y] if filters is not None else y % 5)
        raw += bytes([f]) + _filter_row(f, row, prev, bpp)
        prev = row
    out = _SIG + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if ctype == 3:
        out += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    data = zlib.compress(bytes(raw), level)
    # split the image data over two IDAT chunks (decoders must concatenate them)
    half = len(data) // 2
    out += _chunk(b"IDAT", data[:half]) + _chunk(b"IDAT", data[half:]) + _chunk(b"IEND", b"")
    return out


def decode_png(data):
    """(w, h, rgb uint8 (h, w, 3), top row first) of a non-interlaced PNG."""
    assert data[:8] == _SIG, "not a PNG"
    pos, idat, plte = 8, b"", None
    while pos + 12 <= len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        kind, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
        pos += 12 + n
    assert interlace == 0
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp_bits = depth * chans
    stride, bpp = (w * bpp_bits + 7) // 8, max(1, bpp_bits // 8)
    raw = zlib.decompress(idat)
    rows, prev = [], None
    for y in range(h):
        f, src = raw[(stride + 1) * y], raw[(stride + 1) * y + 1:(stride + 1) * (y + 1)]
        cur = bytearray(stride)
        for i in range(stride):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i] if prev is not None else 0
            c = prev[i - bpp] if (prev is not None and i >= bpp) else 0
            cur[i] = (src[i] + (0, a, b, (a + b) >> 1, _paeth(a, b, c))[f]) & 0xff
        rows.append(bytes(cur))
        prev = cur
    px = np.frombuffer(b"".join(rows), np.uint8).reshape(h, stride)
    if depth == 16:
        s = px.reshape(h, w * chans, 2)[:, :, 0].reshape(h, w, chans).astype(np.int64)
    elif depth == 8:
        s = px[:, :w * chans].reshape(h, w, chans).astype(np.int64)
    else:
        bits = np.unpackbits(px, axis=1)[:, :w * chans * depth].reshape(h, w * chans, depth)
        s = (bits * (1 << np.arange(depth - 1, -1, -1))).sum(axis=2).reshape(h, w, chans)
        if ctype == 0:
            s = s * {1: 255, 2: 85, 4: 17}[depth]
    if ctype == 3:
        rgb = plte[s[:, :, 0]]
    elif ctype in (0, 4):
        rgb = np.repeat(s[:, :, :1], 3, axis=2)
    else:
        rgb = s[:, :, :3]
    return w, h, np.asarray(rgb, np.uint8)


def pyramid(w, h, rgb8, wrap):
    """The fixed mode's pyramid: dict(levels, lod, wrap, rgb=[(h_l, w_l, 3) float32, row 0 the
    bottom row])."""
    # correctly rounded float32 of (c / 255)^2.2 (numpy's own float32 power is off by an ulp for
    # some c; pow in double rounded once is glibc powf's value, which stb_image gets)
    lut = np.array([np.float32(np.power(np.float64(np.float32(c) / np.float32(255)), np.float64(np.float32(2.2))))
                    for c in range(256)], np.float32)
    levels = max(1, int(np.log2(np.float32(max(w, h)))))
    lod = np.float32(levels - 1) + np.log2(np.float32(0.01))
    lv = [lut[rgb8[::-1].astype(np.int64)]]
    for l in range(1, levels):
        p = lv[-1]
        ph, pw = p.shape[:2]
        lw, lh = max(1, w >> l), max(1, h >> l)
        q = np.zeros((2 * lh + 2, 2 * lw + 2, 3), np.float32)
        q[:min(ph, 2 * lh + 2), :min(pw, 2 * lw + 2)] = p[:2 * lh + 2, :2 * lw + 2]
        a, b = q[0:2 * lh:2, 0:2 * lw:2], q[0:2 * lh:2, 1:2 * lw:2]
        c, d = q[1:2 * lh:2, 0:2 * lw:2], q[1:2 * lh:2, 1:2 * lw:2]
        lv.append((np.float32(0.25) * (((a + b) + c) + d)).astype(np.float32))
    return {"levels": levels, "lod": np.float32(lod), "wrap": int(wrap), "rgb": lv}


def _texel(img, l, s, t):
    lv = img["rgb"][l]
    h, w = lv.shape[:2]
    s, t = np.asarray(s, np.int64), np.asarray(t, np.int64)
    if img["wrap"] == 0:
        s, t = np.mod(s, w), np.mod(t, h)
        ok = np.ones(s.shape, bool)
    elif img["wrap"] == 2:
        s, t = np.clip(s, 0, w - 1), np.clip(t, 0, h - 1)
        ok = np.ones(s.shape, bool)
    else:
        ok = (s >= 0) & (s < w) & (t >= 0) & (t < h)
    v = lv[np.where(ok, t, 0), np.where(ok, s, 0)]
    return np.where(ok[..., None], v, np.float32(0)).astype(np.float32)


def _bilerp(img, l, st):
    l = min(max(l, 0), img["levels"] - 1)
    h, w = img["rgb"][l].shape[:2]
    one, half = np.float32(1), np.float32(0.5)
    s = st[:, 0] * np.float32(w) - half
    t = st[:, 1] * np.float32(h) - half
    s0, t0 = np.floor(s).astype(np.int64), np.floor(t).astype(np.int64)
    ds, dt = (s - s0.astype(np.float32)).astype(np.float32), (t - t0.astype(np.float32)).astype(np.float32)
    w00 = ((one - ds) * (one - dt))[:, None]
    w01 = ((one - ds) * dt)[:, None]
    w10 = (ds * (one - dt))[:, None]
    w11 = (ds * dt)[:, None]
    return (((_texel(img, l, s0, t0) * w00 + _texel(img, l, s0, t0 + 1) * w01) + _texel(img, l, s0 + 1, t0) * w10) +
            _texel(img, l, s0 + 1, t0 + 1) * w11).astype(np.float32)


def lookup(img, st):
    """Mipmap::lookUp at width 0.01 for (n, 2) float32 texture coordinates: (n, 3) float32."""
    st = np.asarray(st, np.float32).reshape(-1, 2)
    lod, levels = img["lod"], img["levels"]
    if lod < 0:
        return _bilerp(img, 0, st)
    if lod >= np.float32(levels - 1):
        return np.broadcast_to(_texel(img, levels - 1, np.array([0]), np.array([0])), (len(st), 3)).copy()
    il = int(np.floor(lod))
    delta = np.float32(lod - np.float32(il))
    return (_bilerp(img, il, st) * (np.float32(1) - delta) + _bilerp(img, il + 1, st) * delta).astype(np.float32)
