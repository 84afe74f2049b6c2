"""Test infrastructure (oracle side): a baseline JPEG writer (ITU-T T.81, sequential DCT with
Huffman coding, 8-bit samples) that makes the decoder's test inputs in forms the reference's own
JPEG writer (stbi_write_jpg, extern/stb_image_write.h) never produces: any sampling factors,
greyscale, four components, restart intervals, one scan per component, 16-bit quantisation
tables, SOF1, Adobe colour-transform flags, 'R' 'G' 'B' component ids.  Nothing here decodes:
the expected pixels of every input come from the reference's own reader (stb_image, through
oracle/_ref/lts_ref imread).

Huffman tables are built per image from its symbol counts with the length-limiting procedure of
T.81 Annex K.2 (one reserved code point keeps the all-ones code unused)."""
import heapq
import struct

import numpy as np

ZIGZAG = np.array([0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5, 12, 19, 26, 33, 40, 48, 41, 34, 27, 20,
                   13, 6, 7, 14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51, 58, 59, 52,
                   45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63])  # zig-zag position -> natural index


def _dct_matrix():
    k = np.arange(8)
    c = np.where(k == 0, np.sqrt(1 / 8), np.sqrt(2 / 8))
    return c[:, None] * np.cos((2 * k[None, :] + 1) * k[:, None] * np.pi / 16)


_C = _dct_matrix()


def _fdct(block):
    """Orthonormal 2-D DCT-II of an 8x8 block of level-shifted samples."""
    return _C @ block @ _C.T


def _category(v):
    return 0 if v == 0 else int(abs(v)).bit_length()


def _bits(v, s):
    """The s low bits of coefficient v as T.81 F.1.2.1 codes it (negative: v - 1)."""
    return (v if v >= 0 else v + (1 << s) - 1) & ((1 << s) - 1)


def huffman_lengths(freq):
    """Code lengths <= 16 for the symbols of `freq` (dict symbol -> count) by T.81 K.2: Huffman
    sizes with a reserved symbol of count 1, then lengths above 16 folded down."""
    syms = sorted(freq)
    items = [(freq[s], i, [s]) for i, s in enumerate(syms)] + [(1, len(syms), [None])]
    size = {s: 0 for s in syms}
    size[None] = 0
    heapq.heapify(items)
    tie = len(syms) + 1
    if len(items) == 1:
        size[syms[0]] = 1
    while len(items) > 1:
        f1, _, a = heapq.heappop(items)
        f2, _, b = heapq.heappop(items)
        for s in a + b:
            size[s] += 1
        heapq.heappush(items, (f1 + f2, tie, a + b))
        tie += 1
    bits = [0] * 33
    for s, n in size.items():
        bits[n] += 1
    i = 32
    while i > 16:  # K.2 figure K.3: adjust_bits
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
        i -= 1
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1  # the reserved code point
    # assign the lengths to the symbols, most frequent first
    order = sorted(syms, key=lambda s: (-freq[s], s))
    lengths, k = {}, 0
    for n in range(1, 17):
        for _ in range(bits[n]):
            lengths[order[k]] = n
            k += 1
    return lengths


def canonical(lengths):
    """(counts[16], symbols in code order, {symbol: (code, length)}) of T.81 C.2."""
    order = sorted(lengths, key=lambda s: (lengths[s], s))
    counts = [0] * 16
    for s in order:
        counts[lengths[s] - 1] += 1
    codes, code, prev = {}, 0, 0
    for s in order:
        n = lengths[s]
        code <<= n - prev
        prev = n
        codes[s] = (code, n)
        code += 1
    return counts, order, codes


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def put(self, value, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((value >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)
                self.acc = self.n = 0

    def flush(self):
        """Pad the last byte with 1-bits (T.81 F.1.2.3)."""
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)


def _segment(marker, body):
    return bytes([0xFF, marker]) + struct.pack(">H", len(body) + 2) + body


def encode(planes, factors, quant, *, ids=None, tq=None, restart=0, interleaved=True, sixteen_bit=False,
           sof=0xC0, jfif=True, adobe=None, width=None, height=None):
    """A baseline JPEG of the component sample planes (uint8, each at least its component's
    size).  factors: (h, v) per component; quant: 8x8 quantisation tables (natural order, values
    1..255, or 1..65535 with sixteen_bit); tq: table index per component (default: 0 for the first
    component, 1 for the others); restart: MCUs per restart interval (0: none); interleaved: one
    scan of all components (else one scan per component); adobe: the APP14 colour transform (None:
    no APP14 segment)."""
    nc = len(planes)
    ids = ids if ids is not None else list(range(1, nc + 1))
    tq = tq if tq is not None else [0] + [1] * (nc - 1)
    hmax = max(h for h, _ in factors)
    vmax = max(v for _, v in factors)
    if width is None or height is None:
        height, width = planes[0].shape[0] * vmax // factors[0][1], planes[0].shape[1] * hmax // factors[0][0]
    mcux = -(-width // (8 * hmax))
    mcuy = -(-height // (8 * vmax))
    # coefficient blocks of each component over the MCU grid (edge-replicated padding)
    blocks = []
    for c, (h, v) in enumerate(factors):
        cx = -(-width * h // hmax)
        cy = -(-height * v // vmax)
        p = np.asarray(planes[c], np.float64)[:cy, :cx]
        full = np.pad(p, ((0, mcuy * v * 8 - cy), (0, mcux * h * 8 - cx)), mode="edge")
        q = np.asarray(quant[tq[c]], np.float64).reshape(8, 8)
        by, bx = full.shape[0] // 8, full.shape[1] // 8
        coef = np.zeros((by, bx, 64), np.int64)
        for j in range(by):
            for i in range(bx):
                f = _fdct(full[8 * j:8 * j + 8, 8 * i:8 * i + 8] - 128.0)
                coef[j, i] = np.round(f / q).astype(np.int64).reshape(64)[ZIGZAG]
        blocks.append((coef, -(-cx // 8), -(-cy // 8)))
    table_of = [0] + [1] * (nc - 1)  # Huffman table pair per component

    if interleaved and nc > 1:
        scans = [list(range(nc))]
    else:
        scans = [[c] for c in range(nc)]

    def units(scan):
        """(component, block) sequence of the scan, grouped into restart units."""
        if len(scan) == 1:
            coef, bw, bh = blocks[scan[0]]
            for j in range(bh):
                for i in range(bw):
                    yield [(scan[0], coef[j, i])]
        else:
            for j in range(mcuy):
                for i in range(mcux):
                    mcu = []
                    for c in scan:
                        h, v = factors[c]
                        for y in range(v):
                            for x in range(h):
                                mcu.append((c, blocks[c][0][j * v + y, i * h + x]))
                    yield mcu

    def symbols(scan):
        """Per unit: the (component, kind, symbol, extra bits, extra length) sequence."""
        pred = {c: 0 for c in scan}
        out = []
        for k, unit in enumerate(units(scan)):
            if restart and k and k % restart == 0:
                out.append(None)
                pred = {c: 0 for c in scan}
            for c, z in unit:
                diff = int(z[0]) - pred[c]
                pred[c] = int(z[0])
                s = _category(diff)
                out.append((c, 0, s, _bits(diff, s), s))
                run = 0
                last = max([i for i in range(1, 64) if z[i] != 0], default=0)
                for i in range(1, last + 1):
                    a = int(z[i])
                    if a == 0:
                        run += 1
                        continue
                    while run > 15:
                        out.append((c, 1, 0xF0, 0, 0))
                        run -= 16
                    s = _category(a)
                    out.append((c, 1, (run << 4) | s, _bits(a, s), s))
                    run = 0
                if last < 63:
                    out.append((c, 1, 0x00, 0, 0))
        return out

    seqs = [symbols(s) for s in scans]
    freq = {}
    for seq in seqs:
        for e in seq:
            if e is not None:
                key = (table_of[e[0]], e[1])
                freq.setdefault(key, {})
                freq[key][e[2]] = freq[key].get(e[2], 0) + 1
    huff = {key: canonical(huffman_lengths(f)) for key, f in freq.items()}

    out = bytearray(b"\xFF\xD8")
    if jfif:
        out += _segment(0xE0, b"JFIF\x00\x01\x01\x00\x00\x01\x00\x01\x00\x00")
    if adobe is not None:
        out += _segment(0xEE, b"Adobe\x00" + bytes([100, 0, 0, 0, 0, adobe]))
    for t in sorted(set(tq)):
        q = np.asarray(quant[t]).reshape(64)[ZIGZAG]
        body = bytes([(0x10 if sixteen_bit else 0) | t]) + (
            b"".join(struct.pack(">H", int(x)) for x in q) if sixteen_bit else bytes(int(x) for x in q))
        out += _segment(0xDB, body)
    sofbody = struct.pack(">BHHB", 8, height, width, nc) + b"".join(
        bytes([ids[c], (factors[c][0] << 4) | factors[c][1], tq[c]]) for c in range(nc))
    out += _segment(sof, sofbody)
    for (tab, kind), (counts, order, _) in sorted(huff.items()):
        out += _segment(0xC4, bytes([(kind << 4) | tab]) + bytes(counts) + bytes(order))
    if restart:
        out += _segment(0xDD, struct.pack(">H", restart))
    for scan, seq in zip(scans, seqs):
        body = bytes([len(scan)]) + b"".join(bytes([ids[c], (table_of[c] << 4) | table_of[c]]) for c in scan)
        out += _segment(0xDA, body + b"\x00\x3F\x00")
        bw = _BitWriter()
        rst = 0
        for e in seq:
            if e is None:
                bw.flush()
                out += bw.out
                out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) & 7
                bw = _BitWriter()
                continue
            c, kind, sym, extra, n = e
            code, length = huff[(table_of[c], kind)][2][sym]
            bw.put(code, length)
            if n:
                bw.put(extra, n)
        bw.flush()
        out += bw.out
    out += b"\xFF\xD9"
    return bytes(out)


def test_planes(rng, width, height, factors):
    """Smooth gradients plus noise per component, each at its sampled size."""
    hmax = max(h for h, _ in factors)
    vmax = max(v for _, v in factors)
    planes = []
    for c, (h, v) in enumerate(factors):
        cx, cy = -(-width * h // hmax), -(-height * v // vmax)
        yy, xx = np.mgrid[0:cy, 0:cx]
        base = 128 + 90 * np.sin(xx / (3.0 + c) + yy / (5.0 + 2 * c)) * np.cos(yy / 7.0)
        planes.append(np.clip(base + rng.normal(0, 12, (cy, cx)), 0, 255).astype(np.uint8))
    return planes


def quant_table(scale):
    """A quantisation table growing with frequency, values >= 1 (natural order)."""
    u, v = np.mgrid[0:8, 0:8]
    return np.maximum(1, np.round(scale * (1 + u + v))).astype(np.int64)
