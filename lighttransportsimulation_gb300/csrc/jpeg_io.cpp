// Baseline JPEG decoding (ITU-T T.81: sequential DCT, Huffman coding, 8-bit samples) into 8-bit
// RGB as the reference's image reader produces it.  The reference loads image textures with
// stbi_loadf(file, ..., 3) (core/ImageI.cuh:14) from its vendored stb_image v2.27
// (extern/stb_image.h); for the pixels to match bit for bit this decoder restates the parts of
// that library that are not fixed by the standard:
//   * the integer inverse DCT (stb_image.h:2380-2480): the Loeffler-Ligtenberg-Moschytz
//     factorisation of the IJG "islow" IDCT with 12-bit constants, a column pass keeping two
//     extra bits (rounding shift by 10), a row pass with the +128 level shift folded into the
//     rounding (shift by 17), results clamped to 0..255;
//   * chroma upsampling (stb_image.h:3396-3600): the JFIF-centred triangle filters for factors
//     of two horizontally, vertically or both (weights 3:1, 9:3:3:1), nearest neighbour for other
//     factors, and its row schedule (which input rows feed each output row);
//   * YCbCr to RGB in 20-bit fixed point (stb_image.h:3603-3628), with the Cb term of green
//     truncated to 16 fractional bits; Adobe RGB / CMYK / YCCK handling (stb_image.h:3870-3930);
//   * its marker and bit-buffer behaviour (stb_image.h:2031-2047, 2875-2975, 3059-3392).
// Progressive (SOF2), lossless, arithmetic-coded and 12-bit JPEGs are refused (UNSUPPORTED);
// malformed streams where stb_image would return undefined pixels are refused (PARSE).
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lts_capi.h"
#include "image_io.hpp"

namespace lts {
namespace {

// Natural (row-major) index of the k-th coefficient in zig-zag order (T.81 figure A.6).
const uint8_t kNatural[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                              12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                              35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                              58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct HuffTable {
    bool defined = false;
    uint8_t lookup_len[512];    // 9-bit prefix -> code length (0: longer than 9 bits)
    uint8_t lookup_val[512];    // 9-bit prefix -> symbol
    int32_t maxcode[18];        // largest code of each length, left-aligned to 16 bits, + 1
    int32_t delta[17];          // symbol index - code, per length
    uint8_t vals[256];
};

// Canonical code assignment (T.81 C.2): codes of each length follow the previous length's
// last code, shifted left.  False for a code set that overflows its lengths.
bool build_huff(HuffTable& t, const uint8_t* counts, const uint8_t* symbols, int nsym) {
    memset(t.lookup_len, 0, sizeof(t.lookup_len));
    int code = 0, k = 0;
    for (int len = 1; len <= 16; ++len) {
        t.delta[len] = k - code;
        for (int i = 0; i < counts[len - 1]; ++i, ++k, ++code) {
            if (code >= (1 << len)) return false;  // more codes than the length holds
            if (len <= 9) {
                const int first = code << (9 - len), span = 1 << (9 - len);
                for (int j = 0; j < span; ++j) {
                    t.lookup_len[first + j] = (uint8_t)len;
                    t.lookup_val[first + j] = symbols[k];
                }
            }
        }
        t.maxcode[len] = code << (16 - len);  // exclusive bound on 16-bit prefixes of this length
        code <<= 1;
    }
    t.maxcode[17] = 0x7fffffff;
    memcpy(t.vals, symbols, (size_t)nsym);
    t.defined = true;
    return true;
}

// Entropy-coded segment reader with the byte stuffing of T.81 F.1.2.3: 0xFF 0x00 is a data
// byte 0xFF; 0xFF followed by anything else is a marker, after which the reader supplies zero
// bits.  The buffer holds up to 32 bits, most significant first.
struct Bits {
    const uint8_t* d;
    size_t n, pos;
    uint32_t buf = 0;
    int count = 0;
    bool stopped = false;  // a marker (or the end of the data) was reached
    int marker = -1;
    uint8_t byte() { return pos < n ? d[pos++] : 0; }
    void fill() {
        do {
            uint32_t b = stopped ? 0u : byte();
            if (b == 0xFF) {
                uint8_t c = byte();
                while (c == 0xFF) c = byte();
                if (c != 0) {
                    marker = c;
                    stopped = true;
                    return;
                }
            }
            if (b) buf |= b << (24 - count);  // (past a marker the count may be negative; b is 0)
            count += 8;
        } while (count <= 24);
    }
    void reset() {
        buf = 0;
        count = 0;
        stopped = false;
        marker = -1;
    }
    // One Huffman symbol, or -1 for a code the table does not hold or that runs past the data.
    int decode(const HuffTable& t) {
        if (count < 16) fill();
        const uint32_t top9 = buf >> 23;
        int len = t.lookup_len[top9], sym;
        if (len) {
            sym = t.lookup_val[top9];
        } else {
            const int32_t top16 = (int32_t)(buf >> 16);
            len = 10;
            while (len <= 16 && top16 >= t.maxcode[len]) ++len;
            if (len > 16) return -1;
            const int code = top16 >> (16 - len);
            sym = t.vals[code + t.delta[len]];
        }
        if (len > count) return -1;
        buf <<= len;
        count -= len;
        return sym;
    }
    // n raw bits (1..15) as the signed coefficient value of T.81 F.2.2.1 (EXTEND).
    int receive_extend(int nb) {
        if (count < nb) fill();
        const uint32_t v = buf >> (32 - nb);
        buf <<= nb;
        count -= nb;
        return (v >> (nb - 1)) ? (int)v : (int)v - (1 << nb) + 1;
    }
};

struct Component {
    int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
    int x = 0, y = 0;      // samples covering the image
    int w2 = 0, h2 = 0;    // samples of the whole MCU grid (the plane's stride and height)
    int dc_pred = 0;
    std::vector<uint8_t> plane;
};

inline uint8_t clamp255(int64_t x) { return (uint8_t)(x < 0 ? 0 : x > 255 ? 255 : x); }

// Scaled constants of the islow factorisation as stb_image forms them (stb_image.h:2380): the
// float constant times 4096, plus one half, truncated toward zero -- so a negative constant is
// rounded up, not to nearest (-1.847759065 gives -7567).
constexpr int fix(float c) { return (int)(c * 4096 + 0.5); }
// YCbCr factors (stb_image.h:3603): round(c * 4096) in float, then 8 more fraction bits.
constexpr int color_fix(float c) { return ((int)(c * 4096.0f + 0.5f)) << 8; }

// One 8-point inverse DCT over in[0], in[s], ..., in[7 s] (s the stride), writing the even
// part's sums (x0..x3) and the odd part's (t0..t3) that the caller combines and descales.
// (64-bit sums: the coefficients of a valid stream keep every sum far inside 32 bits, where these
// equal the reference's int arithmetic; a corrupt stream's cannot overflow them.)
struct Idct1d {
    int64_t x0, x1, x2, x3, t0, t1, t2, t3;
    Idct1d(int64_t s0, int64_t s1, int64_t s2, int64_t s3, int64_t s4, int64_t s5, int64_t s6, int64_t s7) {
        // even part: rotation of (s2, s6) by the c6 / c2 terms, butterflies with s0 +- s4
        const int64_t z1 = (s2 + s6) * fix(0.5411961f);
        const int64_t e2 = z1 + s6 * fix(-1.847759065f), e3 = z1 + s2 * fix(0.765366865f);
        const int64_t e0 = (s0 + s4) * 4096, e1 = (s0 - s4) * 4096;
        x0 = e0 + e3;
        x3 = e0 - e3;
        x1 = e1 + e2;
        x2 = e1 - e2;
        // odd part (s7, s5, s3, s1)
        int64_t a0 = s7, a1 = s5, a2 = s3, a3 = s1;
        int64_t p3 = a0 + a2, p4 = a1 + a3, p1 = a0 + a3, p2 = a1 + a2;
        const int64_t p5 = (p3 + p4) * fix(1.175875602f);
        a0 *= fix(0.298631336f);
        a1 *= fix(2.053119869f);
        a2 *= fix(3.072711026f);
        a3 *= fix(1.501321110f);
        p1 = p5 + p1 * fix(-0.899976223f);
        p2 = p5 + p2 * fix(-2.562915447f);
        p3 *= fix(-1.961570560f);
        p4 *= fix(-0.390180644f);
        t3 = a3 + p1 + p4;
        t2 = a2 + p2 + p3;
        t1 = a1 + p2 + p4;
        t0 = a0 + p1 + p3;
    }
};

// 8x8 block of dequantised coefficients (natural order) -> samples at out (row stride `stride`).
void idct_block(const short* c, uint8_t* out, int stride) {
    int64_t tmp[64];
    for (int col = 0; col < 8; ++col) {
        const short* d = c + col;
        int64_t* t = tmp + col;
        if (!(d[8] | d[16] | d[24] | d[32] | d[40] | d[48] | d[56])) {
            const int64_t dc = d[0] * 4;  // a column of DC alone: its exact result
            for (int r = 0; r < 8; ++r) t[8 * r] = dc;
            continue;
        }
        Idct1d f(d[0], d[8], d[16], d[24], d[32], d[40], d[48], d[56]);
        f.x0 += 512;
        f.x1 += 512;
        f.x2 += 512;
        f.x3 += 512;  // 12 fraction bits, keep 2: round at bit 10
        t[0] = (f.x0 + f.t3) >> 10;
        t[56] = (f.x0 - f.t3) >> 10;
        t[8] = (f.x1 + f.t2) >> 10;
        t[48] = (f.x1 - f.t2) >> 10;
        t[16] = (f.x2 + f.t1) >> 10;
        t[40] = (f.x2 - f.t1) >> 10;
        t[24] = (f.x3 + f.t0) >> 10;
        t[32] = (f.x3 - f.t0) >> 10;
    }
    for (int row = 0; row < 8; ++row) {
        const int64_t* t = tmp + 8 * row;
        Idct1d f(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7]);
        // 12 + 2 fraction bits and the two passes' factor 8: 17 bits; round and add 128
        const int64_t bias = 65536 + (128 << 17);
        f.x0 += bias;
        f.x1 += bias;
        f.x2 += bias;
        f.x3 += bias;
        uint8_t* o = out + (size_t)row * stride;
        o[0] = clamp255((f.x0 + f.t3) >> 17);
        o[7] = clamp255((f.x0 - f.t3) >> 17);
        o[1] = clamp255((f.x1 + f.t2) >> 17);
        o[6] = clamp255((f.x1 - f.t2) >> 17);
        o[2] = clamp255((f.x2 + f.t1) >> 17);
        o[5] = clamp255((f.x2 - f.t1) >> 17);
        o[3] = clamp255((f.x3 + f.t0) >> 17);
        o[4] = clamp255((f.x3 - f.t0) >> 17);
    }
}

struct Decoder {
    Decoder(const uint8_t* data, size_t size) : d(data), n(size) { memset(quant, 0, sizeof(quant)); }
    const uint8_t* d;
    size_t n, pos = 0;
    int width = 0, height = 0, ncomp = 0;
    int hmax = 1, vmax = 1, mcux = 0, mcuy = 0;
    int restart = 0;
    bool jfif = false, frame = false;
    int adobe_transform = -1;
    int rgb_ids = 0;  // components whose ids spell 'R', 'G', 'B'
    uint16_t quant[4][64];  // natural order
    HuffTable dc[4], ac[4];
    Component comp[4];
    std::string err;
    int code = LTS_ERR_PARSE;

    bool fail(const char* m, int c = LTS_ERR_PARSE) {
        err = m;
        code = c;
        return false;
    }
    int u8() { return pos < n ? d[pos++] : -1; }
    int u16() {
        const int a = u8(), b = u8();
        return (a < 0 || b < 0) ? -1 : (a << 8 | b);
    }
    // The next marker code: 0xFF, any fill 0xFF bytes, then the code; -1 if the bytes here are
    // not a marker.
    int marker() {
        if (u8() != 0xFF) return -1;
        int c = u8();
        while (c == 0xFF) c = u8();
        return c;
    }

    bool segment(int m) {
        if (m == 0xDD) {  // DRI
            if (u16() != 4) return fail("bad DRI length");
            restart = u16();
            return restart >= 0 || fail("truncated DRI");
        }
        if (m == 0xDB) {  // DQT
            int len = u16() - 2;
            while (len > 0) {
                const int pq = u8();
                if (pq < 0) return fail("truncated DQT");
                const int p = pq >> 4, t = pq & 15;
                if (p > 1 || t > 3) return fail("bad DQT table");
                for (int i = 0; i < 64; ++i) {
                    const int q = p ? u16() : u8();
                    if (q < 0) return fail("truncated DQT");
                    quant[t][kNatural[i]] = (uint16_t)q;
                }
                len -= p ? 129 : 65;
            }
            return len == 0 || fail("bad DQT length");
        }
        if (m == 0xC4) {  // DHT
            int len = u16() - 2;
            while (len > 0) {
                const int tcth = u8();
                if (tcth < 0) return fail("truncated DHT");
                const int tc = tcth >> 4, th = tcth & 15;
                if (tc > 1 || th > 3) return fail("bad DHT header");
                uint8_t counts[16], syms[256];
                int total = 0;
                for (int i = 0; i < 16; ++i) {
                    const int c = u8();
                    if (c < 0) return fail("truncated DHT");
                    counts[i] = (uint8_t)c;
                    total += c;
                }
                if (total > 256) return fail("bad DHT counts");
                for (int i = 0; i < total; ++i) {
                    const int s = u8();
                    if (s < 0) return fail("truncated DHT");
                    syms[i] = (uint8_t)s;
                }
                if (!build_huff(tc ? ac[th] : dc[th], counts, syms, total)) return fail("bad Huffman code lengths");
                len -= 17 + total;
            }
            return len == 0 || fail("bad DHT length");
        }
        if ((m >= 0xE0 && m <= 0xEF) || m == 0xFE) {  // APPn, COM
            int len = u16();
            if (len < 2) return fail("bad segment length");
            len -= 2;
            const size_t start = pos;
            if (m == 0xE0 && len >= 5 && pos + 5 <= n && !memcmp(d + pos, "JFIF\0", 5)) jfif = true;
            if (m == 0xEE && len >= 12 && pos + 12 <= n && !memcmp(d + pos, "Adobe\0", 6)) adobe_transform = d[pos + 11];
            if (start + (size_t)len > n) return fail("truncated segment");
            pos = start + (size_t)len;
            return true;
        }
        return fail("unknown JPEG marker");
    }

    bool frame_header(int m) {
        if (m == 0xC2) return fail("progressive JPEG is not decoded", LTS_ERR_UNSUPPORTED);
        const int len = u16(), p = u8();
        if (len < 11) return fail("bad SOF length");
        if (p != 8) return fail("only 8-bit JPEG is decoded", LTS_ERR_UNSUPPORTED);
        height = u16();
        width = u16();
        ncomp = u8();
        if (height <= 0) return fail("JPEG without a height", LTS_ERR_UNSUPPORTED);
        if (width <= 0) return fail("JPEG of width 0");
        if (width > (1 << 24) || height > (1 << 24)) return fail("JPEG too large");
        if (ncomp != 1 && ncomp != 3 && ncomp != 4) return fail("bad JPEG component count");
        if (len != 8 + 3 * ncomp) return fail("bad SOF length");
        static const char rgb[3] = {'R', 'G', 'B'};
        for (int i = 0; i < ncomp; ++i) {
            Component& c = comp[i];
            c.id = u8();
            const int hv = u8();
            c.tq = u8();
            if (c.tq < 0 || hv < 0) return fail("truncated SOF");
            if (ncomp == 3 && c.id == rgb[i]) ++rgb_ids;
            c.h = hv >> 4;
            c.v = hv & 15;
            if (c.h < 1 || c.h > 4 || c.v < 1 || c.v > 4) return fail("bad sampling factor");
            if (c.tq > 3) return fail("bad quantisation table index");
        }
        if ((double)width * height * ncomp > 2147483647.0) return fail("JPEG too large");
        for (int i = 0; i < ncomp; ++i) {
            hmax = comp[i].h > hmax ? comp[i].h : hmax;
            vmax = comp[i].v > vmax ? comp[i].v : vmax;
        }
        for (int i = 0; i < ncomp; ++i)
            if (hmax % comp[i].h || vmax % comp[i].v) return fail("non-integer sampling ratio");
        mcux = (width + 8 * hmax - 1) / (8 * hmax);
        mcuy = (height + 8 * vmax - 1) / (8 * vmax);
        for (int i = 0; i < ncomp; ++i) {
            Component& c = comp[i];
            c.x = (width * c.h + hmax - 1) / hmax;
            c.y = (height * c.v + vmax - 1) / vmax;
            c.w2 = mcux * c.h * 8;
            c.h2 = mcuy * c.v * 8;
            c.plane.assign((size_t)c.w2 * c.h2, 0);
        }
        frame = true;
        return true;
    }

    bool block(Bits& b, Component& c, short* coef) {
        const HuffTable &hd = dc[c.td], &ha = ac[c.ta];
        if (!hd.defined || !ha.defined) return fail("scan uses an undefined Huffman table");
        const uint16_t* q = quant[c.tq];
        const int t = b.decode(hd);
        if (t < 0 || t > 15) return fail("bad Huffman code");
        memset(coef, 0, 64 * sizeof(short));
        const int diff = t ? b.receive_extend(t) : 0;
        c.dc_pred = (int)((uint32_t)c.dc_pred + (uint32_t)diff);  // wraps, as int arithmetic does in practice
        coef[0] = (short)(uint16_t)((uint32_t)c.dc_pred * q[0]);
        for (int k = 1; k < 64;) {
            const int rs = b.decode(ha);
            if (rs < 0) return fail("bad Huffman code");
            const int r = rs >> 4, s = rs & 15;
            if (s == 0) {
                if (rs != 0xF0) break;  // end of block
                k += 16;                // sixteen zeros
                continue;
            }
            k += r;
            if (k > 63) return fail("coefficient run past the block");
            const int z = kNatural[k++];
            coef[z] = (short)(uint16_t)((uint32_t)b.receive_extend(s) * q[z]);
        }
        return true;
    }

    // One scan's entropy-coded data (T.81 E.2.3-E.2.5): one component in its own block order, or
    // the listed components interleaved MCU by MCU; restart markers every `restart` MCUs.
    bool scan(const int* order, int ns) {
        Bits b{d, n, pos};
        for (int i = 0; i < ncomp; ++i) comp[i].dc_pred = 0;
        int todo = restart ? restart : 0x7fffffff;
        short coef[64];
        // end of one MCU (one block in a single-component scan): count down the restart
        // interval; at its end the next marker must be a restart marker, unless the scan is done
        // (then it is whatever follows the scan)
        long units_left = 0;
        bool stop = false;
        auto next = [&]() {
            --units_left;
            if (--todo > 0) return;
            if (b.count < 24) b.fill();
            if (b.marker < 0xD0 || b.marker > 0xD7) {
                stop = true;
                return;
            }
            b.reset();
            for (int i = 0; i < ncomp; ++i) comp[i].dc_pred = 0;
            todo = restart ? restart : 0x7fffffff;
        };
        if (ns == 1) {
            Component& c = comp[order[0]];
            const int bw = (c.x + 7) >> 3, bh = (c.y + 7) >> 3;
            units_left = (long)bw * bh;
            for (int j = 0; j < bh && !stop; ++j)
                for (int i = 0; i < bw && !stop; ++i) {
                    if (!block(b, c, coef)) return false;
                    idct_block(coef, c.plane.data() + (size_t)c.w2 * j * 8 + i * 8, c.w2);
                    next();
                }
        } else {
            units_left = (long)mcux * mcuy;
            for (int j = 0; j < mcuy && !stop; ++j)
                for (int i = 0; i < mcux && !stop; ++i) {
                    for (int k = 0; k < ns; ++k) {
                        Component& c = comp[order[k]];
                        for (int y = 0; y < c.v; ++y)
                            for (int x = 0; x < c.h; ++x) {
                                if (!block(b, c, coef)) return false;
                                const size_t x2 = (size_t)(i * c.h + x) * 8, y2 = (size_t)(j * c.v + y) * 8;
                                idct_block(coef, c.plane.data() + c.w2 * y2 + x2, c.w2);
                            }
                    }
                    next();
                }
        }
        // a restart marker missing before the scan's end leaves the rest undecoded
        if (stop && units_left > 0) return fail("restart marker missing");
        // continue at the marker the reader stopped on (its code already read), else at the next
        // 0xFF in the stream
        pos = b.pos;
        if (b.stopped) {
            pending = b.marker;
        } else {
            while (pos < n && d[pos] != 0xFF) ++pos;
            pending = -1;
        }
        return true;
    }
    int pending = -1;  // a marker code already read by the entropy decoder

    int next_marker() {
        if (pending >= 0) {
            const int m = pending;
            pending = -1;
            return m;
        }
        return marker();
    }

    bool decode() {
        if (n < 2 || d[0] != 0xFF || d[1] != 0xD8) return fail("not a JPEG file", LTS_ERR_UNSUPPORTED);
        pos = 2;
        int m = marker();
        // tables and application segments up to the frame header
        while (!(m == 0xC0 || m == 0xC1 || m == 0xC2)) {
            if (m < 0) return fail("expected a marker");
            if ((m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC))
                return fail("lossless or arithmetic-coded JPEG is not decoded", LTS_ERR_UNSUPPORTED);
            if (!segment(m)) return false;
            m = marker();
            while (m < 0) {  // padding between segments
                if (pos >= n) return fail("no frame header");
                m = marker();
            }
        }
        if (!frame_header(m)) return false;
        bool scanned = false;
        m = next_marker();
        while (m != 0xD9) {
            if (m == 0xDA) {
                const int ls = u16(), ns = u8();
                if (ns < 1 || ns > 4 || ns > ncomp) return fail("bad SOS component count");
                if (ls != 6 + 2 * ns) return fail("bad SOS length");
                int order[4];
                for (int i = 0; i < ns; ++i) {
                    const int id = u8(), t = u8();
                    int which = 0;
                    while (which < ncomp && comp[which].id != id) ++which;
                    if (which == ncomp || t < 0) return fail("SOS names an unknown component");
                    comp[which].td = t >> 4;
                    comp[which].ta = t & 15;
                    if (comp[which].td > 3 || comp[which].ta > 3) return fail("bad Huffman table index");
                    order[i] = which;
                }
                const int ss = u8(), se = u8(), ahal = u8();
                if (ss != 0 || ahal != 0 || se < 0) return fail("bad SOS spectral selection");
                if (!scan(order, ns)) return false;
                scanned = true;
            } else if (m == 0xDC) {  // DNL
                if (u16() != 4 || u16() != height) return fail("bad DNL");
            } else if (m < 0) {
                return fail("expected a marker");
            } else if (!segment(m)) {
                return false;
            }
            m = next_marker();
        }
        if (!scanned) return fail("JPEG without a scan");
        return true;
    }

    // Row schedule of one component's upsampling (stb_image.h:3850-3888): output row j reads
    // `near` and `far` input rows; far is the neighbour row on the side of the output row.
    struct Resampler {
        int hs, vs, ystep, ypos = 0, wlo;
        const uint8_t *line0, *line1;
    };

    void upsample_row(const Resampler& r, const uint8_t* nearr, const uint8_t* farr, uint8_t* out) const {
        const int w = r.wlo;
        if (r.hs == 1 && r.vs == 1) {
            memcpy(out, nearr, (size_t)w);
        } else if (r.hs == 1 && r.vs == 2) {
            for (int i = 0; i < w; ++i) out[i] = (uint8_t)((3 * nearr[i] + farr[i] + 2) >> 2);
        } else if (r.hs == 2 && r.vs == 1) {
            if (w == 1) {
                out[0] = out[1] = nearr[0];
                return;
            }
            out[0] = nearr[0];
            out[1] = (uint8_t)((nearr[0] * 3 + nearr[1] + 2) >> 2);
            int i = 1;
            for (; i < w - 1; ++i) {
                const int c = 3 * nearr[i] + 2;
                out[2 * i] = (uint8_t)((c + nearr[i - 1]) >> 2);
                out[2 * i + 1] = (uint8_t)((c + nearr[i + 1]) >> 2);
            }
            out[2 * i] = (uint8_t)((nearr[w - 2] * 3 + nearr[w - 1] + 2) >> 2);
            out[2 * i + 1] = nearr[w - 1];
        } else if (r.hs == 2 && r.vs == 2) {
            // vertical 3:1 blend first, then horizontal 3:1 on the blended row (weights 9:3:3:1)
            if (w == 1) {
                out[0] = out[1] = (uint8_t)((3 * nearr[0] + farr[0] + 2) >> 2);
                return;
            }
            int cur = 3 * nearr[0] + farr[0];
            out[0] = (uint8_t)((cur + 2) >> 2);
            for (int i = 1; i < w; ++i) {
                const int prev = cur;
                cur = 3 * nearr[i] + farr[i];
                out[2 * i - 1] = (uint8_t)((3 * prev + cur + 8) >> 4);
                out[2 * i] = (uint8_t)((3 * cur + prev + 8) >> 4);
            }
            out[2 * w - 1] = (uint8_t)((cur + 2) >> 2);
        } else {
            for (int i = 0; i < w; ++i)
                for (int j = 0; j < r.hs; ++j) out[i * r.hs + j] = nearr[i];
        }
    }

    static uint8_t blend(uint8_t x, uint8_t y) {  // x y / 255, rounded (stb_image.h:3804-3808)
        const unsigned t = (unsigned)x * y + 128;
        return (uint8_t)((t + (t >> 8)) >> 8);
    }

    static void ycbcr_to_rgb(uint8_t* out, const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int count) {
        const int kr = color_fix(1.40200f), kgr = -color_fix(0.71414f), kgb = -color_fix(0.34414f),
                  kb = color_fix(1.77200f);
        for (int i = 0; i < count; ++i) {
            const int yf = (y[i] << 20) + (1 << 19);
            const int r_ = cr[i] - 128, b_ = cb[i] - 128;
            const int r = (yf + r_ * kr) >> 20;
            const int g = (yf + r_ * kgr + ((b_ * kgb) & (int)0xffff0000)) >> 20;
            const int b = (yf + b_ * kb) >> 20;
            out[3 * i] = clamp255(r);
            out[3 * i + 1] = clamp255(g);
            out[3 * i + 2] = clamp255(b);
        }
    }

    void to_rgb(std::vector<uint8_t>* rgb) const {
        const bool is_rgb = ncomp == 3 && (rgb_ids == 3 || (adobe_transform == 0 && !jfif));
        Resampler rs[4];
        std::vector<uint8_t> line[4];
        for (int k = 0; k < ncomp; ++k) {
            Resampler& r = rs[k];
            r.hs = hmax / comp[k].h;
            r.vs = vmax / comp[k].v;
            r.ystep = r.vs >> 1;
            r.wlo = (width + r.hs - 1) / r.hs;
            r.line0 = r.line1 = comp[k].plane.data();
            line[k].assign((size_t)width + 3, 0);
        }
        rgb->assign((size_t)width * height * 3, 0);
        const uint8_t* row[4];
        for (int j = 0; j < height; ++j) {
            for (int k = 0; k < ncomp; ++k) {
                Resampler& r = rs[k];
                const bool bottom = r.ystep >= (r.vs >> 1);
                const uint8_t* nearr = bottom ? r.line1 : r.line0;
                const uint8_t* farr = bottom ? r.line0 : r.line1;
                if (r.hs == 1 && r.vs == 1) {
                    row[k] = nearr;
                } else {
                    upsample_row(r, nearr, farr, line[k].data());
                    row[k] = line[k].data();
                }
                if (++r.ystep >= r.vs) {
                    r.ystep = 0;
                    r.line0 = r.line1;
                    if (++r.ypos < comp[k].y) r.line1 += comp[k].w2;
                }
            }
            uint8_t* out = rgb->data() + (size_t)3 * width * j;
            if (ncomp == 1) {
                for (int i = 0; i < width; ++i) out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = row[0][i];
            } else if (ncomp == 3) {
                if (is_rgb) {
                    for (int i = 0; i < width; ++i) {
                        out[3 * i] = row[0][i];
                        out[3 * i + 1] = row[1][i];
                        out[3 * i + 2] = row[2][i];
                    }
                } else {
                    ycbcr_to_rgb(out, row[0], row[1], row[2], width);
                }
            } else if (adobe_transform == 0) {  // CMYK (Adobe inverted), K scales each channel
                for (int i = 0; i < width; ++i)
                    for (int c = 0; c < 3; ++c) out[3 * i + c] = blend(row[c][i], row[3][i]);
            } else if (adobe_transform == 2) {  // YCCK
                ycbcr_to_rgb(out, row[0], row[1], row[2], width);
                for (int i = 0; i < width; ++i)
                    for (int c = 0; c < 3; ++c) out[3 * i + c] = blend((uint8_t)(255 - out[3 * i + c]), row[3][i]);
            } else {  // YCbCr and a fourth channel, which is ignored
                ycbcr_to_rgb(out, row[0], row[1], row[2], width);
            }
        }
    }
};

}  // namespace

std::string decode_jpeg(const uint8_t* data, size_t n, int* w, int* h, std::vector<uint8_t>* rgb, int* code) {
    Decoder dec(data, n);
    if (!dec.decode()) {
        *code = dec.code;
        return dec.err;
    }
    dec.to_rgb(rgb);
    *w = dec.width;
    *h = dec.height;
    *code = LTS_OK;
    return "";
}

}  // namespace lts
