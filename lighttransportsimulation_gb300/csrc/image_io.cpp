// PNG decoding (RFC 2083) with its zlib inflate (RFC 1950 / 1951), and the image-texture pyramid
// of the fixed mode.  The reference reads its images through its vendored stb_image v2.27
// (core/ImageI.cuh:11-34, extern/stb_image.h); this file restates the published formats,
// producing what stbi_load / stbi_loadf give for three requested channels (JPEG: jpeg_io.cpp).
#include "image_io.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>

#include "../../include/lts_capi.h"

namespace lts {
namespace {

// ------------------------------------------------------------------ inflate (RFC 1951)
struct BitIn {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool over = false;
    int bit() {
        if (cnt == 0) {
            if (pos >= n) {
                over = true;
                return 0;
            }
            buf = p[pos++];
            cnt = 8;
        }
        const int b = (int)(buf & 1u);
        buf >>= 1;
        --cnt;
        return b;
    }
    uint32_t bits(int k) {  // k bits, least significant first
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
};

// Canonical Huffman code: codes per length and the symbols in code order.
struct Huff {
    int count[16] = {0};
    std::vector<int> sym;
};

// Returns false for an over-subscribed set of lengths; incomplete codes are accepted (a
// distance code of one symbol is incomplete by design) and fail only if an unused code appears.
bool huff_build(Huff& h, const uint8_t* len, int n) {
    for (int& c : h.count) c = 0;
    for (int i = 0; i < n; ++i) ++h.count[len[i]];
    h.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0) return false;
    }
    int offs[16] = {0};
    for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
    h.sym.assign((size_t)n, 0);
    for (int i = 0; i < n; ++i)
        if (len[i]) h.sym[(size_t)offs[len[i]]++] = i;
    return true;
}

// One symbol: the code is read a bit at a time, most significant first; the codes of each length
// are consecutive integers following those of the shorter lengths.
int huff_decode(BitIn& b, const Huff& h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= b.bit();
        const int c = h.count[l];
        if (code - first < c) return h.sym[(size_t)(index + code - first)];
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

// Length and distance bases and extra bits (RFC 1951 section 3.2.5).
const int kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                          31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const int kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                           193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// Order in which a dynamic block lists its code-length code lengths (section 3.2.7).
const int kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

bool inflate_codes(BitIn& b, const Huff& lit, const Huff& dist, std::vector<uint8_t>& out, std::string* err) {
    for (;;) {
        const int s = huff_decode(b, lit);
        if (s < 0 || b.over) {
            *err = "corrupt deflate data (literal/length code)";
            return false;
        }
        if (s < 256) {
            out.push_back((uint8_t)s);
        } else if (s == 256) {
            return true;
        } else {
            const int li = s - 257;
            if (li >= 29) {
                *err = "corrupt deflate data (length symbol)";
                return false;
            }
            const int len = kLenBase[li] + (int)b.bits(kLenExtra[li]);
            const int ds = huff_decode(b, dist);
            if (ds < 0 || ds >= 30 || b.over) {
                *err = "corrupt deflate data (distance code)";
                return false;
            }
            const size_t d = (size_t)kDistBase[ds] + b.bits(kDistExtra[ds]);
            if (d > out.size()) {
                *err = "corrupt deflate data (distance beyond the output)";
                return false;
            }
            const size_t from = out.size() - d;
            for (int k = 0; k < len; ++k) out.push_back(out[from + (size_t)k]);
        }
    }
}

bool inflate_raw(BitIn& b, std::vector<uint8_t>& out, std::string* err) {
    int last = 0;
    do {
        last = b.bit();
        const uint32_t type = b.bits(2);
        if (b.over) break;
        if (type == 0) {  // stored: byte-aligned LEN, NLEN, then LEN bytes
            b.cnt = 0;
            if (b.pos + 4 > b.n) break;
            const uint32_t len = b.p[b.pos] | (uint32_t)b.p[b.pos + 1] << 8;
            const uint32_t nlen = b.p[b.pos + 2] | (uint32_t)b.p[b.pos + 3] << 8;
            b.pos += 4;
            if ((len ^ 0xffffu) != nlen || b.pos + len > b.n) {
                *err = "corrupt deflate data (stored block)";
                return false;
            }
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {  // fixed codes (section 3.2.6)
            static const Huff* fixed = [] {  // built once (thread-safe static initialisation)
                static Huff codes[2];
                uint8_t l[288];
                for (int i = 0; i < 288; ++i) l[i] = i < 144 ? 8 : (i < 256 ? 9 : (i < 280 ? 7 : 8));
                huff_build(codes[0], l, 288);
                for (int i = 0; i < 30; ++i) l[i] = 5;
                huff_build(codes[1], l, 30);
                return codes;
            }();
            if (!inflate_codes(b, fixed[0], fixed[1], out, err)) return false;
        } else if (type == 2) {  // dynamic codes (section 3.2.7)
            const int nlen = (int)b.bits(5) + 257, ndist = (int)b.bits(5) + 1, ncode = (int)b.bits(4) + 4;
            if (nlen > 286 || ndist > 30) {
                *err = "corrupt deflate data (code counts)";
                return false;
            }
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; ++i) cl[kClOrder[i]] = (uint8_t)b.bits(3);
            Huff clh;
            if (!huff_build(clh, cl, 19)) {
                *err = "corrupt deflate data (code-length code)";
                return false;
            }
            uint8_t lens[316] = {0};
            int i = 0;
            while (i < nlen + ndist) {
                const int s = huff_decode(b, clh);
                if (s < 0 || b.over) {
                    *err = "corrupt deflate data (code lengths)";
                    return false;
                }
                if (s < 16) {
                    lens[i++] = (uint8_t)s;
                    continue;
                }
                int rep = 0, val = 0;
                if (s == 16) {
                    if (i == 0) {
                        *err = "corrupt deflate data (repeat with no previous length)";
                        return false;
                    }
                    val = lens[i - 1];
                    rep = 3 + (int)b.bits(2);
                } else if (s == 17) {
                    rep = 3 + (int)b.bits(3);
                } else {
                    rep = 11 + (int)b.bits(7);
                }
                if (i + rep > nlen + ndist) {
                    *err = "corrupt deflate data (lengths overrun)";
                    return false;
                }
                while (rep--) lens[i++] = (uint8_t)val;
            }
            if (lens[256] == 0) {
                *err = "corrupt deflate data (no end-of-block code)";
                return false;
            }
            Huff lit, dist;
            if (!huff_build(lit, lens, nlen) || !huff_build(dist, lens + nlen, ndist)) {
                *err = "corrupt deflate data (over-subscribed code)";
                return false;
            }
            if (!inflate_codes(b, lit, dist, out, err)) return false;
        } else {
            *err = "corrupt deflate data (block type 3)";
            return false;
        }
    } while (!last);
    if (b.over) {
        *err = "truncated deflate data";
        return false;
    }
    return true;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

int paeth(int a, int b, int c) {  // RFC 2083 section 6.6
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

}  // namespace

bool zlib_inflate(const uint8_t* data, size_t n, std::vector<uint8_t>* out, std::string* err) {
    if (n < 6) {
        *err = "truncated zlib stream";
        return false;
    }
    const int cmf = data[0], flg = data[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0) {
        *err = "bad zlib header";
        return false;
    }
    if (flg & 32) {
        *err = "zlib preset dictionary";
        return false;
    }
    BitIn b{data + 2, n - 2};
    out->clear();
    if (!inflate_raw(b, *out, err)) return false;
    // Adler-32 of the output, big-endian after the deflate data
    if (b.pos + 4 > b.n) {
        *err = "truncated zlib stream (no checksum)";
        return false;
    }
    uint32_t s1 = 1, s2 = 0;
    for (uint8_t c : *out) {
        s1 = (s1 + c) % 65521u;
        s2 = (s2 + s1) % 65521u;
    }
    if (be32(b.p + b.pos) != ((s2 << 16) | s1)) {
        *err = "zlib checksum mismatch";
        return false;
    }
    return true;
}

std::string decode_png(const uint8_t* d, size_t n, int* w_out, int* h_out, std::vector<uint8_t>* rgb, int* code) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    *code = LTS_ERR_PARSE;
    if (n < 8 || memcmp(d, sig, 8) != 0) {
        *code = LTS_ERR_UNSUPPORTED;
        return "not a PNG file (only PNG images are decoded)";
    }
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> plte, idat;
    bool ended = false;
    while (pos + 12 <= n) {
        const uint32_t len = be32(d + pos);
        const uint8_t* type = d + pos + 4;
        if (len > n - pos - 12) return "truncated PNG chunk";
        const uint8_t* body = d + pos + 8;
        if (!memcmp(type, "IHDR", 4)) {
            if (len != 13) return "bad IHDR";
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            if (body[10] != 0 || body[11] != 0) return "unknown PNG compression or filter method";
            interlace = body[12];
        } else if (!memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!memcmp(type, "IEND", 4)) {
            ended = true;
            break;
        }
        pos += 12 + (size_t)len;
    }
    if (!ended) return "PNG without IEND";
    if (w == 0 || h == 0 || w > 65536 || h > 65536) return "bad PNG size";
    int chans = 0;
    bool ok_depth = false;
    switch (ctype) {
        case 0: chans = 1; ok_depth = depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16; break;
        case 2: chans = 3; ok_depth = depth == 8 || depth == 16; break;
        case 3: chans = 1; ok_depth = depth == 1 || depth == 2 || depth == 4 || depth == 8; break;
        case 4: chans = 2; ok_depth = depth == 8 || depth == 16; break;
        case 6: chans = 4; ok_depth = depth == 8 || depth == 16; break;
        default: return "bad PNG colour type";
    }
    if (!ok_depth) return "bad PNG bit depth";
    if (ctype == 3 && (plte.empty() || plte.size() % 3 != 0)) return "PNG palette missing";
    if (interlace != 0) {
        *code = LTS_ERR_UNSUPPORTED;
        return "interlaced PNG images are not decoded";
    }
    std::vector<uint8_t> raw;
    std::string err;
    if (!zlib_inflate(idat.data(), idat.size(), &raw, &err)) return "PNG image data: " + err;
    const size_t bpp_bits = (size_t)depth * chans, stride = ((size_t)w * bpp_bits + 7) / 8;
    const size_t bpp = std::max<size_t>(1, bpp_bits / 8);
    if (raw.size() < (stride + 1) * h) return "PNG image data too short";
    // undo the per-row filters (RFC 2083 section 6) in place
    std::vector<uint8_t> px(stride * h);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t f = raw[(stride + 1) * y];
        const uint8_t* src = &raw[(stride + 1) * y + 1];
        uint8_t* cur = &px[stride * y];
        const uint8_t* prev = y ? &px[stride * (y - 1)] : nullptr;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= bpp ? cur[i - bpp] : 0, b = prev ? prev[i] : 0,
                      c = (prev && i >= bpp) ? prev[i - bpp] : 0;
            int v = src[i];
            switch (f) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: return "bad PNG filter type";
            }
            cur[i] = (uint8_t)v;
        }
    }
    // samples to 8-bit RGB
    static const int kScale[9] = {0, 0xff, 0x55, 0, 0x11, 0, 0, 0, 0x01};  // grey of 1, 2, 4, 8 bits
    rgb->assign((size_t)w * h * 3, 0);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* row = &px[stride * y];
        for (uint32_t x = 0; x < w; ++x) {
            int s[4] = {0, 0, 0, 0};
            for (int c = 0; c < chans; ++c) {
                const size_t k = (size_t)x * chans + c;
                if (depth == 16) {
                    s[c] = row[2 * k];  // the high byte
                } else if (depth == 8) {
                    s[c] = row[k];
                } else {
                    const size_t bit = k * depth;
                    s[c] = (row[bit >> 3] >> (8 - depth - (int)(bit & 7))) & ((1 << depth) - 1);
                    if (ctype == 0) s[c] *= kScale[depth];
                }
            }
            uint8_t* o = &(*rgb)[3 * ((size_t)y * w + x)];
            if (ctype == 3) {
                if ((size_t)s[0] * 3 + 2 >= plte.size()) return "PNG palette index out of range";
                for (int c = 0; c < 3; ++c) o[c] = plte[(size_t)s[0] * 3 + c];
            } else if (ctype == 0 || ctype == 4) {
                o[0] = o[1] = o[2] = (uint8_t)s[0];
            } else {
                for (int c = 0; c < 3; ++c) o[c] = (uint8_t)s[c];
            }
        }
    }
    *w_out = (int)w;
    *h_out = (int)h;
    *code = LTS_OK;
    return "";
}

namespace {
std::string read_file(const std::string& path, std::vector<uint8_t>* data, int* code) {
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) {
        *code = LTS_ERR_IO;
        return "cannot open " + path;
    }
    data->assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    return "";
}
}  // namespace

std::string decode_png_file(const std::string& path, int* w, int* h, std::vector<uint8_t>* rgb, int* code) {
    std::vector<uint8_t> data;
    std::string e = read_file(path, &data, code);
    if (!e.empty()) return e;
    e = decode_png(data.data(), data.size(), w, h, rgb, code);
    return e.empty() ? e : path + ": " + e;
}

std::string decode_image(const uint8_t* d, size_t n, int* w, int* h, std::vector<uint8_t>* rgb, int* code) {
    if (n >= 2 && d[0] == 0xFF && d[1] == 0xD8) return decode_jpeg(d, n, w, h, rgb, code);
    if (n >= 8 && d[0] == 137 && d[1] == 'P' && d[2] == 'N' && d[3] == 'G') return decode_png(d, n, w, h, rgb, code);
    *code = LTS_ERR_UNSUPPORTED;
    return "not a PNG or JPEG file (only these image formats are decoded)";
}

std::string decode_image_file(const std::string& path, int* w, int* h, std::vector<uint8_t>* rgb, int* code) {
    std::vector<uint8_t> data;
    std::string e = read_file(path, &data, code);
    if (!e.empty()) return e;
    e = decode_image(data.data(), data.size(), w, h, rgb, code);
    return e.empty() ? e : path + ": " + e;
}

void build_pyramid(int w, int h, const std::vector<uint8_t>& rgb8, int wrap, HostImage* img) {
    float lut[256];
    // (c / 255)^2.2 correctly rounded to float (pow in double, then rounded once): what glibc's
    // powf gives stb_image for all 256 values, and the same on every host
    for (int c = 0; c < 256; ++c) lut[c] = (float)std::pow((double)((float)c / 255.0f), (double)2.2f);
    int levels = (int)log2f(fmaxf((float)w, (float)h));  // CreateMipMap, Mipmap_kernel.cu:45
    if (levels < 1) levels = 1;
    img->wrap = wrap;
    img->levels = levels;
    img->lod = (float)(levels - 1) + log2f(0.01f);  // Mipmap::lookUp at EVALUATION_WIDTH
    img->w.assign((size_t)levels, 0);
    img->h.assign((size_t)levels, 0);
    img->rgb.assign((size_t)levels, {});
    img->w[0] = w;
    img->h[0] = h;
    std::vector<float>& base = img->rgb[0];
    base.resize(3 * (size_t)w * h);
    for (int v = 0; v < h; ++v)
        for (int u = 0; u < w; ++u)
            for (int c = 0; c < 3; ++c)
                base[3 * ((size_t)v * w + u) + c] = lut[rgb8[3 * ((size_t)(h - 1 - v) * w + u) + c]];
    for (int l = 1; l < levels; ++l) {
        const int pw = img->w[l - 1], ph = img->h[l - 1];
        const int lw = std::max(1, w >> l), lh = std::max(1, h >> l);
        img->w[l] = lw;
        img->h[l] = lh;
        const std::vector<float>& src = img->rgb[l - 1];
        std::vector<float>& dst = img->rgb[l];
        dst.resize(3 * (size_t)lw * lh);
        auto tx = [&](int s, int t, int c) {
            return (s < 0 || s >= pw || t < 0 || t >= ph) ? 0.0f : src[3 * ((size_t)t * pw + s) + c];
        };
        for (int t = 0; t < lh; ++t)
            for (int s = 0; s < lw; ++s)
                for (int c = 0; c < 3; ++c) {
                    const float sum = ((tx(2 * s, 2 * t, c) + tx(2 * s + 1, 2 * t, c)) + tx(2 * s, 2 * t + 1, c)) +
                                      tx(2 * s + 1, 2 * t + 1, c);
                    dst[3 * ((size_t)t * lw + s) + c] = 0.25f * sum;
                }
    }
}

}  // namespace lts
