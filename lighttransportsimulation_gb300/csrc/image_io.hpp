// Image files for image textures: PNG decoding and the mip pyramid of the fixed mode of the
// reference's ImageTexture (materials/textures/ImageTexture.cuh:13-28, Mipmap.cuh:34-73,
// Mipmap_kernel.cu:9-73).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace lts {

// Decodes a PNG file (RFC 2083: every colour type and bit depth, non-interlaced) into 8-bit RGB,
// top row first, as stbi_load with three requested channels gives it: grey replicated, alpha
// dropped, palettes expanded, grey of 1, 2 or 4 bits scaled to 0..255, 16-bit samples reduced to
// their high byte.  Returns "" or an error message; *code receives an LTS_ERR_* value (IO for an
// unreadable file, PARSE for a malformed one, UNSUPPORTED for an interlaced one or another format).
std::string decode_png_file(const std::string& path, int* w, int* h, std::vector<uint8_t>* rgb, int* code);
std::string decode_png(const uint8_t* data, size_t n, int* w, int* h, std::vector<uint8_t>* rgb, int* code);

// Decodes a baseline JPEG (T.81 sequential DCT, Huffman, 8-bit; any sampling factors, restart
// intervals, greyscale, YCbCr, Adobe RGB / CMYK / YCCK) into 8-bit RGB, top row first, as
// stb_image v2.27 does for three requested channels.  Codes as decode_png (UNSUPPORTED for
// progressive, lossless, arithmetic-coded or 12-bit files).
std::string decode_jpeg(const uint8_t* data, size_t n, int* w, int* h, std::vector<uint8_t>* rgb, int* code);

// A PNG or JPEG file by its signature (UNSUPPORTED for any other format).
std::string decode_image(const uint8_t* data, size_t n, int* w, int* h, std::vector<uint8_t>* rgb, int* code);
std::string decode_image_file(const std::string& path, int* w, int* h, std::vector<uint8_t>* rgb, int* code);

// zlib stream (RFC 1950) inflated (RFC 1951: stored, fixed and dynamic Huffman blocks).
bool zlib_inflate(const uint8_t* data, size_t n, std::vector<uint8_t>* out, std::string* err);

// One image texture: its wrap mode (0 repeat, 1 black, 2 clamp: ImageWrap, Mipmap.cuh:10-12)
// and its pyramid, level 0 the image itself, linear RGB, row-major with v = 0 the bottom row
// (loadImageFile_s, ImageI.cuh:11-34, flips the file's rows).
struct HostImage {
    int32_t wrap = 1;
    int32_t levels = 0;
    float lod = 0;  // the lookup's level coordinate: levels - 1 + log2(0.01), ImageTexture.cuh:7-8
    std::vector<int32_t> w, h;
    std::vector<std::vector<float>> rgb;  // [levels][3 w h]
};

// The fixed mode's pyramid from decoded 8-bit RGB (top row first): texel = (c / 255)^2.2 rounded
// to float (stbi_loadf's default LDR-to-linear conversion), rows flipped; floor(log2(max(w, h)))
// levels (at least one), level l of max(1, w >> l) x max(1, h >> l) texels, each the mean of the
// 2 x 2 texels below it with black outside (pyramidInitKernel's box filter over the whole level;
// the reference's kernel only fills 16 >> l texels per axis).
void build_pyramid(int w, int h, const std::vector<uint8_t>& rgb8, int wrap, HostImage* img);

}  // namespace lts
