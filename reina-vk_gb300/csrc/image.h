// Texture image decoding for Scene::defineTexture (src/scene/Scene.cpp:15-25, src/graphics/Image.cpp:10-41):
// an encoded image (PNG or sequential JPEG here; the reference links stb_image) becomes 8-bit RGBA texels,
// first row first.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace rt {

struct Image {
    uint32_t width = 0, height = 0;
    std::vector<uint8_t> rgba;   // width * height * 4 bytes, rows top to bottom
};

// zlib stream (RFC 1950) holding deflate data (RFC 1951).  `limit` bounds the output size; a stream
// that would produce more fails.  Throws Error(REINA_ERR_IO) on malformed input.
std::vector<uint8_t> zlib_inflate(const uint8_t* data, size_t n, size_t limit);

// Decodes an encoded image to RGBA8 the way stbi_load(..., 4) does: PNG of every colour type and bit
// depth (1, 2, 4, 8, 16; 16-bit samples keep their high byte; grey levels below 8 bits are scaled to
// 0..255; tRNS transparency; Adam7 interlacing), and sequential (baseline / extended Huffman, 8-bit) and
// progressive (spectral selection and successive approximation, T.81 Annex G) Huffman JPEG with one or
// three components, any sampling factors, restart markers and multiple scans: inverse DCT in double
// precision, 2:1 chroma upsampling by the triangle filter (replication for other ratios), JFIF YCbCr ->
// RGB (Adobe RGB files kept as RGB).  stb_image's integer IDCT and fixed-point colour conversion can
// give JPEG texels a few units apart from these.  BMP (1/4/8-bit palettes, 16-bit 5-5-5 or bit fields,
// 24 and 32 bits, either row order, uncompressed; a 32-bit alpha that is zero everywhere reads as opaque)
// and TGA (colour-mapped, true-colour 15/16/24/32-bit and grey, raw or run-length encoded, either
// origin), and Radiance RGBE (.hdr, flat or run-length scanlines) tone mapped as stbi_load does for 8-bit
// output (255 x^(1/2.2) + 0.5), and GIF (the first image on a transparent canvas of the logical screen
// size; transparency, interlacing, local tables).  Other formats (lossless, hierarchical or
// arithmetic-coded JPEG, RLE bitmaps, ...) fail with REINA_ERR_IO.
Image decode_image(const uint8_t* data, size_t n);

// Reads and decodes a file; `flip_vertically` reverses the row order (stbi_set_flip_vertically_on_load,
// which the reference sets for textures loaded from a path, src/graphics/Image.cpp:14).
Image load_image(const std::string& path, bool flip_vertically);

void flip_rows(Image& img);

}  // namespace rt
