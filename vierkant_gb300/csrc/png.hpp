// PNG decoding for the glTF loader (host only): zlib / DEFLATE (RFC 1950 / 1951) and the PNG
// scanline filters (PNG specification, 2nd edition), written for the loader's needs.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace vkg
{
// Decodes a PNG file image into RGBA8 (row-major, 4 bytes per texel). Bit depths 1, 2, 4, 8, 16
// (16-bit samples keep their high byte), all five colour types, palettes with tRNS transparency;
// interlaced (Adam7) images are rejected. false with a message on malformed or unsupported input.
bool png_decode(const uint8_t *data, size_t size, std::vector<uint8_t> &rgba, uint32_t &width, uint32_t &height,
                std::string &err);
// raw DEFLATE stream -> bytes (at most max_out); false on malformed input
bool inflate_raw(const uint8_t *data, size_t size, std::vector<uint8_t> &out, size_t max_out, std::string &err);
}// namespace vkg
