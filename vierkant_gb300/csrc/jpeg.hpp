// JPEG decoding for the glTF loader (host only): DCT with Huffman coding, 8-bit samples (ITU-T T.81
// baseline, extended sequential and progressive), written for the loader's needs.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace vkg
{
// Decodes a JPEG file image into RGBA8 (row-major, 4 bytes per texel, alpha 255). One component
// (grey) or three (YCbCr, JFIF conversion; RGB when an Adobe marker says so); any sampling factors
// from 1 to 4, chroma upsampled by replication; interleaved or one-component scans; restart intervals;
// progressive frames (spectral selection, successive approximation, end-of-band runs). Lossless,
// hierarchical, arithmetic-coded, 12-bit and four-component images are rejected: false with a
// message, as on malformed input.
bool jpeg_decode(const uint8_t *data, size_t size, std::vector<uint8_t> &rgba, uint32_t &width, uint32_t &height,
                 std::string &err);
}// namespace vkg
