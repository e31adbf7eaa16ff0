// image_formats.h -- 8-bit image file decoders behind load_image_from_file.
//
// The reference reads every non-HDR image with its vendored stb_image
// (src/utility/image_file.cpp:26-58), which finds the format from the file's
// bytes. These project-written decoders cover the formats it reads that
// scenes use: PNG (image_file.cpp), baseline JPEG, TGA and BMP (here).
// Each returns the pixels top row first, `comp` bytes per pixel (1 grey,
// 3 RGB, 4 RGBA), as stb_image returns them before the reference flips the
// rows; malformed or unsupported files throw TracerError.
#pragma once

#include <cstdint>
#include <vector>

namespace tracer_files {

// Baseline sequential JPEG (SOF0/SOF1): 8-bit samples, Huffman coding, one
// or three components (JFIF YCbCr, or RGB when the component ids say so),
// sampling factors 1..4, restart intervals, any number of scans. Progressive
// and arithmetic-coded files throw TR_ERR_UNSUPPORTED.
std::vector<uint8_t> decode_jpeg(const std::vector<uint8_t>& f, int& w, int& h, int& comp);
// Truevision TGA: colour-mapped, true-colour and grey images (types 1, 2, 3
// and their run-length forms 9, 10, 11) of 8, 15/16, 24 or 32 bits.
std::vector<uint8_t> decode_tga(const std::vector<uint8_t>& f, int& w, int& h, int& comp);
// Windows BMP: 1/4/8-bit palettes, 16/24/32-bit pixels (BI_RGB, BI_BITFIELDS),
// bottom-up or top-down rows.
std::vector<uint8_t> decode_bmp(const std::vector<uint8_t>& f, int& w, int& h, int& comp);
// Whether the bytes start like a JPEG, BMP or TGA file.
bool is_jpeg(const std::vector<uint8_t>& f);
bool is_bmp(const std::vector<uint8_t>& f);
bool is_tga(const std::vector<uint8_t>& f);

}  // namespace tracer_files
