// image_out.cpp -- host writers of the output images, in place of the
// reference's stb-based write_image_to_png / write_image_to_hdr
// (src/utility/image_file.cpp:14-24):
//  * PNG (ISO/IEC 15948): 8-bit RGB, filter type 0 on every row, the zlib
//    stream (RFC 1950) made of stored deflate blocks (RFC 1951, BTYPE 00),
//    CRC-32 per chunk and Adler-32 of the raw rows;
//  * Radiance HDR: the "#?RADIANCE" header, "-Y height +X width", and RGBE
//    scanlines; widths 8..32767 use the run-length scanline form with
//    literal runs only (so no pixel can be mistaken for a run marker), other
//    widths flat pixels.
#include <stdint.h>
#include <stdio.h>

#include <algorithm>
#include <cstddef>
#include <string>
#include <vector>

#include "../../include/tracer_gpu.h"

namespace {

struct CrcTable {
  uint32_t t[256];
  CrcTable() {
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
      t[n] = c;
    }
  }
};

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xffffffffu) {
  static const CrcTable table;  // initialised once, thread-safe
  for (size_t i = 0; i < n; ++i) c = table.t[(c ^ p[i]) & 0xffu] ^ (c >> 8);
  return c;
}

void put32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put32(out, (uint32_t)data.size());
  const size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  put32(out, crc32(out.data() + start, out.size() - start) ^ 0xffffffffu);
}

tr_status write_all(const char* path, const std::vector<uint8_t>& bytes) {
  FILE* f = fopen(path, "wb");
  if (!f) return TR_ERR_ARG;
  const size_t w = fwrite(bytes.data(), 1, bytes.size(), f);
  const int c = fclose(f);
  return (w == bytes.size() && c == 0) ? TR_OK : TR_ERR_ARG;
}

}  // namespace

extern "C" tr_status tr_write_png(const char* path, const uint8_t* rgb8, uint32_t width, uint32_t height) {
  if (!path || !rgb8 || width == 0 || height == 0 || width > (1u << 24) || height > (1u << 24)) return TR_ERR_ARG;
  const size_t row = 1 + 3 * (size_t)width;
  std::vector<uint8_t> raw(row * height);
  for (uint32_t y = 0; y < height; ++y) {
    raw[y * row] = 0;  // filter: none
    const uint8_t* src = rgb8 + 3 * (size_t)width * y;
    std::copy(src, src + 3 * (size_t)width, raw.begin() + (ptrdiff_t)(y * row + 1));
  }
  // zlib: CMF 0x78 (deflate, 32K window), FLG 0x01 (check bits), stored blocks, Adler-32
  std::vector<uint8_t> z;
  z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
  z.push_back(0x78);
  z.push_back(0x01);
  size_t pos = 0;
  do {
    const size_t len = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)(len & 0xff));
    z.push_back((uint8_t)(len >> 8));
    z.push_back((uint8_t)(~len & 0xff));
    z.push_back((uint8_t)((~len >> 8) & 0xff));
    z.insert(z.end(), raw.begin() + (ptrdiff_t)pos, raw.begin() + (ptrdiff_t)(pos + len));
    pos += len;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;
  for (uint8_t v : raw) {
    a = (a + v) % 65521u;
    b = (b + a) % 65521u;
  }
  put32(z, (b << 16) | a);
  std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<uint8_t> ihdr;
  put32(ihdr, width);
  put32(ihdr, height);
  ihdr.push_back(8);  // bit depth
  ihdr.push_back(2);  // colour type: RGB
  ihdr.push_back(0);  // compression: deflate
  ihdr.push_back(0);  // filter method 0
  ihdr.push_back(0);  // no interlace
  chunk(out, "IHDR", ihdr);
  chunk(out, "IDAT", z);
  chunk(out, "IEND", {});
  return write_all(path, out);
}

extern "C" tr_status tr_write_hdr(const char* path, const uint8_t* rgbe, uint32_t width, uint32_t height) {
  if (!path || !rgbe || width == 0 || height == 0) return TR_ERR_ARG;
  const std::string head = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(height) + " +X " +
                           std::to_string(width) + "\n";
  std::vector<uint8_t> out(head.begin(), head.end());
  const bool rle = width >= 8 && width <= 32767;
  out.reserve(out.size() + 4 * (size_t)width * height + (rle ? ((size_t)width / 128 + 2) * 4 * height + 4 * height : 0));
  for (uint32_t y = 0; y < height; ++y) {
    const uint8_t* line = rgbe + 4 * (size_t)width * y;
    if (!rle) {
      out.insert(out.end(), line, line + 4 * (size_t)width);
      continue;
    }
    out.push_back(2);
    out.push_back(2);
    out.push_back((uint8_t)(width >> 8));
    out.push_back((uint8_t)(width & 0xff));
    for (int c = 0; c < 4; ++c)  // each component as literal runs of up to 128
      for (uint32_t x = 0; x < width;) {
        const uint32_t n = std::min<uint32_t>(128, width - x);
        out.push_back((uint8_t)n);
        for (uint32_t k = 0; k < n; ++k) out.push_back(line[4 * (size_t)(x + k) + c]);
        x += n;
      }
  }
  return write_all(path, out);
}
