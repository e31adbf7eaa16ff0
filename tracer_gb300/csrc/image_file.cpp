// image_file.cpp -- the reference's image-file helpers (src/utility/image_file.cpp)
// over project code: the PNG and Radiance HDR writers of image_out.cpp, a
// Radiance HDR reader (G. Ward's RGBE format: a text header, the resolution
// line, then flat or run-length scanlines), and the MTL-to-texture mapping
// of create_texture_from_file.
#include "image_formats.h"
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

#include "../../include/tracer_gb300.hpp"

namespace tracer {
namespace {

// Ward's shared-exponent encoding of one pixel (the largest channel
// v = m * 2^e with m in [0.5, 1) sets the exponent byte e + 128).
void encode_rgbe(const Spectrum& c, uint8_t* out) {
  float v = c.r;
  if (c.g > v) v = c.g;
  if (c.b > v) v = c.b;
  if (!(v >= 1e-32f)) {
    out[0] = out[1] = out[2] = out[3] = 0;
    return;
  }
  int e;
  const float m = std::frexp(v, &e);
  const float s = m * 256.0f / v;
  const float ch[3] = {c.r * s, c.g * s, c.b * s};
  for (int k = 0; k < 3; ++k) out[k] = (uint8_t)(ch[k] > 0.0f ? (ch[k] < 255.0f ? (int)ch[k] : 255) : 0);
  out[3] = (uint8_t)(e + 128);
}

// RGBE bytes to linear floats: byte * 2^(exponent - 128 - 8), zero for exponent 0.
Color3f decode_rgbe(const uint8_t* p) {
  if (p[3] == 0) return Color3f{0, 0, 0};
  const float f = std::ldexp(1.0f, (int)p[3] - 136);
  return Color3f{p[0] * f, p[1] * f, p[2] * f};
}

// ---- inflate (RFC 1950 zlib stream of RFC 1951 deflate blocks)
struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint32_t bitbuf = 0;
  int bitcnt = 0;
  uint32_t bits(int need) {
    while (bitcnt < need) {
      if (pos >= n) throw TracerError(TR_ERR_ARG, "truncated deflate stream");
      bitbuf |= (uint32_t)p[pos++] << bitcnt;
      bitcnt += 8;
    }
    const uint32_t v = bitbuf & ((1u << need) - 1u);
    bitbuf >>= need;
    bitcnt -= need;
    return v;
  }
};

// A canonical Huffman code: codes of each length are consecutive, shorter first.
struct Huffman {
  int count[16] = {0};
  std::vector<int> symbol;
  void build(const uint8_t* lengths, int n) {
    std::memset(count, 0, sizeof(count));
    for (int i = 0; i < n; ++i) count[lengths[i]]++;
    count[0] = 0;
    int offs[16] = {0};
    for (int l = 1; l < 16; ++l) offs[l] = offs[l - 1] + count[l - 1];
    symbol.assign(n, 0);
    for (int i = 0; i < n; ++i)
      if (lengths[i]) symbol[offs[lengths[i]]++] = i;
  }
  int decode(BitReader& br) const {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= (int)br.bits(1);
      const int c = count[l];
      if (code - first < c) return symbol[index + (code - first)];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    throw TracerError(TR_ERR_ARG, "bad Huffman code in deflate stream");
  }
};

// Inflates a zlib stream of at most `limit` output bytes.
std::vector<uint8_t> inflate_zlib(const uint8_t* data, size_t n, size_t limit) {
  if (n < 2 || (data[0] & 0x0f) != 8 || ((data[0] << 8) | data[1]) % 31 != 0 || (data[1] & 0x20))
    throw TracerError(TR_ERR_ARG, "bad zlib header");
  // RFC 1951 section 3.2.5: base values and extra bits of lengths 257..285 and distances 0..29
  static const int kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59,
                                   67, 83, 99, 115, 131, 163, 195, 227, 258};
  static const int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3,
                                    4, 4, 4, 4, 5, 5, 5, 5, 0};
  static const int kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513,
                                    769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
  static const int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8,
                                     9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
  static const int kOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
  BitReader br{data + 2, n - 2};
  std::vector<uint8_t> out;
  for (bool last = false; !last;) {
    last = br.bits(1) != 0;
    const uint32_t type = br.bits(2);
    if (type == 0) {  // stored
      br.bitbuf = 0;
      br.bitcnt = 0;
      if (br.n - br.pos < 4) throw TracerError(TR_ERR_ARG, "truncated stored block");
      const uint32_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8), nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
      br.pos += 4;
      if ((len ^ 0xffffu) != nlen || br.n - br.pos < len) throw TracerError(TR_ERR_ARG, "bad stored block");
      if (out.size() + len > limit) throw TracerError(TR_ERR_ARG, "deflate stream longer than the image");
      out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
      br.pos += len;
      continue;
    }
    if (type == 3) throw TracerError(TR_ERR_ARG, "bad deflate block type");
    Huffman lit, dist;
    uint8_t lengths[320];
    if (type == 1) {  // fixed codes
      for (int i = 0; i < 288; ++i) lengths[i] = i < 144 ? 8 : (i < 256 ? 9 : (i < 280 ? 7 : 8));
      lit.build(lengths, 288);
      for (int i = 0; i < 30; ++i) lengths[i] = 5;
      dist.build(lengths, 30);
    } else {  // dynamic codes
      const int nlit = (int)br.bits(5) + 257, ndist = (int)br.bits(5) + 1, ncode = (int)br.bits(4) + 4;
      if (nlit > 286 || ndist > 30) throw TracerError(TR_ERR_ARG, "bad dynamic block counts");
      uint8_t cl[19] = {0};
      for (int i = 0; i < ncode; ++i) cl[kOrder[i]] = (uint8_t)br.bits(3);
      Huffman clh;
      clh.build(cl, 19);
      for (int i = 0; i < nlit + ndist;) {
        const int sym = clh.decode(br);
        if (sym < 16) {
          lengths[i++] = (uint8_t)sym;
          continue;
        }
        int rep = 0;
        uint8_t val = 0;
        if (sym == 16) {
          if (i == 0) throw TracerError(TR_ERR_ARG, "repeat with no previous length");
          val = lengths[i - 1];
          rep = 3 + (int)br.bits(2);
        } else if (sym == 17) {
          rep = 3 + (int)br.bits(3);
        } else {
          rep = 11 + (int)br.bits(7);
        }
        if (i + rep > nlit + ndist) throw TracerError(TR_ERR_ARG, "code lengths overrun");
        while (rep--) lengths[i++] = val;
      }
      lit.build(lengths, nlit);
      dist.build(lengths + nlit, ndist);
    }
    for (;;) {
      const int sym = lit.decode(br);
      if (out.size() >= limit && sym != 256) throw TracerError(TR_ERR_ARG, "deflate stream longer than the image");
      if (sym < 256) {
        out.push_back((uint8_t)sym);
      } else if (sym == 256) {
        break;
      } else {
        const int li = sym - 257;
        if (li >= 29) throw TracerError(TR_ERR_ARG, "bad length symbol");
        const int len = kLenBase[li] + (int)br.bits(kLenExtra[li]);
        const int di = dist.decode(br);
        if (di >= 30) throw TracerError(TR_ERR_ARG, "bad distance symbol");
        const size_t d = (size_t)kDistBase[di] + br.bits(kDistExtra[di]);
        if (d > out.size()) throw TracerError(TR_ERR_ARG, "distance beyond the output");
        if (out.size() + len > limit) throw TracerError(TR_ERR_ARG, "deflate stream longer than the image");
        for (int k = 0; k < len; ++k) out.push_back(out[out.size() - d]);
      }
    }
  }
  return out;
}

uint32_t be32(const uint8_t* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

// An 8-bit PNG (ISO/IEC 15948): grey, RGB, palette, RGBA; not interlaced.
// Returns the rows top first and the channel count the file stores
// (palette images expand to RGB).
std::vector<uint8_t> decode_png(const std::vector<uint8_t>& f, int& w, int& h, int& comp) {
  static const uint8_t kSig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  if (f.size() < 8 || std::memcmp(f.data(), kSig, 8) != 0) throw TracerError(TR_ERR_ARG, "not a PNG file");
  size_t pos = 8;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<uint8_t> idat, plte;
  w = h = 0;
  while (pos + 8 <= f.size()) {
    const uint32_t len = be32(&f[pos]);
    const std::string type(reinterpret_cast<const char*>(&f[pos + 4]), 4);
    if (f.size() - pos < 12 || f.size() - pos - 12 < len) throw TracerError(TR_ERR_ARG, "truncated PNG chunk");
    const uint8_t* d = &f[pos + 8];
    if (type == "IHDR") {
      if (len < 13) throw TracerError(TR_ERR_ARG, "bad IHDR");
      w = (int)be32(d);
      h = (int)be32(d + 4);
      depth = d[8];
      ctype = d[9];
      interlace = d[12];
    } else if (type == "PLTE") {
      plte.assign(d, d + len);
    } else if (type == "IDAT") {
      idat.insert(idat.end(), d, d + len);
    } else if (type == "IEND") {
      break;
    }
    pos += 12 + len;
  }
  if (w <= 0 || h <= 0 || w > (1 << 16) || h > (1 << 16) || (size_t)w * h > (size_t(1) << 28))
    throw TracerError(TR_ERR_ARG, "bad PNG size");
  if (depth != 8) throw TracerError(TR_ERR_UNSUPPORTED, "PNG bit depth other than 8");
  if (interlace) throw TracerError(TR_ERR_UNSUPPORTED, "interlaced PNG");
  const int ch = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : ctype == 6 ? 4 : 0;
  if (!ch) throw TracerError(TR_ERR_ARG, "bad PNG colour type");
  if (ctype == 3 && plte.size() < 3) throw TracerError(TR_ERR_ARG, "palette PNG without PLTE");
  const size_t stride = (size_t)w * ch;
  const std::vector<uint8_t> raw = inflate_zlib(idat.data(), idat.size(), (stride + 1) * h);
  if (raw.size() < (stride + 1) * h) throw TracerError(TR_ERR_ARG, "short PNG image data");
  std::vector<uint8_t> px(stride * h);
  for (int y = 0; y < h; ++y) {
    const uint8_t filter = raw[(stride + 1) * y];
    const uint8_t* src = &raw[(stride + 1) * y + 1];
    uint8_t* row = &px[stride * y];
    const uint8_t* prev = y ? &px[stride * (y - 1)] : nullptr;
    for (size_t i = 0; i < stride; ++i) {
      const int a = i >= (size_t)ch ? row[i - ch] : 0, b = prev ? prev[i] : 0,
                c = (prev && i >= (size_t)ch) ? prev[i - ch] : 0;
      int v = src[i];
      if (filter == 1) v += a;
      else if (filter == 2) v += b;
      else if (filter == 3) v += (a + b) >> 1;
      else if (filter == 4) {  // Paeth predictor
        const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
        v += (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
      } else if (filter != 0) {
        throw TracerError(TR_ERR_ARG, "bad PNG filter type");
      }
      row[i] = (uint8_t)v;
    }
  }
  comp = ch;
  if (ctype != 3) return px;
  std::vector<uint8_t> rgb((size_t)w * h * 3);
  for (size_t i = 0; i < (size_t)w * h; ++i) {
    if ((size_t)px[i] * 3 + 2 >= plte.size()) throw TracerError(TR_ERR_ARG, "palette index out of range");
    std::memcpy(&rgb[3 * i], &plte[3 * (size_t)px[i]], 3);
  }
  comp = 3;
  return rgb;
}

std::string extension(const std::string& filename) {
  const size_t dot = filename.find_last_of('.'), slash = filename.find_last_of("/\\");
  if (dot == std::string::npos || (slash != std::string::npos && dot < slash))
    throw TracerError(TR_ERR_ARG, "invalid filename for image: " + filename);
  return filename.substr(dot);
}

// _create_texture_from_file (src/utility/image_file.cpp:98-128)
RC<Texture2D> texture_of(const std::string& name, real r, real g, real b) {
  if (name.empty()) return create_constant_texture2d(Spectrum(r, g, b));
  if (!r && !g && !b) r = g = b = 1;
  const std::string ext = extension(name);
  if (ext == ".png" || ext == ".jpg" || ext == ".jpeg") {
    // 8-bit maps: bytes / 255 raised to 2.2, back to bytes, times the scale
    // (each step truncating to a byte, as Point3<uint8_t> does)
    auto img = load_image_from_file(name);
    const real gamma = 2.2f;
    for (int y = 0; y < img->height(); ++y)
      for (int x = 0; x < img->width(); ++x) {
        Color3b& c = img->at(x, y);
        const real t[3] = {std::pow((real)c.x / 255, gamma), std::pow((real)c.y / 255, gamma),
                           std::pow((real)c.z / 255, gamma)};
        c = Color3b{(uint8_t)(t[0] * 255), (uint8_t)(t[1] * 255), (uint8_t)(t[2] * 255)};
        c = Color3b{(uint8_t)(c.x * r), (uint8_t)(c.y * g), (uint8_t)(c.z * b)};
      }
    return create_image_texture2d(img);
  }
  // is_float_image (src/utility/image_file.cpp:83-98): ".jpg", ".jpeg" and
  // ".png" are 8-bit, ".hdr" float, everything else (".bmp" too: the
  // reference compares with "bmp", without the dot) is refused
  if (ext != ".hdr") throw TracerError(TR_ERR_ARG, "unsupported image format: " + name);
  auto img = load_hdr_from_file(name);
  for (int y = 0; y < img->height(); ++y)
    for (int x = 0; x < img->width(); ++x) {
      Color3f& c = img->at(x, y);
      c.x *= r;
      c.y *= g;
      c.z *= b;
    }
  return create_hdr_texture2d(img);
}

}  // namespace

void write_image_to_hdr(const Image2D<Spectrum>& image, const std::string& filename) {
  const int w = image.width(), h = image.height();
  std::vector<uint8_t> rgbe(4 * (size_t)w * h);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) encode_rgbe(image.at(x, y), &rgbe[4 * ((size_t)y * w + x)]);
  if (tr_write_hdr(filename.c_str(), rgbe.data(), (uint32_t)w, (uint32_t)h) != TR_OK)
    throw TracerError(TR_ERR_ARG, "cannot write " + filename);
}

void write_image_to_png(const Image2D<Color3b>& image, const std::string& filename) {
  const int w = image.width(), h = image.height();
  std::vector<uint8_t> rgb(3 * (size_t)w * h);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const Color3b& c = image.at(x, y);
      uint8_t* o = &rgb[3 * ((size_t)y * w + x)];
      o[0] = c.x;
      o[1] = c.y;
      o[2] = c.z;
    }
  if (tr_write_png(filename.c_str(), rgb.data(), (uint32_t)w, (uint32_t)h) != TR_OK)
    throw TracerError(TR_ERR_ARG, "cannot write " + filename);
}

RC<Image2D<Color3f>> load_hdr_from_file(const std::string& filename) {
  std::ifstream f(filename, std::ios::binary);
  if (!f) throw TracerError(TR_ERR_ARG, "load image failed: " + filename);
  const std::vector<uint8_t> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  size_t pos = 0;
  auto line = [&]() {
    std::string s;
    while (pos < buf.size() && buf[pos] != '\n') s.push_back((char)buf[pos++]);
    if (pos >= buf.size()) throw TracerError(TR_ERR_ARG, "truncated HDR header: " + filename);
    ++pos;
    return s;
  };
  const std::string magic = line();
  if (magic != "#?RADIANCE" && magic != "#?RGBE") throw TracerError(TR_ERR_ARG, "not a Radiance HDR file: " + filename);
  for (std::string s; !(s = line()).empty();)
    if (s.rfind("FORMAT=", 0) == 0 && s != "FORMAT=32-bit_rle_rgbe")
      throw TracerError(TR_ERR_UNSUPPORTED, "HDR pixel format " + s.substr(7) + ": " + filename);
  int w = 0, h = 0;
  {
    const std::string res = line();
    char ya[3] = {0}, xa[3] = {0};
    if (std::sscanf(res.c_str(), "%2s %d %2s %d", ya, &h, xa, &w) != 4 || std::strcmp(ya, "-Y") != 0 ||
        std::strcmp(xa, "+X") != 0 || w <= 0 || h <= 0 || w > (1 << 16) || h > (1 << 16) ||
        (size_t)w * h > (size_t(1) << 28))
      throw TracerError(TR_ERR_UNSUPPORTED, "HDR resolution line '" + res + "' (only -Y h +X w): " + filename);
  }
  auto img = std::make_shared<Image2D<Color3f>>(w, h);
  std::vector<uint8_t> row(4 * (size_t)w);
  auto need = [&](size_t n) {
    if (buf.size() - pos < n) throw TracerError(TR_ERR_ARG, "truncated HDR pixel data: " + filename);
  };
  for (int y = 0; y < h; ++y) {
    const bool rle = w >= 8 && w < 32768 && buf.size() - pos >= 4 && buf[pos] == 2 && buf[pos + 1] == 2 &&
                     (((int)buf[pos + 2] << 8) | buf[pos + 3]) == w;
    if (!rle) {  // flat RGBE pixels
      need(4 * (size_t)w);
      std::memcpy(row.data(), &buf[pos], 4 * (size_t)w);
      pos += 4 * (size_t)w;
    } else {  // each component as runs (count > 128: repeat the next byte) or literals
      pos += 4;
      for (int c = 0; c < 4; ++c)
        for (int x = 0; x < w;) {
          need(1);
          int n = buf[pos++];
          if (n > 128) {
            n -= 128;
            need(1);
            if (x + n > w) throw TracerError(TR_ERR_ARG, "bad HDR run length: " + filename);
            const uint8_t v = buf[pos++];
            for (int k = 0; k < n; ++k) row[4 * (size_t)(x + k) + c] = v;
          } else {
            if (n == 0 || x + n > w) throw TracerError(TR_ERR_ARG, "bad HDR literal run: " + filename);
            need((size_t)n);
            for (int k = 0; k < n; ++k) row[4 * (size_t)(x + k) + c] = buf[pos++];
          }
          x += n;
        }
    }
    for (int x = 0; x < w; ++x) img->at(x, y) = decode_rgbe(&row[4 * (size_t)x]);
  }
  return img;
}

RC<Image2D<Color3b>> load_image_from_file(const std::string& filename) {
  std::ifstream f(filename, std::ios::binary);
  if (!f) throw TracerError(TR_ERR_ARG, "load image failed: " + filename);
  const std::vector<uint8_t> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  int w = 0, h = 0, comp = 0;
  std::vector<uint8_t> px;
  try {
    // the format from the file's bytes, as stb_image finds it
    if (buf.size() >= 8 && std::memcmp(buf.data(), "\x89PNG\r\n\x1a\n", 8) == 0) px = decode_png(buf, w, h, comp);
    else if (tracer_files::is_jpeg(buf)) px = tracer_files::decode_jpeg(buf, w, h, comp);
    else if (tracer_files::is_bmp(buf)) px = tracer_files::decode_bmp(buf, w, h, comp);
    else if (tracer_files::is_tga(buf)) px = tracer_files::decode_tga(buf, w, h, comp);
    else throw TracerError(TR_ERR_ARG, "unknown image format");
  } catch (const TracerError& e) {
    throw TracerError(e.status, std::string(e.what()) + ": " + filename);
  }
  // load_image_from_file (src/utility/image_file.cpp:26-58): rows flipped
  // (the file's last row is row 0); 1 and 4 channels map to RGB, 2 is refused
  if (comp == 2) throw TracerError(TR_ERR_ARG, "invalid image component: " + filename);
  auto img = std::make_shared<Image2D<Color3b>>(w, h);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = &px[((size_t)(h - 1 - y) * w + x) * comp];
      img->at(x, y) = comp == 1 ? Color3b{p[0], p[0], p[0]} : Color3b{p[0], p[1], p[2]};
    }
  return img;
}

RC<const Texture2D> create_texture2d_from_file(const std::string& filename) {
  const std::string ext = extension(filename);
  if (ext == ".hdr") return create_hdr_texture2d(load_hdr_from_file(filename));
  if (ext == ".png" || ext == ".jpg" || ext == ".jpeg") return create_image_texture2d(load_image_from_file(filename));
  throw TracerError(TR_ERR_ARG, "unsupported image format: " + filename);
}

MaterialTexture create_texture_from_file(const material_t& m) {
  MaterialTexture t;
  t.map_ka = texture_of(m.map_ka, m.ambient[0], m.ambient[1], m.ambient[2]);
  t.map_kd = texture_of(m.map_kd, m.diffuse[0], m.diffuse[1], m.diffuse[2]);
  t.map_ks = texture_of(m.map_ks, m.specular[0], m.specular[1], m.specular[2]);
  t.map_ns = texture_of(m.map_ns, m.shininess, m.shininess, m.shininess);
  t.map_ke = texture_of(m.map_ke, m.emission[0], m.emission[1], m.emission[2]);
  if (m.emission[0] > 0 || m.emission[1] > 0 || m.emission[2] > 0) t.has_emission = true;
  if (m.ior > 1) {
    if (t.map_ks->evaluate_s(Point2f{0.5f, 0.5f}) == 0) t.map_ks = create_constant_texture2d(Spectrum(1, 1, 1));
    t.map_kt = t.map_ks;
    t.as_glass = true;
    t.ior = texture_of("", m.ior, m.ior, m.ior);
  }
  return t;
}

}  // namespace tracer
