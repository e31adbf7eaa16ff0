// image_file.cpp -- the reference's image-file helpers (src/utility/image_file.cpp)
// over project code: the PNG and Radiance HDR writers of image_out.cpp, a
// Radiance HDR reader (G. Ward's RGBE format: a text header, the resolution
// line, then flat or run-length scanlines), and the MTL-to-texture mapping
// of create_texture_from_file.
#include <cmath>
#include <cstdio>
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
  if (ext != ".hdr") {
    if (ext == ".jpg" || ext == ".jpeg" || ext == ".png")
      throw TracerError(TR_ERR_UNSUPPORTED, "8-bit image files have no reader here (convert to .hdr): " + name);
    throw TracerError(TR_ERR_ARG, "unsupported image format: " + name);
  }
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
        std::strcmp(xa, "+X") != 0 || w <= 0 || h <= 0 || w > (1 << 16) || h > (1 << 16))
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

RC<const Texture2D> create_texture2d_from_file(const std::string& filename) {
  const std::string ext = extension(filename);
  if (ext == ".hdr") return create_hdr_texture2d(load_hdr_from_file(filename));
  if (ext == ".jpg" || ext == ".jpeg" || ext == ".png")
    throw TracerError(TR_ERR_UNSUPPORTED, "8-bit image files have no reader here (convert to .hdr): " + filename);
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
