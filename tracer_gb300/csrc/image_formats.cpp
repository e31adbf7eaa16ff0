// image_formats.cpp -- baseline JPEG, TGA and BMP decoders (see image_formats.h).
//
// Project-written from the formats' specifications: ITU-T T.81 (JPEG) with
// the JFIF colour space, the Truevision TGA 2.0 file format and the Windows
// BMP file format. Where the standard leaves the integer arithmetic open --
// the inverse DCT's fixed point, the chroma upsampling filter, the YCbCr
// conversion's rounding -- the choices are those of the reader the reference
// uses (its vendored stb_image v2.26), so that the decoded bytes are the
// reference's; tests/test_image_formats.py compares them with the
// reference's own reader on files written by the reference's own encoders.

#include "image_formats.h"

#include <climits>
#include <cstring>
#include <string>

#include "../../include/tracer_gb300.hpp"

namespace tracer_files {

namespace {

[[noreturn]] void bad(const std::string& what) { throw tracer::TracerError(TR_ERR_ARG, what); }

// ================================================================== JPEG
// Natural (row-major) position of the k-th coefficient in zig-zag order (T.81 Figure A.6).
const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

// A Huffman table as the canonical code of T.81 Annex C: per code length the
// smallest and largest code and the index of its first value (Figure F.16).
struct Huffman {
  bool defined = false;
  uint8_t values[256] = {};
  int mincode[17] = {}, maxcode[18] = {}, valptr[17] = {};
  void build(const uint8_t* counts, int total) {
    int code = 0, k = 0;
    for (int len = 1; len <= 16; ++len) {
      valptr[len] = k;
      mincode[len] = code;
      code += counts[len - 1];
      k += counts[len - 1];
      maxcode[len] = counts[len - 1] ? code - 1 : -1;
      code <<= 1;
    }
    maxcode[17] = INT_MAX;
    (void)total;
    defined = true;
  }
};

struct Component {
  int id = 0, h = 1, v = 1, tq = 0;
  int td = 0, ta = 0;     // Huffman tables of the current scan
  int bw = 0, bh = 0;     // blocks per row and column (MCU-padded)
  int pred = 0;           // DC predictor
  std::vector<uint8_t> plane;  // bw * 8 x bh * 8 samples
};

// Entropy-coded data: bits MSB first, 0xFF00 stuffing removed; a marker ends
// the data (zeros are supplied after it, as T.81 F.2.2.5 suggests).
struct BitReader {
  const std::vector<uint8_t>& f;
  size_t pos;
  uint32_t acc = 0;
  int nbits = 0;
  bool at_marker = false;
  BitReader(const std::vector<uint8_t>& f_, size_t p) : f(f_), pos(p) {}
  void fill() {
    while (nbits <= 24) {
      uint32_t b = 0;
      if (!at_marker && pos < f.size()) {
        b = f[pos];
        if (b == 0xFF) {
          const uint32_t nxt = pos + 1 < f.size() ? f[pos + 1] : 0xD9;
          if (nxt == 0x00) {
            pos += 2;
          } else {
            at_marker = true;  // a marker: leave pos on it
            b = 0;
          }
        } else {
          ++pos;
        }
      }
      acc |= b << (24 - nbits);
      nbits += 8;
    }
  }
  int bit() {
    if (nbits <= 0) fill();
    const int b = (int)(acc >> 31);
    acc <<= 1;
    --nbits;
    return b;
  }
  int bits(int n) {
    int v = 0;
    for (int i = 0; i < n; ++i) v = (v << 1) | bit();
    return v;
  }
  int decode(const Huffman& t) {
    int code = 0;
    for (int len = 1; len <= 16; ++len) {
      code = (code << 1) | bit();
      if (code <= t.maxcode[len]) return t.values[(t.valptr[len] + code - t.mincode[len]) & 255];
    }
    bad("corrupt JPEG Huffman code");
  }
  // receive + extend (T.81 F.2.2.1): an s-bit magnitude category
  int receive_extend(int s) {
    if (s == 0) return 0;
    if (s > 16) bad("corrupt JPEG coefficient");
    const int v = bits(s);
    return v < (1 << (s - 1)) ? v - (1 << s) + 1 : v;
  }
  // restart: the bits left in the byte are discarded, the next marker (RSTn) skipped
  void restart() {
    acc = 0;
    nbits = 0;
    at_marker = false;
    while (pos + 1 < f.size() && !(f[pos] == 0xFF && f[pos + 1] >= 0xD0 && f[pos + 1] <= 0xD7)) ++pos;
    if (pos + 1 < f.size()) pos += 2;
  }
};

// The inverse DCT of one dequantised block (natural order) to 8x8 samples:
// the Loeffler-Ligtenberg-Moschytz factorisation with 12-bit fixed-point
// constants, columns first (2 extra fraction bits kept), then rows, each
// output rounded, level-shifted by 128 and clamped to a byte.
inline int fix(double x) { return (int)(x * 4096.0 + 0.5); }

struct Idct1D {
  int o[8];
  void run(int s0, int s1, int s2, int s3, int s4, int s5, int s6, int s7) {
    // even part
    const int z1 = (s2 + s6) * fix(0.5411961);
    const int e2 = z1 + s6 * fix(-1.847759065);
    const int e3 = z1 + s2 * fix(0.765366865);
    const int e0 = (s0 + s4) * 4096, e1 = (s0 - s4) * 4096;
    const int a0 = e0 + e3, a3 = e0 - e3, a1 = e1 + e2, a2 = e1 - e2;
    // odd part
    const int q1 = s7 + s1, q2 = s5 + s3, q3 = s7 + s3, q4 = s5 + s1;
    const int q5 = (q3 + q4) * fix(1.175875602);
    const int b0 = s7 * fix(0.298631336) + q1 * fix(-0.899976223) + q3 * fix(-1.96157056) + q5;
    const int b1 = s5 * fix(2.053119869) + q2 * fix(-2.562915447) + q4 * fix(-0.390180644) + q5;
    const int b2 = s3 * fix(3.072711026) + q2 * fix(-2.562915447) + q3 * fix(-1.96157056) + q5;
    const int b3 = s1 * fix(1.50132111) + q1 * fix(-0.899976223) + q4 * fix(-0.390180644) + q5;
    o[0] = a0 + b3;
    o[7] = a0 - b3;
    o[1] = a1 + b2;
    o[6] = a1 - b2;
    o[2] = a2 + b1;
    o[5] = a2 - b1;
    o[3] = a3 + b0;
    o[4] = a3 - b0;
  }
};

inline uint8_t clamp_byte(int x) { return (uint8_t)(x < 0 ? 0 : (x > 255 ? 255 : x)); }

void idct_block(const int16_t* in, uint8_t* out, int stride) {
  int tmp[64];
  Idct1D d;
  for (int c = 0; c < 8; ++c) {
    d.run(in[c], in[8 + c], in[16 + c], in[24 + c], in[32 + c], in[40 + c], in[48 + c], in[56 + c]);
    for (int r = 0; r < 8; ++r) tmp[r * 8 + c] = (d.o[r] + 512) >> 10;
  }
  for (int r = 0; r < 8; ++r) {
    const int* t = tmp + r * 8;
    d.run(t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7]);
    for (int c = 0; c < 8; ++c) out[r * stride + c] = clamp_byte((d.o[c] + 65536 + (128 << 17)) >> 17);
  }
}

inline int div4(int x) { return x >> 2; }
inline int div16(int x) { return x >> 4; }

// One upsampled row of a subsampled component: `near` the chroma row nearest
// the output row, `far` the next nearest; hs, vs the horizontal and vertical
// factors. 2x: a triangle filter (3/4 of the nearer sample, 1/4 of the other,
// edges copied); other factors replicate the nearest sample.
void upsample_row(const uint8_t* near, const uint8_t* far, int w, int hs, int vs, uint8_t* out) {
  if (hs == 1 && vs == 1) {
    std::memcpy(out, near, (size_t)w);
  } else if (hs == 1 && vs == 2) {
    for (int i = 0; i < w; ++i) out[i] = (uint8_t)div4(3 * near[i] + far[i] + 2);
  } else if (hs == 2 && vs == 1) {
    if (w == 1) {
      out[0] = out[1] = near[0];
      return;
    }
    out[0] = near[0];
    out[1] = (uint8_t)div4(near[0] * 3 + near[1] + 2);
    for (int i = 1; i < w - 1; ++i) {
      const int n = 3 * near[i] + 2;
      out[2 * i] = (uint8_t)div4(n + near[i - 1]);
      out[2 * i + 1] = (uint8_t)div4(n + near[i + 1]);
    }
    out[2 * (w - 1)] = (uint8_t)div4(near[w - 2] * 3 + near[w - 1] + 2);
    out[2 * (w - 1) + 1] = near[w - 1];
  } else if (hs == 2 && vs == 2) {
    if (w == 1) {
      out[0] = out[1] = (uint8_t)div4(3 * near[0] + far[0] + 2);
      return;
    }
    int t1 = 3 * near[0] + far[0];
    out[0] = (uint8_t)div4(t1 + 2);
    for (int i = 1; i < w; ++i) {
      const int t0 = t1;
      t1 = 3 * near[i] + far[i];
      out[2 * i - 1] = (uint8_t)div16(3 * t0 + t1 + 8);
      out[2 * i] = (uint8_t)div16(3 * t1 + t0 + 8);
    }
    out[2 * w - 1] = (uint8_t)div4(t1 + 2);
  } else {
    for (int i = 0; i < w; ++i)
      for (int j = 0; j < hs; ++j) out[i * hs + j] = near[i];
  }
}

// JFIF YCbCr -> RGB (the JFIF matrix in fixed point, 20 fraction bits).
inline int cfix(float x) { return ((int)(x * 4096.0f + 0.5f)) << 8; }

void ycbcr_row(const uint8_t* y, const uint8_t* cb, const uint8_t* cr, int w, uint8_t* out) {
  for (int i = 0; i < w; ++i) {
    const int yf = (y[i] << 20) + (1 << 19);
    const int r = cr[i] - 128, b = cb[i] - 128;
    const int R = yf + r * cfix(1.40200f);
    const int G = yf + r * -cfix(0.71414f) + (int)((unsigned)(b * -cfix(0.34414f)) & 0xffff0000u);
    const int B = yf + b * cfix(1.77200f);
    out[3 * i] = clamp_byte(R >> 20);
    out[3 * i + 1] = clamp_byte(G >> 20);
    out[3 * i + 2] = clamp_byte(B >> 20);
  }
}

}  // namespace

bool is_jpeg(const std::vector<uint8_t>& f) { return f.size() >= 3 && f[0] == 0xFF && f[1] == 0xD8 && f[2] == 0xFF; }

std::vector<uint8_t> decode_jpeg(const std::vector<uint8_t>& f, int& w, int& h, int& comp) {
  if (!is_jpeg(f)) bad("not a JPEG file");
  uint16_t qt[4][64] = {};
  bool qt_defined[4] = {};
  Huffman dc[4], ac[4];
  std::vector<Component> cs;
  int hmax = 1, vmax = 1, restart_interval = 0, adobe_transform = -1;
  bool frame = false, done = false, any_scan = false;
  w = h = 0;
  size_t pos = 2;
  auto u16 = [&](size_t p) -> int {
    if (p + 1 >= f.size()) bad("truncated JPEG file");
    return (f[p] << 8) | f[p + 1];
  };
  while (!done) {
    // next marker (fill bytes 0xFF allowed)
    while (pos < f.size() && f[pos] != 0xFF) ++pos;
    while (pos < f.size() && f[pos] == 0xFF) ++pos;
    if (pos >= f.size()) break;
    const int m = f[pos++];
    if (m == 0xD9) break;                 // EOI
    if (m >= 0xD0 && m <= 0xD7) continue;  // a stray RSTn
    if (m == 0x01) continue;              // TEM
    const int len = u16(pos);
    if (len < 2 || pos + len > f.size()) bad("truncated JPEG segment");
    const size_t seg = pos + 2, end = pos + len;
    if (m == 0xDB) {  // DQT
      size_t p = seg;
      while (p < end) {
        const int pq = f[p] >> 4, tq = f[p] & 15;
        if (tq > 3 || pq > 1) bad("invalid JPEG quantisation table");
        ++p;
        for (int k = 0; k < 64; ++k) {
          if (p + (pq ? 1 : 0) >= end + (pq ? 0 : 1)) bad("truncated JPEG quantisation table");
          qt[tq][k] = pq ? (uint16_t)u16(p) : f[p];
          p += pq ? 2 : 1;
        }
        qt_defined[tq] = true;
      }
    } else if (m == 0xC4) {  // DHT
      size_t p = seg;
      while (p < end) {
        const int tc = f[p] >> 4, th = f[p] & 15;
        if (tc > 1 || th > 3 || p + 17 > end) bad("invalid JPEG Huffman table");
        const uint8_t* counts = &f[p + 1];
        int total = 0;
        for (int i = 0; i < 16; ++i) total += counts[i];
        if (total > 256 || p + 17 + total > end) bad("invalid JPEG Huffman table");
        Huffman& t = tc ? ac[th] : dc[th];
        std::memcpy(t.values, &f[p + 17], (size_t)total);
        t.build(counts, total);
        p += 17 + total;
      }
    } else if (m == 0xDD) {  // DRI
      restart_interval = u16(seg);
    } else if (m == 0xEE) {  // APP14 (Adobe): colour transform flag
      if (len >= 14 && std::memcmp(&f[seg], "Adobe", 5) == 0) adobe_transform = f[seg + 11];
    } else if (m == 0xC0 || m == 0xC1) {  // SOF0/SOF1: baseline / extended sequential, Huffman
      if (frame) bad("several JPEG frames");
      if (f[seg] != 8) throw tracer::TracerError(TR_ERR_UNSUPPORTED, "JPEG samples of other than 8 bits");
      h = u16(seg + 1);
      w = u16(seg + 3);
      const int nc = f[seg + 5];
      if (w <= 0 || h <= 0) bad("JPEG without image size");
      if ((long long)w * h > (1ll << 28)) bad("JPEG image too large");
      if (nc != 1 && nc != 3)
        throw tracer::TracerError(TR_ERR_UNSUPPORTED, "JPEG with " + std::to_string(nc) + " components");
      if (len < 8 + 3 * nc) bad("truncated JPEG frame header");
      cs.resize(nc);
      for (int i = 0; i < nc; ++i) {
        cs[i].id = f[seg + 6 + 3 * i];
        cs[i].h = f[seg + 7 + 3 * i] >> 4;
        cs[i].v = f[seg + 7 + 3 * i] & 15;
        cs[i].tq = f[seg + 8 + 3 * i];
        if (cs[i].h < 1 || cs[i].h > 4 || cs[i].v < 1 || cs[i].v > 4 || cs[i].tq > 3)
          bad("invalid JPEG component");
        hmax = std::max(hmax, cs[i].h);
        vmax = std::max(vmax, cs[i].v);
      }
      const int mcux = (w + 8 * hmax - 1) / (8 * hmax), mcuy = (h + 8 * vmax - 1) / (8 * vmax);
      for (Component& c : cs) {
        c.bw = mcux * c.h;
        c.bh = mcuy * c.v;
        c.plane.assign((size_t)c.bw * 8 * c.bh * 8, 0);
      }
      frame = true;
    } else if (m == 0xC2 || m == 0xC6 || m == 0xCA || m == 0xCE) {
      throw tracer::TracerError(TR_ERR_UNSUPPORTED, "progressive JPEG files have no reader here");
    } else if ((m >= 0xC3 && m <= 0xCF) && m != 0xC4 && m != 0xC8 && m != 0xCC) {
      throw tracer::TracerError(TR_ERR_UNSUPPORTED, "lossless, hierarchical or arithmetic-coded JPEG");
    } else if (m == 0xDA) {  // SOS
      if (!frame) bad("JPEG scan before the frame header");
      const int ns = f[seg];
      if (ns < 1 || ns > 4 || len < 6 + 2 * ns) bad("invalid JPEG scan header");
      std::vector<Component*> sc;
      for (int i = 0; i < ns; ++i) {
        const int id = f[seg + 1 + 2 * i];
        Component* c = nullptr;
        for (Component& x : cs)
          if (x.id == id) c = &x;
        if (!c) bad("JPEG scan names a missing component");
        c->td = f[seg + 2 + 2 * i] >> 4;
        c->ta = f[seg + 2 + 2 * i] & 15;
        if (c->td > 3 || c->ta > 3 || !dc[c->td].defined || !ac[c->ta].defined || !qt_defined[c->tq])
          bad("JPEG scan without its tables");
        c->pred = 0;
        sc.push_back(c);
      }
      BitReader br(f, end);
      int16_t blk[64];
      auto block = [&](Component& c, int bx, int by) {
        std::memset(blk, 0, sizeof(blk));
        const uint16_t* q = qt[c.tq];
        const int t = br.decode(dc[c.td]);
        c.pred += br.receive_extend(t);
        blk[0] = (int16_t)(c.pred * q[0]);
        for (int k = 1; k < 64;) {
          const int rs = br.decode(ac[c.ta]);
          const int r = rs >> 4, s = rs & 15;
          if (s == 0) {
            if (r != 15) break;  // end of block
            k += 16;
            continue;
          }
          k += r;
          if (k > 63) bad("corrupt JPEG block");
          blk[kZigzag[k]] = (int16_t)(br.receive_extend(s) * q[k]);
          ++k;
        }
        const int stride = c.bw * 8;
        idct_block(blk, c.plane.data() + (size_t)by * 8 * stride + (size_t)bx * 8, stride);
      };
      long long mcus;
      int mx_n;
      if (ns == 1) {
        // a non-interleaved scan: the component's blocks that cover the image, row by row
        Component& c = *sc[0];
        const int cw = (w * c.h + hmax - 1) / hmax, ch = (h * c.v + vmax - 1) / vmax;
        mx_n = (cw + 7) / 8;
        mcus = (long long)mx_n * ((ch + 7) / 8);
      } else {
        mx_n = (w + 8 * hmax - 1) / (8 * hmax);
        mcus = (long long)mx_n * ((h + 8 * vmax - 1) / (8 * vmax));
      }
      for (long long i = 0; i < mcus; ++i) {
        if (restart_interval && i && i % restart_interval == 0) {
          br.restart();
          for (Component* c : sc) c->pred = 0;
        }
        const int mx = (int)(i % mx_n), my = (int)(i / mx_n);
        if (ns == 1) {
          block(*sc[0], mx, my);
        } else {
          for (Component* c : sc)
            for (int v = 0; v < c->v; ++v)
              for (int u = 0; u < c->h; ++u) block(*c, mx * c->h + u, my * c->v + v);
        }
      }
      // continue after the scan's data: the next marker (skipping stuffing and RSTn)
      pos = br.pos;
      while (pos + 1 < f.size()) {
        if (f[pos] == 0xFF && f[pos + 1] != 0x00 && !(f[pos + 1] >= 0xD0 && f[pos + 1] <= 0xD7)) break;
        ++pos;
      }
      any_scan = true;
      continue;
    }
    pos = end;
  }
  if (!frame || !any_scan) bad("JPEG file without image data");
  // colour: one component is grey; three are YCbCr unless the file says RGB
  // (component ids 'R', 'G', 'B', or an Adobe transform of 0)
  const int nc = (int)cs.size();
  comp = nc;
  std::vector<uint8_t> out((size_t)w * h * comp);
  std::vector<std::vector<uint8_t>> rows(nc, std::vector<uint8_t>((size_t)w + 4 * hmax));
  for (int y = 0; y < h; ++y) {
    for (int k = 0; k < nc; ++k) {
      const Component& c = cs[k];
      const int hs = hmax / c.h, vs = vmax / c.v;
      const int cw = (w * c.h + hmax - 1) / hmax, ch = (h * c.v + vmax - 1) / vmax;
      const int stride = c.bw * 8;
      int near_row, far_row;
      if (vs == 2 && hs <= 2) {
        near_row = y >> 1;
        far_row = (y & 1) ? std::min(near_row + 1, ch - 1) : std::max(near_row - 1, 0);
      } else {
        near_row = far_row = std::min(y / vs, ch - 1);
      }
      upsample_row(c.plane.data() + (size_t)near_row * stride, c.plane.data() + (size_t)far_row * stride, cw, hs,
                   (vs == 2 && hs <= 2) ? 2 : 1, rows[k].data());
    }
    uint8_t* o = out.data() + (size_t)y * w * comp;
    if (nc == 1) {
      std::memcpy(o, rows[0].data(), (size_t)w);
    } else {
      const bool rgb = (cs[0].id == 'R' && cs[1].id == 'G' && cs[2].id == 'B') || adobe_transform == 0;
      if (rgb) {
        for (int x = 0; x < w; ++x)
          for (int k = 0; k < 3; ++k) o[3 * x + k] = rows[k][x];
      } else {
        ycbcr_row(rows[0].data(), rows[1].data(), rows[2].data(), w, o);
      }
    }
  }
  return out;
}

// =================================================================== TGA
namespace {
inline int le16(const std::vector<uint8_t>& f, size_t p) { return f[p] | (f[p + 1] << 8); }
}  // namespace

bool is_tga(const std::vector<uint8_t>& f) {
  if (f.size() < 18) return false;
  const int cmap = f[1], type = f[2], bpp = f[16];
  if (cmap > 1) return false;
  if (cmap == 1 && type != 1 && type != 9) return false;
  if (cmap == 0 && type != 2 && type != 3 && type != 10 && type != 11) return false;
  if (cmap == 1 && bpp != 8 && bpp != 16) return false;
  if (cmap == 1) {
    const int ebpp = f[7];
    if (ebpp != 8 && ebpp != 15 && ebpp != 16 && ebpp != 24 && ebpp != 32) return false;
  } else if (bpp != 8 && bpp != 15 && bpp != 16 && bpp != 24 && bpp != 32) {
    return false;
  }
  return le16(f, 12) > 0 && le16(f, 14) > 0;
}

std::vector<uint8_t> decode_tga(const std::vector<uint8_t>& f, int& w, int& h, int& comp) {
  if (!is_tga(f)) bad("not a TGA file");
  const int idlen = f[0], cmap = f[1], type = f[2];
  const int cmap_first = le16(f, 3), cmap_len = le16(f, 5), cmap_bpp = f[7];
  w = le16(f, 12);
  h = le16(f, 14);
  const int bpp = f[16], desc = f[17];
  const bool rle = type >= 9, grey = type == 3 || type == 11;
  const int pix_bpp = cmap ? cmap_bpp : bpp;  // bits of an output pixel's source
  // components: 8-bit grey 1, 15/16-bit 3, 24-bit 3, 32-bit 4
  comp = grey ? 1 : (pix_bpp == 32 ? 4 : (pix_bpp == 8 ? 1 : 3));
  size_t p = 18 + idlen;
  std::vector<uint8_t> pal;
  const int pe = (cmap_bpp + 7) / 8;
  if (cmap) {
    if (p + (size_t)cmap_len * pe > f.size()) bad("truncated TGA colour map");
    pal.assign(f.begin() + (ptrdiff_t)p, f.begin() + (ptrdiff_t)(p + (size_t)cmap_len * pe));
    p += (size_t)cmap_len * pe;
  }
  const int ib = (bpp + 7) / 8;  // bytes per stored pixel or index
  auto expand = [&](const uint8_t* s, int nbits, uint8_t* o) {
    if (nbits == 15 || nbits == 16) {  // 5-5-5 (stored little-endian, BGR), each to 8 bits
      const int v = s[0] | (s[1] << 8);
      o[0] = (uint8_t)(((v >> 10) & 31) * 255 / 31);
      o[1] = (uint8_t)(((v >> 5) & 31) * 255 / 31);
      o[2] = (uint8_t)((v & 31) * 255 / 31);
    } else if (nbits == 8) {
      o[0] = s[0];
    } else {  // BGR(A)
      o[0] = s[2];
      o[1] = s[1];
      o[2] = s[0];
      if (nbits == 32) o[3] = s[3];
    }
  };
  std::vector<uint8_t> out((size_t)w * h * comp);
  uint8_t px[4] = {};
  int run = 0;
  bool packet_rle = false;
  for (size_t i = 0; i < (size_t)w * h; ++i) {
    bool read = true;
    if (rle) {
      if (run == 0) {
        if (p >= f.size()) bad("truncated TGA image");
        const int hdr = f[p++];
        run = (hdr & 127) + 1;
        packet_rle = (hdr & 128) != 0;
        read = true;
      } else {
        read = !packet_rle;
      }
      --run;
    }
    if (read) {
      if (p + ib > f.size()) bad("truncated TGA image");
      if (cmap) {
        int idx = ib == 1 ? f[p] : le16(f, p);
        idx -= cmap_first;
        if (idx < 0 || idx >= cmap_len) idx = 0;
        expand(&pal[(size_t)idx * pe], cmap_bpp, px);
      } else {
        expand(&f[p], bpp, px);
      }
      p += ib;
    }
    std::memcpy(&out[i * comp], px, (size_t)comp);
  }
  // rows stored bottom-up unless the descriptor's top-left bit is set
  if (!(desc & 0x20)) {
    std::vector<uint8_t> row((size_t)w * comp);
    for (int y = 0; y < h / 2; ++y) {
      uint8_t* a = &out[(size_t)y * w * comp];
      uint8_t* b = &out[(size_t)(h - 1 - y) * w * comp];
      std::memcpy(row.data(), a, row.size());
      std::memcpy(a, b, row.size());
      std::memcpy(b, row.data(), row.size());
    }
  }
  return out;
}

// =================================================================== BMP
namespace {
inline uint32_t le32(const std::vector<uint8_t>& f, size_t p) {
  return (uint32_t)f[p] | ((uint32_t)f[p + 1] << 8) | ((uint32_t)f[p + 2] << 16) | ((uint32_t)f[p + 3] << 24);
}
// Bits of a channel mask as an 8-bit value (shifted to the top, then
// replicated into the low bits).
int masked(uint32_t v, uint32_t mask) {
  if (!mask) return 0;
  int shift = 0, bits = 0;
  while (!((mask >> shift) & 1)) ++shift;
  while ((mask >> (shift + bits)) & 1) ++bits;
  uint32_t x = (v & mask) >> shift;
  if (bits >= 8) return (int)(x >> (bits - 8));
  int r = 0, have = 0;
  while (have < 8) {
    r = (r << bits) | (int)x;
    have += bits;
  }
  return r >> (have - 8);
}
}  // namespace

bool is_bmp(const std::vector<uint8_t>& f) {
  if (f.size() < 26 || f[0] != 'B' || f[1] != 'M') return false;
  const uint32_t hs = le32(f, 14);
  return hs == 12 || hs == 40 || hs == 56 || hs == 108 || hs == 124;
}

std::vector<uint8_t> decode_bmp(const std::vector<uint8_t>& f, int& w, int& h, int& comp) {
  if (!is_bmp(f)) bad("not a BMP file");
  const uint32_t offset = le32(f, 10), hsz = le32(f, 14);
  int bpp, planes;
  uint32_t compression = 0, rmask = 0, gmask = 0, bmask = 0, amask = 0, ncolors = 0;
  bool top_down = false;
  if (hsz == 12) {
    w = le16(f, 18);
    h = le16(f, 20);
    planes = le16(f, 22);
    bpp = le16(f, 24);
  } else {
    if (f.size() < 14 + 40) bad("truncated BMP header");
    w = (int)le32(f, 18);
    int32_t hh = (int32_t)le32(f, 22);
    top_down = hh < 0;
    h = top_down ? -hh : hh;
    planes = le16(f, 26);
    bpp = le16(f, 28);
    compression = le32(f, 30);
    ncolors = le32(f, 46);
    if (compression == 3) {  // BI_BITFIELDS: masks after the header (or in it)
      const size_t mp = hsz >= 56 ? 54 : 54;
      if (f.size() < mp + 12) bad("truncated BMP masks");
      rmask = le32(f, mp);
      gmask = le32(f, mp + 4);
      bmask = le32(f, mp + 8);
      if (hsz >= 56 && f.size() >= mp + 16) amask = le32(f, mp + 12);
    } else if (compression != 0) {
      throw tracer::TracerError(TR_ERR_UNSUPPORTED, "run-length or other compressed BMP files have no reader here");
    }
  }
  if (planes != 1) bad("invalid BMP planes");
  if (w <= 0 || h <= 0 || (long long)w * h > (1ll << 28)) bad("invalid BMP size");
  if (bpp != 1 && bpp != 4 && bpp != 8 && bpp != 16 && bpp != 24 && bpp != 32)
    throw tracer::TracerError(TR_ERR_UNSUPPORTED, "BMP of " + std::to_string(bpp) + " bits per pixel");
  if (bpp == 16 && compression == 0) {  // 5-5-5
    rmask = 0x7c00;
    gmask = 0x03e0;
    bmask = 0x001f;
  }
  const bool alpha = bpp == 32 && (compression == 0 || amask != 0);
  comp = alpha ? 4 : 3;
  // palette
  std::vector<uint8_t> pal;
  if (bpp <= 8) {
    const size_t pe = hsz == 12 ? 3 : 4;
    size_t n = ncolors ? ncolors : (1u << bpp);
    const size_t pp = 14 + hsz;
    if (pp + n * pe > f.size()) bad("truncated BMP palette");
    for (size_t i = 0; i < n; ++i) {
      pal.push_back(f[pp + i * pe + 2]);
      pal.push_back(f[pp + i * pe + 1]);
      pal.push_back(f[pp + i * pe]);
    }
  }
  const size_t row_bytes = (((size_t)w * bpp + 31) / 32) * 4;
  if ((size_t)offset + row_bytes * h > f.size()) bad("truncated BMP pixels");
  std::vector<uint8_t> out((size_t)w * h * comp);
  bool all_alpha_zero = true;
  for (int y = 0; y < h; ++y) {
    const int src_row = top_down ? y : h - 1 - y;
    const uint8_t* r = &f[offset + (size_t)src_row * row_bytes];
    uint8_t* o = &out[(size_t)y * w * comp];
    for (int x = 0; x < w; ++x, o += comp) {
      if (bpp <= 8) {
        const int bit = x * bpp;
        int idx = (r[bit >> 3] >> (8 - bpp - (bit & 7))) & ((1 << bpp) - 1);
        if ((size_t)idx * 3 + 2 >= pal.size()) idx = 0;
        o[0] = pal[idx * 3];
        o[1] = pal[idx * 3 + 1];
        o[2] = pal[idx * 3 + 2];
      } else if (bpp == 24) {
        o[0] = r[3 * x + 2];
        o[1] = r[3 * x + 1];
        o[2] = r[3 * x];
      } else if (bpp == 32 && compression == 0) {
        o[0] = r[4 * x + 2];
        o[1] = r[4 * x + 1];
        o[2] = r[4 * x];
        o[3] = r[4 * x + 3];
        all_alpha_zero &= o[3] == 0;
      } else {
        const uint32_t v = bpp == 16 ? (uint32_t)(r[2 * x] | (r[2 * x + 1] << 8)) : le32(f, (size_t)(r - f.data()) + 4 * x);
        o[0] = (uint8_t)masked(v, rmask);
        o[1] = (uint8_t)masked(v, gmask);
        o[2] = (uint8_t)masked(v, bmask);
        if (comp == 4) {
          o[3] = amask ? (uint8_t)masked(v, amask) : 255;
          all_alpha_zero &= o[3] == 0;
        }
      }
    }
  }
  // a 32-bit file whose alpha is zero everywhere is opaque
  if (comp == 4 && all_alpha_zero)
    for (size_t i = 3; i < out.size(); i += 4) out[i] = 255;
  return out;
}

}  // namespace tracer_files
