// env_tex.cuh -- the environment map lookup, shared by the host table build
// and the device kernels: HDRTexture2D::evaluate_impl
// (src/texture/hdr_texture.cpp:27-30) behind Texture2D::evaluate with the
// repeat wrap (src/core/texture.hpp:57-95), i.e. LinearSampler::Sample2D
// (src/utility/sampler.hpp:16-29) in double with float texels: each
// texel-times-weight product is a double product rounded to float
// (Point3<float>::operator*(double), src/utility/geometry.hpp:268-271), the
// sums are float.
#pragma once

#include <cuda_runtime.h>

#include "tr_math.cuh"

namespace trg {

// texel (x, y) at tex[x + y * w]; (u, v) in texture coordinates
TR_HD f3 env_tex_eval(const float4* tex, int w, int h, float u_in, float v_in) {
  // wrap_repeat: clamp(x - floor(x), 0, 1)
  float uw = u_in - floorf(u_in), vw = v_in - floorf(v_in);
  uw = uw < 0.0f ? 0.0f : (1.0f < uw ? 1.0f : uw);
  vw = vw < 0.0f ? 0.0f : (1.0f < vw ? 1.0f : vw);
  double u = (double)uw, v = (double)vw;
  u = (u < 0.0 ? 0.0 : (1.0 < u ? 1.0 : u)) * (double)(w - 1);
  v = (v < 0.0 ? 0.0 : (1.0 < v ? 1.0 : v)) * (double)(h - 1);
  int u0 = (int)u, v0 = (int)v;
  u0 = u0 < 0 ? 0 : (u0 > w - 1 ? w - 1 : u0);
  v0 = v0 < 0 ? 0 : (v0 > h - 1 ? h - 1 : v0);
  const int u1 = u0 + 1 > w - 1 ? w - 1 : u0 + 1;
  const int v1 = v0 + 1 > h - 1 ? h - 1 : v0 + 1;
  const double du = u - u0, dv = v - v0;
  const double eu = 1.0 - du, ev = 1.0 - dv;
  const float4 a = tex[u0 + (size_t)v0 * w], b = tex[u1 + (size_t)v0 * w];
  const float4 c = tex[u0 + (size_t)v1 * w], d = tex[u1 + (size_t)v1 * w];
  // ((a eu + b du) ev) + ((c eu + d du) dv), per channel
  const float tr = (float)(eu * a.x) + (float)(du * b.x), br = (float)(eu * c.x) + (float)(du * d.x);
  const float tg = (float)(eu * a.y) + (float)(du * b.y), bg = (float)(eu * c.y) + (float)(du * d.y);
  const float tb = (float)(eu * a.z) + (float)(du * b.z), bb = (float)(eu * c.z) + (float)(du * d.z);
  return mk3((float)(ev * tr) + (float)(dv * br), (float)(ev * tg) + (float)(dv * bg),
             (float)(ev * tb) + (float)(dv * bb));
}

// ImageTexture2D::evaluate_impl (src/texture/image_texture2d.cpp:26-30) over
// Image2D<Color3b>: the same bilinear weights, but each weighted texel is a
// Point3<uint8_t> (the double product truncated to a byte) and the sums are
// bytes; the result is divided by 255.
TR_HD f3 env_tex_eval8(const uchar4* tex, int w, int h, float u_in, float v_in) {
  float uw = u_in - floorf(u_in), vw = v_in - floorf(v_in);
  uw = uw < 0.0f ? 0.0f : (1.0f < uw ? 1.0f : uw);
  vw = vw < 0.0f ? 0.0f : (1.0f < vw ? 1.0f : vw);
  double u = (double)uw, v = (double)vw;
  u = (u < 0.0 ? 0.0 : (1.0 < u ? 1.0 : u)) * (double)(w - 1);
  v = (v < 0.0 ? 0.0 : (1.0 < v ? 1.0 : v)) * (double)(h - 1);
  int u0 = (int)u, v0 = (int)v;
  u0 = u0 < 0 ? 0 : (u0 > w - 1 ? w - 1 : u0);
  v0 = v0 < 0 ? 0 : (v0 > h - 1 ? h - 1 : v0);
  const int u1 = u0 + 1 > w - 1 ? w - 1 : u0 + 1;
  const int v1 = v0 + 1 > h - 1 ? h - 1 : v0 + 1;
  const double du = u - u0, dv = v - v0;
  const double eu = 1.0 - du, ev = 1.0 - dv;
  const uchar4 a = tex[u0 + (size_t)v0 * w], b = tex[u1 + (size_t)v0 * w];
  const uchar4 c = tex[u0 + (size_t)v1 * w], d = tex[u1 + (size_t)v1 * w];
  auto by = [](double f, int x) { return (int)(f * (double)x) & 0xff; };
  auto ch = [&](int ta, int tb, int tc, int td) {
    const int top = (by(eu, ta) + by(du, tb)) & 0xff, bot = (by(eu, tc) + by(du, td)) & 0xff;
    return (float)((by(ev, top) + by(dv, bot)) & 0xff) / 255.0f;
  };
  return mk3(ch(a.x, b.x, c.x, d.x), ch(a.y, b.y, c.y, d.y), ch(a.z, b.z, c.z, d.z));
}

}  // namespace trg
