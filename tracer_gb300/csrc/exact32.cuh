// exact32.cuh -- the reference's double-precision vector expressions,
// evaluated in single precision with a proof of the result.
//
// GB300 runs FP64 at a small fraction of its FP32 rate, and the reference
// computes normalize(), cross() and cos() through doubles
// (src/utility/geometry.hpp:429-445, 570-590, 943-949). Each function here
//  1. computes the exact real value of the expression to about 2^-43
//     relative in float-float arithmetic (FMA-based error-free products and
//     sums, one Newton step on rsqrt),
//  2. rounds that to float and checks, with a rigorous error bound that also
//     covers the reference's intermediate double roundings (at most a few
//     2^-53 relative), that the true value lies strictly inside the rounding
//     interval of that float -- then the reference's float(double(...)) is
//     the same float,
//  3. otherwise evaluates the reference's double expression directly.
// Step 3 is needed only when the value lies within ~2^-40 relative of a
// float rounding boundary or outside a safe exponent range (rare), so
// results equal the reference bit for bit while the common case uses the
// FP32 pipes. Device checks against the double expressions run through
// tr_selftest (tests/test_gpu_exact32.py); host builds of the same code are
// checked in tests/test_exact32_host.py.
#pragma once

#include "tr_math.cuh"

namespace trg {

TR_HD uint32_t fbits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t b;
  memcpy(&b, &x, 4);
  return b;
#endif
}
TR_HD float bitsf(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}
TR_HD float ffma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
TR_HD float frsqrt(float x) {
#if defined(__CUDA_ARCH__)
  return rsqrtf(x);
#else
  return 1.0f / std::sqrt(x);
#endif
}

// |x| in [2^-60, 2^60]: float-float steps below neither overflow nor lose
// their error terms to underflow.
TR_HD bool in_range(float x) {
  const uint32_t e = (fbits(x) >> 23) & 0xffu;
  return e >= 67u && e <= 187u;
}

// True when every real within err of (y + r) rounds to y, where y is a
// normal float and r the exact residual of the approximation (|r| at most
// half a spacing). Both neighbouring half-spacings are checked.
TR_HD bool rounds_to(float y, float r, float err) {
  const uint32_t b = fbits(y) & 0x7fffffffu;
  if (b < 0x01000000u || b >= 0x7e800000u) return false;  // tiny, huge, inf, nan
  const float ulp = bitsf(b & 0x7f800000u) * 1.1920928955078125e-07f;  // 2^(e-23)
  float half = 0.5f * ulp;
  if ((b & 0x007fffffu) == 0u) half *= 0.5f;  // power of two: smaller spacing below
  return fabsf(r) + err < half;
}

// (s, e) with s = RN(a + b) and s + e = a + b exactly.
TR_HD float two_sum(float a, float b, float& e) {
  const float s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
  return s;
}

// 1/sqrt(L) ~ r0 + c (relative error below 2^-43 for L in range).
TR_HD void rsqrt_ff(float L, float& r0, float& c) {
  r0 = frsqrt(L);
  const float th = r0 * r0;
  const float tl = ffma(r0, r0, -th);
  const float uh = L * th;
  const float ul = ffma(L, th, -uh) + L * tl;
  const float res = (1.0f - uh) - ul;
  c = r0 * res * 0.5f;
}

TR_HD_COLD float cross1_d(float a, float b, float c, float d) {
  return (float)((double)a * (double)b - (double)c * (double)d);
}

// float(double(a) * b - double(c) * d): one component of the reference's cross().
TR_HD float cross1(float a, float b, float c, float d) {
  const float ph = a * b, qh = c * d;
  const bool pz = (a == 0.0f) | (b == 0.0f), qz = (c == 0.0f) | (d == 0.0f);
  if (pz | qz) {
    if (pz & qz) return ph - qh;  // exact zeros, with the double result's sign
    return pz ? -qh : ph;         // the other product, exactly rounded once
  }
  if (in_range(ph) & in_range(qh)) {
    const float pl = ffma(a, b, -ph), ql = ffma(c, d, -qh);
    float e;
    const float s = two_sum(ph, -qh, e);
    const float w = e + (pl - ql);
    float r;
    const float y = two_sum(s, w, r);
    const float err = 1.4210855e-14f * (fabsf(ph) + fabsf(qh)) + 8.8817842e-16f * fabsf(y);  // 2^-46, 2^-50
    if (rounds_to(y, r, err)) return y;
  }
  return cross1_d(a, b, c, d);
}

TR_HD f3 cross_x(f3 a, f3 b) {
  return mk3(cross1(a.y, b.z, a.z, b.y), cross1(a.z, b.x, a.x, b.z), cross1(a.x, b.y, a.y, b.x));
}

// The reference's normalize(v): float(x * (1.0 / sqrt(double(|v|^2_float)))).
TR_HD f3 normalize_x(f3 v) {
  const float L = len2f(v);
  if (L >= 8.6736174e-19f && L <= 1.1529215e+18f) {  // [2^-60, 2^60]
    float r0, c;
    rsqrt_ff(L, r0, c);
    float o[3];
    const float in[3] = {v.x, v.y, v.z};
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
      const float x = in[k];
      if (x == 0.0f) {
        o[k] = x;  // +-0 * positive finite
        continue;
      }
      if (!in_range(x)) {
        ok = false;
        break;
      }
      const float ph = x * r0;
      const float pl = ffma(x, r0, -ph);
      const float zl = pl + x * c;
      float r;
      const float y = two_sum(ph, zl, r);
      if (!rounds_to(y, r, 9.094947e-13f * fabsf(y))) {  // 2^-40
        ok = false;
        break;
      }
      o[k] = y;
    }
    if (ok) return mk3(o[0], o[1], o[2]);
  }
  return normalize_d(v);
}

// float(double(dot32(a, b)) / (sqrt(double(La)) * sqrt(double(Lb)))), the
// reference's cos(w1, w2).
TR_HD float cos_x(f3 a, f3 b) {
  const float d = dot(a, b);
  const float La = len2f(a), Lb = len2f(b);
  if (d == 0.0f && La > 0.0f && Lb > 0.0f && La <= 1e30f && Lb <= 1e30f) return d;
  if (La >= 8.6736174e-19f && La <= 1.1529215e+18f && Lb >= 8.6736174e-19f && Lb <= 1.1529215e+18f &&
      in_range(d)) {
    float ra, ca, rb, cb;
    rsqrt_ff(La, ra, ca);
    rsqrt_ff(Lb, rb, cb);
    const float Rh = ra * rb;
    const float Rl = ffma(ra, rb, -Rh) + (ra * cb + rb * ca);
    const float ph = d * Rh;
    if (in_range(ph)) {
      const float zl = ffma(d, Rh, -ph) + d * Rl;
      float r;
      const float y = two_sum(ph, zl, r);
      if (rounds_to(y, r, 1.8189894e-12f * fabsf(y))) return y;  // 2^-39
    }
  }
  return cosv_d(a, b);
}
TR_HD float abs_cos_x(f3 a, f3 b) { return fabsf(cos_x(a, b)); }

TR_HD_COLD float dist_minus_eps_d(float L, bool& le_eps) {
  const double dd = sqrt((double)L) - (double)kEps;
  le_eps = dd <= (double)kEps;
  return (float)dd;
}

// sqrt(double(L)) - eps in double, rounded to float, and whether that
// double is <= eps (src/renderer/direct_illumination.cpp:45-47).
TR_HD float dist_minus_eps(float L, bool& le_eps) {
  if (L >= 8.6736174e-19f && L <= 1.1529215e+18f) {
    float r0, c;
    rsqrt_ff(L, r0, c);
    // sqrt(L) = L * r ~ sh + sl
    const float sh = L * r0;
    const float sl = ffma(L, r0, -sh) + L * c;
    float e1;
    const float t = two_sum(sh, -kEps, e1);
    const float w = e1 + sl;
    float r;
    const float y = two_sum(t, w, r);
    // error: 2^-43 |sqrt L| from r, plus the reference's two double roundings
    const float err = 2.2737368e-13f * sh;  // 2^-42
    if (rounds_to(y, r, err)) {
      const float margin = 2.0f * err + 1.1920929e-07f * kEps;
      if (y > kEps + margin) {
        le_eps = false;
        return y;
      }
      if (y < kEps - margin) {
        le_eps = true;
        return y;
      }
    }
  }
  return dist_minus_eps_d(L, le_eps);
}

TR_HD_COLD float area_to_solid_pdf_d(float A, float d, float L) {
  return (float)((double)A / fabs((double)d / sqrt((double)L)));
}

// float(double(A) / fabs(double(dot) / sqrt(double(L)))): the light
// sampling pdf of DiffuseLight::sample_li (src/light/diffuse_light.cpp:50-51).
TR_HD float area_to_solid_pdf(float A, float d, float L) {
  if (A > 0.0f && in_range(A) && in_range(d) && L >= 8.6736174e-19f && L <= 1.1529215e+18f) {
    float r0, c;
    rsqrt_ff(L, r0, c);
    const float ad = fabsf(d);
    // q = |d| / sqrt(L) = |d| * r ~ qh + ql
    const float qh = ad * r0;
    const float ql = ffma(ad, r0, -qh) + ad * c;
    // A / (qh + ql): y0 = A / qh, then one correction
    const float y0 = A / qh;
    const float res = ffma(-y0, qh, A) - y0 * ql;
    const float corr = res / qh;
    float r;
    const float y = two_sum(y0, corr, r);
    if (rounds_to(y, r, 1.8189894e-12f * fabsf(y))) return y;  // 2^-39
  }
  return area_to_solid_pdf_d(A, d, L);
}

// Vector3 / f for a float f (src/utility/geometry.hpp:429-433):
// float(x * (1.0 / double(f))) per component.
TR_HD f3 div_x(f3 v, float f) {
  if (in_range(f)) {
    const float i0 = 1.0f / f;
    const float i1 = i0 * ffma(-i0, f, 1.0f);  // 1/f ~ i0 + i1
    float o[3];
    const float in[3] = {v.x, v.y, v.z};
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
      const float x = in[k];
      if (x == 0.0f) {
        o[k] = (f > 0.0f) ? x : -x;
        continue;
      }
      if (!in_range(x)) {
        ok = false;
        break;
      }
      const float ph = x * i0;
      if (!in_range(ph)) {
        ok = false;
        break;
      }
      const float zl = ffma(x, i0, -ph) + x * i1;
      float r;
      const float y = two_sum(ph, zl, r);
      if (!rounds_to(y, r, 9.094947e-13f * fabsf(y))) {  // 2^-40
        ok = false;
        break;
      }
      o[k] = y;
    }
    if (ok) return mk3(o[0], o[1], o[2]);
  }
  return divd(v, (double)f);
}

// The kernels' names for the reference's vector functions.
TR_HD f3 normalize(f3 v) { return normalize_x(v); }
TR_HD f3 cross(f3 a, f3 b) { return cross_x(a, b); }
TR_HD float cosv(f3 a, f3 b) { return cos_x(a, b); }
TR_HD float abs_cos(f3 a, f3 b) { return fabsf(cos_x(a, b)); }

// coordinate(v1, v2, v3) (geometry.hpp:887-894): the divisor is a float sqrt
TR_HD void coordinate(f3 v1, f3& v2, f3& v3) {
  if (fabsf(v1.x) > fabsf(v1.y))
    v2 = div_x(mk3(-v1.z, 0.0f, v1.x), sqrtf(v1.x * v1.x + v1.z * v1.z));
  else
    v2 = div_x(mk3(0.0f, v1.z, -v1.y), sqrtf(v1.y * v1.y + v1.z * v1.z));
  v3 = cross(v1, v2);
}

// compute_ss_ts (utility/coordinate.hpp:54-68)
TR_HD void compute_ss_ts(f3 AB, f3 AC, float m00, float m01, float m10, float m11, f3 n, f3& ss, f3& ts) {
  const float det = m00 * m11 - m01 * m10;
  if (det) {
    const float inv_det = 1.0f / det;
    ss = scale(AB, m11 * inv_det) - scale(AC, m01 * inv_det);
    ts = scale(AB, m10 * inv_det) - scale(AC, m00 * inv_det);
  } else {
    coordinate(n, ss, ts);
  }
}

// Orthonormal frame (utility/coordinate.hpp:15-116): the constructor
// normalises each axis.
struct Frame {
  f3 x, y, z;
};
TR_HD Frame make_frame(f3 a, f3 b, f3 c) {
  Frame f;
  f.x = normalize(a);
  f.y = normalize(b);
  f.z = normalize(c);
  return f;
}
TR_HD Frame frame_from_z(f3 z) {
  f3 nz = normalize(z), ny;
  if (fabsf(nz.x) > fabsf(nz.y))
    ny = normalize(mk3(-nz.z, 0.0f, nz.x));
  else
    ny = normalize(mk3(0.0f, nz.z, -nz.y));
  return make_frame(cross(ny, nz), ny, nz);
}
TR_HD f3 to_local(const Frame& f, f3 v) { return mk3(dot(f.x, v), dot(f.y, v), dot(f.z, v)); }
TR_HD f3 to_global(const Frame& f, f3 v) { return scale(f.x, v.x) + scale(f.y, v.y) + scale(f.z, v.z); }
TR_HD bool pos_hemi(const Frame& f, f3 v) { return dot(v, f.z) > 0.0f; }

}  // namespace trg
