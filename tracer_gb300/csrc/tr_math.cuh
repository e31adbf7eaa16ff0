// tr_math.cuh -- vector arithmetic with the reference's exact float/double
// semantics, shared by host set-up code and device kernels.
//
// Every translation unit that includes this is compiled without multiply-add
// contraction (nvcc --fmad=false, host -ffp-contract=off), so each operator
// below is one IEEE operation, in the order the reference writes it:
//  * length_squared(): float sum left to right, widened to double
//    (src/utility/geometry.hpp:444-445);
//  * operator/(f): double reciprocal, double product, float result
//    (src/utility/geometry.hpp:429-433) -> normalize (:570-572);
//  * cross(): evaluated in double, rounded to float (:584-590);
//  * dot(): float, left to right (:866-884).
// The *_d functions evaluate the double expressions as written; kernels use
// the certified single-precision forms in exact32.cuh, which return the same
// floats and fall back to these.
#pragma once

#include <stdint.h>
#include <string.h>

#include <cmath>

#if defined(__CUDACC__)
#define TR_HD __host__ __device__ __forceinline__
#define TR_HD_COLD static __host__ __device__ inline
#else
#define TR_HD inline
#define TR_HD_COLD static inline
#endif

namespace trg {

constexpr float kEps = 3e-4f;  // common.hpp:47
// PI<float> and the constants derived from it in float (common.hpp:50-73)
constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 1.0f / kPi;
constexpr float kInv2Pi = 1.0f / (2.0f * kPi);
constexpr float kPiOver2 = kPi / 2.0f;
constexpr float kPiOver4 = kPi / 4.0f;
constexpr float kRealMax = 3.402823466e+38f;

struct f3 {
  float x, y, z;
};
TR_HD f3 mk3(float x, float y, float z) {
  f3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}
TR_HD f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
TR_HD f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
TR_HD f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
// Vector3<T>::operator*(float s): s * x in float
TR_HD f3 scale(f3 v, float s) { return mk3(s * v.x, s * v.y, s * v.z); }
TR_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
TR_HD float len2f(f3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
TR_HD double lengthd(f3 v) { return sqrt((double)len2f(v)); }
TR_HD_COLD f3 divd(f3 v, double f) {
  double inv = 1.0 / f;
  return mk3((float)(v.x * inv), (float)(v.y * inv), (float)(v.z * inv));
}
TR_HD_COLD f3 normalize_d(f3 v) { return divd(v, lengthd(v)); }
TR_HD_COLD f3 cross_d(f3 a, f3 b) {
  double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
  return mk3((float)((ay * bz) - (az * by)), (float)((az * bx) - (ax * bz)), (float)((ax * by) - (ay * bx)));
}
// cos(w1, w2) = dot / (len1 * len2) in double, returned as float (geometry.hpp:943-949)
TR_HD_COLD float cosv_d(f3 a, f3 b) { return (float)(dot(a, b) / (lengthd(a) * lengthd(b))); }
TR_HD bool all_zero(f3 v) { return !v.x && !v.y && !v.z; }

// std::min / std::max argument semantics
TR_HD float smin(float a, float b) { return (b < a) ? b : a; }
TR_HD float smax(float a, float b) { return (a < b) ? b : a; }

// Transform application (utility/transform.hpp:70-95), row-major 4x4
TR_HD f3 xform_point(const float* m, f3 p) {
  float x = p.x, y = p.y, z = p.z;
  float xp = m[0] * x + m[1] * y + m[2] * z + m[3];
  float yp = m[4] * x + m[5] * y + m[6] * z + m[7];
  float zp = m[8] * x + m[9] * y + m[10] * z + m[11];
  float wp = m[12] * x + m[13] * y + m[14] * z + m[15];
  if (wp == 1.0f) return mk3(xp, yp, zp);
  double inv = 1.0 / (double)wp;
  return mk3((float)(inv * xp), (float)(inv * yp), (float)(inv * zp));
}
TR_HD f3 xform_vec(const float* m, f3 v) {
  float x = v.x, y = v.y, z = v.z;
  return mk3(m[0] * x + m[1] * y + m[2] * z, m[4] * x + m[5] * y + m[6] * z, m[8] * x + m[9] * y + m[10] * z);
}
TR_HD f3 xform_normal_inv(const float* inv, f3 n) {
  float x = n.x, y = n.y, z = n.z;
  return mk3(inv[0] * x + inv[4] * y + inv[8] * z, inv[1] * x + inv[5] * y + inv[9] * z,
             inv[2] * x + inv[6] * y + inv[10] * z);
}

// The slab test's `tMax *= 1 + 0.0000001` (geometry.hpp:848,849,859) is
// float(double(x) * 1.0000001). For a finite non-zero x the result is x
// moved away from zero by 0, 1 or 2 units in the last place, as a function
// of x's significand m only: 2 for normal m >= 15000000 (except m = 2^24 - 1,
// whose sum crosses into the next binade, where one unit of the larger
// spacing wins), else 1; for subnormals 1 from m = 5000001 on, else 0.
// One correctly rounded fma(x, c, x) with c = float(1e-7) (slightly above
// 1e-7, below 1.5 / 14999999) adds m * c units and rounds to nearest: the
// same unit counts for every m except the subnormal tie m = 5000000, whose
// exact sum m + 0.5 rounds to even (m) in double but lies just above the
// tie here. Zero, inf and nan pass unchanged, and the largest finite values
// overflow to inf as the double expression does. Exhaustively checked
// against the double expression over all 2^32 inputs.
TR_HD float slab_scale(float x) {
#if defined(__CUDA_ARCH__)
  const float tie = __uint_as_float(5000000u);  // the subnormal 5000000 * 2^-149
#else
  const uint32_t tb = 5000000u;
  float tie;
  memcpy(&tie, &tb, 4);
#endif
  const float r = fmaf(x, 1e-7f, x);
  return fabsf(x) == tie ? x : r;
}

}  // namespace trg
