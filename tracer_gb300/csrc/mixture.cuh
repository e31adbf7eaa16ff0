// mixture.cuh -- the guiding network's 8-lobe von Mises-Fisher mixture.
//
// The network's 40 outputs per vertex (lobe j: weight logit, log kappa,
// unnormalised mean direction) are decoded once, in the epilogue of the
// forward pass that guided rendering runs, into 48 floats laid out lobe-
// major for vector loads:
//   pi[8]     lobe weights (softmax of the logits)
//   c[8]      pi * kappa / (2 pi (1 - exp(-2 kappa))), the density scale
//   kappa[8]  concentrations, exp of the clamped log kappa
//   mu x[8], y[8], z[8]   unit mean directions
// so that the density at a direction (evaluated per light sample) costs 8
// exponentials, and sampling needs no decoding.
#pragma once

#include <math.h>

#include "tr_math.cuh"
#include "tracer_gpu.h"

namespace trg {

constexpr int kMixLobes = 8;
constexpr int kMixFloats = 48;

// z: one row of 40 network outputs; d: its 48 decoded floats.
__device__ __forceinline__ void mixture_decode(const float (&z)[48], float (&d)[48]) {
  float amax = -INFINITY;
#pragma unroll
  for (int j = 0; j < kMixLobes; ++j) amax = fmaxf(amax, z[5 * j]);
  float sum = 0.0f;
#pragma unroll
  for (int j = 0; j < kMixLobes; ++j) {
    d[j] = expf(z[5 * j] - amax);
    sum += d[j];
  }
#pragma unroll
  for (int j = 0; j < kMixLobes; ++j) {
    const float pi = d[j] / sum;
    const float kappa = expf(fminf(fmaxf(z[5 * j + 1], TR_GUIDE_LOG_KAPPA_MIN), TR_GUIDE_LOG_KAPPA_MAX));
    const float norm = kappa / (6.283185307179586f * -expm1f(-2.0f * kappa));
    const float mx = z[5 * j + 2], my = z[5 * j + 3], mz = z[5 * j + 4];
    const float len = sqrtf(mx * mx + my * my + mz * mz) + 1e-6f;
    d[j] = pi;
    d[8 + j] = pi * norm;
    d[16 + j] = kappa;
    d[24 + j] = mx / len;
    d[32 + j] = my / len;
    d[40 + j] = mz / len;
  }
}

// A decoded row in global memory (16-byte aligned).
struct Mixture {
  const float* __restrict__ d;

  // The hardware exponential (relative error about 1e-6, the arguments are
  // <= 0): the density enters only MIS weights and the guided estimate's
  // denominator, evaluated the same way for every strategy.
  __device__ float pdf(f3 w) const {
    const float4* q = reinterpret_cast<const float4*>(d);
    float p = 0.0f;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float4 c = q[2 + h], k = q[4 + h], x = q[6 + h], y = q[8 + h], z = q[10 + h];
      p += c.x * __expf(k.x * (x.x * w.x + y.x * w.y + z.x * w.z - 1.0f));
      p += c.y * __expf(k.y * (x.y * w.x + y.y * w.y + z.y * w.z - 1.0f));
      p += c.z * __expf(k.z * (x.z * w.x + y.z * w.y + z.z * w.z - 1.0f));
      p += c.w * __expf(k.w * (x.w * w.x + y.w * w.y + z.w * w.z - 1.0f));
    }
    return p;
  }

  // Lobe by u_lobe, then the numerically stable vMF sampling of W. Jakob,
  // "Numerically stable sampling of the von Mises-Fisher distribution on
  // S^2" (2012), in the frame of the lobe's mean (Duff et al. 2017 basis).
  __device__ f3 sample(float u_lobe, float u1, float u2) const {
    int j = 0;
    float c = d[0];
    while (j < kMixLobes - 1 && u_lobe >= c) c += d[++j];
    const float k = d[16 + j];
    float w = 1.0f + logf(u1 + (1.0f - u1) * expf(-2.0f * k)) / k;
    w = fminf(fmaxf(w, -1.0f), 1.0f);
    const float r = sqrtf(fmaxf(0.0f, 1.0f - w * w));
    float sp, cp;
    sincosf(6.283185307179586f * u2, &sp, &cp);
    const f3 n = mk3(d[24 + j], d[32 + j], d[40 + j]);
    const float sgn = copysignf(1.0f, n.z);
    const float a = -1.0f / (sgn + n.z);
    const float b = n.x * n.y * a;
    const f3 b1 = mk3(1.0f + sgn * n.x * n.x * a, sgn * b, -sgn * n.x);
    const f3 b2 = mk3(b, sgn + n.y * n.y * a, -n.y);
    return scale(b1, r * cp) + scale(b2, r * sp) + scale(n, w);
  }
};

}  // namespace trg
