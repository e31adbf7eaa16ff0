// post.cu -- the output path on the device: Film::write_render_target
// (src/core/render.hpp:105-115), the ACES tone mapper and gamma corrector
// post-processors (src/post_processor/aces.cpp, src/post_processor/gamma.cpp),
// the demo driver's 8-bit image (src/main.hpp:171-178) and the RGBE bytes of
// a Radiance HDR file. One thread per channel value or pixel; HBM-bound
// elementwise passes over the image, launched on the context's stream.
#include <cuda_runtime.h>

#include "context.h"

namespace trg {
namespace post {

// sum / weight per channel where the weight is positive, else 0
__global__ void k_resolve(const float4* __restrict__ film, const double2* __restrict__ film64, size_t n,
                          float* __restrict__ rgb) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float r = 0.0f, g = 0.0f, b = 0.0f;
    if (film) {
      const float4 s = film[i];
      if (s.w > 0.0f) {
        r = s.x / s.w;
        g = s.y / s.w;
        b = s.z / s.w;
      }
    } else {
      const double2 a = film64[2 * i], c = film64[2 * i + 1];
      if (c.y > 0.0) {
        r = (float)(a.x / c.y);
        g = (float)(a.y / c.y);
        b = (float)(c.x / c.y);
      }
    }
    rgb[3 * i] = r;
    rgb[3 * i + 1] = g;
    rgb[3 * i + 2] = b;
  }
}

// clamp(x (2.51 x + 0.03) / (x (2.43 x + 0.59) + 0.14), 0, 1), x = c * exposure
// (std::clamp keeps a NaN)
__global__ void k_aces(float* __restrict__ v, size_t n, float exposure) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float x = v[i] * exposure;
    const float y = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
    v[i] = y < 0.0f ? 0.0f : (1.0f < y ? 1.0f : y);
  }
}

__global__ void k_gamma(float* __restrict__ v, size_t n, float gamma) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    v[i] = powf(v[i], gamma);
}

// clamp<int>(pow(c, inv_gamma) * 255, 0, 255); the float-to-int conversion
// truncates and saturates (NaN: 0)
__global__ void k_rgb8(const float* __restrict__ v, size_t n, float inv_gamma, uint8_t* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int iv = __float2int_rz(powf(v[i], inv_gamma) * 255.0f);
    out[i] = (uint8_t)(iv < 0 ? 0 : (iv > 255 ? 255 : iv));
  }
}

// Radiance RGBE (G. Ward, "Real Pixels", Graphics Gems II): the largest
// channel v = m 2^e (m in [0.5, 1)) gives the shared exponent e + 128, each
// channel floor(c m 256 / v); v < 1e-32 encodes as zeros
__global__ void k_rgbe(const float* __restrict__ rgb, size_t n, uchar4* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
    float v = r;
    if (g > v) v = g;
    if (b > v) v = b;
    if (!(v >= 1e-32f)) {
      out[i] = make_uchar4(0, 0, 0, 0);
      continue;
    }
    int e;
    const float m = frexpf(v, &e);
    const float s = m * 256.0f / v;
    const float c[3] = {r * s, g * s, b * s};
    uint8_t q[3];
    for (int k = 0; k < 3; ++k) q[k] = (uint8_t)(c[k] > 0.0f ? (c[k] < 255.0f ? (int)c[k] : 255) : 0);
    out[i] = make_uchar4(q[0], q[1], q[2], (uint8_t)(e + 128));
  }
}

int grid(const tr_ctx* ctx, size_t n) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const size_t want = (n + 255) / 256;
  const size_t cap = (size_t)(sms > 0 ? sms : 1) * 16;
  return (int)(want < cap ? (want ? want : 1) : cap);
}

bool aligned(const void* p, size_t a) { return ((uintptr_t)p & (a - 1)) == 0; }

}  // namespace post
}  // namespace trg

using namespace trg;

extern "C" tr_status tr_film_resolve_dev(tr_ctx* ctx, const float* d_rgbw, const double* d_rgbw64, size_t pixels,
                                         float* d_rgb) {
  if (!ctx || !d_rgb || ((d_rgbw == nullptr) == (d_rgbw64 == nullptr))) return TR_ERR_ARG;
  if (pixels == 0) return TR_OK;
  if (!post::aligned(d_rgbw ? (const void*)d_rgbw : (const void*)d_rgbw64, 16))
    return set_err(ctx, TR_ERR_ARG, "film buffer must be 16-byte aligned");
  TR_DEVICE_SCOPE(ctx);
  post::k_resolve<<<post::grid(ctx, pixels), 256, 0, ctx->stream>>>(
      reinterpret_cast<const float4*>(d_rgbw), reinterpret_cast<const double2*>(d_rgbw64), pixels, d_rgb);
  TR_CUDA(ctx, cudaGetLastError());
  return TR_OK;
}

extern "C" tr_status tr_aces_tone_map_dev(tr_ctx* ctx, float* d_rgb, size_t pixels, float exposure) {
  if (!ctx || (pixels && !d_rgb)) return TR_ERR_ARG;
  if (pixels == 0) return TR_OK;
  if (exposure < 0.0f) exposure = 1.0f;  // ACESToneMapper's constructor resets an invalid exposure
  TR_DEVICE_SCOPE(ctx);
  post::k_aces<<<post::grid(ctx, 3 * pixels), 256, 0, ctx->stream>>>(d_rgb, 3 * pixels, exposure);
  TR_CUDA(ctx, cudaGetLastError());
  return TR_OK;
}

extern "C" tr_status tr_gamma_correct_dev(tr_ctx* ctx, float* d_rgb, size_t pixels, float gamma) {
  if (!ctx || (pixels && !d_rgb)) return TR_ERR_ARG;
  if (pixels == 0) return TR_OK;
  if (!(gamma > 0.0f)) gamma = 1.0f;  // GammaCorrector's constructor resets an invalid gamma
  TR_DEVICE_SCOPE(ctx);
  post::k_gamma<<<post::grid(ctx, 3 * pixels), 256, 0, ctx->stream>>>(d_rgb, 3 * pixels, gamma);
  TR_CUDA(ctx, cudaGetLastError());
  return TR_OK;
}

extern "C" tr_status tr_to_rgb8_dev(tr_ctx* ctx, const float* d_rgb, size_t pixels, float inv_gamma,
                                    uint8_t* d_rgb8) {
  if (!ctx || (pixels && (!d_rgb || !d_rgb8))) return TR_ERR_ARG;
  if (pixels == 0) return TR_OK;
  TR_DEVICE_SCOPE(ctx);
  post::k_rgb8<<<post::grid(ctx, 3 * pixels), 256, 0, ctx->stream>>>(d_rgb, 3 * pixels, inv_gamma, d_rgb8);
  TR_CUDA(ctx, cudaGetLastError());
  return TR_OK;
}

extern "C" tr_status tr_to_rgbe_dev(tr_ctx* ctx, const float* d_rgb, size_t pixels, uint8_t* d_rgbe) {
  if (!ctx || (pixels && (!d_rgb || !d_rgbe))) return TR_ERR_ARG;
  if (pixels == 0) return TR_OK;
  if (!post::aligned(d_rgbe, 4)) return set_err(ctx, TR_ERR_ARG, "RGBE buffer must be 4-byte aligned");
  TR_DEVICE_SCOPE(ctx);
  post::k_rgbe<<<post::grid(ctx, pixels), 256, 0, ctx->stream>>>(d_rgb, pixels, reinterpret_cast<uchar4*>(d_rgbe));
  TR_CUDA(ctx, cudaGetLastError());
  return TR_OK;
}
