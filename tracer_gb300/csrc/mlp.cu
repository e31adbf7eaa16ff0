// mlp.cu -- the path-guiding network on Blackwell tensor cores.
//
// No reference counterpart: Tracer has no path guiding. The network maps a
// path vertex (position normalised to the scene box, outgoing direction,
// roughness: 7 inputs) through four hidden layers of 64 ReLU units to the 40
// parameters of an 8-lobe von Mises-Fisher mixture. Weights and activations
// are fp16, accumulation fp32 (tcgen05.mma kind::f16 into tensor memory).
//
// Forward kernel: persistent CTAs of 128 threads, one 128-row tile at a
// time. All weights live in shared memory in the core-matrix layout of
// tc05.cuh; a layer is K/16 MMAs (M = 128, N = 64 or 48) issued by one
// thread into a 64-column TMEM accumulator; the four warps read their 32
// rows back (tcgen05.ld), add the bias, apply ReLU and write fp16 into the
// next layer's A operand.

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <utility>
#include <cstring>
#include <vector>

#include "context.h"
#include "mixture.cuh"
#include "mlp.h"
#include "tc05.cuh"

namespace trg {
namespace mlp {

// shared-memory image: W0..W4 (fp16, core layout), biases (fp32)
__host__ __device__ constexpr uint32_t w_off(int l) {
  return l == 0 ? 0u : (l == 1 ? 2048u : (l == 2 ? 10240u : (l == 3 ? 18432u : 26624u)));
}
constexpr uint32_t kBiasOff = 32768;                        // 4 x 64 + 48 floats
constexpr uint32_t kPackedBytes = kBiasOff + 304 * 4;        // 33984
constexpr uint32_t kAOff = 34048;                            // 128 x 64 fp16
constexpr uint32_t kMbarOff = kAOff + kTile * kHid * 2;      // 50432
constexpr uint32_t kSlotOff = kMbarOff + 8;
constexpr uint32_t kSmemBytes = kSlotOff + 8;
static_assert(kPackedBytes % 16 == 0, "packed image is copied in 16-byte units");
static_assert(w_off(4) + kOutPad * kHid * 2 == kBiasOff, "weight image layout");

__host__ __device__ constexpr int layer_k(int l) { return l == 0 ? kInPad : kHid; }
__host__ __device__ constexpr int layer_n(int l) { return l == 4 ? kOutPad : kHid; }
__host__ __device__ constexpr int layer_kin(int l) { return l == 0 ? kIn : kHid; }
__host__ __device__ constexpr int layer_nout(int l) { return l == 4 ? kOut : kHid; }

// Offsets of W_l (nout x kin, row-major) and b_l in the flat fp32 parameter vector.
__host__ __device__ constexpr int param_w(int l) {
  return l == 0 ? 0 : (l == 1 ? 512 : (l == 2 ? 4672 : (l == 3 ? 8832 : 12992)));
}
__host__ __device__ constexpr int param_b(int l) { return param_w(l) + layer_nout(l) * layer_kin(l); }
static_assert(param_b(4) + kOut == kParams, "parameter layout");

// Writes the shared-memory image (fp16 weights in core layout, fp32 biases)
// from the fp32 parameters; one thread per image element.
__global__ void k_pack(const float* __restrict__ p, uint8_t* __restrict__ img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  // weights: element (n, k) of layer l
  int base = 0;
  for (int l = 0; l < kLayers; ++l) {
    const int N = layer_n(l), K = layer_k(l);
    if (i < base + N * K) {
      const int e = i - base, n = e / K, k = e % K;
      const float v = (n < layer_nout(l) && k < layer_kin(l)) ? p[param_w(l) + n * layer_kin(l) + k] : 0.0f;
      *reinterpret_cast<__half*>(img + w_off(l) + tc05::core_off(n, k, K)) = __float2half_rn(v);
      return;
    }
    base += N * K;
  }
  const int j = i - base;
  if (j < 304) {
    const int l = j < 256 ? j / 64 : 4, c = j < 256 ? j % 64 : j - 256;
    reinterpret_cast<float*>(img + kBiasOff)[j] = c < layer_nout(l) ? p[param_b(l) + c] : 0.0f;
  }
}
constexpr int kPackThreads = 64 * 16 + 3 * 64 * 64 + 48 * 64 + 304;  // W0, W1..W3, W4, biases

// x: n x 7 fp32; out: n x 40 fp32. With acts != null, the fp16 outputs of
// the four hidden layers are stored too (acts[l][row][64]) for training.
__global__ void __launch_bounds__(128, 1)
    k_forward(const uint8_t* __restrict__ img, const float* __restrict__ x, int n, float* __restrict__ out,
              __half* __restrict__ acts, int* err, const unsigned int* __restrict__ n_dev, int decode) {
  extern __shared__ __align__(1024) uint8_t sm[];
  if (n_dev) n = (int)*n_dev;  // row count produced on the device (guided rendering)
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < (int)(kPackedBytes / 16); i += blockDim.x)
    reinterpret_cast<int4*>(sm)[i] = reinterpret_cast<const int4*>(img)[i];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kMbarOff);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kSlotOff);
  if (tid == 0) tc05::mbar_init(mbar, 1);
  if (warp == 0) {
    tc05::tmem_alloc(slot, 64);
    tc05::tmem_relinquish();  // at once: the SM's other CTAs allocate their columns meanwhile
  }
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  const float* bias = reinterpret_cast<const float*>(sm + kBiasOff);
  uint8_t* A = sm + kAOff;
  const uint32_t a_addr = tc05::smem_u32(A);
  const uint32_t w_addr = tc05::smem_u32(sm);
  uint32_t phase = 0;
  bool ok = true;
  const int ntiles = (n + kTile - 1) / kTile;
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int row = t * kTile + tid;
    {  // inputs, zero-padded to 16
      __align__(16) __half h[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) h[j] = __float2half_rn(j < kIn && row < n ? x[(size_t)row * kIn + j] : 0.0f);
      *reinterpret_cast<int4*>(A + tc05::core_off(tid, 0, kInPad)) = *reinterpret_cast<const int4*>(h);
      *reinterpret_cast<int4*>(A + tc05::core_off(tid, 8, kInPad)) = *reinterpret_cast<const int4*>(h + 8);
    }
    tc05::fence_proxy_async();
    __syncthreads();
    for (int l = 0; l < kLayers && ok; ++l) {
      const int K = layer_k(l), N = layer_n(l);
      if (tid == 0) {
        tc05::fence_after();
        const uint32_t sbo = (uint32_t)(K / 8) * 128u;
        for (int kk = 0; kk < K / 16; ++kk)
          tc05::mma_f16(tmem, tc05::smem_desc(a_addr + kk * 256u, 128u, sbo),
                        tc05::smem_desc(w_addr + w_off(l) + kk * 256u, 128u, sbo),
                        tc05::idesc_f16_f32(128, (uint32_t)N), kk > 0 ? 1u : 0u);
        tc05::commit(mbar);
      }
      const bool got = tc05::mbar_wait(mbar, phase);
      ok = __syncthreads_and(got) != 0;
      if (!ok) break;
      phase ^= 1u;
      tc05::fence_after();
      if (l < kLayers - 1) {
        for (int c0 = 0; c0 < N; c0 += 16) {
          float v[16];
          tc05::tmem_ld16(tmem + lane_base + (uint32_t)c0, v);
          __align__(16) __half h[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) h[j] = __float2half_rn(fmaxf(v[j] + bias[l * 64 + c0 + j], 0.0f));
          *reinterpret_cast<int4*>(A + tc05::core_off(tid, c0, kHid)) = *reinterpret_cast<const int4*>(h);
          *reinterpret_cast<int4*>(A + tc05::core_off(tid, c0 + 8, kHid)) = *reinterpret_cast<const int4*>(h + 8);
          if (acts && row < n) {
            __half* dst = acts + ((size_t)l * n + row) * kHid + c0;
            *reinterpret_cast<int4*>(dst) = *reinterpret_cast<const int4*>(h);
            *reinterpret_cast<int4*>(dst + 8) = *reinterpret_cast<const int4*>(h + 8);
          }
        }
      } else {
        // the output row, whole in this thread: raw, or decoded into the
        // mixture's lobe parameters (guided rendering)
        float o[kOutPad];
#pragma unroll
        for (int c = 0; c < kOutPad / 16; ++c) {
          float v[16];
          tc05::tmem_ld16(tmem + lane_base + (uint32_t)(16 * c), v);
#pragma unroll
          for (int j = 0; j < 16; ++j) o[16 * c + j] = 16 * c + j < kOut ? v[j] + bias[256 + 16 * c + j] : 0.0f;
        }
        if (row < n) {
          if (decode) {
            float dd[kMixFloats];
            mixture_decode(o, dd);
            float4* dst = reinterpret_cast<float4*>(out + (size_t)row * kMixFloats);
#pragma unroll
            for (int q = 0; q < kMixFloats / 4; ++q)
              dst[q] = make_float4(dd[4 * q], dd[4 * q + 1], dd[4 * q + 2], dd[4 * q + 3]);
          } else {
#pragma unroll
            for (int j = 0; j < kOut; ++j) out[(size_t)row * kOut + j] = o[j];
          }
        }
      }
      tc05::fence_before();
      tc05::fence_proxy_async();
      __syncthreads();
    }
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
    tc05::mbar_wait(mbar, phase);  // the same phase, bounded: let an MMA still in flight finish
  }
  __syncthreads();
  if (warp == 0) {
    tc05::tmem_dealloc(tmem, 64);
  }
}

// ------------------------------------------------------------ backward
//
// For a 128-row tile and layer l = 4 .. 0, with in_l the layer's input
// (x for l = 0, h_{l-1} otherwise):
//   dW_l (+)= dZ_l^T in_l       M = 128 (rows of dZ^T: the layer's outputs,
//                                zero-padded), N = 16 or 80, K = 128 rows;
//                                in_l^T carries a row of ones after its
//                                inputs, so the same MMA yields db_l
//   dH     = dZ_l W_l           M = 128 rows, N = 64, K = 48 or 64
//   dZ_{l-1} = dH * (h_{l-1} > 0)
// dW accumulates in tensor memory over all tiles of the CTA and is added to
// the global gradient once at the end.

// transposed weights W_l^T (k_in x n_out, core layout, K = n_out padded) for l = 1..4
__host__ __device__ constexpr uint32_t wt_off(int l) { return (uint32_t)(l - 1) * 8192u; }
constexpr uint32_t kWtBytes = 3 * 8192 + 64 * 48 * 2;  // 30720
__host__ __device__ constexpr int bk_n(int l) { return l == 0 ? 16 : 80; }                 // dW MMA N
__host__ __device__ constexpr uint32_t bk_col(int l) { return l == 0 ? 64u : 80u + 80u * (uint32_t)(l - 1); }
constexpr uint32_t kBDz = kWtBytes;                   // dZ tile, 128 x 64 (K = 48 or 64)
constexpr uint32_t kBDzT = kBDz + 16384;              // dZ^T tile, 128 (outputs) x 128 (rows)
constexpr uint32_t kBInT = kBDzT + 32768;             // in^T tile, 80 x 128
constexpr uint32_t kBMbar = kBInT + 80 * 128 * 2;
constexpr uint32_t kBSlot = kBMbar + 8;
constexpr uint32_t kBSmemBytes = kBSlot + 8;

__global__ void k_pack_t(const float* __restrict__ p, uint8_t* __restrict__ img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;  // element (k, n) of W_l^T, l = 1..4
  int base = 0;
  for (int l = 1; l < kLayers; ++l) {
    const int KK = layer_n(l);  // MMA K of dH: the layer's outputs (48 or 64)
    if (i < base + 64 * KK) {
      const int e = i - base, k = e / KK, n = e % KK;
      const float v = n < layer_nout(l) ? p[param_w(l) + n * kHid + k] : 0.0f;
      *reinterpret_cast<__half*>(img + wt_off(l) + tc05::core_off(k, n, KK)) = __float2half_rn(v);
      return;
    }
    base += 64 * KK;
  }
}
constexpr int kPackTThreads = 3 * 64 * 64 + 64 * 48;

__device__ __forceinline__ void st_half(uint8_t* base, uint32_t off, float v) {
  *reinterpret_cast<__half*>(base + off) = __float2half_rn(v);
}

// x: n x 7, acts: 4 x n x 64 (fp16, forward outputs of the hidden layers),
// dout: n x 40 (gradient of the loss w.r.t. the network outputs).
// grads (fp32, parameter layout) += this CTA's share.
__global__ void __launch_bounds__(128, 1)
    k_backward(const uint8_t* __restrict__ wt_img, const float* __restrict__ x, const __half* __restrict__ acts,
               const float* __restrict__ dout, int n, float* __restrict__ grads, int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < (int)(kWtBytes / 16); i += blockDim.x)
    reinterpret_cast<int4*>(sm)[i] = reinterpret_cast<const int4*>(wt_img)[i];
  for (int i = tid; i < (int)((kBMbar - kBDz) / 16); i += blockDim.x)
    reinterpret_cast<int4*>(sm + kBDz)[i] = make_int4(0, 0, 0, 0);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kBMbar);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kBSlot);
  if (tid == 0) tc05::mbar_init(mbar, 1);
  if (warp == 0) {
    tc05::tmem_alloc(slot, 512);
    tc05::tmem_relinquish();
  }
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
  uint8_t* Dz = sm + kBDz;
  uint8_t* DzT = sm + kBDzT;
  uint8_t* InT = sm + kBInT;
  const uint32_t a_dz = tc05::smem_u32(Dz), a_dzt = tc05::smem_u32(DzT), a_int = tc05::smem_u32(InT),
                 a_wt = tc05::smem_u32(sm);
  uint32_t phase = 0;
  bool ok = true;
  int tiles_done = 0;
  const int ntiles = (n + kTile - 1) / kTile;
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int r = tid, g = t * kTile + tid;
    const bool live = g < n;
    // layer 4: dZ4 = dout, in_4 = h3
    float hin[64];  // in_l of the current layer (the ReLU mask of the next dZ)
    {
      float dz[48];
#pragma unroll
      for (int c = 0; c < 48; ++c) dz[c] = (live && c < kOut) ? dout[(size_t)g * kOut + c] : 0.0f;
#pragma unroll
      for (int c = 0; c < 48; ++c) st_half(Dz, tc05::core_off(r, c, 48), dz[c]);
#pragma unroll
      for (int c = 0; c < 64; ++c) st_half(DzT, tc05::core_off(c, r, 128), c < 48 ? dz[c] : 0.0f);
    }
#pragma unroll
    for (int k = 0; k < 64; ++k) hin[k] = live ? __half2float(acts[((size_t)3 * n + g) * kHid + k]) : 0.0f;
#pragma unroll
    for (int k = 0; k < 80; ++k)
      st_half(InT, tc05::core_off(k, r, 128), k < 64 ? hin[k] : (k == 64 && live ? 1.0f : 0.0f));
    for (int l = kLayers - 1; l >= 0 && ok; --l) {
      tc05::fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        tc05::fence_after();
        const uint32_t acc0 = tiles_done > 0 ? 1u : 0u;
        for (int kk = 0; kk < 8; ++kk)
          tc05::mma_f16(tmem + bk_col(l), tc05::smem_desc(a_dzt + kk * 256u, 128u, 2048u),
                        tc05::smem_desc(a_int + kk * 256u, 128u, 2048u), tc05::idesc_f16_f32(128, bk_n(l)),
                        (acc0 || kk > 0) ? 1u : 0u);
        if (l > 0) {
          const int KK = layer_n(l);
          const uint32_t sbo = (uint32_t)(KK / 8) * 128u;
          for (int kk = 0; kk < KK / 16; ++kk)
            tc05::mma_f16(tmem, tc05::smem_desc(a_dz + kk * 256u, 128u, sbo),
                          tc05::smem_desc(a_wt + wt_off(l) + kk * 256u, 128u, sbo), tc05::idesc_f16_f32(128, 64),
                          kk > 0 ? 1u : 0u);
        }
        tc05::commit(mbar);
      }
      const bool got = tc05::mbar_wait(mbar, phase);
      ok = __syncthreads_and(got) != 0;
      if (!ok) break;
      phase ^= 1u;
      if (l == 0) break;
      tc05::fence_after();
      // dZ_{l-1} = dH * (h_{l-1} > 0); h_{l-1} is this layer's input (hin)
      float dz[64];
#pragma unroll
      for (int c0 = 0; c0 < 64; c0 += 16) {
        float v[16];
        tc05::tmem_ld16(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) dz[c0 + j] = hin[c0 + j] > 0.0f ? v[j] : 0.0f;
      }
      tc05::fence_before();
#pragma unroll
      for (int c = 0; c < 64; ++c) st_half(Dz, tc05::core_off(r, c, 64), dz[c]);
#pragma unroll
      for (int c = 0; c < 64; ++c) st_half(DzT, tc05::core_off(c, r, 128), dz[c]);
      // the input of layer l-1
      if (l - 1 > 0) {
#pragma unroll
        for (int k = 0; k < 64; ++k)
          hin[k] = live ? __half2float(acts[((size_t)(l - 2) * n + g) * kHid + k]) : 0.0f;
#pragma unroll
        for (int k = 0; k < 80; ++k)
          st_half(InT, tc05::core_off(k, r, 128), k < 64 ? hin[k] : (k == 64 && live ? 1.0f : 0.0f));
      } else {
#pragma unroll
        for (int k = 0; k < 16; ++k)
          st_half(InT, tc05::core_off(k, r, 128),
                  k < kIn ? (live ? x[(size_t)g * kIn + k] : 0.0f) : (k == kIn && live ? 1.0f : 0.0f));
      }
    }
    ++tiles_done;
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
    tc05::mbar_wait(mbar, phase);
  }
  __syncthreads();
  tc05::fence_after();
  if (ok && tiles_done > 0 && warp < 2) {
    // rows (lanes) 0..63 of the dW accumulators: output unit `o` of each layer
    const int o = tid;
    for (int l = 0; l < kLayers; ++l) {
      const int N = bk_n(l), kin = layer_kin(l);
      for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        tc05::tmem_ld16(tmem + lane_base + bk_col(l) + (uint32_t)c0, v);
        if (o < layer_nout(l)) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int k = c0 + j;
            if (k < kin) atomicAdd(grads + param_w(l) + o * kin + k, v[j]);
            else if (k == kin) atomicAdd(grads + param_b(l) + o, v[j]);
          }
        }
      }
    }
  }
  tc05::fence_before();
  __syncthreads();
  if (warp == 0) {
    tc05::tmem_dealloc(tmem, 512);
  }
}

// ------------------------------------------------------------ loss, Adam
//
// Negative log-likelihood of the directions under the 8-lobe vMF mixture,
// weighted per row: loss = -sum_i w_i log p(omega_i | x_i) / sum_i w_i.
// Lobe j of row i: out[5j] weight logit, out[5j+1] log kappa (clamped to
// [TR_GUIDE_LOG_KAPPA_MIN, TR_GUIDE_LOG_KAPPA_MAX]), out[5j+2..4]
// unnormalised mean direction;
// vMF(omega) = kappa / (2 pi (1 - exp(-2 kappa))) exp(kappa (mu.omega - 1)).

struct Lobe {
  float pi, kappa, mlen, c;
  float3 mu;
};

__device__ __forceinline__ float vmf_log_norm(float kappa) {
  // log(kappa / (2 pi (1 - exp(-2 kappa))))
  return logf(kappa) - 1.8378770664093453f - log1pf(-expf(-2.0f * kappa));
}

// log p(omega | z) of one row, and d[0..39] = the gradient of -wi log p
// w.r.t. the row's 40 network outputs z.
__device__ __forceinline__ float row_nll_grad(const float* z, float3 om, float wi, float* d) {
  float a_max = -INFINITY;
  for (int j = 0; j < kLobes; ++j) a_max = fmaxf(a_max, z[5 * j]);
  float esum = 0.0f, lq[kLobes], pi[kLobes];
  for (int j = 0; j < kLobes; ++j) {
    pi[j] = expf(z[5 * j] - a_max);
    esum += pi[j];
  }
  float lmax = -INFINITY;
  Lobe L[kLobes];
  for (int j = 0; j < kLobes; ++j) {
    pi[j] /= esum;
    const float s = fminf(fmaxf(z[5 * j + 1], TR_GUIDE_LOG_KAPPA_MIN), TR_GUIDE_LOG_KAPPA_MAX);
    const float kappa = expf(s);
    const float3 m = make_float3(z[5 * j + 2], z[5 * j + 3], z[5 * j + 4]);
    const float mlen = sqrtf(m.x * m.x + m.y * m.y + m.z * m.z) + 1e-6f;
    const float3 mu = make_float3(m.x / mlen, m.y / mlen, m.z / mlen);
    const float c = mu.x * om.x + mu.y * om.y + mu.z * om.z;
    L[j] = Lobe{pi[j], kappa, mlen, c, mu};
    lq[j] = logf(fmaxf(pi[j], 1e-30f)) + vmf_log_norm(kappa) + kappa * (c - 1.0f);
    lmax = fmaxf(lmax, lq[j]);
  }
  float qs = 0.0f;
  for (int j = 0; j < kLobes; ++j) qs += expf(lq[j] - lmax);
  const float logp = lmax + logf(qs);
  for (int j = 0; j < kLobes; ++j) {
    const float q = expf(lq[j] - logp);  // responsibility
    const Lobe& b = L[j];
    d[5 * j] = -wi * (q - b.pi);
    const float s = z[5 * j + 1];
    const float e2 = expf(-2.0f * b.kappa);
    const float dlogk = 1.0f - 2.0f * b.kappa * e2 / fmaxf(-expm1f(-2.0f * b.kappa), 1e-30f) + b.kappa * (b.c - 1.0f);
    d[5 * j + 1] = (s > TR_GUIDE_LOG_KAPPA_MIN && s < TR_GUIDE_LOG_KAPPA_MAX) ? -wi * q * dlogk : 0.0f;
    const float f = -wi * q * b.kappa / b.mlen;
    d[5 * j + 2] = f * (om.x - b.c * b.mu.x);
    d[5 * j + 3] = f * (om.y - b.c * b.mu.y);
    d[5 * j + 4] = f * (om.z - b.c * b.mu.z);
  }
  return logp;
}

__global__ void k_loss(const float* __restrict__ out, const float* __restrict__ dir, const float* __restrict__ w,
                       int n, const float* __restrict__ wsum, float* __restrict__ dout, float* __restrict__ loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float li = 0.0f;
  if (i < n) {
    const float3 om = make_float3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    const float wi = w[i] / fmaxf(*wsum, 1e-30f);
    li = -wi * row_nll_grad(out + (size_t)i * kOut, om, wi, dout + (size_t)i * kOut);
  }
  // block sum of the loss
  for (int o = 16; o > 0; o >>= 1) li += __shfl_xor_sync(0xffffffffu, li, o);
  if ((threadIdx.x & 31) == 0 && li != 0.0f) atomicAdd(loss, li);
}

__global__ void k_sum(const float* __restrict__ w, int n, float* __restrict__ out) {
  float s = 0.0f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s += w[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, float lr, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float gi = g[i];
  const float mi = 0.9f * m[i] + 0.1f * gi;
  const float vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

// ------------------------------------------------------------ fused training step
//
// One Adam step on a batch is two launches: k_train and k_update.
//
// k_train does the batch's forward pass, loss and backward pass on the
// tensor cores. CTAs (one per SM, 256 threads, all 512 TMEM columns) walk
// 128-row tiles. A tile's rows are gathered from the record arrays; each
// layer's input is kept in shared memory twice, as the forward MMA's A
// operand and transposed (in_l^T) as the B operand of the weight-gradient
// MMA; the last layer's epilogue evaluates the loss and its gradient; the
// backward chain is the one of k_backward, with the ReLU masks held in
// registers. Weight gradients accumulate in TMEM over the CTA's tiles and are
// written once per CTA as a partial sum (no atomics).
//
// k_update sums the partials in a fixed order (the step is deterministic),
// takes the Adam step and writes the updated fp16 weights and fp32 biases
// into both packed images in place.
//
// Loss weighting: loss = sum_i -w_i log p_i / sum_i w_i. The rows carry
// s * w_i into the fp16 gradient chain, s = N / (64 W) for the weight sum W
// of N rows (the whole record set, or the batch), so the per-row values sit
// in fp16's normal range; k_update divides by s * sum_i w_i.

constexpr uint32_t kTWt = 34048;                           // transposed weights, kWtBytes
constexpr uint32_t kTA = kTWt + kWtBytes;                  // forward A operand / backward dZ (128 x 64)
constexpr uint32_t kTDzT = kTA + kTile * kHid * 2;         // dZ^T (128 x 128)
constexpr uint32_t kTIn = kTDzT + 128 * kTile * 2;         // in_l^T, l = 0..4
__host__ __device__ constexpr uint32_t tin_off(int l) {
  return l == 0 ? kTIn : kTIn + (uint32_t)kInPad * kTile * 2 + (uint32_t)(l - 1) * 80u * kTile * 2;
}
constexpr uint32_t kTRed = tin_off(4) + 80u * kTile * 2;   // block-reduction scratch
constexpr uint32_t kTMbar = kTRed + 64;
constexpr uint32_t kTSlot = kTMbar + 8;
constexpr uint32_t kTSmemBytes = kTSlot + 8;
static_assert(kPackedBytes <= kTWt && kTWt % 128 == 0 && kTA % 128 == 0 && kTIn % 128 == 0, "k_train layout");
static_assert(kTSmemBytes <= 227 * 1024, "k_train shared memory");
constexpr int kPartStride = kParams + 16;  // per-CTA partial: gradients, then weight sum and loss sum
constexpr int kWsumParts = 128;            // blocks of k_wsum
constexpr float kRowScale = 1.0f / 64.0f;
constexpr int kTrainThreads = 256;         // k_train: two warps per TMEM lane quarter
static_assert(kTRed + 8 * kTrainThreads / 32 <= kTMbar, "k_train reduction scratch");

// The batch's row i: a record index drawn by a hash of (seed, i).
__device__ __forceinline__ unsigned int batch_record(unsigned long long seed, unsigned int i, unsigned int count) {
  unsigned long long h = seed * 0x9E3779B97F4A7C15ull + i * 0xBF58476D1CE4E5B9ull + 0x94D049BB133111EBull;
  h ^= h >> 31;
  h *= 0xD6E8FEB86659FD93ull;
  h ^= h >> 32;
  return (unsigned int)(h % count);
}

// Per-block sums of w[0..n) in a fixed order (kWsumParts blocks of 256).
__global__ void k_wsum(const float* __restrict__ w, unsigned int n, float* __restrict__ parts) {
  __shared__ float red[256];
  float s = 0.0f;
  for (unsigned int i = blockIdx.x * 256u + threadIdx.x; i < n; i += kWsumParts * 256u) s += w[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) parts[blockIdx.x] = red[0];
}

// The row scale s = nrows / (64 W) from k_wsum's partial sums, in a fixed order.
__global__ void k_scale(const float* __restrict__ parts, float nrows, float* __restrict__ scale) {
  __shared__ float red[kWsumParts];
  red[threadIdx.x] = parts[threadIdx.x];
  __syncthreads();
  for (int o = kWsumParts / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *scale = nrows * kRowScale / fmaxf(red[0], 1e-30f);
}

__device__ __forceinline__ __half sat_half(float v) {
  return __float2half_rn(fminf(fmaxf(v, -65504.0f), 65504.0f));
}

// rec_in: count x 7, rec_dir: count x 3, rec_w: count. gather != 0: row i of
// the batch is record batch_record(seed, i, count); else record i.
// part: gridDim.x x kPartStride floats.
//
// Eight warps: warp w reads TMEM lanes 32 (w % 4) .. + 31, so threads t and
// t + 128 own the same tile row; in the epilogues of the hidden layers and of
// the backward chain each of the two takes half of the row's 64 columns
// (grp = w / 4). The loss epilogue, which needs a whole output row, runs on
// the first four warps.
__global__ void __launch_bounds__(kTrainThreads, 1)
    k_train(const uint8_t* __restrict__ img, const uint8_t* __restrict__ img_t, const float* __restrict__ rin,
            const float* __restrict__ rdir, const float* __restrict__ rw, unsigned int count, int n,
            unsigned long long seed, int gather, const float* __restrict__ scale, float* __restrict__ part,
            int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5;
  const int grp = warp >> 2;                         // column half of the epilogues
  const int r = ((warp & 3) << 5) | (tid & 31);      // this thread's tile row (TMEM lane)
  for (int i = tid; i < (int)(kPackedBytes / 16); i += blockDim.x)
    reinterpret_cast<int4*>(sm)[i] = reinterpret_cast<const int4*>(img)[i];
  for (int i = tid; i < (int)(kWtBytes / 16); i += blockDim.x)
    reinterpret_cast<int4*>(sm + kTWt)[i] = reinterpret_cast<const int4*>(img_t)[i];
  // operands start zero: padding rows and columns are never written again
  for (int i = tid; i < (int)((kTRed - kTA) / 16); i += blockDim.x)
    reinterpret_cast<int4*>(sm + kTA)[i] = make_int4(0, 0, 0, 0);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kTMbar);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kTSlot);
  if (tid == 0) tc05::mbar_init(mbar, 1);
  if (warp == 0) {
    tc05::tmem_alloc(slot, 512);
    tc05::tmem_relinquish();
  }
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
  const uint32_t tmem = *slot;
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
  const float* bias = reinterpret_cast<const float*>(sm + kBiasOff);
  uint8_t* A = sm + kTA;
  uint8_t* DzT = sm + kTDzT;
  const uint32_t w_addr = tc05::smem_u32(sm), wt_addr = tc05::smem_u32(sm + kTWt), a_addr = tc05::smem_u32(A),
                 dzt_addr = tc05::smem_u32(DzT);
  const float s = *scale;
  float w_acc = 0.0f, l_acc = 0.0f;
  uint32_t phase = 0;
  bool ok = true;
  int tiles_done = 0;
  const int ntiles = (n + kTile - 1) / kTile;
  for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const int i = t * kTile + r;
    const bool live = i < n;
    float x[kIn], om[3], w = 0.0f;
    {
      const unsigned int j = live ? (gather ? batch_record(seed, (unsigned int)i, count) : (unsigned int)i) : 0u;
#pragma unroll
      for (int k = 0; k < kIn; ++k) x[k] = live ? rin[(size_t)j * kIn + k] : 0.0f;
#pragma unroll
      for (int k = 0; k < 3; ++k) om[k] = live ? rdir[(size_t)j * 3 + k] : 0.0f;
      if (live) w = rw[j];
    }
    // layer 0's input: the A operand (zero-padded to 16; first four warps) and
    // in_0^T (ones row at 7 for the bias; last four)
    if (grp == 0) {
      __align__(16) __half h[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) h[k] = __float2half_rn(k < kIn ? x[k] : 0.0f);
      *reinterpret_cast<int4*>(A + tc05::core_off(r, 0, kInPad)) = *reinterpret_cast<const int4*>(h);
      *reinterpret_cast<int4*>(A + tc05::core_off(r, 8, kInPad)) = *reinterpret_cast<const int4*>(h + 8);
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k)
        st_half(sm + tin_off(0), tc05::core_off(k, r, kTile), k < kIn ? x[k] : (k == kIn && live ? 1.0f : 0.0f));
    }
    uint32_t mask[4];  // ReLU masks (h > 0 in fp16) of this thread's 32 hidden units per layer
    tc05::fence_proxy_async();
    __syncthreads();
    // ---- forward
    for (int l = 0; l < kLayers && ok; ++l) {
      const int K = layer_k(l), N = layer_n(l);
      if (tid == 0) {
        tc05::fence_after();
        const uint32_t sbo = (uint32_t)(K / 8) * 128u;
        for (int kk = 0; kk < K / 16; ++kk)
          tc05::mma_f16(tmem, tc05::smem_desc(a_addr + kk * 256u, 128u, sbo),
                        tc05::smem_desc(w_addr + w_off(l) + kk * 256u, 128u, sbo),
                        tc05::idesc_f16_f32(128, (uint32_t)N), kk > 0 ? 1u : 0u);
        tc05::commit(mbar);
      }
      const bool got = tc05::mbar_wait(mbar, phase);
      ok = __syncthreads_and(got) != 0;
      if (!ok) break;
      phase ^= 1u;
      tc05::fence_after();
      if (l < kLayers - 1) {
        uint8_t* inT = sm + tin_off(l + 1);
        uint32_t mk = 0u;
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
          const int c0 = 32 * grp + 16 * hf;
          float v[16];
          tc05::tmem_ld16(tmem + lane_base + (uint32_t)c0, v);
          __align__(16) __half h[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            h[j] = __float2half_rn(fmaxf(v[j] + bias[l * 64 + c0 + j], 0.0f));
            if (__half2float(h[j]) > 0.0f) mk |= 1u << (16 * hf + j);
            *reinterpret_cast<__half*>(inT + tc05::core_off(c0 + j, r, kTile)) = h[j];
          }
          *reinterpret_cast<int4*>(A + tc05::core_off(r, c0, kHid)) = *reinterpret_cast<const int4*>(h);
          *reinterpret_cast<int4*>(A + tc05::core_off(r, c0 + 8, kHid)) = *reinterpret_cast<const int4*>(h + 8);
        }
        mask[l] = mk;
        if (grp == 1) st_half(inT, tc05::core_off(kHid, r, kTile), live ? 1.0f : 0.0f);
      } else if (grp == 0) {
        // loss and its gradient w.r.t. the outputs: dZ_4 into dZ (K = 48) and dZ^T
        float z[kOutPad];
#pragma unroll
        for (int c = 0; c < kOutPad / 16; ++c) {
          float v[16];
          tc05::tmem_ld16(tmem + lane_base + (uint32_t)(16 * c), v);
#pragma unroll
          for (int j = 0; j < 16; ++j) z[16 * c + j] = 16 * c + j < kOut ? v[j] + bias[256 + 16 * c + j] : 0.0f;
        }
        float d[kOut];
        if (live) {
          const float logp = row_nll_grad(z, make_float3(om[0], om[1], om[2]), w * s, d);
          w_acc += w;
          l_acc -= w * logp;
        } else {
#pragma unroll
          for (int c = 0; c < kOut; ++c) d[c] = 0.0f;
        }
#pragma unroll
        for (int c = 0; c < kOutPad; ++c)
          *reinterpret_cast<__half*>(A + tc05::core_off(r, c, kOutPad)) = sat_half(c < kOut ? d[c] : 0.0f);
#pragma unroll
        for (int c = 0; c < kHid; ++c)
          *reinterpret_cast<__half*>(DzT + tc05::core_off(c, r, kTile)) = sat_half(c < kOut ? d[c] : 0.0f);
      }
      tc05::fence_before();
      tc05::fence_proxy_async();
      __syncthreads();
    }
    // ---- backward: dW_l (+)= dZ_l^T in_l, dH = dZ_l W_l, dZ_{l-1} = dH * mask
    for (int l = kLayers - 1; l >= 0 && ok; --l) {
      if (tid == 0) {
        tc05::fence_after();
        const uint32_t acc0 = tiles_done > 0 ? 1u : 0u;
        for (int kk = 0; kk < kTile / 16; ++kk)
          tc05::mma_f16(tmem + bk_col(l), tc05::smem_desc(dzt_addr + kk * 256u, 128u, 2048u),
                        tc05::smem_desc(tc05::smem_u32(sm + tin_off(l)) + kk * 256u, 128u, 2048u),
                        tc05::idesc_f16_f32(128, bk_n(l)), (acc0 || kk > 0) ? 1u : 0u);
        if (l > 0) {
          const int KK = layer_n(l);
          const uint32_t sbo = (uint32_t)(KK / 8) * 128u;
          for (int kk = 0; kk < KK / 16; ++kk)
            tc05::mma_f16(tmem, tc05::smem_desc(a_addr + kk * 256u, 128u, sbo),
                          tc05::smem_desc(wt_addr + wt_off(l) + kk * 256u, 128u, sbo), tc05::idesc_f16_f32(128, 64),
                          kk > 0 ? 1u : 0u);
        }
        tc05::commit(mbar);
      }
      const bool got = tc05::mbar_wait(mbar, phase);
      ok = __syncthreads_and(got) != 0;
      if (!ok) break;
      phase ^= 1u;
      if (l == 0) break;
      tc05::fence_after();
      const uint32_t mk = mask[l - 1];
#pragma unroll
      for (int hf = 0; hf < 2; ++hf) {
        const int c0 = 32 * grp + 16 * hf;
        float v[16];
        tc05::tmem_ld16(tmem + lane_base + (uint32_t)c0, v);
        __align__(16) __half h[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          h[j] = sat_half((mk >> (16 * hf + j)) & 1u ? v[j] : 0.0f);
          *reinterpret_cast<__half*>(DzT + tc05::core_off(c0 + j, r, kTile)) = h[j];
        }
        *reinterpret_cast<int4*>(A + tc05::core_off(r, c0, kHid)) = *reinterpret_cast<const int4*>(h);
        *reinterpret_cast<int4*>(A + tc05::core_off(r, c0 + 8, kHid)) = *reinterpret_cast<const int4*>(h + 8);
      }
      tc05::fence_before();
      tc05::fence_proxy_async();
      __syncthreads();
    }
    ++tiles_done;
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
    tc05::mbar_wait(mbar, phase);  // the same phase, bounded: let an MMA still in flight finish
  }
  __syncthreads();
  tc05::fence_after();
  // this CTA's partial: weight gradients from TMEM lanes 0..63 (one output
  // unit per lane; warps 0, 1, 4, 5), the two column halves' 16-column
  // chunks alternating
  float* mine = part + (size_t)blockIdx.x * kPartStride;
  if ((warp & 3) < 2) {
    const int o = r;
    for (int l = 0; l < kLayers; ++l) {
      const int N = bk_n(l), kin = layer_kin(l);
      for (int c0 = 16 * grp; c0 < N; c0 += 32) {
        float v[16];
        tc05::tmem_ld16(tmem + lane_base + bk_col(l) + (uint32_t)c0, v);
        if (o < layer_nout(l)) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int k = c0 + j;
            const float g = (ok && tiles_done > 0) ? v[j] : 0.0f;
            if (k < kin) mine[param_w(l) + o * kin + k] = g;
            else if (k == kin) mine[param_b(l) + o] = g;
          }
        }
      }
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    w_acc += __shfl_xor_sync(0xffffffffu, w_acc, off);
    l_acc += __shfl_xor_sync(0xffffffffu, l_acc, off);
  }
  float* red = reinterpret_cast<float*>(sm + kTRed);
  if ((tid & 31) == 0) {
    red[2 * warp] = w_acc;
    red[2 * warp + 1] = l_acc;
  }
  tc05::fence_before();
  __syncthreads();
  if (tid == 0) {
    float ws = 0.0f, ls = 0.0f;
    for (int k = 0; k < kTrainThreads / 32; ++k) {
      ws += red[2 * k];
      ls += red[2 * k + 1];
    }
    mine[kParams] = ws;
    mine[kParams + 1] = ls;
  }
  if (warp == 0) {
    tc05::tmem_dealloc(tmem, 512);
  }
}

// Sums the nparts partials (32 parameters x 8 partial slices per block),
// takes the Adam step, and writes the new weight (or bias) into the forward
// image and, for layers 1..4, the transposed image. loss_out (optional)
// receives the batch loss.
__global__ void __launch_bounds__(256)
    k_update(const float* __restrict__ part, int nparts, const float* __restrict__ scale,
             float* __restrict__ p, float* __restrict__ m, float* __restrict__ v, float lr, float c1, float c2,
             uint8_t* __restrict__ img, uint8_t* __restrict__ img_t, float* __restrict__ loss_out) {
  __shared__ float red[8][33];
  __shared__ float tot[8][2];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i = blockIdx.x * 32 + tx;
  float g = 0.0f, ws = 0.0f, ls = 0.0f;
  for (int c = ty; c < nparts; c += 8) {
    const float* pc = part + (size_t)c * kPartStride;
    if (i < kParams) g += pc[i];
    if (tx == 0) {
      ws += pc[kParams];
      ls += pc[kParams + 1];
    }
  }
  red[ty][tx] = g;
  if (tx == 0) {
    tot[ty][0] = ws;
    tot[ty][1] = ls;
  }
  __syncthreads();
  if (ty != 0 || i >= kParams) return;
  g = 0.0f;
  ws = 0.0f;
  ls = 0.0f;
#pragma unroll
  for (int y = 0; y < 8; ++y) {
    g += red[y][tx];
    ws += tot[y][0];
    ls += tot[y][1];
  }
  if (loss_out && i == 0) *loss_out = ls / fmaxf(ws, 1e-30f);
  const float denom = *scale * ws;
  g = denom > 1e-30f ? g / denom : 0.0f;
  const float mi = 0.9f * m[i] + 0.1f * g;
  const float vi = 0.999f * v[i] + 0.001f * g * g;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
  p[i] = pi;
  int l = kLayers - 1;
  while (l > 0 && i < param_w(l)) --l;
  const int kin = layer_kin(l), e = i - param_w(l);
  if (e < layer_nout(l) * kin) {
    const int o = e / kin, k = e % kin;
    *reinterpret_cast<__half*>(img + w_off(l) + tc05::core_off(o, k, layer_k(l))) = __float2half_rn(pi);
    if (l > 0) *reinterpret_cast<__half*>(img_t + wt_off(l) + tc05::core_off(k, o, layer_n(l))) = __float2half_rn(pi);
  } else {
    const int o = e - layer_nout(l) * kin;
    reinterpret_cast<float*>(img + kBiasOff)[l < kLayers - 1 ? l * 64 + o : 256 + o] = pi;
  }
}

}  // namespace mlp

// ------------------------------------------------------------------ host

namespace {

uint32_t pcg_next(uint64_t& s) {
  const uint64_t old = s;
  s = old * 6364136223846793005ull + 1442695040888963407ull;
  const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
  const uint32_t rot = (uint32_t)(old >> 59u);
  return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

}  // namespace

tr_status guide_reserve(tr_ctx* ctx) {
  if (!ctx->guide) ctx->guide = new GuideModel();
  GuideModel* g = ctx->guide;
  if (g->params.p) return TR_OK;
  cudaError_t e = cudaSuccess;
  for (auto pr : {std::make_pair(&g->params, (size_t)mlp::kParams * 4), std::make_pair(&g->img, (size_t)mlp::kPackedBytes),
                  std::make_pair(&g->img_t, (size_t)mlp::kWtBytes), std::make_pair(&g->grads, (size_t)mlp::kParams * 4),
                  std::make_pair(&g->adam_m, (size_t)mlp::kParams * 4),
                  std::make_pair(&g->adam_v, (size_t)mlp::kParams * 4),
                  std::make_pair(&g->scal, (size_t)(16 + mlp::kWsumParts) * 4)})
    if ((e = pr.first->reserve(pr.second)) != cudaSuccess) return cuda_fail(ctx, e, "guide model allocation");
  if (!g->attr_set) {
    if ((e = cudaFuncSetAttribute(mlp::k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::kSmemBytes)) !=
            cudaSuccess ||
        (e = cudaFuncSetAttribute(mlp::k_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::kBSmemBytes)) !=
            cudaSuccess ||
        (e = cudaFuncSetAttribute(mlp::k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::kTSmemBytes)) !=
            cudaSuccess)
      return cuda_fail(ctx, e, "guide kernels' shared memory");
    g->attr_set = true;
  }
  return TR_OK;
}

// Resets the Adam state (new parameters start a new optimisation).
static tr_status guide_reset_adam(tr_ctx* ctx) {
  GuideModel* g = ctx->guide;
  TR_CUDA(ctx, cudaMemsetAsync(g->adam_m.p, 0, mlp::kParams * 4, ctx->stream));
  TR_CUDA(ctx, cudaMemsetAsync(g->adam_v.p, 0, mlp::kParams * 4, ctx->stream));
  g->step = 0;
  return TR_OK;
}

tr_status guide_pack(tr_ctx* ctx) {
  GuideModel* g = ctx->guide;
  mlp::k_pack<<<(mlp::kPackThreads + 255) / 256, 256, 0, ctx->stream>>>(g->params.as<float>(), g->img.as<uint8_t>());
  mlp::k_pack_t<<<(mlp::kPackTThreads + 255) / 256, 256, 0, ctx->stream>>>(g->params.as<float>(),
                                                                            g->img_t.as<uint8_t>());
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "guide weight packing");
}

// Forward: up to four CTAs per SM (50 KB of shared memory and 64 TMEM
// columns each), so that one CTA's MMAs overlap another's epilogue.
// Backward: one per SM (each holds 512 TMEM columns, the whole SM's).
static int guide_grid(tr_ctx* ctx, int n, int per_sm) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const int tiles = (n + mlp::kTile - 1) / mlp::kTile;
  return std::max(1, std::min(tiles, sms * per_sm));
}

tr_status guide_forward(tr_ctx* ctx, const float* d_in, int n, float* d_out, __half* d_acts) {
  mlp::k_forward<<<guide_grid(ctx, n, 4), 128, mlp::kSmemBytes, ctx->stream>>>(
      ctx->guide->img.as<uint8_t>(), d_in, n, d_out, d_acts, ctx->d_err.as<int>() + 2, nullptr, 0);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "k_forward");
}

tr_status guide_forward_rows_on_device(tr_ctx* ctx, const float* d_in, const unsigned int* d_n, float* d_out) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  mlp::k_forward<<<std::max(sms, 1) * 4, 128, mlp::kSmemBytes, ctx->stream>>>(
      ctx->guide->img.as<uint8_t>(), d_in, 0, d_out, nullptr, ctx->d_err.as<int>() + 2, d_n, 1);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "k_forward");
}

// The row scale of a training pass or step (scal[2]) from the weights w[0..n).
static tr_status guide_scale(tr_ctx* ctx, const float* w, unsigned int n) {
  float* scal = ctx->guide->scal.as<float>();
  mlp::k_wsum<<<mlp::kWsumParts, 256, 0, ctx->stream>>>(w, n, scal + 16);
  mlp::k_scale<<<1, mlp::kWsumParts, 0, ctx->stream>>>(scal + 16, (float)n, scal + 2);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "guide weight sum");
}

// One Adam step on n rows (gather: drawn from `count` records by seed), two
// launches: k_train, k_update. The batch loss lands in *d_loss (device).
static tr_status guide_fused_step(tr_ctx* ctx, const float* in, const float* dir, const float* w, unsigned int count,
                                  int n, int gather, unsigned long long seed, float lr, float* d_loss) {
  GuideModel* g = ctx->guide;
  const int grid = guide_grid(ctx, n, 1);
  cudaError_t e;
  if ((e = g->part.reserve((size_t)grid * mlp::kPartStride * 4)) != cudaSuccess)
    return cuda_fail(ctx, e, "guide gradient partials");
  const float* scale = g->scal.as<float>() + 2;
  mlp::k_train<<<grid, mlp::kTrainThreads, mlp::kTSmemBytes, ctx->stream>>>(g->img.as<uint8_t>(), g->img_t.as<uint8_t>(), in, dir, w,
                                                              count, n, seed, gather, scale, g->part.as<float>(),
                                                              ctx->d_err.as<int>() + 2);
  ++g->step;
  const float c1 = 1.0f - std::pow(0.9f, (float)g->step), c2 = 1.0f - std::pow(0.999f, (float)g->step);
  mlp::k_update<<<(mlp::kParams + 31) / 32, dim3(32, 8), 0, ctx->stream>>>(
      g->part.as<float>(), grid, scale, g->params.as<float>(), g->adam_m.as<float>(), g->adam_v.as<float>(), lr, c1,
      c2, g->img.as<uint8_t>(), g->img_t.as<uint8_t>(), d_loss);
  e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "guide training step");
}

tr_status guide_train_on(tr_ctx* ctx, const float* rec_in, const float* rec_dir, const float* rec_w, unsigned int count,
                         int steps, unsigned int batch, float lr, unsigned long long seed, float* mean_loss) {
  GuideModel* g = ctx->guide;
  cudaError_t e;
  if ((e = g->losses.reserve((size_t)std::max(steps, 1) * 4)) != cudaSuccess)
    return cuda_fail(ctx, e, "training losses");
  tr_status st = guide_scale(ctx, rec_w, count);
  if (st != TR_OK) return st;
  for (int s = 0; s < steps; ++s) {
    st = guide_fused_step(ctx, rec_in, rec_dir, rec_w, count, (int)batch, 1, seed * 1000003ull + (unsigned long long)s,
                          lr, g->losses.as<float>() + s);
    if (st != TR_OK) return st;
  }
  std::vector<float> l((size_t)steps);
  if (steps)
    TR_CUDA(ctx, cudaMemcpyAsync(l.data(), g->losses.p, (size_t)steps * 4, cudaMemcpyDeviceToHost, ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double sum = 0.0;
  for (float v : l) sum += v;
  if (mean_loss) *mean_loss = steps ? (float)(sum / steps) : 0.0f;
  return TR_OK;
}

static tr_status guide_workspace(tr_ctx* ctx, int n) {
  GuideModel* g = ctx->guide;
  cudaError_t e;
  if ((e = g->acts.reserve((size_t)4 * n * mlp::kHid * 2)) != cudaSuccess ||
      (e = g->out.reserve((size_t)n * mlp::kOut * 4)) != cudaSuccess ||
      (e = g->dout.reserve((size_t)n * mlp::kOut * 4)) != cudaSuccess)
    return cuda_fail(ctx, e, "guide training workspace");
  return TR_OK;
}

tr_status guide_backward(tr_ctx* ctx, const float* d_in, const float* d_dout, int n, float* d_grads) {
  tr_status s = guide_workspace(ctx, n);
  if (s != TR_OK) return s;
  GuideModel* g = ctx->guide;
  s = guide_forward(ctx, d_in, n, g->out.as<float>(), g->acts.as<__half>());
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaMemsetAsync(d_grads, 0, mlp::kParams * 4, ctx->stream));
  mlp::k_backward<<<guide_grid(ctx, n, 1), 128, mlp::kBSmemBytes, ctx->stream>>>(
      g->img_t.as<uint8_t>(), d_in, g->acts.as<__half>(), d_dout, n, d_grads, ctx->d_err.as<int>() + 2);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "k_backward");
}

// Loss and its gradient w.r.t. the network outputs (g->dout) for a batch;
// the loss lands in scal[1].
static tr_status guide_loss(tr_ctx* ctx, const float* d_in, const float* d_dir, const float* d_w, int n) {
  tr_status s = guide_workspace(ctx, n);
  if (s != TR_OK) return s;
  GuideModel* g = ctx->guide;
  s = guide_forward(ctx, d_in, n, g->out.as<float>(), g->acts.as<__half>());
  if (s != TR_OK) return s;
  float* scal = g->scal.as<float>();
  TR_CUDA(ctx, cudaMemsetAsync(scal, 0, 8, ctx->stream));
  mlp::k_sum<<<64, 256, 0, ctx->stream>>>(d_w, n, scal);
  mlp::k_loss<<<(n + 255) / 256, 256, 0, ctx->stream>>>(g->out.as<float>(), d_dir, d_w, n, scal,
                                                         g->dout.as<float>(), scal + 1);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "k_loss");
}

tr_status guide_train_step(tr_ctx* ctx, const float* d_in, const float* d_dir, const float* d_w, int n, float lr) {
  tr_status s = guide_scale(ctx, d_w, (unsigned int)n);
  if (s != TR_OK) return s;
  return guide_fused_step(ctx, d_in, d_dir, d_w, (unsigned int)n, n, 0, 0ull, lr, ctx->guide->scal.as<float>() + 1);
}

// Synchronises and turns a timed-out tensor-core wait into an error.
static tr_status guide_check(tr_ctx* ctx) {
  int e = 0;
  TR_CUDA(ctx, cudaMemcpyAsync(&e, ctx->d_err.as<int>() + 2, 4, cudaMemcpyDeviceToHost, ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (e) {
    cudaMemsetAsync(ctx->d_err.as<int>() + 2, 0, 4, ctx->stream);
    return set_err(ctx, TR_ERR_TIMEOUT, "tensor-core MMA wait timed out");
  }
  return TR_OK;
}

void release_guide(tr_ctx* ctx) {
  if (!ctx->guide) return;
  GuideModel* g = ctx->guide;
  for (DevBuf* b : {&g->params, &g->img, &g->img_t, &g->grads, &g->adam_m, &g->adam_v, &g->acts, &g->out, &g->dout,
                    &g->scal, &g->part, &g->losses})
    b->release();
  delete g;
  ctx->guide = nullptr;
}

}  // namespace trg

using namespace trg;

extern "C" {

tr_status tr_guide_init(tr_ctx* ctx, uint64_t seed) {
  if (!ctx) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  tr_status s = guide_reserve(ctx);
  if (s != TR_OK) return s;
  // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) for weights and biases
  std::vector<float> p(mlp::kParams);
  uint64_t st = seed * 2 + 1;
  for (int l = 0; l < mlp::kLayers; ++l) {
    const float bound = 1.0f / std::sqrt((float)mlp::layer_kin(l));
    const int nw = mlp::layer_nout(l) * mlp::layer_kin(l);
    for (int i = 0; i < nw + mlp::layer_nout(l); ++i) {
      const float u = (float)(pcg_next(st) >> 8) * (1.0f / 16777216.0f);
      p[mlp::param_w(l) + i] = (2.0f * u - 1.0f) * bound;
    }
  }
  return tr_guide_set_params(ctx, p.data(), p.size());
}

tr_status tr_guide_set_params(tr_ctx* ctx, const float* params, size_t n) {
  if (!ctx || !params || n != (size_t)mlp::kParams) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  tr_status s = guide_reserve(ctx);
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->guide->params.p, params, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  s = guide_reset_adam(ctx);
  if (s != TR_OK) return s;
  s = guide_pack(ctx);
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TR_OK;
}

tr_status tr_guide_get_params(tr_ctx* ctx, float* params, size_t n) {
  if (!ctx || !params || n != (size_t)mlp::kParams) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  TR_DEVICE_SCOPE(ctx);
  TR_CUDA(ctx, cudaMemcpyAsync(params, ctx->guide->params.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TR_OK;
}

tr_status tr_guide_forward_dev(tr_ctx* ctx, const float* d_in, size_t n, float* d_out) {
  if (!ctx || (n && (!d_in || !d_out))) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  if (n > (1u << 30)) return set_err(ctx, TR_ERR_ARG, "too many rows");
  if (n == 0) return TR_OK;
  TR_DEVICE_SCOPE(ctx);
  tr_status s = guide_forward(ctx, d_in, (int)n, d_out, nullptr);
  return s != TR_OK ? s : guide_check(ctx);
}

tr_status tr_guide_backward_dev(tr_ctx* ctx, const float* d_in, const float* d_dout, size_t n, float* d_grads) {
  if (!ctx || !d_grads || (n && (!d_in || !d_dout))) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  if (n > (1u << 26)) return set_err(ctx, TR_ERR_ARG, "too many rows");
  TR_DEVICE_SCOPE(ctx);
  if (n == 0) {
    TR_CUDA(ctx, cudaMemsetAsync(d_grads, 0, mlp::kParams * 4, ctx->stream));
    return guide_check(ctx);
  }
  tr_status s = guide_backward(ctx, d_in, d_dout, (int)n, d_grads);
  return s != TR_OK ? s : guide_check(ctx);
}

tr_status tr_guide_loss_dev(tr_ctx* ctx, const float* d_in, const float* d_dir, const float* d_weight, size_t n,
                            float* d_dout, float* loss) {
  if (!ctx || !loss || !d_dout || n == 0 || !d_in || !d_dir || !d_weight) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  if (n > (1u << 26)) return set_err(ctx, TR_ERR_ARG, "too many rows");
  TR_DEVICE_SCOPE(ctx);
  tr_status s = guide_loss(ctx, d_in, d_dir, d_weight, (int)n);
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaMemcpyAsync(d_dout, ctx->guide->dout.p, n * mlp::kOut * 4, cudaMemcpyDeviceToDevice, ctx->stream));
  TR_CUDA(ctx, cudaMemcpyAsync(loss, ctx->guide->scal.as<float>() + 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
  return guide_check(ctx);
}

tr_status tr_guide_train_step_dev(tr_ctx* ctx, const float* d_in, const float* d_dir, const float* d_weight,
                                  size_t n, float lr, float* loss) {
  if (!ctx || n == 0 || !d_in || !d_dir || !d_weight || !(lr > 0.0f)) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  if (n > (1u << 26)) return set_err(ctx, TR_ERR_ARG, "too many rows");
  TR_DEVICE_SCOPE(ctx);
  tr_status s = guide_train_step(ctx, d_in, d_dir, d_weight, (int)n, lr);
  if (s != TR_OK) return s;
  float l = 0.0f;
  TR_CUDA(ctx, cudaMemcpyAsync(&l, ctx->guide->scal.as<float>() + 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
  s = guide_check(ctx);
  if (loss) *loss = l;
  return s;
}

}  // extern "C"
