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

#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
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
              __half* __restrict__ acts, int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < (int)(kPackedBytes / 16); i += blockDim.x)
    reinterpret_cast<int4*>(sm)[i] = reinterpret_cast<const int4*>(img)[i];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kMbarOff);
  uint32_t* slot = reinterpret_cast<uint32_t*>(sm + kSlotOff);
  if (tid == 0) tc05::mbar_init(mbar, 1);
  if (warp == 0) tc05::tmem_alloc(slot, 64);
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
      for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        tc05::tmem_ld16(tmem + lane_base + (uint32_t)c0, v);
        if (l < kLayers - 1) {
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
        } else if (row < n) {
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (c0 + j < kOut) out[(size_t)row * kOut + c0 + j] = v[j] + bias[256 + c0 + j];
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
    tc05::tmem_relinquish();
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
  cudaError_t e;
  if ((e = g->params.reserve(mlp::kParams * 4)) != cudaSuccess || (e = g->img.reserve(mlp::kPackedBytes)) != cudaSuccess)
    return cuda_fail(ctx, e, "guide model allocation");
  if (!g->attr_set) {
    if ((e = cudaFuncSetAttribute(mlp::k_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, mlp::kSmemBytes)) !=
        cudaSuccess)
      return cuda_fail(ctx, e, "forward kernel shared memory");
    g->attr_set = true;
  }
  return TR_OK;
}

tr_status guide_pack(tr_ctx* ctx) {
  mlp::k_pack<<<(mlp::kPackThreads + 255) / 256, 256, 0, ctx->stream>>>(ctx->guide->params.as<float>(),
                                                                         ctx->guide->img.as<uint8_t>());
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "k_pack");
}

tr_status guide_forward(tr_ctx* ctx, const float* d_in, int n, float* d_out, __half* d_acts) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  const int tiles = (n + mlp::kTile - 1) / mlp::kTile;
  const int grid = std::max(1, std::min(tiles, sms));
  mlp::k_forward<<<grid, 128, mlp::kSmemBytes, ctx->stream>>>(ctx->guide->img.as<uint8_t>(), d_in, n, d_out, d_acts,
                                                              ctx->d_err.as<int>() + 2);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "k_forward");
}

void release_guide(tr_ctx* ctx) {
  if (!ctx->guide) return;
  GuideModel* g = ctx->guide;
  for (DevBuf* b : {&g->params, &g->img}) b->release();
  delete g;
  ctx->guide = nullptr;
}

}  // namespace trg

using namespace trg;

extern "C" {

tr_status tr_guide_init(tr_ctx* ctx, uint64_t seed) {
  if (!ctx) return TR_ERR_ARG;
  TR_CUDA(ctx, cudaSetDevice(ctx->device));
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
  TR_CUDA(ctx, cudaSetDevice(ctx->device));
  tr_status s = guide_reserve(ctx);
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->guide->params.p, params, n * 4, cudaMemcpyHostToDevice, ctx->stream));
  s = guide_pack(ctx);
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TR_OK;
}

tr_status tr_guide_get_params(tr_ctx* ctx, float* params, size_t n) {
  if (!ctx || !params || n != (size_t)mlp::kParams) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  TR_CUDA(ctx, cudaSetDevice(ctx->device));
  TR_CUDA(ctx, cudaMemcpyAsync(params, ctx->guide->params.p, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TR_OK;
}

tr_status tr_guide_forward_dev(tr_ctx* ctx, const float* d_in, size_t n, float* d_out) {
  if (!ctx || (n && (!d_in || !d_out))) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  if (n > (1u << 30)) return set_err(ctx, TR_ERR_ARG, "too many rows");
  if (n == 0) return TR_OK;
  TR_CUDA(ctx, cudaSetDevice(ctx->device));
  tr_status s = guide_forward(ctx, d_in, (int)n, d_out, nullptr);
  if (s != TR_OK) return s;
  int e = 0;
  TR_CUDA(ctx, cudaMemcpyAsync(&e, ctx->d_err.as<int>() + 2, 4, cudaMemcpyDeviceToHost, ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (e) {
    cudaMemsetAsync(ctx->d_err.as<int>() + 2, 0, 4, ctx->stream);
    return set_err(ctx, TR_ERR_TIMEOUT, "tensor-core MMA wait timed out");
  }
  return TR_OK;
}

}  // extern "C"
