// selftest.cu -- device checks of the certified single-precision functions
// (exact32.cuh) and the slab-test scale (tr_math.cuh) against the double
// expressions they stand for, evaluated on the same device.

#include <cuda_runtime.h>

#include "context.h"
#include "exact32.cuh"
#include "shade.cuh"

namespace trg {

// splitmix64: a deterministic stream of test inputs per index
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// A float whose magnitude class depends on the draw: unit-scale values,
// wide exponents, exact zeros, small integers, and values near 1.
__device__ float test_float(unsigned long long& s) {
  s = mix64(s);
  const unsigned cls = (unsigned)(s & 15u);
  const unsigned bits = (unsigned)(s >> 32);
  const float u = (float)(bits >> 8) * 5.9604645e-08f * 2.0f - 1.0f;  // [-1, 1)
  switch (cls) {
    case 0:
      return 0.0f;
    case 1: {
      const int k = (int)((s >> 8) & 63u) - 32;  // 2^-32 .. 2^31
      return ldexpf(u, k);
    }
    case 2:
      return (float)((int)((s >> 8) & 15u) - 8);
    case 3:
      return 1.0f - fabsf(u) * 1e-6f;
    default:
      return u;
  }
}

__device__ f3 test_vec(unsigned long long& s) { return mk3(test_float(s), test_float(s), test_float(s)); }

__device__ __forceinline__ bool same(float a, float b) {
  return __float_as_uint(a) == __float_as_uint(b) || (a != a && b != b);
}

__global__ void k_selftest(int which, unsigned long long n, unsigned long long seed, unsigned long long* bad) {
  unsigned long long nb = 0;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    unsigned long long s = mix64(seed ^ (i * 0x632be59bd9b4e019ull));
    switch (which) {
      case 0: {  // slab scale, exhaustive over the 2^32 bit patterns when n = 2^32
        const float x = __uint_as_float((unsigned)i);
        float t = x;
        const float r = (float)((double)t * (1 + 0.0000001));
        if (!same(slab_scale(x), r)) ++nb;
        break;
      }
      case 1: {  // cross, including nearly parallel pairs
        f3 a = test_vec(s), b = test_vec(s);
        if ((s >> 60) == 0) b = a + scale(b, 1e-5f);
        const f3 c = cross_x(a, b), r = cross_d(a, b);
        if (!same(c.x, r.x) || !same(c.y, r.y) || !same(c.z, r.z)) ++nb;
        break;
      }
      case 2: {  // normalize, including already-normalised vectors
        f3 a = test_vec(s);
        if ((s >> 61) == 0) a = normalize_d(a);
        const f3 c = normalize_x(a), r = normalize_d(a);
        if (!same(c.x, r.x) || !same(c.y, r.y) || !same(c.z, r.z)) ++nb;
        break;
      }
      case 3: {  // cos
        const f3 a = test_vec(s), b = test_vec(s);
        if (!same(cos_x(a, b), cosv_d(a, b))) ++nb;
        break;
      }
      case 4: {  // Vector3 / float
        const f3 a = test_vec(s);
        const float f = test_float(s);
        const f3 c = div_x(a, f), r = divd(a, (double)f);
        if (!same(c.x, r.x) || !same(c.y, r.y) || !same(c.z, r.z)) ++nb;
        break;
      }
      case 5: {  // shadow-ray distance and its comparison with eps
        float L = fabsf(test_float(s));
        if ((s >> 62) == 0) L = 3.6e-7f * (1.0f + test_float(s) * 1e-3f);  // near (2 eps)^2
        bool le;
        const float d = dist_minus_eps(L, le);
        const double dd = sqrt((double)L) - (double)kEps;
        if (!same(d, (float)dd) || le != (dd <= (double)kEps)) ++nb;
        break;
      }
      case 6: {  // light sampling pdf
        const float A = fabsf(test_float(s)) + 1e-3f, d = test_float(s), L = fabsf(test_float(s));
        const float r = (float)((double)A / fabs((double)d / sqrt((double)L)));
        if (!same(area_to_solid_pdf(A, d, L), r)) ++nb;
        break;
      }
      case 7: {  // Disney Fd90 and the subsurface term
        const float L = test_float(s), rgh = fabsf(test_float(s)), Fss = test_float(s);
        const float S = fabsf(test_float(s)) + fabsf(test_float(s));
        const float f1 = (float)(0.5 + 2.0 * (double)L * (double)L * (double)rgh);
        const float f2 = (float)(1.25 * ((double)Fss * (1.0 / (double)S - 0.5) + 0.5));
        if (!same(disney_fd90(L, rgh), f1) || !same(disney_ss(Fss, S), f2)) ++nb;
        break;
      }
      default:
        break;
    }
  }
  if (nb) atomicAdd(bad, nb);
}

}  // namespace trg

using namespace trg;

extern "C" tr_status tr_selftest(tr_ctx* ctx, int which, uint64_t n, uint64_t seed, uint64_t* mismatches) {
  if (!ctx || !mismatches || which < 0 || which > 7) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  unsigned long long* d_bad = nullptr;
  cudaError_t e = cudaMalloc(&d_bad, sizeof(unsigned long long));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "selftest counter");
  cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), ctx->stream);
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
  k_selftest<<<sms * 8, 256, 0, ctx->stream>>>(which, (unsigned long long)n, (unsigned long long)seed, d_bad);
  e = cudaGetLastError();
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_bad, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_bad);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "selftest");
  *mismatches = h;
  return TR_OK;
}
