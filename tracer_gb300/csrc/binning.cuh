// binning.cuh -- ray binning before traversal.
//
// A queue of rays is regrouped by a key: the direction's octant (most
// significant), then the Morton code of the origin's cell in a grid of
// 2^b x 2^b x 2^b cells over the root box of the ray's scene. A counting sort
// in three launches -- histogram of the keys, a one-block exclusive scan,
// scatter -- writes the queue's items in key order to a second array, which
// the persistent traversal kernels then read instead of the queue. A
// traversal's result depends only on its own ray, so the reordering changes
// no result; it only makes the 32 lanes of a warp walk alike paths (fewer
// idle lanes per instruction, node fetches shared across the warp).
//
// Within a bin the order follows the atomics (not fixed from run to run),
// which again affects nothing but timing.
//
// Src: unsigned count() const;             queue length (read on the device)
//      void ray(unsigned i, f3& o, f3& d, int& scene) const;
//      int item(unsigned i) const;          the queue entry written out
#pragma once

#include "scene_types.h"

namespace trg {

constexpr int kBinCountMax = 1 << (3 + 3 * kBinBitsMax);         // octant x cells
constexpr int kBinScanThreads = 1024;

// The low 10 bits of v spread to every third bit.
__device__ __forceinline__ unsigned int spread3(unsigned int v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

__device__ __forceinline__ unsigned int ray_bin_key(const DScene& sc, int scene, f3 o, f3 d, int bits) {
  const SceneRoot& R = sc.roots[scene];
  const float cells = (float)(1 << bits);
  const float oo[3] = {o.x, o.y, o.z};
  unsigned int c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float ext = R.hi[k] - R.lo[k];
    float u = ext > 0.0f ? (oo[k] - R.lo[k]) * (cells / ext) : 0.0f;
    u = fminf(fmaxf(u, 0.0f), cells - 1.0f);  // NaN (empty scene boxes) -> 0
    c[k] = (unsigned int)u;
  }
  const unsigned int oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
  return (oct << (3 * bits)) | (spread3(c[0]) << 2) | (spread3(c[1]) << 1) | spread3(c[2]);
}

// Histogram: keys[i] and cnt[key] += 1 (cnt zeroed by the caller).
template <class Src>
__global__ void __launch_bounds__(128) k_bin_count(Src src, const DScene sc, unsigned int* cnt, unsigned int* keys,
                                                   int bits) {
  const unsigned int n = src.count();
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    f3 o, d;
    int scene;
    src.ray(i, o, d, scene);
    const unsigned int key = ray_bin_key(sc, scene, o, d, bits);  // < 8 << 3 * bits
    keys[i] = key;
    // lanes with the same key add once
    const unsigned int active = __activemask();
    const unsigned int peers = __match_any_sync(active, key);
    if ((int)(threadIdx.x & 31u) == __ffs(peers) - 1) atomicAdd(cnt + key, (unsigned int)__popc(peers));
  }
}

// Exclusive scan of cnt[0 .. nb) in place, one block of kBinScanThreads.
static __global__ void __launch_bounds__(kBinScanThreads) k_bin_scan(unsigned int* cnt, int nb) {
  __shared__ unsigned int warp_sum[kBinScanThreads / 32];
  const int t = threadIdx.x;
  const int per = (nb + kBinScanThreads - 1) / kBinScanThreads;
  const int b0 = min(t * per, nb), b1 = min(b0 + per, nb);
  unsigned int s = 0;
  for (int b = b0; b < b1; ++b) s += cnt[b];
  // inclusive scan of the per-thread sums over the block
  const int lane = t & 31, warp = t >> 5;
  unsigned int x = s;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned int y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) warp_sum[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned int w = warp_sum[lane];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned int y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    warp_sum[lane] = w;
  }
  __syncthreads();
  unsigned int run = x - s + (warp > 0 ? warp_sum[warp - 1] : 0u);  // exclusive prefix of this thread's bins
  for (int b = b0; b < b1; ++b) {
    const unsigned int c = cnt[b];
    cnt[b] = run;
    run += c;
  }
}

// Scatter: out[cnt[key]++] = item (cnt holds the exclusive offsets).
template <class Src>
__global__ void __launch_bounds__(128) k_bin_scatter(Src src, unsigned int* cnt, const unsigned int* keys, int* out) {
  // The offsets were counted over the same n keys, so every position is
  // below n.
  const unsigned int n = src.count();
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned int key = keys[i];
    const unsigned int active = __activemask();
    const unsigned int peers = __match_any_sync(active, key);
    const int lane = (int)(threadIdx.x & 31u);
    const int leader = __ffs(peers) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(cnt + key, (unsigned int)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    out[base + (unsigned int)__popc(peers & ((1u << lane) - 1u))] = src.item(i);
  }
}

}  // namespace trg
