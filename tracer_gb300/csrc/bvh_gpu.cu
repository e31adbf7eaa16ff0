// bvh_gpu.cu -- BVH construction on the device (TR_BVH_DEVICE): Parallel
// Locally-Ordered Clustering (D. Meister and J. Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction",
// IEEE TVCG 2018), the fast alternative to the host build of the
// reference's binned-SAH tree (src/accelerator/bvh.cpp:191-306).
//
// Per scene of an uploaded set:
//   1. bounds of the primitive centroids (block reduction);
//   2. a 63-bit Morton code per centroid (21 bits per axis), primitives
//      sorted by it (the radix sort of the CUDA toolkit's CUB);
//   3. clusters = the sorted primitives (one leaf each); repeatedly every
//      cluster finds, within `kRadius` positions of the cluster array, the
//      one whose merged box has the least surface area (ties broken by the
//      pair's positions: a strict total order, so the best pair of the
//      whole array is mutual and every round merges at least once), mutual
//      nearest neighbours merge into a new node, and the array is compacted
//      in order (prefix sums, so node numbering is deterministic);
//   4. every node made also gets its primitive count, and a node with at
//      most the scene's max_leaf_prims primitives becomes a leaf (the
//      reference's leaf rule, bvh.cpp:268-280);
//   5. slot offsets top-down (round by round from the root: a left child
//      starts at its parent's offset, a right child after the left's
//      primitives), so every leaf's primitives are contiguous slots;
//   6. the tree is written as the traversal's child-pair DNodes: a node's
//      children are ordered along the axis of largest separation of their
//      box centres (that axis picks the near child at traversal time), and
//      the slots are gathered in leaf order.
// The tree differs from the reference's, so closest hits can differ where
// two primitives are hit at the same distance and where the reference's
// slab test culls a box it touches (images are compared, not hits: the
// fast mode is for uploads where the host build would dominate).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"
#include "traverse.cuh"

namespace trg {
namespace ploc {

constexpr int kRadius = 16;
constexpr int kMaxRounds = 4096;  // a bound on the merging rounds (each merges at least one pair)

__device__ __forceinline__ float half_area(float4 lo, float4 hi) {
  const float x = hi.x - lo.x, y = hi.y - lo.y, z = hi.z - lo.z;
  return x * y + y * z + z * x;
}

// Centroid bounds: per-block minima and maxima, then one block over those.
__global__ void k_centroid_bounds(const float* __restrict__ lo, const float* __restrict__ hi, int n,
                                  float* __restrict__ part) {
  __shared__ float s[6][256];
  float m[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int c = 0; c < 3; ++c) {
      const float v = 0.5f * (lo[3 * i + c] + hi[3 * i + c]);
      m[c] = fminf(m[c], v);
      m[3 + c] = fmaxf(m[3 + c], v);
    }
  for (int c = 0; c < 6; ++c) s[c][threadIdx.x] = m[c];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w)
      for (int c = 0; c < 6; ++c)
        s[c][threadIdx.x] = c < 3 ? fminf(s[c][threadIdx.x], s[c][threadIdx.x + w])
                                  : fmaxf(s[c][threadIdx.x], s[c][threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int c = 0; c < 6; ++c) part[6 * blockIdx.x + c] = s[c][0];
}

__global__ void k_centroid_bounds_final(const float* __restrict__ part, int nparts, float* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float m[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int b = 0; b < nparts; ++b)
    for (int c = 0; c < 6; ++c) m[c] = c < 3 ? fminf(m[c], part[6 * b + c]) : fmaxf(m[c], part[6 * b + c]);
  for (int c = 0; c < 6; ++c) out[c] = m[c];
}

__device__ __forceinline__ unsigned long long spread21(unsigned int v) {
  unsigned long long x = v & 0x1fffffu;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

__global__ void k_morton(const float* __restrict__ lo, const float* __restrict__ hi, int n,
                         const float* __restrict__ cb, unsigned long long* __restrict__ keys,
                         unsigned int* __restrict__ vals) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned int q[3];
  for (int c = 0; c < 3; ++c) {
    const float ext = cb[3 + c] - cb[c];
    const float v = 0.5f * (lo[3 * i + c] + hi[3 * i + c]);
    const float t = ext > 0.0f ? (v - cb[c]) / ext : 0.5f;
    q[c] = (unsigned int)fminf(fmaxf(t * 2097152.0f, 0.0f), 2097151.0f);
  }
  keys[i] = spread21(q[0]) << 2 | spread21(q[1]) << 1 | spread21(q[2]);
  vals[i] = (unsigned int)i;
}

// Leaves: node id i is the i-th primitive in Morton order.
// Per node: box (blo, bhi), children, primitive count, whether it is a leaf
// of the final tree, its height in that tree and its first slot (off).
struct Nodes {
  float4 *blo, *bhi;
  int *left, *right, *height, *cnt, *leaf, *off;
};

__global__ void k_leaves(const unsigned int* __restrict__ order, const float* __restrict__ lo,
                         const float* __restrict__ hi, int n, Nodes t, int* __restrict__ clusters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned int p = order[i];
  t.blo[i] = make_float4(lo[3 * p], lo[3 * p + 1], lo[3 * p + 2], 0.0f);
  t.bhi[i] = make_float4(hi[3 * p], hi[3 * p + 1], hi[3 * p + 2], 0.0f);
  t.height[i] = 0;
  t.cnt[i] = 1;
  t.leaf[i] = 1;
  clusters[i] = i;
}

// Nearest neighbour of every cluster within the window, by the surface area
// of the merged box; ties by the pair (min position, max position).
__global__ void k_nearest(const int* __restrict__ C, int n, const float4* __restrict__ blo,
                          const float4* __restrict__ bhi, int* __restrict__ nn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 al = blo[C[i]], ah = bhi[C[i]];
  int best = -1;
  float bd = INFINITY;
  const int j0 = max(0, i - kRadius), j1 = min(n - 1, i + kRadius);
  for (int j = j0; j <= j1; ++j) {
    if (j == i) continue;
    const float4 bl = blo[C[j]], bh = bhi[C[j]];
    const float4 ul = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
    const float4 uh = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
    const float d = half_area(ul, uh);
    // j ascends, and so does the pair (min(i, j), max(i, j)): (j, i) for
    // j < i, then (i, j); keeping the first least d keeps the least pair
    if (d < bd) {
      bd = d;
      best = j;
    }
  }
  nn[i] = best;
}

__global__ void k_merge_flags(const int* __restrict__ nn, int n, int* __restrict__ create, int* __restrict__ keep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = nn[i];
  const bool mutual = j >= 0 && nn[j] == i;
  create[i] = mutual && i < j;
  keep[i] = !(mutual && i > j);
}

__global__ void k_merge_apply(const int* __restrict__ C, const int* __restrict__ nn, int n,
                              const int* __restrict__ create, const int* __restrict__ cid,
                              const int* __restrict__ keep, const int* __restrict__ kid, int next_id, int max_leaf,
                              Nodes t, int* __restrict__ Cout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  int id = C[i];
  if (create[i]) {
    const int a = C[i], b = C[nn[i]];
    id = next_id + cid[i];
    const float4 al = t.blo[a], ah = t.bhi[a], bl = t.blo[b], bh = t.bhi[b];
    const float4 lo = make_float4(fminf(al.x, bl.x), fminf(al.y, bl.y), fminf(al.z, bl.z), 0.0f);
    const float4 hi = make_float4(fmaxf(ah.x, bh.x), fmaxf(ah.y, bh.y), fmaxf(ah.z, bh.z), 0.0f);
    t.blo[id] = lo;
    t.bhi[id] = hi;
    t.left[id] = a;
    t.right[id] = b;
    const int c = t.cnt[a] + t.cnt[b];
    const bool leaf = c <= max_leaf;
    t.cnt[id] = c;
    t.leaf[id] = leaf ? 1 : 0;
    t.height[id] = leaf ? 0 : 1 + max(t.height[a], t.height[b]);
  }
  Cout[kid[i]] = id;
}

// Slot offsets of the children of the nodes made in one round.
__global__ void k_offsets(int id0, int id1, Nodes t) {
  const int id = id0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= id1) return;
  const int a = t.left[id], b = t.right[id], o = t.off[id];
  t.off[a] = o;
  t.off[b] = o + t.cnt[a];
}

// Internal node N + k as DNode node_off + k (nodes inside a leaf are
// written too, and never referenced).
__global__ void k_emit(int N, Nodes t, int node_off, int slot_off, DNode* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= N - 1) return;
  const int id = N + k;
  int a = t.left[id], b = t.right[id];
  float4 al = t.blo[a], ah = t.bhi[a], bl = t.blo[b], bh = t.bhi[b];
  const float d[3] = {(bl.x + bh.x) - (al.x + ah.x), (bl.y + bh.y) - (al.y + ah.y), (bl.z + bh.z) - (al.z + ah.z)};
  int axis = 0;
  if (fabsf(d[1]) > fabsf(d[axis])) axis = 1;
  if (fabsf(d[2]) > fabsf(d[axis])) axis = 2;
  if (d[axis] < 0.0f) {  // first child lower along the axis
    const int t = a;
    a = b;
    b = t;
    const float4 tl = al, th = ah;
    al = bl;
    ah = bh;
    bl = tl;
    bh = th;
  }
  DNode n;
  n.a = make_float4(al.x, al.y, al.z, ah.x);
  n.b = make_float4(ah.y, ah.z, bl.x, bl.y);
  n.c = make_float4(bl.z, bh.x, bh.y, bh.z);
  const bool la = t.leaf[a], lb = t.leaf[b];
  const int aref = la ? slot_off + t.off[a] : node_off + (a - N), bref = lb ? slot_off + t.off[b] : node_off + (b - N);
  const unsigned int acnt = la ? (unsigned int)t.cnt[a] : 0u, bcnt = lb ? (unsigned int)t.cnt[b] : 0u;
  n.d = make_int4(aref, bref, (int)(acnt | bcnt << 16), axis);
  out[node_off + k] = n;
}

// Slots in tree order: the primitive of leaf node i (order[i] of the
// scene) goes to slot slot_off + off[i].
__global__ void k_gather_slots(const float4* __restrict__ src, const unsigned int* __restrict__ order, int n,
                               const int* __restrict__ off, int prim_off, int slot_off, float4* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t s = (size_t)(prim_off + (int)order[i]), d = (size_t)slot_off + (size_t)off[i];
  for (int c = 0; c < 3; ++c) dst[3 * d + c] = src[3 * s + c];
}

}  // namespace ploc

namespace {

int blocks(int n, int t) { return (n + t - 1) / t; }

}  // namespace

// Builds every scene's tree on the device and uploads the scene set
// (TR_BVH_DEVICE). hs holds the primitive bounds instead of a host tree.
tr_status upload_device_built(tr_ctx* ctx) {
  HostScene& hs = ctx->hs;
  const size_t np = hs.prims.size(), nsc = hs.scene_prim.size();
  if (hs.blo.size() != 3 * np || hs.bhi.size() != 3 * np) return set_err(ctx, TR_ERR_STATE, "missing primitive bounds");
  if (np >= (1u << 26)) return set_err(ctx, TR_ERR_UNSUPPORTED, "more than 2^26 primitives in one upload");
  auto put = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t e = b.reserve(bytes ? bytes : 16);
    if (e != cudaSuccess) return e;
    if (bytes) return cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    return cudaSuccess;
  };
  // unordered slots (primitive order), bounds
  std::vector<float4> src(3 * np);
  for (size_t p = 0; p < np; ++p) {
    const DPrim& pr = hs.prims[p];
    if (pr.kind == PRIM_TRIANGLE) {
      const f3 A = hs.A[pr.shape], AB = hs.AB[pr.shape], AC = hs.AC[pr.shape];
      int idv = (int)p, neg = -1;
      float fid, fneg;
      std::memcpy(&fid, &idv, 4);
      std::memcpy(&fneg, &neg, 4);
      src[3 * p] = float4{A.x, A.y, A.z, fid};
      src[3 * p + 1] = float4{AB.x, AB.y, AB.z, fneg};
      src[3 * p + 2] = float4{AC.x, AC.y, AC.z, 0.0f};
    } else {
      int idv = (int)p, sv = pr.shape;
      float fid, fs;
      std::memcpy(&fid, &idv, 4);
      std::memcpy(&fs, &sv, 4);
      src[3 * p] = float4{0.0f, 0.0f, 0.0f, fid};
      src[3 * p + 1] = float4{0.0f, 0.0f, 0.0f, fs};
      src[3 * p + 2] = float4{0.0f, 0.0f, 0.0f, 0.0f};
    }
  }
  DevBuf d_src, d_lo, d_hi, scratch;
  struct Release {
    DevBuf *a, *b, *c, *d;
    ~Release() {
      a->release();
      b->release();
      c->release();
      d->release();
    }
  } release{&d_src, &d_lo, &d_hi, &scratch};
  TR_CUDA(ctx, put(d_src, src.data(), src.size() * sizeof(float4)));
  TR_CUDA(ctx, put(d_lo, hs.blo.data(), hs.blo.size() * 4));
  TR_CUDA(ctx, put(d_hi, hs.bhi.data(), hs.bhi.size() * 4));
  src.clear();
  src.shrink_to_fit();

  // per-scene sizes and offsets: scene k owns primitives / slots
  // [scene_prim[k], next) and DNodes [node_off, node_off + n - 1)
  std::vector<int> sp0(nsc), sn(nsc), soff(nsc);
  size_t total_nodes = 0;
  int nmax = 0;
  for (size_t k = 0; k < nsc; ++k) {
    sp0[k] = (int)hs.scene_prim[k];
    sn[k] = (int)((k + 1 < nsc ? hs.scene_prim[k + 1] : np) - hs.scene_prim[k]);
    soff[k] = (int)total_nodes;
    total_nodes += sn[k] > 1 ? (size_t)(sn[k] - 1) : 0;
    nmax = std::max(nmax, sn[k]);
  }
  TR_CUDA(ctx, ctx->d_nodes.reserve(std::max<size_t>(total_nodes, 1) * sizeof(DNode)));
  TR_CUDA(ctx, ctx->d_slots.reserve(std::max<size_t>(3 * np, 1) * sizeof(float4)));

  // scratch for the largest scene
  const size_t N = (size_t)std::max(nmax, 1), M = 2 * N;
  size_t sort_bytes = 0, scan_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, (unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (unsigned int*)nullptr, (unsigned int*)nullptr, (int)N, 0, 63);
  cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, (int*)nullptr, (int*)nullptr, (int)N);
  const size_t tmp_bytes = std::max(sort_bytes, scan_bytes);
  // layout (8-byte aligned pieces)
  size_t off = 0;
  auto carve = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  const size_t o_keys = carve(N * 8), o_keys2 = carve(N * 8), o_vals = carve(N * 4), o_vals2 = carve(N * 4);
  const size_t o_blo = carve(M * 16), o_bhi = carve(M * 16), o_left = carve(M * 4), o_right = carve(M * 4);
  const size_t o_height = carve(M * 4), o_c = carve(N * 4), o_c2 = carve(N * 4), o_nn = carve(N * 4);
  const size_t o_cnt = carve(M * 4), o_leaf = carve(M * 4), o_off = carve(M * 4);
  const size_t o_create = carve(N * 4), o_cid = carve(N * 4), o_keep = carve(N * 4), o_kid = carve(N * 4);
  const size_t o_part = carve(6 * 1024 * 4), o_cb = carve(64), o_tmp = carve(tmp_bytes);
  TR_CUDA(ctx, scratch.reserve(off));
  char* base = scratch.as<char>();
  auto* keys = reinterpret_cast<unsigned long long*>(base + o_keys);
  auto* keys2 = reinterpret_cast<unsigned long long*>(base + o_keys2);
  auto* vals = reinterpret_cast<unsigned int*>(base + o_vals);
  auto* vals2 = reinterpret_cast<unsigned int*>(base + o_vals2);
  ploc::Nodes t;
  t.blo = reinterpret_cast<float4*>(base + o_blo);
  t.bhi = reinterpret_cast<float4*>(base + o_bhi);
  t.left = reinterpret_cast<int*>(base + o_left);
  t.right = reinterpret_cast<int*>(base + o_right);
  t.height = reinterpret_cast<int*>(base + o_height);
  t.cnt = reinterpret_cast<int*>(base + o_cnt);
  t.leaf = reinterpret_cast<int*>(base + o_leaf);
  t.off = reinterpret_cast<int*>(base + o_off);
  auto* C = reinterpret_cast<int*>(base + o_c);
  auto* C2 = reinterpret_cast<int*>(base + o_c2);
  auto* nn = reinterpret_cast<int*>(base + o_nn);
  auto* create = reinterpret_cast<int*>(base + o_create);
  auto* cid = reinterpret_cast<int*>(base + o_cid);
  auto* keep = reinterpret_cast<int*>(base + o_keep);
  auto* kid = reinterpret_cast<int*>(base + o_kid);
  auto* part = reinterpret_cast<float*>(base + o_part);
  auto* cb = reinterpret_cast<float*>(base + o_cb);
  void* tmp = base + o_tmp;
  cudaStream_t st = ctx->stream;

  std::vector<SceneRoot> roots(nsc);
  int max_lights = 0, max_height = 0;
  for (size_t k = 0; k < nsc; ++k) {
    SceneRoot& R = roots[k];
    std::memset(&R, 0, sizeof(R));
    R.light_base = (int)hs.scene_light[k];
    R.num_lights = (int)hs.scene_nlight[k];
    max_lights = std::max(max_lights, R.num_lights);
    const int n = sn[k], p0 = sp0[k];
    if (n == 0) continue;
    const float* lo = d_lo.as<float>() + 3 * (size_t)p0;
    const float* hi = d_hi.as<float>() + 3 * (size_t)p0;
    const int nparts = std::min(1024, blocks(n, 256));
    ploc::k_centroid_bounds<<<nparts, 256, 0, st>>>(lo, hi, n, part);
    ploc::k_centroid_bounds_final<<<1, 32, 0, st>>>(part, nparts, cb);
    ploc::k_morton<<<blocks(n, 256), 256, 0, st>>>(lo, hi, n, cb, keys, vals);
    size_t tb = tmp_bytes;
    TR_CUDA(ctx, cub::DeviceRadixSort::SortPairs(tmp, tb, keys, keys2, vals, vals2, n, 0, 63, st));
    ploc::k_leaves<<<blocks(n, 256), 256, 0, st>>>(vals2, lo, hi, n, t, C);
    const int max_leaf = std::max(1, std::min(hs.scene_leaf[k], 65535));
    std::vector<int> round_start;
    int live = n, next_id = n, rounds = 0;
    while (live > 1) {
      if (++rounds > ploc::kMaxRounds) return set_err(ctx, TR_ERR_STATE, "device BVH build did not converge");
      ploc::k_nearest<<<blocks(live, 128), 128, 0, st>>>(C, live, t.blo, t.bhi, nn);
      ploc::k_merge_flags<<<blocks(live, 256), 256, 0, st>>>(nn, live, create, keep);
      tb = tmp_bytes;
      TR_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tb, create, cid, live, st));
      tb = tmp_bytes;
      TR_CUDA(ctx, cub::DeviceScan::ExclusiveSum(tmp, tb, keep, kid, live, st));
      ploc::k_merge_apply<<<blocks(live, 256), 256, 0, st>>>(C, nn, live, create, cid, keep, kid, next_id, max_leaf,
                                                             t, C2);
      int tail[4];
      TR_CUDA(ctx, cudaMemcpyAsync(&tail[0], cid + live - 1, 4, cudaMemcpyDeviceToHost, st));
      TR_CUDA(ctx, cudaMemcpyAsync(&tail[1], create + live - 1, 4, cudaMemcpyDeviceToHost, st));
      TR_CUDA(ctx, cudaMemcpyAsync(&tail[2], kid + live - 1, 4, cudaMemcpyDeviceToHost, st));
      TR_CUDA(ctx, cudaMemcpyAsync(&tail[3], keep + live - 1, 4, cudaMemcpyDeviceToHost, st));
      TR_CUDA(ctx, cudaStreamSynchronize(st));
      const int made = tail[0] + tail[1];
      if (made <= 0) return set_err(ctx, TR_ERR_STATE, "device BVH build made no progress");
      round_start.push_back(next_id);
      next_id += made;
      live = tail[2] + tail[3];
      std::swap(C, C2);
    }
    if (next_id != 2 * n - 1) return set_err(ctx, TR_ERR_STATE, "device BVH build lost primitives");
    const int root = n - 1 + n - 1;  // the last node made
    // slot offsets top-down: the nodes of later rounds are the parents
    TR_CUDA(ctx, cudaMemsetAsync(t.off + root, 0, 4, st));
    for (int r = (int)round_start.size() - 1; r >= 0; --r) {
      const int id0 = round_start[r], id1 = r + 1 < (int)round_start.size() ? round_start[r + 1] : next_id;
      ploc::k_offsets<<<blocks(id1 - id0, 256), 256, 0, st>>>(id0, id1, t);
    }
    float4 rl, rh;
    int rheight = 0, rleaf = 1;
    TR_CUDA(ctx, cudaMemcpyAsync(&rl, t.blo + root, 16, cudaMemcpyDeviceToHost, st));
    TR_CUDA(ctx, cudaMemcpyAsync(&rh, t.bhi + root, 16, cudaMemcpyDeviceToHost, st));
    TR_CUDA(ctx, cudaMemcpyAsync(&rheight, t.height + root, 4, cudaMemcpyDeviceToHost, st));
    TR_CUDA(ctx, cudaMemcpyAsync(&rleaf, t.leaf + root, 4, cudaMemcpyDeviceToHost, st));
    if (n > 1) ploc::k_emit<<<blocks(n - 1, 256), 256, 0, st>>>(n, t, soff[k], p0, ctx->d_nodes.as<DNode>());
    ploc::k_gather_slots<<<blocks(n, 256), 256, 0, st>>>(d_src.as<float4>(), vals2, n, t.off, p0, p0,
                                                         ctx->d_slots.as<float4>());
    TR_CUDA(ctx, cudaGetLastError());
    TR_CUDA(ctx, cudaStreamSynchronize(st));
    if (rheight >= kMaxDepth)
      return set_err(ctx, TR_ERR_UNSUPPORTED, "device BVH of scene " + std::to_string(k) + " is " +
                                                  std::to_string(rheight) + " levels deep (limit " +
                                                  std::to_string(kMaxDepth) + ")");
    max_height = std::max(max_height, rheight);
    R.lo[0] = rl.x;
    R.lo[1] = rl.y;
    R.lo[2] = rl.z;
    R.hi[0] = rh.x;
    R.hi[1] = rh.y;
    R.hi[2] = rh.z;
    if (rleaf) {  // one leaf: the whole scene
      R.kind = 2;
      R.offset = p0;
      R.count = n;
    } else {
      R.kind = 1;
      R.offset = soff[k] + (root - n);
    }
  }
  if (total_nodes >= (1u << 26)) return set_err(ctx, TR_ERR_UNSUPPORTED, "more than 2^26 interior nodes in one upload");
  hs.depth = max_height;
  TR_CUDA(ctx, put(ctx->d_spheres, hs.spheres.data(), hs.spheres.size() * sizeof(DSphere)));
  TR_CUDA(ctx, put(ctx->d_prims, hs.prims.data(), hs.prims.size() * sizeof(DPrim)));
  TR_CUDA(ctx, put(ctx->d_tshade, hs.tshade.data(), hs.tshade.size() * sizeof(DTriShade)));
  TR_CUDA(ctx, put(ctx->d_mats, hs.mats.data(), hs.mats.size() * sizeof(DMat)));
  TR_CUDA(ctx, put(ctx->d_lights, hs.lights.data(), hs.lights.size() * sizeof(DLight)));
  TR_CUDA(ctx, put(ctx->d_roots, roots.data(), roots.size() * sizeof(SceneRoot)));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->any4_nodes = 0;  // the four-wide any-hit tree is built from host trees only
  ctx->any4_stack = 0;
  DScene& sc = ctx->dsc;
  sc.nodes = ctx->d_nodes.as<DNode>();
  sc.nodes4 = nullptr;
  sc.treelet = nullptr;  // no host copy of the device-built tree to stage from
  sc.treelet_n = 0;
  sc.slot_leaf = nullptr;  // nor the leaf of every slot: no occluder cache
  hs.dnodes.clear();
  hs.root0 = -1;
  sc.slots = ctx->d_slots.as<float4>();
  sc.spheres = ctx->d_spheres.as<DSphere>();
  sc.prims = ctx->d_prims.as<DPrim>();
  sc.tshade = ctx->d_tshade.as<DTriShade>();
  sc.mats = ctx->d_mats.as<DMat>();
  sc.lights = ctx->d_lights.as<DLight>();
  sc.roots = ctx->d_roots.as<SceneRoot>();
  sc.num_scenes = (int)nsc;
  sc.max_lights = max_lights;
  sc.has_glass = 0;
  sc.has_metal = 0;
  sc.has_disney15 = 0;
  for (const DMat& m : hs.mats) {
    sc.has_glass |= m.kind == MAT_GLASS;
    sc.has_metal |= m.kind == MAT_METAL;
    sc.has_disney15 |= m.kind == MAT_DISNEY15;
  }
  tr_status es = upload_envs(ctx);
  if (es != TR_OK) return es;
  es = upload_textures(ctx);
  if (es != TR_OK) return es;
  ctx->has_scene = true;
  return TR_OK;
}

}  // namespace trg
