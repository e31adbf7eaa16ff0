// render.cu -- wavefront path tracer: PathTraceRenderer::eval_pixel_li
// (src/renderer/path_trace_renderer.cpp:27-210) for every camera sample of
// PixelSamplerRenderer::render (src/renderer/pixel_sampler_renderer.cpp:24-109).
//
// One path slot per pixel. A slot draws its pixel's pcg32 stream in the
// reference's order and runs its spp samples one after another, so the
// random numbers, the rays and the film sums are the reference's. Each
// wavefront iteration runs these kernels over compacted queues:
//
//   extend       closest hit for every queued ray (continuation and MIS rays)
//   logic        per live slot: add the previous vertex's direct lighting
//                (shadow results + MIS hit), finish samples (film) and start
//                the next camera sample, add emission at depth 0, and queue
//                hits by material
//   material<K>  per hit of material K: BSDF sample, the light-sample draws,
//                the MIS ray, the throughput update, Russian roulette and the
//                next continuation ray
//   nee<K>       per (hit of material K, light): the light sample, BSDF eval
//                and pdf, and a shadow ray with its would-be contribution
//   shadow       any hit for every queued shadow ray (zeroes blocked ones)
//
// Splitting by material keeps each kernel's code small (the shading code of
// one monolithic kernel overflowed the instruction cache) and its warps on
// one code path. All random draws of a vertex happen in `material`, before
// any of its rays is traced, in the reference's order (its draws never depend
// on ray results); the contributions are summed back in the reference's
// order in `logic`. Queues are appended with warp-aggregated atomics.

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "context.h"
#include "mixture.cuh"
#include "mlp.h"
#include "binning.cuh"
#include "mega.h"
#include "render_common.cuh"
#include "shade.cuh"
#include "traverse.cuh"

namespace trg {

enum : int {
  F_PENDING = 1,    // the previous vertex's direct lighting is still to be added
  F_MIS = 2,        // ...and it includes a MIS ray
  F_TERMINATE = 4,  // the path ends once that lighting is added
  F_REC = 8,        // the previous vertex wrote a guiding record awaiting its radiance
  F_GCONT = 16,     // ...and its guided continuation is an MIS strategy of its direct lighting
  F_GX = 32,        // ...and so is a ray drawn from the mixture alone (in the MIS slot)
  F_SPEC = 64,      // the continuation was sampled from a delta BSDF: emission it reaches counts
};

// light-sample queue of a material kind (glass has none)
__host__ __device__ constexpr int nee_index(int kind) {
  return kind == MAT_METAL ? 2 : (kind == MAT_DISNEY15 ? 3 : kind);
}

enum : int {  // counter slots
  C_EXT = 0,      // 2: extend queue sizes (double-buffered)
  C_ACT = 2,      // 2: live-slot list sizes
  C_SH = 4,       // shadow queue size
  C_MAT = 5,      // 5: per-material hit queue sizes (Phong, Disney12, glass, metal, Disney15)
  C_NEE = 10,     // 4: light-sample queue sizes (Phong, Disney12, metal, Disney15; glass has none)
  C_FEXT = 14,    // extend kernel's work-fetch position
  C_FSH = 15,     // shadow kernel's work-fetch position
  C_TB = 16,      // guiding training records written (whole render)
  C_ERR = 17,     // traversal error word
  C_ORD = 18,     // live slots written in slot order (this iteration)
  C_GROW = 19,    // network rows of this iteration's guided vertices
};
constexpr int kCtrWords = 32;  // the counter array
// Statistics words: samples, extend rays, shadow rays, shade items, visit
// counts (4-7), occluder-cache hits (8).
constexpr int kStatWords = 16;
// render_mode auto: renders of at most this many pixels use the persistent kernel
constexpr long long kMegaAutoSlots = 1 << 17;
// Material code in the shading context: the material index, or with this bit
// set the slot's own set-up in Launch::MT (a Phong material with maps).
constexpr int kMatScratch = 1 << 30;

struct RenderBuffers {
  int n = 0, nl = 0;
  DevBuf P0, P1, P2, P3, P4, rng, M0, M1, M2, HC, HM, SC, NU, SH, SHC, acc, q_ext, q_act, q_mat, q_nee, q_sh, ctr,
      stats;
  DevBuf VR, NV, gfeat, gout, tb;  // path guiding: vertex records, network rows, training records
  DevBuf GX;                        // path guiding: the continuation's MIS data (4 float4 per slot)
  DevBuf grow;                      // path guiding: per slot, the network row of its vertex
  DevBuf MT;                        // Phong set-ups at hits with image maps (one DMat per slot)
  DevBuf jobs;                      // JobDev table of the current render
  DevBuf q_srt, bin_key, bin_cnt;   // ray binning: the reordered queue, keys, bin counts
  DevBuf OC;                        // occluder cache, one int per (slot, light)
  DevBuf q_ord, act_flag;           // the live-slot list in slot order, per-slot marks
  unsigned int tb_count = 0, tb_cap = 0;  // training records of the last guided render
  unsigned int* h_active = nullptr;  // pinned: live-slot count per check
  std::vector<cudaEvent_t> ev_pool;  // reused by stage timing
};

struct Launch {
  DScene sc;
  const JobDev* jobs;
  int njobs, nslots;
  int nl_max;  // stride of the per-(slot, light) records
  int refill;  // traversal lane-refill threshold (tr_tuning)
  int tl_n;    // treelet nodes the binary traversal kernels stage (their launches give tl_n * 64 bytes)
  float4 *P0, *P1, *P2, *P3, *P4;  // cont o|flags, cont d|depth, coef|sample, L|px, coef_prev|py
  unsigned long long* rng;
  float4 *M0, *M1, *M2;  // mis o|bsdf_pdf, mis d|abs_cos, bsdf_f (guided: o|p_guided, d|p_bsdf, f_eval|p_plain)
  float4 *HC, *HM;       // hits: prim, t_attr, alpha, beta
  float4* SC;            // shading context for nee: 7 per slot (pos|mat, wo, g, s frames; the last
                         // also holds the guided vertex's network row, normal correction and |cos|)
  float2* NU;            // light-sample draws per (slot, light)
  float4* SH;            // shadow rays: 2 per (slot, light): o|t_max, d|estimate
  float4* SHC;           // per (slot, light): the light sample's contribution|valid (0: none or occluded)
  DMat* MT;              // per slot: the Phong set-up at a hit with image maps (null without maps)
  int* q_ext[2];
  int* q_act[2];
  int* q_mat[kMatKinds];
  int* q_nee[kNeeKinds];
  int* q_sh;
  // ray binning (bin_bits > 0): the extend or shadow queue reordered by ray
  // key, read by the traversal kernels instead of the queue
  int bin_bits;
  int* q_srt;
  unsigned int *bin_key, *bin_cnt;
  // occluder cache (null: off): per (slot, light) item, the slot that last
  // blocked its shadow ray, or -1
  int* OC;
  // the live-slot list in slot order (null: k_logic reads the list as appended)
  int* q_ord;
  int mis_all;  // trace every MIS ray (visit-counting renders match the oracle's queries)
  // guided renders: vertices at path depth < guide_depth (0: all) are
  // guided; grow: per slot, the network row of its vertex (-1: not guided)
  int guide_depth;
  int* grow;
  unsigned char* act_flag;
  unsigned int* ctr;
  unsigned long long* stats;  // samples, extend rays, shadow rays, shade items, visit counts (4-7)
  // path guiding (alpha > 0: sample Lambertian continuations from the network's mixture;
  // record: keep training records)
  float guide_alpha;
  int guide_record, maxd;  // record: 0 off, n > 0 every n-th sample of a pixel
  float gbox_lo[3], gbox_scale[3];
  float* gfeat;  // network inputs, one row per entry of q_mat[0]
  float* gout;   // decoded mixtures (kMixFloats per row), same rows
  float4* GX;    // 4 per slot: continuation o|p_g, d|p_bsdf, f_eval|p_plain, (nc, |cos|, p_mix, p_g of the mixture ray)
  float4* VR;    // 4 per (slot, vertex): features 0-3 | features 4-6, pdf | direction, throughput | radiance
  int* NV;       // records of the slot's current sample
  float *tb_in, *tb_dir, *tb_w;
  unsigned int tb_cap;
  // learned light sampling (lg_cdf null: the reference's uniform light
  // sample): per (cell of lg_grid over the guide box, light) the cumulative
  // distribution over lg_bins x lg_bins cells of the light's sample square;
  // lg_acc non-null: unoccluded light samples add to its statistics
  const float* lg_cdf;
  float* lg_acc;
  int lg_grid[3], lg_bins;
};

// The light-table entry of position `pos` and light l: the cell of the grid
// over the guide box (clamped) times the lights plus l, times bins^2 floats.
__device__ __forceinline__ size_t lg_table(const Launch& P, f3 pos, int l) {
  const float q[3] = {pos.x, pos.y, pos.z};
  int c[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    // gbox_scale maps the box to [0, 2]
    const float u = (q[k] - P.gbox_lo[k]) * P.gbox_scale[k] * 0.5f * (float)P.lg_grid[k];
    c[k] = (int)fminf(fmaxf(u, 0.0f), (float)(P.lg_grid[k] - 1));
  }
  const int cell = (c[2] * P.lg_grid[1] + c[1]) * P.lg_grid[0] + c[0];
  return ((size_t)cell * P.nl_max + l) * (size_t)(P.lg_bins * P.lg_bins);
}

// A learned light sample: the bin by the first draw's inverse CDF, the
// position inside the bin from that draw's remainder and the second draw.
// Returns the point in the light's sample square, the bin, and the ratio of
// the uniform density to the table's there.
__device__ __forceinline__ float2 lg_sample(const Launch& P, size_t tab, float2 uv, int& bin, float& ratio) {
  const float* cdf = P.lg_cdf + tab;
  const int nb = P.lg_bins * P.lg_bins;
  int lo = 0, hi = nb - 1;  // the first bin whose cumulative value is above u (the last is exactly 1)
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cdf[mid] > uv.x) hi = mid;
    else lo = mid + 1;
  }
  bin = lo;
  const float c0 = lo ? cdf[lo - 1] : 0.0f;
  const float pm = cdf[lo] - c0;
  float r = pm > 0.0f ? (uv.x - c0) / pm : 0.5f;
  r = fminf(fmaxf(r, 0.0f), 0.99999994f);
  ratio = 1.0f / (pm * (float)nb);
  const int bx = lo % P.lg_bins, by = lo / P.lg_bins;
  return make_float2(((float)bx + r) / (float)P.lg_bins, ((float)by + uv.y) / (float)P.lg_bins);
}

// The job a path slot belongs to.
__device__ __forceinline__ const JobDev& job_of(const Launch& P, int slot) { return job_of(P.jobs, P.njobs, slot); }

// Network inputs of a vertex: position in the scene box mapped to [-1, 1],
// outgoing direction, roughness.
__device__ __forceinline__ void guide_features(const Launch& P, f3 pos, f3 wo, float rough, float (&f)[7]) {
  f[0] = (pos.x - P.gbox_lo[0]) * P.gbox_scale[0] - 1.0f;
  f[1] = (pos.y - P.gbox_lo[1]) * P.gbox_scale[1] - 1.0f;
  f[2] = (pos.z - P.gbox_lo[2]) * P.gbox_scale[2] - 1.0f;
  f[3] = wo.x;
  f[4] = wo.y;
  f[5] = wo.z;
  f[6] = rough;
}

// Warp-aggregated queue append. The active lanes are grouped by counter
// address (__match_any_sync): one call site can target different queues per
// lane (the per-material hit queues), and each group reserves its own range.
__device__ __forceinline__ int append(unsigned int* ctr) {
  const unsigned int active = __activemask();
  const unsigned int peers = __match_any_sync(active, (unsigned long long)ctr);
  const int lane = (int)(threadIdx.x & 31u);
  const int leader = __ffs(peers) - 1;
  unsigned int base = 0;
  if (lane == leader) base = atomicAdd(ctr, (unsigned int)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  return (int)(base + (unsigned int)__popc(peers & ((1u << lane) - 1u)));
}

// Warp-aggregated add to a 64-bit statistics counter (lanes grouped by
// address, as in append); per-lane values are per-kernel tallies well below
// 2^32 / 32.
__device__ __forceinline__ void count_add(unsigned long long* c, unsigned int v) {
  const unsigned int active = __activemask();
  const unsigned int peers = __match_any_sync(active, (unsigned long long)c);
  const unsigned int s = __reduce_add_sync(peers, v);
  if ((int)(threadIdx.x & 31u) == __ffs(peers) - 1 && s) atomicAdd(c, (unsigned long long)s);
}

// Starts the slot's next camera sample, finishing samples that Russian
// roulette ends before their first vertex. Returns false when the pixel has
// no samples left.
__device__ __forceinline__ bool start_sample(const Launch& P, int slot, unsigned long long& st, int sample,
                                             int next_q, unsigned int& finished) {
  const JobDev& J = job_of(P, slot);
  const int pix = slot - J.slot_base;
  const int x = pix % J.W, y = pix / J.W;
  while (sample < J.spp) {
    const float fu = Pcg::next(st), fv = Pcg::next(st);
    const float lu = Pcg::next(st), lv = Pcg::next(st);
    const float px = (float)x + fu, py = (float)y + fv;
    f3 o, d;
    camera_ray(J.cam, px / (float)J.W, py / (float)J.H, lu, lv, o, d);
    f3 coef = mk3(1.0f, 1.0f, 1.0f);
    bool dead = false;
    if (0 > J.min_depth) {  // Russian roulette at depth 0
      if (Pcg::next(st) > 0.9f) dead = true;
      else coef = divs(coef, 0.9f);
    }
    if (!dead && !valid3(coef)) dead = true;
    if (dead) {
      film_add(J, slot, px, py, mk3(0.0f, 0.0f, 0.0f));
      ++finished;
      ++sample;
      continue;
    }
    P.P0[slot] = make_float4(o.x, o.y, o.z, __int_as_float(0));
    P.P1[slot] = make_float4(d.x, d.y, d.z, __int_as_float(0));
    P.P2[slot] = make_float4(coef.x, coef.y, coef.z, __int_as_float(sample));
    P.P3[slot] = make_float4(0.0f, 0.0f, 0.0f, px);
    P.P4[slot] = make_float4(0.0f, 0.0f, 0.0f, py);
    P.q_ext[next_q][append(P.ctr + C_EXT + next_q)] = 2 * slot;
    return true;
  }
  return false;
}

// Ends the slot's current sample (film) and starts its next one.
__device__ void finish_sample(const Launch& P, int slot, unsigned long long& st, f3 L, int nxt,
                              unsigned int& finished) {
  if (!valid3(L)) L = mk3(0.0f, 0.0f, 0.0f);  // eval_pixel_li returns {} (path_trace_renderer.cpp:204-209)
  if (P.guide_record) {
    // training records of this sample's vertices: the radiance that arrived
    // along each continuation direction, (L - L_after_vertex) / throughput,
    // where L_after_vertex leaves out the emission the continuation reached
    // (so that emission is part of the target), times |cos| over the pdf
    // the direction was drawn with
    const int nv = P.NV[slot];
    for (int k = 0; k < nv; ++k) {
      const float4* r = P.VR + ((size_t)slot * P.maxd + k) * 4;
      const float4 a = r[0], b = r[1], c = r[2], d = r[3];
      const float li = lum(mk3(L.x - d.x, L.y - d.y, L.z - d.z)) / fmaxf(c.w, 1e-20f);
      const float w = li / b.w;
      if (!(w > 0.0f) || !(w < 1e30f)) continue;
      const unsigned int idx = (unsigned int)append(P.ctr + C_TB);
      if (idx >= P.tb_cap) continue;
      float* fi = P.tb_in + (size_t)idx * 7;
      fi[0] = a.x; fi[1] = a.y; fi[2] = a.z; fi[3] = a.w; fi[4] = b.x; fi[5] = b.y; fi[6] = b.z;
      float* di = P.tb_dir + (size_t)idx * 3;
      di[0] = c.x; di[1] = c.y; di[2] = c.z;
      P.tb_w[idx] = w;
    }
    P.NV[slot] = 0;
  }
  const float px = P.P3[slot].w, py = P.P4[slot].w;
  film_add(job_of(P, slot), slot, px, py, L);
  ++finished;
  const int sample = __float_as_int(P.P2[slot].w) + 1;
  if (start_sample(P, slot, st, sample, nxt, finished)) P.q_act[nxt][append(P.ctr + C_ACT + nxt)] = slot;
}

__global__ void __launch_bounds__(256) k_init(Launch P) {
  const int n = P.nslots;
  unsigned int finished = 0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const JobDev& J = job_of(P, s);
    const int pix = s - J.slot_base;
    const int x = pix % J.W, y = pix / J.W;
    unsigned long long st = Pcg::seed((int)(J.seed_base + (unsigned)y * (unsigned)J.W + (unsigned)x));
    if (P.guide_record) P.NV[s] = 0;
    const bool live = start_sample(P, s, st, 0, 0, finished);
    P.rng[s] = st;
    if (live) P.q_act[0][append(P.ctr + C_ACT)] = s;
  }
  count_add(P.stats, finished);
}

// Work items of the extend kernel: queue entry 2*slot (+1 for the MIS ray).
struct ExtendJob {
  const Launch& P;
  int cur;
  const int* q;  // the queue, or its binned order
  __device__ ExtendJob(const Launch& P_, int cur_) : P(P_), cur(cur_), q(P_.bin_bits ? P_.q_srt : P_.q_ext[cur_]) {}
  __device__ __forceinline__ unsigned int count() const { return P.ctr[C_EXT + cur]; }
  __device__ __forceinline__ int cached(unsigned int) const { return -1; }
  __device__ __forceinline__ void load(unsigned int i, f3& o, f3& d, float& t_min, float& t_max, int& scene) const {
    const int e = q[i];
    const int slot = e >> 1;
    scene = job_of(P, slot).scene;
    const float4 a = (e & 1) ? P.M0[slot] : P.P0[slot];
    const float4 b = (e & 1) ? P.M1[slot] : P.P1[slot];
    o = mk3(a.x, a.y, a.z);
    d = mk3(b.x, b.y, b.z);
    t_min = 0.0f;
    t_max = kRealMax;
  }
  __device__ __forceinline__ void store(unsigned int i, const Hit& h, float, bool) const {
    const int e = q[i];
    const float4 rec = make_float4(__int_as_float(h.prim), h.t_attr, h.alpha, h.beta);
    if (e & 1) P.HM[e >> 1] = rec;
    else P.HC[e >> 1] = rec;
  }
};

// Work items of the shadow kernel: shadow records o|t_max, d, contrib|valid.
struct ShadowJob {
  const Launch& P;
  const int* q;  // the queue (shadow rays keep queue order: a vertex's rays to every light are adjacent)
  __device__ explicit ShadowJob(const Launch& P_) : P(P_), q(P_.q_sh) {}
  __device__ __forceinline__ unsigned int count() const { return P.ctr[C_SH]; }
  // the slot that last blocked this (pixel slot, light) item's shadow ray
  __device__ __forceinline__ int cached(unsigned int i) const { return P.OC ? P.OC[q[i]] : -1; }
  __device__ __forceinline__ void load(unsigned int i, f3& o, f3& d, float& t_min, float& t_max, int& scene) const {
    const int r = q[i];
    scene = job_of(P, r / P.nl_max).scene;
    const float4 a = P.SH[2 * r], b = P.SH[2 * r + 1];
    o = mk3(a.x, a.y, a.z);
    d = mk3(b.x, b.y, b.z);
    t_min = kEps;
    t_max = a.w;
  }
  __device__ __forceinline__ void store(unsigned int i, const Hit& h, float, bool occluded) const {
    if (occluded) {
      P.SHC[q[i]].w = 0.0f;
      if (P.OC) P.OC[q[i]] = h.prim;
    }
  }
};

// The extend queue as a source of ray binning (binning.cuh): entries in
// queue order with their rays. (The shadow queue is not binned: k_nee appends
// a vertex's rays to all lights next to each other, an order binning loses;
// measured slower on the occluded room.)
struct ExtendSrc {
  Launch P;
  int cur;
  __device__ __forceinline__ unsigned int count() const { return P.ctr[C_EXT + cur]; }
  __device__ __forceinline__ int item(unsigned int i) const { return P.q_ext[cur][i]; }
  __device__ __forceinline__ void ray(unsigned int i, f3& o, f3& d, int& scene) const {
    const int e = P.q_ext[cur][i];
    const int slot = e >> 1;
    scene = job_of(P, slot).scene;
    const float4 a = (e & 1) ? P.M0[slot] : P.P0[slot];
    const float4 b = (e & 1) ? P.M1[slot] : P.P1[slot];
    o = mk3(a.x, a.y, a.z);
    d = mk3(b.x, b.y, b.z);
  }
};

template <bool COUNT>
__global__ void __launch_bounds__(128) k_extend(Launch P, int cur) {
  ExtendJob job(P, cur);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(P.stats + 1, (unsigned long long)job.count());
  VisitCount vc;
  persistent_traverse<false, COUNT>(P.sc, job, P.ctr + C_FEXT, (int*)(P.ctr + C_ERR), vc, P.refill, P.tl_n);
  if (COUNT) {
    count_add(P.stats + 4, vc.boxes);
    count_add(P.stats + 5, vc.prims);
  }
}

template <bool COUNT, bool WIDE = false>
__global__ void __launch_bounds__(128) k_shadow(Launch P) {
  ShadowJob job(P);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(P.stats + 2, (unsigned long long)job.count());
  VisitCount vc;
  persistent_traverse<true, COUNT, WIDE>(P.sc, job, P.ctr + C_FSH, (int*)(P.ctr + C_ERR), vc, P.refill, P.tl_n);
  if (P.OC) count_add(P.stats + 8, vc.cache_hits);
  if (COUNT) {
    count_add(P.stats + 6, vc.boxes);
    count_add(P.stats + 7, vc.prims);
  }
}

// sample_bsdf's contribution once its ray has been traced
// (src/renderer/direct_illumination.cpp:144-198).
__device__ f3 mis_contribution(const Launch& P, int slot) {
  const float4 hit = P.HM[slot];
  const int pid = __float_as_int(hit.x);
  if (pid < 0) {
    // the ray left the scene: the environment light's share (:156-174)
    const int ei = job_of(P, slot).env;
    if (ei < 0) return mk3(0.0f, 0.0f, 0.0f);
    const DEnv& e = P.sc.envs[ei];
    const float4 m0 = P.M0[slot], m1 = P.M1[slot], m2 = P.M2[slot];
    const f3 d = mk3(m1.x, m1.y, m1.z);
    const f3 Le = env_emit(e, d);
    if (black(Le)) return mk3(0.0f, 0.0f, 0.0f);
    const f3 f = muls(mulc(Le, mk3(m2.x, m2.y, m2.z)), m1.w);
    const float w = power_heuristic(m0.w, env_pdf(e, d));
    return divs(muls(f, w), m0.w);
  }
  const DPrim& pr = P.sc.prims[pid];
  if (!pr.emissive) return mk3(0.0f, 0.0f, 0.0f);
  const float4 m0 = P.M0[slot], m1 = P.M1[slot], m2 = P.M2[slot];
  const f3 o = mk3(m0.x, m0.y, m0.z), d = mk3(m1.x, m1.y, m1.z);
  const f3 gz = P.sc.tshade[pr.shape].gz;
  // light_emit(t_isect, t_isect.wo) with wo = -ray.d
  if (!(dot(gz, -d) > 0.0f)) return mk3(0.0f, 0.0f, 0.0f);
  const f3 f = muls(mulc(pr.emission, mk3(m2.x, m2.y, m2.z)), m1.w);
  const f3 pos = o + scale(d, hit.y);
  const float lpdf = light_pdf_at(pr.area, o, pos, gz);
  const float w = power_heuristic(m0.w, lpdf);
  return divs(muls(f, w), m0.w);
}

// Power-heuristic weight of a strategy of density a against one of density
// b, zero when a is (no 0/0).
__device__ __forceinline__ float mis_w(float a, float b) { return a > 0.0f ? power_heuristic(a, b) : 0.0f; }

// The direct-lighting integrand of a Lambertian vertex over incident
// direction w, per unit emitted radiance and |cos|: what the reference's
// two strategies sum to in expectation (sample_area_light with the BSDF's
// eval and pdf, sample_bsdf with the sampler's own integrand and density,
// src/renderer/direct_illumination.cpp:35-71,144-198). fe, pb: eval and pdf
// at w; fs, ps: the plain sampler's integrand and density at w; lpdf: the
// light's solid-angle density at w; lq: the light density the reference's
// sample_bsdf weighs against (lpdf for area lights, IBL::pdf for the
// environment light, :156-174).
__device__ __forceinline__ f3 direct_integrand(f3 fe, float pb, f3 fs, float ps, float lpdf, float lq) {
  return muls(fe, mis_w(lpdf, pb)) + muls(fs, mis_w(ps, lq));
}

// Emission reached by a ray of a guided vertex that is one of its MIS
// strategies for direct lighting, weighted by the power heuristic against
// next-event estimation and the other guided strategy (the other half of
// guided_nee_factor). The ray's data: origin o, direction d, its own density
// pr, the other strategy's density there po (0: two strategies), the BSDF's
// eval fe and pdf pb, the plain sampler's density ps, the normal correction
// nc and |cos|. `hit` is the ray's hit.
__device__ f3 guided_strategy_emission(const Launch& P, int slot, float4 hit, f3 o, f3 d, float pr, float po, f3 fe,
                                       float pb, float ps, float nc, float cosv) {
  const int pid = __float_as_int(hit.x);
  f3 Le;
  float lpdf, lq;
  if (pid < 0) {  // left the scene: the environment light, if any
    const int ei = job_of(P, slot).env;
    if (ei < 0) return mk3(0.0f, 0.0f, 0.0f);
    const DEnv& e = P.sc.envs[ei];
    Le = env_emit(e, d);
    if (black(Le)) return mk3(0.0f, 0.0f, 0.0f);
    lpdf = env_sample_density(e, d);
    lq = env_pdf(e, d);
  } else {
    const DPrim& pr_ = P.sc.prims[pid];
    if (!pr_.emissive) return mk3(0.0f, 0.0f, 0.0f);
    const f3 gz = P.sc.tshade[pr_.shape].gz;
    if (!(dot(gz, -d) > 0.0f)) return mk3(0.0f, 0.0f, 0.0f);
    Le = pr_.emission;
    lpdf = light_pdf_at(pr_.area, o, o + scale(d, hit.y), gz);
    lq = lpdf;
  }
  const int mcode = __float_as_int(P.SC[7 * (size_t)slot].w);
  const DMat& mat = (mcode & kMatScratch) ? P.MT[slot] : P.sc.mats[mcode];
  const f3 fs = ps > 0.0f ? muls(mat.diffuse_coef, nc) : mk3(0.0f, 0.0f, 0.0f);
  const f3 g = direct_integrand(fe, pb, fs, ps, lpdf, lq);
  const float w = pr * pr / (pr * pr + lpdf * lpdf + po * po);
  return muls(mulc(Le, g), cosv * w / pr);
}

// The strategy in the MIS slot (M0-M2, normal correction and |cos| in the
// shading context): the continuation of a vertex whose path ends there, or
// the mixture ray (whose continuation-density is in GX).
__device__ f3 guided_mis_slot_emission(const Launch& P, int slot, bool mixture_ray) {
  const float4 m0 = P.M0[slot], m1 = P.M1[slot], m2 = P.M2[slot], sc6 = P.SC[7 * (size_t)slot + 6];
  const float po = mixture_ray ? P.GX[4 * (size_t)slot + 3].w : 0.0f;
  return guided_strategy_emission(P, slot, P.HM[slot], mk3(m0.x, m0.y, m0.z), mk3(m1.x, m1.y, m1.z), m0.w, po,
                                  mk3(m2.x, m2.y, m2.z), m1.w, m2.w, sc6.z, sc6.w);
}

// The continuation of a vertex whose path goes on (data in GX, hit in HC),
// against next-event estimation and the mixture ray.
__device__ f3 guided_continuation_emission(const Launch& P, int slot) {
  const float4* g = P.GX + 4 * (size_t)slot;
  const float4 a = g[0], b = g[1], c = g[2], e = g[3];
  return guided_strategy_emission(P, slot, P.HC[slot], mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), a.w, e.z,
                                  mk3(c.x, c.y, c.z), b.w, c.w, e.x, e.y);
}

// Emission the continuation of a recorded vertex reaches (full, unweighted):
// part of the radiance that arrived along it, and so of the training target.
__device__ __forceinline__ f3 continuation_emission(const Launch& P, int slot, float4 hit) {
  const int pid = __float_as_int(hit.x);
  if (pid < 0) {
    const int ei = job_of(P, slot).env;
    const float4 p1 = P.P1[slot];
    return ei < 0 ? mk3(0.0f, 0.0f, 0.0f) : env_emit(P.sc.envs[ei], mk3(p1.x, p1.y, p1.z));
  }
  const DPrim& pr = P.sc.prims[pid];
  if (!pr.emissive) return mk3(0.0f, 0.0f, 0.0f);
  const float4 p1 = P.P1[slot];
  if (!(dot(P.sc.tshade[pr.shape].gz, mk3(-p1.x, -p1.y, -p1.z)) > 0.0f)) return mk3(0.0f, 0.0f, 0.0f);
  return pr.emission;
}

// Marks the slots of the live-slot list, which is in append order.
__global__ void __launch_bounds__(256) k_act_mark(Launch P, int cur) {
  const unsigned int n = P.ctr[C_ACT + cur];
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    P.act_flag[P.q_act[cur][i]] = 1;
}

// The marked slots in slot order within each 256-slot range (the ranges in
// the order their blocks reach the counter), marks cleared. k_logic then
// reads the path state of consecutive slots together, and the queues it
// fills, so the kernels after it, follow slot order too; the order of work
// changes no result.
__global__ void __launch_bounds__(256) k_act_order(Launch P) {
  __shared__ unsigned int wsum[8];
  __shared__ unsigned int base;
  const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
  for (unsigned int b0 = blockIdx.x * 256u; b0 < (unsigned int)P.nslots; b0 += gridDim.x * 256u) {
    const unsigned int s = b0 + threadIdx.x;
    const bool live = s < (unsigned int)P.nslots && P.act_flag[s];
    const unsigned int m = __ballot_sync(0xffffffffu, live);
    if (lane == 0) wsum[warp] = (unsigned int)__popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned int t = 0;
      for (int w = 0; w < 8; ++w) {
        const unsigned int c = wsum[w];
        wsum[w] = t;
        t += c;
      }
      base = t ? atomicAdd(P.ctr + C_ORD, t) : 0u;
    }
    __syncthreads();
    if (live) {
      P.q_ord[base + wsum[warp] + (unsigned int)__popc(m & ((1u << lane) - 1u))] = (int)s;
      P.act_flag[s] = 0;
    }
    __syncthreads();
  }
}

__global__ void __launch_bounds__(128) k_logic(Launch P, int cur) {
  const int nxt = cur ^ 1;
  const unsigned int n = P.ctr[C_ACT + cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(P.stats + 3, (unsigned long long)n);
  unsigned int finished = 0;
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int slot = P.q_ord ? P.q_ord[i] : P.q_act[cur][i];
    const float4 p0 = P.P0[slot], p3 = P.P3[slot];
    const int flags = __float_as_int(p0.w);
    f3 L = mk3(p3.x, p3.y, p3.z);
    if (flags & F_PENDING) {
      // direct lighting of the previous vertex, in the reference's order:
      // lights in scene order, then the MIS term, then L += direct
      const float4 p4 = P.P4[slot];
      f3 direct = mk3(0.0f, 0.0f, 0.0f);
      const int nl = job_of(P, slot).nl;
      for (int l = 0; l < nl; ++l) {
        const float4 c = P.SHC[slot * P.nl_max + l];
        if (c.w != 0.0f) direct = direct + mk3(c.x, c.y, c.z);
        if (P.lg_acc && c.w != 0.0f) {
          // an unoccluded learned light sample: its estimate into the
          // statistics of its (cell, light) bin (environment-light items
          // carry no estimate)
          const float v = P.SH[2 * (slot * P.nl_max + l) + 1].w;
          if (v > 0.0f && v < 1e30f) {
            const float4 s0 = P.SC[7 * (size_t)slot];
            atomicAdd(P.lg_acc + lg_table(P, mk3(s0.x, s0.y, s0.z), l) + ((int)c.w - 1), v);
          }
        }
      }
      if (flags & F_MIS) direct = direct + mulc(mk3(p4.x, p4.y, p4.z), mis_contribution(P, slot));
      if (flags & (F_GCONT | F_GX)) {
        f3 ge = mk3(0.0f, 0.0f, 0.0f);
        if ((flags & F_GCONT) && (flags & F_TERMINATE)) ge = guided_mis_slot_emission(P, slot, false);
        if ((flags & F_GCONT) && !(flags & F_TERMINATE)) ge = guided_continuation_emission(P, slot);
        if (flags & F_GX) ge = ge + guided_mis_slot_emission(P, slot, true);
        direct = direct + mulc(mk3(p4.x, p4.y, p4.z), ge);
      }
      L = L + direct;
      if (flags & F_REC) {
        // the record's baseline leaves out the continuation's own emission,
        // so the target is the whole radiance that arrived along it
        const float4 p2 = P.P2[slot];
        const f3 Lb = L - mulc(mk3(p2.x, p2.y, p2.z), continuation_emission(P, slot, P.HC[slot]));
        P.VR[((size_t)slot * P.maxd + P.NV[slot] - 1) * 4 + 3] = make_float4(Lb.x, Lb.y, Lb.z, 0.0f);
      }
    }
    const float4 hit = P.HC[slot];
    const int pid = __float_as_int(hit.x);
    if (!(flags & F_TERMINATE) && pid < 0 && (path_depth(P.P1[slot].w) == 0 || (flags & F_SPEC))) {
      // a camera ray or one after a delta sample left the scene: the
      // environment light's radiance along it (path_trace_renderer.cpp:66-81)
      const int ei = job_of(P, slot).env;
      if (ei >= 0) {
        const float4 p1 = P.P1[slot], p2 = P.P2[slot];
        L = L + mulc(mk3(p2.x, p2.y, p2.z), env_emit(P.sc.envs[ei], mk3(p1.x, p1.y, p1.z)));
      }
    }
    if ((flags & F_TERMINATE) || pid < 0) {
      unsigned long long st = P.rng[slot];
      finish_sample(P, slot, st, L, nxt, finished);
      P.rng[slot] = st;
      continue;
    }
    const DPrim& pr = P.sc.prims[pid];
    if ((path_depth(P.P1[slot].w) == 0 || (flags & F_SPEC)) && pr.emissive) {
      // emission seen by the camera ray or after a delta sample:
      // light_emit(isect, -ray.d); only triangles emit on this path
      const f3 gz = P.sc.tshade[pr.shape].gz;
      const float4 p1 = P.P1[slot], p2 = P.P2[slot];
      if (dot(gz, mk3(-p1.x, -p1.y, -p1.z)) > 0.0f) L = L + mulc(mk3(p2.x, p2.y, p2.z), pr.emission);
    }
    P.P3[slot] = make_float4(L.x, L.y, L.z, p3.w);
    const int kind = P.sc.mats[pr.material].kind;
    const int qi = append(P.ctr + C_MAT + kind);
    P.q_mat[kind][qi] = slot;
    if (kind == MAT_PHONG && P.guide_alpha > 0.0f) {
      // network inputs of the vertex, a row of this iteration's forward pass
      const float4 p1 = P.P1[slot];
      int row = -1;
      if (P.guide_depth == 0 || path_depth(p1.w) < P.guide_depth) {
        row = append(P.ctr + C_GROW);
        const f3 d = mk3(p1.x, p1.y, p1.z);
        float f[7];
        guide_features(P, mk3(p0.x, p0.y, p0.z) + scale(d, hit.y), -d, 1.0f, f);
        float* out = P.gfeat + (size_t)row * 7;
        for (int k = 0; k < 7; ++k) out[k] = f[k];
      }
      P.grow[slot] = row;
    }
  }
  count_add(P.stats, finished);
}

template <int KIND>
struct MatOps {
  static __device__ __forceinline__ BsdfSample sample(const Bsdf& b, f3 wo, float u, float v, float w) {
    if (KIND == MAT_GLASS) return b.glass_sample(wo, u);
    if (KIND == MAT_METAL) return b.metal_sample(wo, u, v, w);
    if (KIND == MAT_DISNEY15) return b.d15_sample(wo, u, v, w);
    return KIND == MAT_PHONG ? b.phong_sample_agg(wo, u, v, w) : b.disney_sample(wo, u, v, w);
  }
  static __device__ __forceinline__ f3 eval(const Bsdf& b, f3 wi, f3 wo) {
    if (KIND == MAT_GLASS) return mk3(0.0f, 0.0f, 0.0f);
    if (KIND == MAT_METAL) return b.metal_eval(wi, wo);
    if (KIND == MAT_DISNEY15) return b.d15_eval(wi, wo);
    return KIND == MAT_PHONG ? b.phong_eval_agg(wi, wo) : b.disney_eval(wi, wo);
  }
  static __device__ __forceinline__ float pdf(const Bsdf& b, f3 wi, f3 wo) {
    if (KIND == MAT_GLASS) return 0.0f;
    if (KIND == MAT_METAL) return b.metal_pdf(wi, wo);
    if (KIND == MAT_DISNEY15) return b.d15_pdf(wi, wo);
    return KIND == MAT_PHONG ? b.phong_pdf_agg(wi, wo) : b.disney_pdf(wi, wo);
  }
};

// Guided directions at a Lambertian vertex (Phong with no specular lobe, not
// a fringe vertex). The integrand is exactly what the plain sampler returns
// for a direction -- diffuse_coef times the normal correction, zero where
// the plain sampler rejects (cosine pdf below 0.001) -- and the BSDF's
// density there is the cosine pdf, so a one-sample MIS of the network's
// mixture (probability alpha) and the BSDF keeps the plain estimator's
// expectation.
__device__ __forceinline__ float lambert_plain_pdf(const Bsdf& bsdf, f3 wo, f3 wi) {
  const f3 lwo = normalize(to_local(bsdf.s, wo)), lwi = normalize(to_local(bsdf.s, wi));
  const float pb = cosine_pdf(lwi.z);
  return (lwo.z > 0.0f && pb >= 0.001f) ? pb : 0.0f;
}

// Replaces the plain sample `bs` by the one-sample MIS choice: with
// probability alpha (sel < alpha) a mixture direction, else the plain
// sample itself (which may be invalid: then nothing is returned). ps, nc
// and pm receive the plain sampler's density at the chosen direction, the
// normal correction of its integrand (0 where that density is 0) and the
// mixture's density.
__device__ __noinline__ void guided_pick(const Launch& P, const Bsdf& bsdf, const Isect& is, unsigned int row,
                                         float sel, float g0, float g1, BsdfSample& bs, float& ps, float& nc,
                                         float& pm) {
  const Mixture mx{P.gout + (size_t)row * kMixFloats};
  f3 wi;
  if (sel < P.guide_alpha) {
    wi = normalize(mx.sample(sel / P.guide_alpha, g0, g1));
  } else {
    if (!bs.valid()) return;
    wi = bs.wi;
  }
  ps = lambert_plain_pdf(bsdf, is.wo, wi);
  nc = ps > 0.0f ? normal_correct(bsdf.g, bsdf.s, wi) : 0.0f;
  pm = mx.pdf(wi);
  bs.wi = wi;
  bs.f = muls(bsdf.m->diffuse_coef, nc);
  bs.pdf = P.guide_alpha * pm + (1.0f - P.guide_alpha) * ps;
}

// A guided vertex's ray for one MIS strategy of its direct lighting: its
// direction, the densities of the strategies there and what the direct
// integrand needs (the BSDF's eval and pdf, the plain sampler's density,
// the normal correction, |cos|).
struct GuidedRay {
  f3 wi, fe;
  float p_mix, p_g, pb, ps, nc, cosv;
  bool trace;  // the direct integrand can be non-zero along it
};

// The mixture ray: a direction drawn from the mixture alone (lobe u, v, w).
__device__ __noinline__ void guided_mixture_ray(const Launch& P, const Bsdf& bsdf, const Isect& is, unsigned int row,
                                                float u, float v, float w, GuidedRay& r) {
  const Mixture mx{P.gout + (size_t)row * kMixFloats};
  r.wi = normalize(mx.sample(u, v, w));
  r.p_mix = mx.pdf(r.wi);
  r.ps = lambert_plain_pdf(bsdf, is.wo, r.wi);
  r.nc = r.ps > 0.0f ? normal_correct(bsdf.g, bsdf.s, r.wi) : 0.0f;
  r.p_g = P.guide_alpha * r.p_mix + (1.0f - P.guide_alpha) * r.ps;
  const f3 wc = normalize(r.wi);
  r.fe = bsdf.phong_eval_agg(wc, is.wo);
  r.pb = bsdf.phong_pdf_agg(wc, is.wo);
  r.cosv = abs_cos(is.g.z, wc);
  r.trace = r.p_mix >= kEps && (r.ps > 0.0f || !black(r.fe));
}

// Next-event estimation at a guided vertex: the light sample of direction
// wl, weighted against the guided continuation (density p_g at wl) and,
// when the vertex also traced a mixture ray, the mixture (p_mix), instead
// of the plain BSDF sample. With guided_strategy_emission it estimates the
// same direct-lighting integral as the reference's pair of strategies.
// Returns that integrand times |cos| per unit emission, times the weight.
__device__ __noinline__ f3 guided_nee_factor(const Launch& P, const Bsdf& bsdf, f3 wo, f3 wl, int row, bool three,
                                             float lpdf, float lq) {
  const Mixture mx{P.gout + (size_t)row * kMixFloats};
  const float ps = lambert_plain_pdf(bsdf, wo, wl);
  const f3 fs = ps > 0.0f ? muls(bsdf.m->diffuse_coef, normal_correct(bsdf.g, bsdf.s, wl)) : mk3(0.0f, 0.0f, 0.0f);
  const f3 g = direct_integrand(bsdf.phong_eval_agg(wl, wo), bsdf.phong_pdf_agg(wl, wo), fs, ps, lpdf, lq);
  const float pm = mx.pdf(wl);
  const float pg = P.guide_alpha * pm + (1.0f - P.guide_alpha) * ps;
  const float po = three ? pm : 0.0f;
  const float w = lpdf * lpdf / (lpdf * lpdf + pg * pg + po * po);
  return muls(g, abs_cos(wl, bsdf.g.z) * w);
}

// The BSDF sample, shared out of line by the two call sites of k_material
// (the path's sample and the MIS sample): one copy of the sampling code
// instead of two keeps the kernel within the instruction cache.
template <int KIND>
__device__ __noinline__ BsdfSample sample_bsdf_shared(const Bsdf& b, f3 wo, float u, float v, float w) {
  return MatOps<KIND>::sample(b, wo, u, v, w);
}

// One path vertex on a material of kind KIND: the body of eval_pixel_li
// from the BSDF sample to the next continuation ray
// (src/renderer/path_trace_renderer.cpp:125-163).
// Resident blocks per SM, measured on the room: Phong runs faster at five
// (96 registers, little spill) than at eight (64 registers, ~200 bytes of
// spill), Disney12 the other way round.
template <int KIND, bool GUIDED = false>
__global__ void __launch_bounds__(128, KIND == MAT_DISNEY12 ? 8 : 5) k_material(Launch P, int cur) {
  const int nxt = cur ^ 1;
  const unsigned int n = P.ctr[C_MAT + KIND];
  unsigned int finished = 0;
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int slot = P.q_mat[KIND][i];
    unsigned long long st = P.rng[slot];
    const float4 p0 = P.P0[slot], p1 = P.P1[slot], p2 = P.P2[slot];
    const f3 ro = mk3(p0.x, p0.y, p0.z), rd = mk3(p1.x, p1.y, p1.z);
    int depth = path_depth(p1.w), sdepth = spec_depth(p1.w);
    f3 coef = mk3(p2.x, p2.y, p2.z);
    const float4 hit = P.HC[slot];
    Isect is;
    make_isect(P.sc, hit, ro, rd, is);
    int mat = P.sc.prims[is.prim].material;
    Bsdf bsdf;
    bsdf.m = P.sc.mats + mat;
    if (P.MT && bsdf.m->tex_any) {
      // image maps: the material set up at this hit's uv, in the slot's record
      float u, v;
      hit_uv(P.sc, hit, ro, rd, u, v);
      material_at(P.sc, mat, u, v, P.MT + slot);
      bsdf.m = P.MT + slot;
      mat |= kMatScratch;
    }
    bsdf.g = is.g;
    bsdf.s = is.s;
    const float u0 = Pcg::next(st), u1 = Pcg::next(st), u2 = Pcg::next(st);
    BsdfSample bs = sample_bsdf_shared<KIND>(bsdf, is.wo, u0, u1, u2);
    if (black(bs.f) || bs.pdf < kEps) {
      const float4 p3 = P.P3[slot];
      finish_sample(P, slot, st, mk3(p3.x, p3.y, p3.z), nxt, finished);
      P.rng[slot] = st;
      continue;
    }
    // Guided continuation. The plain sample above still decides, as in the
    // reference, whether this vertex gets direct lighting at all; a guided
    // direction without contribution only ends the path after it.
    // At a guided vertex the continuation is also an MIS strategy of the
    // direct lighting (traced even when the path ends here, as long as the
    // integrand can be non-zero along it), so emission it reaches counts.
    bool guided_end = false, g_trace = false;
    float g_ps = 0.0f, g_nc = 0.0f, g_pb = 0.0f, g_cos = 0.0f, g_pm = 0.0f;
    f3 g_fe = mk3(0.0f, 0.0f, 0.0f);
    const int row = GUIDED && KIND == MAT_PHONG && P.guide_alpha > 0.0f ? P.grow[slot] : -1;
    const bool gv = GUIDED && KIND == MAT_PHONG && P.guide_alpha > 0.0f && row >= 0 && bsdf.m->w_specular == 0.0f &&
                    !bsdf.fringe(is.wo);
    if (gv) {
      const float sel = Pcg::next(st), g0 = Pcg::next(st), g1 = Pcg::next(st);
      guided_pick(P, bsdf, is, row, sel, g0, g1, bs, g_ps, g_nc, g_pm);
      guided_end = black(bs.f) || bs.pdf < kEps;
      if (bs.pdf >= kEps) {
        const f3 wc = normalize(normalize(bs.wi));
        g_fe = bsdf.phong_eval_agg(wc, is.wo);
        g_pb = bsdf.phong_pdf_agg(wc, is.wo);
        g_cos = abs_cos(is.g.z, wc);
        g_trace = !black(bs.f) || !black(g_fe);
      }
    }
    // next-event estimation on every light (sample_area_light): the draws
    // happen here, the rest in k_nee
    const JobDev& J = job_of(P, slot);
    const float pos_mag = fabsf(is.pos.x) + fabsf(is.pos.y) + fabsf(is.pos.z);
    for (int l = 0; l < J.nl; ++l) {
      const int item = slot * P.nl_max + l;
      // A vertex well behind a light's plane gets nothing from it:
      // k_nee's test dot(n, pos - light point) > 0 fails for every point
      // of the (planar) light. The margin covers the rounding of the
      // sampled point and of that dot product, so only items the exact test
      // would reject are skipped here (their five draws only advance the
      // stream). Of a kept light's five draws the sample uses the first two.
      const DLight& lt = P.sc.lights[J.light_base + l];
      const float side = dot(lt.gz, is.pos - lt.A);
      const float tol = 1e-4f * (pos_mag + lt.extent);
      if (side < -tol) {
        Pcg::skip<5>(st);
        P.SHC[item] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        continue;
      }
      const float lu = Pcg::next(st), lv = Pcg::next(st);
      Pcg::skip<3>(st);
      P.NU[item] = make_float2(lu, lv);
      P.q_nee[nee_index(KIND)][append(P.ctr + C_NEE + nee_index(KIND))] = item;
    }
    float4* sc = P.SC + 7 * (size_t)slot;
    sc[0] = make_float4(is.pos.x, is.pos.y, is.pos.z, __int_as_float(mat));
    sc[1] = make_float4(is.wo.x, is.wo.y, is.wo.z, is.g.x.x);
    sc[2] = make_float4(is.g.x.y, is.g.x.z, is.g.y.x, is.g.y.y);
    sc[3] = make_float4(is.g.y.z, is.g.z.x, is.g.z.y, is.g.z.z);
    sc[4] = make_float4(is.s.x.x, is.s.x.y, is.s.x.z, is.s.y.x);
    sc[5] = make_float4(is.s.y.y, is.s.y.z, is.s.z.x, is.s.z.y);
    // MIS BSDF ray (sample_bsdf, src/renderer/direct_illumination.cpp:144-155);
    // a guided vertex draws a direction from the mixture alone instead
    int flags = F_PENDING;
    GuidedRay gx;
    gx.trace = false;
    if (gv) {
      const float x0 = Pcg::next(st), x1 = Pcg::next(st), x2 = Pcg::next(st);
      guided_mixture_ray(P, bsdf, is, row, x0, x1, x2, gx);
    } else {
      const float v0 = Pcg::next(st), v1 = Pcg::next(st), v2 = Pcg::next(st);
      const BsdfSample ms = sample_bsdf_shared<KIND>(bsdf, is.wo, v0, v1, v2);
      if (ms.valid()) {
        const f3 wi = normalize(ms.wi);
        const f3 mo = is.eps_offset(wi);
        const f3 md = normalize(wi);
        P.M0[slot] = make_float4(mo.x, mo.y, mo.z, ms.pdf);
        P.M1[slot] = make_float4(md.x, md.y, md.z, abs_cos(is.g.z, md));
        P.M2[slot] = make_float4(ms.f.x, ms.f.y, ms.f.z, 0.0f);
        if (P.mis_all || mis_may_hit_light(P.sc, J, mo, md))
          P.q_ext[nxt][append(P.ctr + C_EXT + nxt)] = 2 * slot + 1;
        else
          P.HM[slot] = make_float4(__int_as_float(-1), 0.0f, 0.0f, 0.0f);  // the zero of a miss
        flags |= F_MIS;
      }
    }
    P.P4[slot] = make_float4(coef.x, coef.y, coef.z, P.P4[slot].w);
    coef = mulc(coef, divs(muls(bs.f, abs_cos(is.g.z, bs.wi)), bs.pdf));
    bool term = guided_end || !valid3(coef);
    if (!term) {
      ++depth;
      if (depth >= J.max_depth) {
        term = true;
      } else if (depth > J.min_depth) {
        if (Pcg::next(st) > 0.9f) term = true;
        else {
          coef = divs(coef, 0.9f);
          if (!valid3(coef)) term = true;
        }
      }
    }
    // The guided strategies of the direct lighting. A path that ends here
    // traces its continuation in the MIS slot for its emission only (next-
    // event estimation and the continuation); a path that goes on traces
    // the continuation (hit in HC, its data in GX) and the mixture ray in
    // the MIS slot (three strategies; bit 30 of the shading context's row
    // tells k_nee).
    int gcode = gv ? row : -1;
    float sc6z = 0.0f, sc6w = 0.0f;
    if (gv && g_trace) {
      const f3 mo = is.eps_offset(bs.wi);
      const f3 md = normalize(normalize(bs.wi));
      flags |= F_GCONT;
      if (term) {
        P.M0[slot] = make_float4(mo.x, mo.y, mo.z, bs.pdf);
        P.M1[slot] = make_float4(md.x, md.y, md.z, g_pb);
        P.M2[slot] = make_float4(g_fe.x, g_fe.y, g_fe.z, g_ps);
        sc6z = g_nc;
        sc6w = g_cos;
        // (as the plain MIS ray: its emission is all it gives)
        if (P.mis_all || mis_may_hit_light(P.sc, J, mo, md))
          P.q_ext[nxt][append(P.ctr + C_EXT + nxt)] = 2 * slot + 1;
        else
          P.HM[slot] = make_float4(__int_as_float(-1), 0.0f, 0.0f, 0.0f);
      } else {
        gcode |= 1 << 30;
        float4* gxr = P.GX + 4 * (size_t)slot;
        gxr[0] = make_float4(mo.x, mo.y, mo.z, bs.pdf);
        gxr[1] = make_float4(md.x, md.y, md.z, g_pb);
        gxr[2] = make_float4(g_fe.x, g_fe.y, g_fe.z, g_ps);
        gxr[3] = make_float4(g_nc, g_cos, g_pm, gx.p_g);
        if (gx.trace) {
          const f3 xo = is.eps_offset(gx.wi);
          const f3 xd = normalize(gx.wi);
          P.M0[slot] = make_float4(xo.x, xo.y, xo.z, gx.p_mix);
          P.M1[slot] = make_float4(xd.x, xd.y, xd.z, gx.pb);
          P.M2[slot] = make_float4(gx.fe.x, gx.fe.y, gx.fe.z, gx.ps);
          sc6z = gx.nc;
          sc6w = gx.cosv;
          flags |= F_GX;
          if (P.mis_all || mis_may_hit_light(P.sc, J, xo, xd))
            P.q_ext[nxt][append(P.ctr + C_EXT + nxt)] = 2 * slot + 1;
          else
            P.HM[slot] = make_float4(__int_as_float(-1), 0.0f, 0.0f, 0.0f);
        }
      }
    }
    sc[6] = make_float4(is.s.z.z, __int_as_float(gcode), sc6z, sc6w);
    if (term) {
      flags |= F_TERMINATE;
      P.P0[slot] = make_float4(p0.x, p0.y, p0.z, __int_as_float(flags));
    } else {
      const f3 no = is.eps_offset(bs.wi);
      const f3 nd = normalize(normalize(bs.wi));
      if (P.guide_record && __float_as_int(p2.w) % P.guide_record == 0) {
        const int nv = P.NV[slot];
        if (nv < P.maxd) {
          float f[7];
          const float t = P.HC[slot].y;
          guide_features(P, ro + scale(rd, t), -rd, KIND == MAT_PHONG ? 1.0f : bsdf.m->roughness, f);
          float4* r = P.VR + ((size_t)slot * P.maxd + nv) * 4;
          r[0] = make_float4(f[0], f[1], f[2], f[3]);
          // training target: incident radiance times |cos| (the Lambertian
          // product), over the pdf the direction was drawn with
          r[1] = make_float4(f[4], f[5], f[6], bs.pdf / fmaxf(abs_cos(is.g.z, bs.wi), 1e-6f));
          r[2] = make_float4(nd.x, nd.y, nd.z, lum(coef));
          P.NV[slot] = nv + 1;
          flags |= F_REC;
        }
      }
      P.P0[slot] = make_float4(no.x, no.y, no.z, __int_as_float(flags));
      P.P1[slot] = make_float4(nd.x, nd.y, nd.z, __int_as_float(depth | sdepth << 16));
      P.q_ext[nxt][append(P.ctr + C_EXT + nxt)] = 2 * slot;
    }
    P.P2[slot] = make_float4(coef.x, coef.y, coef.z, p2.w);
    P.q_act[nxt][append(P.ctr + C_ACT + nxt)] = slot;
    P.rng[slot] = st;
  }
  count_add(P.stats, finished);
}

// A vertex on glass, a delta BSDF (src/material/glass.cpp:29-80): the body of
// eval_pixel_li for a delta sample (src/renderer/path_trace_renderer.cpp:125-163).
// No direct lighting (and no draws for it); up to kMaxSpecularDepth delta
// samples of a path do not count toward its depth; the emission the next
// ray reaches counts (F_SPEC, read by k_logic).
__global__ void __launch_bounds__(128) k_glass(Launch P, int cur) {
  const int nxt = cur ^ 1;
  const unsigned int n = P.ctr[C_MAT + MAT_GLASS];
  unsigned int finished = 0;
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int slot = P.q_mat[MAT_GLASS][i];
    unsigned long long st = P.rng[slot];
    const float4 p0 = P.P0[slot], p1 = P.P1[slot], p2 = P.P2[slot];
    int depth = path_depth(p1.w), sdepth = spec_depth(p1.w);
    f3 coef = mk3(p2.x, p2.y, p2.z);
    Isect is;
    make_isect(P.sc, P.HC[slot], mk3(p0.x, p0.y, p0.z), mk3(p1.x, p1.y, p1.z), is);
    Bsdf bsdf;
    bsdf.m = P.sc.mats + P.sc.prims[is.prim].material;
    if (P.MT && bsdf.m->tex_any) {  // image maps: the material at this hit's uv
      float u, v;
      hit_uv(P.sc, P.HC[slot], mk3(p0.x, p0.y, p0.z), mk3(p1.x, p1.y, p1.z), u, v);
      material_at(P.sc, P.sc.prims[is.prim].material, u, v, P.MT + slot);
      bsdf.m = P.MT + slot;
    }
    bsdf.g = is.g;
    bsdf.s = is.s;
    const float u0 = Pcg::next(st);
    Pcg::skip<2>(st);  // the rest of sample3()
    const BsdfSample bs = bsdf.glass_sample(is.wo, u0);
    bool term = black(bs.f) || bs.pdf < kEps;
    if (!term) {
      const bool counted = sdepth >= kMaxSpecularDepth;
      if (!counted) ++sdepth;
      coef = mulc(coef, divs(muls(bs.f, abs_cos(is.g.z, bs.wi)), bs.pdf));
      term = !valid3(coef);
      if (!term) {
        if (counted) ++depth;
        const JobDev& J = job_of(P, slot);
        if (depth >= J.max_depth) {
          term = true;
        } else if (depth > J.min_depth) {
          if (Pcg::next(st) > 0.9f) term = true;
          else {
            coef = divs(coef, 0.9f);
            if (!valid3(coef)) term = true;
          }
        }
      }
    }
    if (term) {
      const float4 p3 = P.P3[slot];
      finish_sample(P, slot, st, mk3(p3.x, p3.y, p3.z), nxt, finished);
      P.rng[slot] = st;
      continue;
    }
    const f3 no = is.eps_offset(bs.wi);
    const f3 nd = normalize(normalize(bs.wi));
    P.P0[slot] = make_float4(no.x, no.y, no.z, __int_as_float(F_SPEC));
    P.P1[slot] = make_float4(nd.x, nd.y, nd.z, __int_as_float(depth | sdepth << 16));
    P.P2[slot] = make_float4(coef.x, coef.y, coef.z, p2.w);
    P.q_ext[nxt][append(P.ctr + C_EXT + nxt)] = 2 * slot;
    P.q_act[nxt][append(P.ctr + C_ACT + nxt)] = slot;
    P.rng[slot] = st;
  }
  count_add(P.stats, finished);
}

// sample_environment_light (src/renderer/direct_illumination.cpp:73-106) for
// one (vertex, environment light) item; false: no shadow ray. gcode: the
// guided vertex's network row (bit 30: three strategies), else -1.
template <int KIND>
__device__ __noinline__ bool nee_env_item(const Launch& P, int item, int slot, int env, f3 pos, f3 wo,
                                          const Bsdf& bsdf, float2 uv, int gcode, float4* rec, float4* recc) {
  bool ok = false;
  // sample_environment_light (src/renderer/direct_illumination.cpp:73-106)
  f3 Le, lpos;
  float lpdf;
  if (env_sample(P.sc.envs[env], pos, uv.x, uv.y, Le, lpdf, lpos) && !black(Le)) {
    f3 to_light = lpos - pos;
    bool too_close;
    const float dist = dist_minus_eps(len2f(to_light), too_close);
    if (!too_close) {
      to_light = normalize(to_light);
      const float4 p4 = P.P4[slot];
      f3 cc = mk3(0.0f, 0.0f, 0.0f);
      bool trace = false;
      if (KIND == MAT_PHONG && gcode >= 0) {
        const f3 fw = guided_nee_factor(P, bsdf, wo, to_light, gcode & 0x3fffffff, (gcode >> 30) & 1, lpdf,
                                        env_pdf(P.sc.envs[env], normalize(to_light)));
        trace = !black(fw);
        cc = mulc(mk3(p4.x, p4.y, p4.z), divs(mulc(Le, fw), lpdf));
      } else {
        const f3 bf = MatOps<KIND>::eval(bsdf, to_light, wo);
        trace = !black(bf);
        if (trace) {
          const float bpdf = MatOps<KIND>::pdf(bsdf, to_light, wo);
          const f3 fl = muls(mulc(Le, bf), abs_cos(to_light, bsdf.g.z));
          const float w = power_heuristic(lpdf, bpdf);
          cc = mulc(mk3(p4.x, p4.y, p4.z), divs(muls(fl, w), lpdf));
        }
      }
      if (trace) {
        const f3 sd = normalize(to_light);
        rec[0] = make_float4(pos.x, pos.y, pos.z, dist);
        rec[1] = make_float4(sd.x, sd.y, sd.z, 0.0f);
        *recc = make_float4(cc.x, cc.y, cc.z, 1.0f);
        P.q_sh[append(P.ctr + C_SH)] = item;
        ok = true;
      }
    }
  }
  return ok;
}

// sample_area_light (src/renderer/direct_illumination.cpp:35-71) for one
// (vertex, light) pair: the shadow ray is traced by k_shadow, which zeroes
// the contribution when it is blocked.
// Six resident blocks per SM (80 registers, a few bytes of spill) measured
// faster than the five its free allocation (91 registers) allows.
template <int KIND, bool MAPS = false>  // MAPS: hits of materials with image maps carry per-slot set-ups
__global__ void __launch_bounds__(128, 6) k_nee(Launch P) {
  const unsigned int n = P.ctr[C_NEE + nee_index(KIND)];
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int item = P.q_nee[nee_index(KIND)][i];
    const int slot = item / P.nl_max, l = item - slot * P.nl_max;
    const float4* sc = P.SC + 7 * (size_t)slot;
    const float4 a = sc[0], b = sc[1], c = sc[2], d = sc[3], e = sc[4], f = sc[5], g = sc[6];
    const f3 pos = mk3(a.x, a.y, a.z), wo = mk3(b.x, b.y, b.z);
    Bsdf bsdf;
    const int mcode = __float_as_int(a.w);
    bsdf.m = (MAPS && (mcode & kMatScratch)) ? P.MT + slot : P.sc.mats + mcode;
    bsdf.g.x = mk3(b.w, c.x, c.y);
    bsdf.g.y = mk3(c.z, c.w, d.x);
    bsdf.g.z = mk3(d.y, d.z, d.w);
    bsdf.s.x = mk3(e.x, e.y, e.z);
    bsdf.s.y = mk3(e.w, f.x, f.y);
    bsdf.s.z = mk3(f.z, f.w, g.x);
    const float2 uv = P.NU[item];
    const DLight& lt = P.sc.lights[job_of(P, slot).light_base + l];
    float4* rec = P.SH + 2 * (size_t)item;
    float4* recc = P.SHC + item;
    bool ok = false;
    if (lt.env >= 0) {  // out of line: its registers would otherwise count for every item
      if (!nee_env_item<KIND>(P, item, slot, lt.env, pos, wo, bsdf, uv, __float_as_int(g.y), rec, recc))
        *recc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      continue;
    }
    // Triangle::sample via UniformSampleTriangle (src/shape/triangle.cpp:61-97),
    // at the light table's point of the sample square when it is learned
    float2 su = uv;
    int lbin = 0;
    float lratio = 1.0f;
    if (P.lg_cdf) su = lg_sample(P, lg_table(P, pos, l), uv, lbin, lratio);
    const float su0 = sqrtf(su.x);
    const float bx = 1.0f - su0, by = su.y * su0;
    const f3 lpos = scale(lt.A, bx) + scale(lt.B, by) + scale(lt.C, 1.0f - bx - by);
    const f3 sp2ref = pos - lpos;
    if (dot(lt.gz, sp2ref) > 0.0f) {
      const float dist2 = len2f(sp2ref);
      const float lpdf = area_to_solid_pdf(lt.area_pdf * dist2, dot(lt.gz, sp2ref), dist2);
      if (lpdf) {
        f3 to_light = lpos - pos;
        bool too_close;
        const float dist = dist_minus_eps(len2f(to_light), too_close);
        if (!too_close) {
          to_light = normalize(to_light);
          const int gcode = __float_as_int(g.y);  // guided vertex: network row (bit 30: three strategies), else -1
          const int grow = gcode < 0 ? -1 : (gcode & 0x3fffffff);
          f3 cc = mk3(0.0f, 0.0f, 0.0f);          // contribution before the shadow test
          bool trace = false;
          const float4 p4 = P.P4[slot];
          // the estimate per unit path throughput; a learned light sample's
          // is divided by the table's density over the uniform one (the MIS
          // weights stay those of the uniform sample)
          f3 inner = mk3(0.0f, 0.0f, 0.0f);
          if (KIND == MAT_PHONG && grow >= 0) {
            const f3 fw = guided_nee_factor(P, bsdf, wo, to_light, grow, (gcode >> 30) & 1, lpdf, lpdf);
            trace = !black(fw);
            inner = divs(mulc(lt.emission, fw), lpdf);
          } else {
            const f3 bf = MatOps<KIND>::eval(bsdf, to_light, wo);
            trace = !black(bf);
            if (trace) {
              const float bpdf = MatOps<KIND>::pdf(bsdf, to_light, wo);
              const f3 fl = muls(mulc(lt.emission, bf), abs_cos(to_light, bsdf.g.z));
              const float w = power_heuristic(lpdf, bpdf);
              inner = divs(muls(fl, w), lpdf);
            }
          }
          if (P.lg_cdf) inner = muls(inner, lratio);
          cc = mulc(mk3(p4.x, p4.y, p4.z), inner);
          if (trace) {
            const f3 sd = normalize(to_light);
            rec[0] = make_float4(pos.x, pos.y, pos.z, dist);
            // statistics of the light table: the estimate's luminance, the bin + 1
            rec[1] = make_float4(sd.x, sd.y, sd.z, P.lg_acc ? lum(inner) : 0.0f);
            *recc = make_float4(cc.x, cc.y, cc.z, P.lg_acc ? (float)(lbin + 1) : 1.0f);
            P.q_sh[append(P.ctr + C_SH)] = item;
            ok = true;
          }
        }
      }
    }
    if (!ok) *recc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

void release_render(tr_ctx* ctx) {
  if (!ctx->rb) return;
  RenderBuffers* rb = ctx->rb;
  for (DevBuf* b : {&rb->P0, &rb->P1, &rb->P2, &rb->P3, &rb->P4, &rb->rng, &rb->M0, &rb->M1, &rb->M2, &rb->HC,
                    &rb->HM, &rb->SC, &rb->NU, &rb->SH, &rb->SHC, &rb->acc, &rb->q_ext, &rb->q_act, &rb->q_mat, &rb->q_nee,
                    &rb->q_sh, &rb->ctr, &rb->stats, &rb->VR, &rb->NV, &rb->gfeat, &rb->gout, &rb->tb, &rb->jobs,
                    &rb->GX, &rb->grow, &rb->MT, &rb->q_srt, &rb->bin_key, &rb->bin_cnt, &rb->OC, &rb->q_ord,
                    &rb->act_flag})
    b->release();
  if (rb->h_active) cudaFreeHost(rb->h_active);
  for (cudaEvent_t e : rb->ev_pool) cudaEventDestroy(e);
  delete rb;
  ctx->rb = nullptr;
}

namespace {

tr_status reserve_render(tr_ctx* ctx, int n, int nl) {
  if (!ctx->rb) ctx->rb = new RenderBuffers();
  RenderBuffers* rb = ctx->rb;
  const size_t N = (size_t)n;
  const size_t NL = (size_t)std::max(nl, 1);
  const size_t f4 = sizeof(float4);
  struct Need {
    DevBuf* b;
    size_t bytes;
  } needs[] = {{&rb->P0, N * f4},           {&rb->P1, N * f4},          {&rb->P2, N * f4},
               {&rb->P3, N * f4},           {&rb->P4, N * f4},          {&rb->rng, N * 8},
               {&rb->M0, N * f4},           {&rb->M1, N * f4},          {&rb->M2, N * f4},
               {&rb->HC, N * f4},           {&rb->HM, N * f4},          {&rb->SC, N * 7 * f4},
               {&rb->NU, N * NL * 8},       {&rb->SH, N * NL * 2 * f4}, {&rb->SHC, N * NL * f4}, {&rb->acc, N * 32},
               {&rb->q_ext, 2 * 2 * N * 4}, {&rb->q_act, 2 * N * 4},   {&rb->q_mat, kMatKinds * N * 4},
               {&rb->q_nee, kNeeKinds * N * NL * 4}, {&rb->q_sh, N * NL * 4},  {&rb->ctr, kCtrWords * 4},
               {&rb->stats, kStatWords * 8}};
  for (auto& nd : needs) {
    cudaError_t e = nd.b->reserve(nd.bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "render buffer allocation");
  }
  if (!rb->h_active) {
    cudaError_t e = cudaHostAlloc((void**)&rb->h_active, 64, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "pinned counter allocation");
  }
  rb->n = n;
  rb->nl = nl;
  return TR_OK;
}

void setup_camera(Cam& c, const tr_camera& p) {
  // look_at (src/utility/transform.cpp:96-124) and the ThinLensCamera
  // constructor (src/camera/thin_lens_camera.cpp:23-36), host arithmetic
  const f3 pos = mk3(p.pos[0], p.pos[1], p.pos[2]), target = mk3(p.target[0], p.target[1], p.target[2]);
  const f3 up = mk3(p.up[0], p.up[1], p.up[2]);
  const f3 dir = normalize(target - pos);
  const f3 right = normalize(cross(normalize(up), dir));
  const f3 new_up = cross(dir, right);
  const float m[16] = {right.x, new_up.x, dir.x, pos.x, right.y, new_up.y, dir.y, pos.y,
                       right.z, new_up.z, dir.z, pos.z, 0.0f,    0.0f,     0.0f,  1.0f};
  std::memcpy(c.m, m, sizeof(m));
  c.focal = p.focal_dist;
  c.lens_radius = p.lens_radius;
  c.film_h = (float)(2 * p.focal_dist * std::tan(p.fov * 0.5));
  c.film_w = p.film_aspect * c.film_h;
}

}  // namespace

// One render of a batch as the host describes it.
struct JobSpec {
  int scene;
  tr_camera cam;
  tr_filter filter;
  tr_render_params prm;
  void* film;  // device sums (float4 or 2 x double2 per pixel); null: the context's film buffer
  bool fp64;
};

static tr_status validate_job(tr_ctx* ctx, const JobSpec& j) {
  const tr_render_params* prm = &j.prm;
  if (j.scene < 0 || j.scene >= ctx->dsc.num_scenes) return set_err(ctx, TR_ERR_ARG, "scene index out of range");
  if (prm->width <= 0 || prm->height <= 0 || prm->spp <= 0 || prm->max_depth < 0)
    return set_err(ctx, TR_ERR_ARG, "invalid render size, spp or depth");
  if (prm->max_depth > kMaxPathDepth)
    return set_err(ctx, TR_ERR_ARG, "max_depth above 65515 (the path depth is kept in 16 bits)");
  if ((long long)prm->width * prm->height > (1ll << 28)) return set_err(ctx, TR_ERR_ARG, "film too large");
  if (prm->direct_light_sample_num != 1)
    return set_err(ctx, TR_ERR_UNSUPPORTED, "direct_light_sample_num must be 1 on the GPU path");
  if (!(j.filter.radius > 0.0f) || j.filter.radius > 16.0f) return set_err(ctx, TR_ERR_ARG, "invalid filter radius");
  if (j.film && ((uintptr_t)j.film & 15u) != 0) return set_err(ctx, TR_ERR_ARG, "film buffer must be 16-byte aligned");
  return TR_OK;
}

static JobDev make_job_dev(tr_ctx* ctx, const JobSpec& j, int slot_base, void* film) {
  JobDev J;
  std::memset(&J, 0, sizeof(J));
  setup_camera(J.cam, j.cam);
  J.W = j.prm.width;
  J.H = j.prm.height;
  J.spp = j.prm.spp;
  J.min_depth = j.prm.min_depth;
  J.max_depth = j.prm.max_depth;
  J.seed_base = j.prm.seed_base;
  J.scene = j.scene;
  J.slot_base = slot_base;
  J.light_base = (int)ctx->hs.scene_light[j.scene];
  J.nl = (int)ctx->hs.scene_nlight[j.scene];
  J.env = J.nl > 0 ? ctx->hs.lights[J.light_base + J.nl - 1].env : -1;
  J.mis_always = ctx->hs.scene_unlisted[j.scene];
  // the sphere of mis_may_hit_light: around the box of the area-light
  // triangles as the triangle test sees them (A, A + AB, A + AC), widened
  // by 1e-3 of the radius and of the coordinates' scale
  {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, scale = 1.0;
    int tris = 0;
    for (int l = 0; l < J.nl; ++l) {
      const DLight& L = ctx->hs.lights[J.light_base + l];
      if (L.env >= 0) continue;
      const double A[3] = {L.A.x, L.A.y, L.A.z}, AB[3] = {L.AB.x, L.AB.y, L.AB.z}, AC[3] = {L.AC.x, L.AC.y, L.AC.z};
      for (int k = 0; k < 3; ++k)
        for (double v : {A[k], A[k] + AB[k], A[k] + AC[k]}) {
          lo[k] = std::min(lo[k], v);
          hi[k] = std::max(hi[k], v);
          scale = std::max(scale, std::fabs(v));
        }
      ++tris;
    }
    if (tris) {
      double r2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        J.lsph[k] = (float)(0.5 * (lo[k] + hi[k]));
        const double e = 0.5 * (hi[k] - lo[k]) + std::fabs(0.5 * (lo[k] + hi[k]) - (double)J.lsph[k]);
        r2 += e * e;
      }
      J.lsph[3] = (float)(std::sqrt(r2) * (1.0 + 1e-3) + 1e-3 * scale);
      J.lsph_cn = (float)std::sqrt((double)J.lsph[0] * J.lsph[0] + (double)J.lsph[1] * J.lsph[1] +
                                   (double)J.lsph[2] * J.lsph[2]);
    } else {
      J.lsph[3] = -1.0f;
    }
  }
  J.filter_radius = j.filter.radius;
  J.filter_alpha = j.filter.alpha;
  J.filter_exp = std::exp(-j.filter.alpha * j.filter.radius * j.filter.radius);  // GaussianFilter ctor
  J.fp64 = j.fp64 ? 1 : 0;
  J.film = static_cast<float4*>(film);
  return J;
}

tr_status render_jobs(tr_ctx* ctx, const JobSpec* jobs, int njobs, uint32_t flags, tr_stats* stats,
                      const tr_guide_params* gp = nullptr) {
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (njobs <= 0) return set_err(ctx, TR_ERR_ARG, "no jobs");
  long long total = 0;
  // every slot finishes within spp * (max_depth + 2) iterations, plus the
  // delta samples that do not count toward the depth
  long long max_iters = 0;
  const int extra = ctx->dsc.has_glass ? kMaxSpecularDepth : 0;
  for (int k = 0; k < njobs; ++k) {
    tr_status v = validate_job(ctx, jobs[k]);
    if (v != TR_OK) return v;
    if (!jobs[k].film && njobs != 1) return set_err(ctx, TR_ERR_ARG, "batch jobs need device films");
    total += (long long)jobs[k].prm.width * jobs[k].prm.height;
    max_iters = std::max(max_iters, (long long)jobs[k].prm.spp * ((long long)jobs[k].prm.max_depth + 2 + extra) + 4);
  }
  if (total > (1ll << 28)) return set_err(ctx, TR_ERR_ARG, "batch too large");
  const int n = (int)total;
  const int nl = ctx->dsc.max_lights;
  if ((long long)n * std::max(nl, 1) > (1ll << 30)) return set_err(ctx, TR_ERR_ARG, "too many shadow records");
  tr_status s = reserve_render(ctx, n, nl);
  if (s != TR_OK) return s;
  RenderBuffers* rb = ctx->rb;
  cudaStream_t st = ctx->stream;
  cudaError_t ce = rb->jobs.reserve((size_t)njobs * sizeof(JobDev));
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "job table");
  std::vector<JobDev> jd(njobs);
  {
    int base = 0;
    for (int k = 0; k < njobs; ++k) {
      jd[k] = make_job_dev(ctx, jobs[k], base, jobs[k].film ? jobs[k].film : rb->acc.p);
      base += jobs[k].prm.width * jobs[k].prm.height;
    }
  }
  ce = cudaMemcpyAsync(rb->jobs.p, jd.data(), jd.size() * sizeof(JobDev), cudaMemcpyHostToDevice, st);
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "job table upload");

  Launch P;
  std::memset(&P, 0, sizeof(P));
  P.sc = ctx->dsc;
  P.jobs = rb->jobs.as<JobDev>();
  P.njobs = njobs;
  P.nslots = n;
  P.mis_all = (flags & TR_RENDER_COUNT_VISITS) != 0;
  P.nl_max = std::max(nl, 1);
  P.P0 = rb->P0.as<float4>();
  P.P1 = rb->P1.as<float4>();
  P.P2 = rb->P2.as<float4>();
  P.P3 = rb->P3.as<float4>();
  P.P4 = rb->P4.as<float4>();
  P.rng = rb->rng.as<unsigned long long>();
  P.M0 = rb->M0.as<float4>();
  P.M1 = rb->M1.as<float4>();
  P.M2 = rb->M2.as<float4>();
  P.HC = rb->HC.as<float4>();
  P.HM = rb->HM.as<float4>();
  P.SC = rb->SC.as<float4>();
  P.NU = rb->NU.as<float2>();
  P.SH = rb->SH.as<float4>();
  P.SHC = rb->SHC.as<float4>();
  P.MT = nullptr;
  if (ctx->dsc.has_textures) {
    cudaError_t e = rb->MT.reserve((size_t)n * sizeof(DMat));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "per-slot material set-ups");
    P.MT = rb->MT.as<DMat>();
  }
  for (int k = 0; k < 2; ++k) {
    P.q_ext[k] = rb->q_ext.as<int>() + (size_t)k * 2 * n;
    P.q_act[k] = rb->q_act.as<int>() + (size_t)k * n;
  }
  for (int k = 0; k < kNeeKinds; ++k) P.q_nee[k] = rb->q_nee.as<int>() + (size_t)k * n * std::max(nl, 1);
  for (int k = 0; k < kMatKinds; ++k) P.q_mat[k] = rb->q_mat.as<int>() + (size_t)k * n;
  P.q_sh = rb->q_sh.as<int>();
  P.ctr = rb->ctr.as<unsigned int>();
  P.stats = rb->stats.as<unsigned long long>();
  {
    cudaError_t e;
    if ((e = rb->q_ord.reserve((size_t)n * 4)) != cudaSuccess || (e = rb->act_flag.reserve((size_t)n)) != cudaSuccess)
      return cuda_fail(ctx, e, "ordered live-slot list");
    P.q_ord = rb->q_ord.as<int>();
    P.act_flag = rb->act_flag.as<unsigned char>();
  }
  P.OC = nullptr;
  if (ctx->tune.occluder_cache && ctx->dsc.slot_leaf && !(flags & TR_RENDER_COUNT_VISITS)) {
    // (a counting render keeps the reference's walks: its visit counts are the oracle's)
    const cudaError_t e = rb->OC.reserve((size_t)n * std::max(nl, 1) * 4);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "occluder cache");
    P.OC = rb->OC.as<int>();
  }
  P.bin_bits = ctx->tune.ray_bin_bits;
  if (P.bin_bits) {
    const size_t cap = (size_t)2 * n;
    cudaError_t e;
    if ((e = rb->q_srt.reserve(cap * 4)) != cudaSuccess || (e = rb->bin_key.reserve(cap * 4)) != cudaSuccess ||
        (e = rb->bin_cnt.reserve((size_t)4 << (3 + 3 * P.bin_bits))) != cudaSuccess)
      return cuda_fail(ctx, e, "ray binning buffers");
    P.q_srt = rb->q_srt.as<int>();
    P.bin_key = rb->bin_key.as<unsigned int>();
    P.bin_cnt = rb->bin_cnt.as<unsigned int>();
  }
  if (gp) {
    if (njobs != 1) return set_err(ctx, TR_ERR_ARG, "guided rendering takes one job");
    if (!(gp->alpha >= 0.0f && gp->alpha < 1.0f)) return set_err(ctx, TR_ERR_ARG, "guide alpha must be in [0, 1)");
    if (gp->alpha > 0.0f && (!ctx->guide || !ctx->guide->params.p))
      return set_err(ctx, TR_ERR_STATE, "guide model not initialised");
    for (int k = 0; k < 3; ++k) {
      if (!(gp->box_hi[k] > gp->box_lo[k])) return set_err(ctx, TR_ERR_ARG, "empty guide box");
      P.gbox_lo[k] = gp->box_lo[k];
      P.gbox_scale[k] = 2.0f / (gp->box_hi[k] - gp->box_lo[k]);
    }
    P.guide_alpha = gp->alpha;
    if (gp->record < 0) return set_err(ctx, TR_ERR_ARG, "guide record stride must be >= 0");
    P.guide_record = gp->record;
    if (gp->light_record && !gp->light_guide)
      return set_err(ctx, TR_ERR_ARG, "light_record needs light_guide (the statistics are kept per table bin)");
    if (gp->light_guide) {
      if (!ctx->d_lg_cdf.p || ctx->lg_nl != std::max(nl, 1))
        return set_err(ctx, TR_ERR_STATE, "light table not initialised for this scene (tr_guide_light_init)");
      P.lg_cdf = ctx->d_lg_cdf.as<float>();
      P.lg_acc = gp->light_record ? ctx->d_lg_acc.as<float>() : nullptr;
      for (int k = 0; k < 3; ++k) P.lg_grid[k] = ctx->lg_grid[k];
      P.lg_bins = ctx->lg_bins;
    }
    P.maxd = std::max(jobs[0].prm.max_depth, 1);
    const size_t N = (size_t)n;
    const unsigned int cap = gp->max_records ? gp->max_records : (4u << 20);
    cudaError_t e = cudaSuccess;
    if (P.guide_alpha > 0.0f) {
      if ((e = rb->gfeat.reserve(N * 7 * 4)) != cudaSuccess || (e = rb->gout.reserve(N * kMixFloats * 4)) != cudaSuccess ||
          (e = rb->GX.reserve(N * 4 * sizeof(float4))) != cudaSuccess || (e = rb->grow.reserve(N * 4)) != cudaSuccess)
        return cuda_fail(ctx, e, "guide inference buffers");
      P.gfeat = rb->gfeat.as<float>();
      P.gout = rb->gout.as<float>();
      P.GX = rb->GX.as<float4>();
      P.grow = rb->grow.as<int>();
      if (gp->max_depth < 0) return set_err(ctx, TR_ERR_ARG, "guide max_depth must be >= 0");
      P.guide_depth = gp->max_depth;
    }
    if (P.guide_record) {
      if ((e = rb->VR.reserve(N * P.maxd * 64)) != cudaSuccess || (e = rb->NV.reserve(N * 4)) != cudaSuccess ||
          (e = rb->tb.reserve((size_t)cap * 11 * 4)) != cudaSuccess)
        return cuda_fail(ctx, e, "guide record buffers");
      P.VR = rb->VR.as<float4>();
      P.NV = rb->NV.as<int>();
      P.tb_in = rb->tb.as<float>();
      P.tb_dir = P.tb_in + (size_t)cap * 7;
      P.tb_w = P.tb_dir + (size_t)cap * 3;
      P.tb_cap = cap;
      rb->tb_cap = cap;
    }
  }

  int sms = 0;
  {
    const cudaError_t ae = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (ae != cudaSuccess) return cuda_fail(ctx, ae, "cudaDeviceGetAttribute(multiprocessor count)");
  }
  if (sms <= 0) sms = 1;
  const int grid = sms * ctx->tune.shade_blocks_per_sm, grid_init = sms * 8;
  // the treelet staged by the binary traversal kernels
  P.tl_n = treelet_nodes(ctx);
  const size_t tl_smem = (size_t)P.tl_n * sizeof(DNode);
  for (const void* k : {(const void*)k_extend<false>, (const void*)k_extend<true>, (const void*)k_shadow<false>,
                        (const void*)k_shadow<true>}) {
    const cudaError_t ae = allow_dynamic_smem(k, tl_smem);
    if (ae != cudaSuccess) return cuda_fail(ctx, ae, "traversal shared memory");
  }
  const int grid_ext = traversal_grid(ctx, (const void*)k_extend<false>, tl_smem);
  const bool wide = any_wide(ctx);
  const size_t sh_smem = wide ? 0 : tl_smem;
  const int grid_sh =
      traversal_grid(ctx, wide ? (const void*)k_shadow<false, true> : (const void*)k_shadow<false>, sh_smem);
  P.refill = ctx->tune.trav_refill_lanes;

  ctx->cancel.store(0);
  cudaEvent_t e0, e1, chk;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreateWithFlags(&chk, cudaEventDisableTiming);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t gexec = nullptr;
  const bool timed = (flags & TR_RENDER_TIME_STAGES) != 0;
  const bool count = (flags & TR_RENDER_COUNT_VISITS) != 0;
  // the persistent kernel (tr_tuning.render_mode) for plain renders whose
  // scenes have at most kMegaLights lights; by default for renders of at most
  // kMegaAutoSlots pixels, which the wavefront's launches cannot fill the GPU with
  bool mega = false;
  unsigned mmask = 0;
  int mgrid = 0, mthreads = kMegaThreads;
  if (!gp && !timed && !count && nl <= kMegaLights && ctx->tune.render_mode != TR_RENDER_MODE_WAVEFRONT) {
    mega = ctx->tune.render_mode == TR_RENDER_MODE_PERSISTENT || (long long)n <= kMegaAutoSlots;
    if (mega) {
      bool d12 = false;
      for (const DMat& m : ctx->hs.mats) d12 |= m.kind == MAT_DISNEY12;
      mmask = mega_kernel_mask(ctx->dsc, d12);
      // full 512-thread blocks even when fewer than the SMs: spreading a
      // 65k-pixel render over all 152 SMs in 448-thread blocks was slower
      // (70.7 against 75.7 Msamples/s on the Cornell box)
      const long long want = ((long long)n + kMegaThreads - 1) / kMegaThreads;
      mgrid = (int)std::min<long long>(want, (long long)sms * mega_blocks_per_sm(mmask));
    }
  }
  std::vector<cudaEvent_t>& ev = rb->ev_pool;
  size_t nev = 0;
  auto cleanup = [&]() {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(chk);
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
  };
#define RCHK(call)                      \
  do {                                  \
    cudaError_t e_ = (call);            \
    if (e_ != cudaSuccess) {            \
      cleanup();                        \
      return cuda_fail(ctx, e_, #call); \
    }                                   \
  } while (0)
  if (mega) {
    // The persistent kernel: every sample of every job in one launch. With
    // graphs enabled, the zeroing of the films and counters and the launch
    // are captured into one CUDA graph and replayed as one launch.
    MegaLaunch M;
    M.sc = P.sc;
    M.jobs = P.jobs;
    M.njobs = njobs;
    M.nslots = n;
    M.nl_max = nl;
    M.occluder_cache = ctx->tune.occluder_cache;
    M.fetch = P.ctr + C_FEXT;
    M.err = (int*)(P.ctr + C_ERR);
    M.stats = P.stats;
    const bool use_graph = ctx->tune.graph_iterations > 0;
    RCHK(cudaEventRecord(e0, st));
    if (use_graph) RCHK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaSuccess;
    for (int k = 0; k < njobs && le == cudaSuccess; ++k)
      le = cudaMemsetAsync(jd[k].film, 0, (size_t)jd[k].W * jd[k].H * (jd[k].fp64 ? 32 : 16), st);
    if (le == cudaSuccess) le = cudaMemsetAsync(P.ctr, 0, kCtrWords * 4, st);
    if (le == cudaSuccess) le = cudaMemsetAsync(P.stats, 0, kStatWords * 8, st);
    if (le == cudaSuccess) le = launch_mega(M, mmask, mgrid, mthreads, st);
    if (use_graph) {
      const cudaError_t ce = cudaStreamEndCapture(st, &graph);
      if (le == cudaSuccess) le = ce;
      if (le == cudaSuccess) le = cudaGraphInstantiate(&gexec, graph, 0);
      if (le == cudaSuccess) le = cudaGraphLaunch(gexec, st);
    }
    RCHK(le);
    RCHK(cudaEventRecord(e1, st));
    RCHK(cudaEventSynchronize(e1));
    unsigned long long hs[kStatWords] = {};
    RCHK(cudaMemcpy(hs, P.stats, sizeof(hs), cudaMemcpyDeviceToHost));
    unsigned int ctrs[kCtrWords];
    RCHK(cudaMemcpy(ctrs, P.ctr, sizeof(ctrs), cudaMemcpyDeviceToHost));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cleanup();
    tr_status result = TR_OK;
    if (ctrs[C_ERR] & 1u) result = set_err(ctx, TR_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
    else if (ctrs[C_ERR] & 2u) result = set_err(ctx, TR_ERR_TIMEOUT, "a path slot ran past its vertex bound");
    rb->tb_count = 0;
    if (stats) {
      std::memset(stats, 0, sizeof(*stats));
      stats->samples = hs[0];
      stats->extend_rays = hs[1];
      stats->shadow_rays = hs[2];
      stats->shade_items = hs[3];
      stats->iterations = 1;
      stats->device_ms = ms;
      stats->occluder_hits = hs[8];
    }
    return result;
  }
  for (int k = 0; k < njobs; ++k)
    RCHK(cudaMemsetAsync(jd[k].film, 0, (size_t)jd[k].W * jd[k].H * (jd[k].fp64 ? 32 : 16), st));
  RCHK(cudaMemsetAsync(P.ctr, 0, kCtrWords * 4, st));
  RCHK(cudaMemsetAsync(P.stats, 0, kStatWords * 8, st));
  if (P.OC) RCHK(cudaMemsetAsync(P.OC, 0xff, (size_t)n * P.nl_max * 4, st));
  if (P.act_flag) RCHK(cudaMemsetAsync(P.act_flag, 0, (size_t)n, st));
  RCHK(cudaEventRecord(e0, st));
  k_init<<<grid_init, 256, 0, st>>>(P);
  RCHK(cudaGetLastError());

  // optional per-kernel timing: an event before the first kernel of every
  // iteration and after each of its kernels, summed once drained
  auto mark = [&]() {
    if (!timed) return;
    if (nev == ev.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev.push_back(e);
    }
    cudaEventRecord(ev[nev++], st);
  };
  // one wavefront iteration; returns the first launch error
  const int bin_nb = P.bin_bits ? 1 << (3 + 3 * P.bin_bits) : 0;
  auto iteration = [&](int cur) -> tr_status {
    const int nxt = cur ^ 1;
    mark();
    if (P.bin_bits) {  // the extend queue in ray-key order
      cudaMemsetAsync(P.bin_cnt, 0, (size_t)bin_nb * 4, st);
      k_bin_count<<<grid, 128, 0, st>>>(ExtendSrc{P, cur}, P.sc, P.bin_cnt, P.bin_key, P.bin_bits);
      k_bin_scan<<<1, kBinScanThreads, 0, st>>>(P.bin_cnt, bin_nb);
      k_bin_scatter<<<grid, 128, 0, st>>>(ExtendSrc{P, cur}, P.bin_cnt, P.bin_key, P.q_srt);
    }
    mark();
    if (count) k_extend<true><<<grid_ext, 128, tl_smem, st>>>(P, cur);
    else k_extend<false><<<grid_ext, 128, tl_smem, st>>>(P, cur);
    mark();
    // next iteration's extend and live counts; this iteration's shadow,
    // material and light-sample counts and the fetch positions
    cudaMemsetAsync(P.ctr + C_EXT + nxt, 0, 4, st);
    cudaMemsetAsync(P.ctr + C_ACT + nxt, 0, 4, st);
    cudaMemsetAsync(P.ctr + C_SH, 0, 4 * (C_FSH + 1 - C_SH), st);  // C_SH, C_MAT, C_NEE, C_FEXT, C_FSH
    if (P.guide_alpha > 0.0f) cudaMemsetAsync(P.ctr + C_GROW, 0, 4, st);
    mark();
    if (P.q_ord) {  // the live slots in slot order (timed with k_logic)
      cudaMemsetAsync(P.ctr + C_ORD, 0, 4, st);
      k_act_mark<<<grid, 256, 0, st>>>(P, cur);
      k_act_order<<<grid_init, 256, 0, st>>>(P);
    }
    k_logic<<<grid, 128, 0, st>>>(P, cur);
    if (P.guide_alpha > 0.0f) {
      // decoded mixtures for this iteration's Phong-material vertices (inputs written by k_logic)
      tr_status gs = guide_forward_rows_on_device(ctx, P.gfeat, P.ctr + C_GROW, P.gout);
      if (gs != TR_OK) return gs;
    }
    mark();
    // the guided instantiation only when guiding (its code would slow the plain kernel)
    if (P.guide_alpha > 0.0f) k_material<MAT_PHONG, true><<<grid, 128, 0, st>>>(P, cur);
    else k_material<MAT_PHONG><<<grid, 128, 0, st>>>(P, cur);
    mark();
    k_material<MAT_DISNEY12><<<grid, 128, 0, st>>>(P, cur);
    if (P.sc.has_glass) k_glass<<<grid, 128, 0, st>>>(P, cur);  // timed with Disney12
    if (P.sc.has_metal) k_material<MAT_METAL><<<grid, 128, 0, st>>>(P, cur);
    if (P.sc.has_disney15) k_material<MAT_DISNEY15><<<grid, 128, 0, st>>>(P, cur);
    mark();
    if (P.MT) k_nee<MAT_PHONG, true><<<grid, 128, 0, st>>>(P);
    else k_nee<MAT_PHONG><<<grid, 128, 0, st>>>(P);
    mark();
    // (MAPS instantiations: hits of materials with image maps read the slot's set-up)
    if (P.MT) k_nee<MAT_DISNEY12, true><<<grid, 128, 0, st>>>(P);
    else k_nee<MAT_DISNEY12><<<grid, 128, 0, st>>>(P);
    if (P.sc.has_metal) {  // timed with Disney12
      if (P.MT) k_nee<MAT_METAL, true><<<grid, 128, 0, st>>>(P);
      else k_nee<MAT_METAL><<<grid, 128, 0, st>>>(P);
    }
    if (P.sc.has_disney15) {
      if (P.MT) k_nee<MAT_DISNEY15, true><<<grid, 128, 0, st>>>(P);
      else k_nee<MAT_DISNEY15><<<grid, 128, 0, st>>>(P);
    }
    mark();
    if (count && wide) k_shadow<true, true><<<grid_sh, 128, 0, st>>>(P);
    else if (count) k_shadow<true><<<grid_sh, 128, sh_smem, st>>>(P);
    else if (wide) k_shadow<false, true><<<grid_sh, 128, 0, st>>>(P);
    else k_shadow<false><<<grid_sh, 128, sh_smem, st>>>(P);
    mark();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? TR_OK : cuda_fail(ctx, e, "wavefront launch");
  };
  // Without per-kernel instrumentation, a chunk of iterations (an even
  // number, so each chunk starts on the same queue parity) is captured once
  // into a CUDA graph and replayed: one launch per chunk instead of ten
  // per iteration. The host still polls the live count between chunks.
  const int chunk = (!timed && !count && ctx->tune.graph_iterations > 0) ? (ctx->tune.graph_iterations + 1) & ~1 : 4;
  if (!timed && !count && ctx->tune.graph_iterations > 0) {
    RCHK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    tr_status cs = TR_OK;
    for (int c = 0; c < chunk && cs == TR_OK; ++c) cs = iteration(c & 1);
    cudaError_t ee = cudaStreamEndCapture(st, &graph);
    if (cs != TR_OK) {
      cleanup();
      return cs;
    }
    RCHK(ee);
    RCHK(cudaGraphInstantiate(&gexec, graph, 0));
  }
  long long it = 0;
  bool done = false, chk_pending = false;
  tr_status result = TR_OK;
  while (!done) {
    if (gexec) {
      RCHK(cudaGraphLaunch(gexec, st));
      it += chunk;
    } else {
      for (int c = 0; c < chunk && it < max_iters; ++c, ++it) {
        tr_status is = iteration((int)(it & 1));
        if (is != TR_OK) {
          cleanup();
          return is;
        }
      }
    }
    RCHK(cudaGetLastError());
    if (chk_pending) {
      RCHK(cudaEventSynchronize(chk));
      if (rb->h_active[0] == 0) done = true;
    }
    if (!done) {
      const int nxt_after = (int)(it & 1);
      RCHK(cudaMemcpyAsync(rb->h_active, P.ctr + C_ACT + nxt_after, 4, cudaMemcpyDeviceToHost, st));
      RCHK(cudaEventRecord(chk, st));
      chk_pending = true;
      if (it >= max_iters) {
        RCHK(cudaEventSynchronize(chk));
        if (rb->h_active[0] != 0)
          result = set_err(ctx, TR_ERR_TIMEOUT, "wavefront did not drain within its iteration bound");
        done = true;
      }
    }
    if (ctx->cancel.load()) {
      result = set_err(ctx, TR_ERR_CANCELLED, "render cancelled");
      done = true;
    }
  }
  RCHK(cudaEventRecord(e1, st));
  RCHK(cudaEventSynchronize(e1));
  unsigned long long hs[kStatWords] = {};
  RCHK(cudaMemcpy(hs, P.stats, sizeof(hs), cudaMemcpyDeviceToHost));
  unsigned int ctrs[kCtrWords];
  RCHK(cudaMemcpy(ctrs, P.ctr, sizeof(ctrs), cudaMemcpyDeviceToHost));
  // event k of an iteration's 10 precedes kernel group k; stage of each interval
  static const int kStageOf[9] = {TR_STAGE_BIN,       TR_STAGE_EXTEND,          TR_STAGE_RESET,
                                  TR_STAGE_LOGIC,     TR_STAGE_MATERIAL_PHONG,  TR_STAGE_MATERIAL_DISNEY,
                                  TR_STAGE_NEE_PHONG, TR_STAGE_NEE_DISNEY,      TR_STAGE_SHADOW};
  double stage[TR_NUM_STAGES] = {};
  for (size_t k = 0; k + 10 <= nev; k += 10)
    for (int j = 0; j < 9; ++j) {
      float a = 0.0f;
      cudaEventElapsedTime(&a, ev[k + j], ev[k + j + 1]);
      stage[kStageOf[j]] += a;
    }
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cleanup();
  if (ctrs[C_ERR] != 0 && result == TR_OK) result = set_err(ctx, TR_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
  rb->tb_count = P.guide_record ? std::min(ctrs[C_TB], P.tb_cap) : 0;
  if (P.guide_alpha > 0.0f && result == TR_OK) {
    int ge = 0;
    RCHK(cudaMemcpy(&ge, ctx->d_err.as<int>() + 2, 4, cudaMemcpyDeviceToHost));
    if (ge) {
      cudaMemset(ctx->d_err.as<int>() + 2, 0, 4);
      result = set_err(ctx, TR_ERR_TIMEOUT, "tensor-core MMA wait timed out");
    }
  }
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->samples = hs[0];
    stats->extend_rays = hs[1];
    stats->shadow_rays = hs[2];
    stats->shade_items = hs[3];
    stats->iterations = (uint64_t)it;
    stats->device_ms = ms;
    for (int k = 0; k < TR_NUM_STAGES; ++k) stats->stage_ms[k] = stage[k];
    stats->closest_boxes = hs[4];
    stats->closest_prims = hs[5];
    stats->any_boxes = hs[6];
    stats->any_prims = hs[7];
    stats->guide_records = rb->tb_count;
    stats->occluder_hits = hs[8];
  }
  return result;
#undef RCHK
}

tr_status render_impl(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter, const tr_render_params* prm,
                      void* d_out, bool fp64, tr_stats* stats, const tr_guide_params* gp = nullptr) {
  JobSpec j;
  j.scene = 0;
  j.cam = *cam;
  j.filter = *filter;
  j.prm = *prm;
  j.film = d_out;
  j.fp64 = fp64;
  return render_jobs(ctx, &j, 1, prm->flags, stats, gp);
}

}  // namespace trg

using namespace trg;

extern "C" {

tr_status tr_render_dev(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter, const tr_render_params* params,
                        float* d_rgbw, double* d_rgbw64, tr_stats* stats) {
  if (!ctx || !cam || !filter || !params || ((d_rgbw == nullptr) == (d_rgbw64 == nullptr))) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  void* out = d_rgbw ? (void*)d_rgbw : (void*)d_rgbw64;
  if (((uintptr_t)out & 15u) != 0) return set_err(ctx, TR_ERR_ARG, "film buffer must be 16-byte aligned");
  return render_impl(ctx, cam, filter, params, out, d_rgbw64 != nullptr, stats);
}

tr_status tr_render(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter, const tr_render_params* params,
                    float* rgbw, double* rgbw64, tr_stats* stats) {
  if (!ctx || !cam || !filter || !params || ((rgbw == nullptr) == (rgbw64 == nullptr))) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  tr_status s = render_impl(ctx, cam, filter, params, nullptr, rgbw64 != nullptr, stats);
  if (s != TR_OK) return s;
  const size_t n = (size_t)params->width * params->height;
  cudaError_t e = rgbw64 ? cudaMemcpy(rgbw64, ctx->rb->acc.p, n * 32, cudaMemcpyDeviceToHost)
                         : cudaMemcpy(rgbw, ctx->rb->acc.p, n * 16, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "film copy");
  return TR_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// No-allocation render (tr_render_dev_noalloc). The same kernels as
// render_impl, with every scratch buffer carved from one file-scope device
// array instead of cudaMalloc'd RenderBuffers, a fixed iteration count instead
// of polling a pinned live count, and no CUDA events.

namespace trg {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB per device
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mtx;
void* g_noalloc_base[kMaxDevices] = {};

// Scratch bytes a film of n pixels with nl lights needs (each buffer 256-byte aligned).
struct NoAllocLayout {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t at = off;
    off = (off + bytes + 255) & ~size_t(255);
    return at;
  }
};

}  // namespace

tr_status render_noalloc_impl(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter,
                              const tr_render_params* prm, float* d_rgbw, tr_stats* stats) {
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (prm->width <= 0 || prm->height <= 0 || prm->spp <= 0 || prm->max_depth < 0)
    return set_err(ctx, TR_ERR_ARG, "invalid render size, spp or depth");
  if (prm->max_depth > kMaxPathDepth)
    return set_err(ctx, TR_ERR_ARG, "max_depth above 65515 (the path depth is kept in 16 bits)");
  if (prm->direct_light_sample_num != 1)
    return set_err(ctx, TR_ERR_UNSUPPORTED, "direct_light_sample_num must be 1 on the GPU path");
  if (!(filter->radius > 0.0f) || filter->radius > 16.0f) return set_err(ctx, TR_ERR_ARG, "invalid filter radius");
  if (ctx->device < 0 || ctx->device >= kMaxDevices) return set_err(ctx, TR_ERR_ARG, "device ordinal out of range");
  if (ctx->dsc.has_textures)  // their per-slot material set-ups have no room in the static scratch
    return set_err(ctx, TR_ERR_UNSUPPORTED, "tr_render_dev_noalloc does not take materials with image maps");
  const long long npix = (long long)prm->width * prm->height;
  const int nl = ctx->dsc.max_lights;
  const size_t NL = (size_t)std::max(nl, 1);
  // carve the layout first: reject what does not fit before touching the device
  const size_t N = npix > (1ll << 24) ? (size_t(1) << 24) : (size_t)npix;
  NoAllocLayout L;
  const size_t f4 = sizeof(float4);
  const size_t oP = L.take(5 * N * f4), oRng = L.take(N * 8), oM = L.take(3 * N * f4), oH = L.take(2 * N * f4),
               oSC = L.take(N * 7 * f4), oNU = L.take(N * NL * 8), oSH = L.take(N * NL * 2 * f4),
               oSHC = L.take(N * NL * f4),
               oQe = L.take(2 * 2 * N * 4), oQa = L.take(2 * N * 4), oQm = L.take(kMatKinds * N * 4),
               oQn = L.take(kNeeKinds * N * NL * 4), oQs = L.take(N * NL * 4), oCtr = L.take(kCtrWords * 4),
               oSt = L.take(kStatWords * 8),
               oJob = L.take(sizeof(JobDev));
  if (npix > (1ll << 24) || L.off > kNoAllocScratchBytes) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "film %dx%d with %d lights needs %zu bytes of scratch; tr_render_dev_noalloc has %zu "
                  "(about 324 + 76 * lights bytes per pixel)",
                  prm->width, prm->height, nl, (size_t)L.off, kNoAllocScratchBytes);
    return set_err(ctx, TR_ERR_ARG, msg);
  }
  const int n = (int)npix;
  unsigned char* base = nullptr;
  {
    // once per device: the address of this device's copy of the array
    std::lock_guard<std::mutex> lk(g_noalloc_mtx);
    if (!g_noalloc_base[ctx->device]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress(scratch)");
      g_noalloc_base[ctx->device] = p;
    }
    base = static_cast<unsigned char*>(g_noalloc_base[ctx->device]);
  }
  cudaStream_t st = ctx->stream;
#define NCHK(call)                                      \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)
  JobSpec spec;
  spec.scene = 0;
  spec.cam = *cam;
  spec.filter = *filter;
  spec.prm = *prm;
  spec.film = d_rgbw;
  spec.fp64 = false;
  const JobDev job = make_job_dev(ctx, spec, 0, d_rgbw);
  // the job record is copied from host stack memory into the array
  NCHK(cudaMemcpyAsync(base + oJob, &job, sizeof(job), cudaMemcpyHostToDevice, st));

  Launch P;
  std::memset(&P, 0, sizeof(P));
  P.sc = ctx->dsc;
  P.jobs = reinterpret_cast<const JobDev*>(base + oJob);
  P.njobs = 1;
  P.nslots = n;
  P.nl_max = (int)NL;
  P.refill = ctx->tune.trav_refill_lanes;
  float4* Pb = reinterpret_cast<float4*>(base + oP);
  P.P0 = Pb;
  P.P1 = Pb + N;
  P.P2 = Pb + 2 * N;
  P.P3 = Pb + 3 * N;
  P.P4 = Pb + 4 * N;
  P.rng = reinterpret_cast<unsigned long long*>(base + oRng);
  float4* Mb = reinterpret_cast<float4*>(base + oM);
  P.M0 = Mb;
  P.M1 = Mb + N;
  P.M2 = Mb + 2 * N;
  P.HC = reinterpret_cast<float4*>(base + oH);
  P.HM = P.HC + N;
  P.SC = reinterpret_cast<float4*>(base + oSC);
  P.NU = reinterpret_cast<float2*>(base + oNU);
  P.SH = reinterpret_cast<float4*>(base + oSH);
  P.SHC = reinterpret_cast<float4*>(base + oSHC);
  int* qe = reinterpret_cast<int*>(base + oQe);
  int* qa = reinterpret_cast<int*>(base + oQa);
  int* qm = reinterpret_cast<int*>(base + oQm);
  int* qn = reinterpret_cast<int*>(base + oQn);
  for (int k = 0; k < 2; ++k) {
    P.q_ext[k] = qe + (size_t)k * 2 * N;
    P.q_act[k] = qa + (size_t)k * N;
  }
  for (int k = 0; k < kNeeKinds; ++k) P.q_nee[k] = qn + (size_t)k * N * NL;
  for (int k = 0; k < kMatKinds; ++k) P.q_mat[k] = qm + (size_t)k * N;
  P.q_sh = reinterpret_cast<int*>(base + oQs);
  P.ctr = reinterpret_cast<unsigned int*>(base + oCtr);
  P.stats = reinterpret_cast<unsigned long long*>(base + oSt);

  int sms = 0;
  {
    const cudaError_t ae = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (ae != cudaSuccess) return cuda_fail(ctx, ae, "cudaDeviceGetAttribute(multiprocessor count)");
  }
  if (sms <= 0) sms = 1;
  const int grid = sms * ctx->tune.shade_blocks_per_sm, grid_init = sms * 8;
  const int grid_ext = traversal_grid(ctx, (const void*)k_extend<false>);
  const bool wide = any_wide(ctx);
  const int grid_sh = traversal_grid(ctx, wide ? (const void*)k_shadow<false, true> : (const void*)k_shadow<false>);
  // the counters, statistics and film start at zero on every call; the
  // rest of the scratch is written before it is read
  NCHK(cudaMemsetAsync(d_rgbw, 0, (size_t)n * 16, st));
  NCHK(cudaMemsetAsync(P.ctr, 0, kCtrWords * 4, st));
  NCHK(cudaMemsetAsync(P.stats, 0, kStatWords * 8, st));
  k_init<<<grid_init, 256, 0, st>>>(P);
  NCHK(cudaGetLastError());
  // Every slot finishes within spp * (max_depth + 2) iterations (plus the
  // delta samples that do not count toward the depth): that bound is the
  // ceiling. Every kDrainCheck iterations the live-slot count is copied into
  // a host stack variable (a pageable copy: nothing is allocated), and the
  // loop stops once the wavefront has drained or tr_cancel was called.
  const long long iters =
      (long long)prm->spp * ((long long)prm->max_depth + 2 + (ctx->dsc.has_glass ? kMaxSpecularDepth : 0)) + 4;
  constexpr int kDrainCheck = 16;  // even: the count read is the list the next iteration starts from
  ctx->cancel.store(0);
  long long it = 0;
  unsigned int live = 1;
  bool cancelled = false;
  while (it < iters && live != 0 && !cancelled) {
    const int cur = (int)(it & 1), nxt = cur ^ 1;
    k_extend<false><<<grid_ext, 128, 0, st>>>(P, cur);
    NCHK(cudaMemsetAsync(P.ctr + C_EXT + nxt, 0, 4, st));
    NCHK(cudaMemsetAsync(P.ctr + C_ACT + nxt, 0, 4, st));
    NCHK(cudaMemsetAsync(P.ctr + C_SH, 0, 4 * (C_FSH + 1 - C_SH), st));  // C_SH, C_MAT, C_NEE, C_FEXT, C_FSH
    k_logic<<<grid, 128, 0, st>>>(P, cur);
    k_material<MAT_PHONG><<<grid, 128, 0, st>>>(P, cur);
    k_material<MAT_DISNEY12><<<grid, 128, 0, st>>>(P, cur);
    if (P.sc.has_glass) k_glass<<<grid, 128, 0, st>>>(P, cur);
    if (P.sc.has_metal) k_material<MAT_METAL><<<grid, 128, 0, st>>>(P, cur);
    if (P.sc.has_disney15) k_material<MAT_DISNEY15><<<grid, 128, 0, st>>>(P, cur);
    k_nee<MAT_PHONG><<<grid, 128, 0, st>>>(P);
    k_nee<MAT_DISNEY12><<<grid, 128, 0, st>>>(P);
    if (P.sc.has_metal) k_nee<MAT_METAL><<<grid, 128, 0, st>>>(P);
    if (P.sc.has_disney15) k_nee<MAT_DISNEY15><<<grid, 128, 0, st>>>(P);
    if (wide) k_shadow<false, true><<<grid_sh, 128, 0, st>>>(P);
    else k_shadow<false><<<grid_sh, 128, 0, st>>>(P);
    ++it;
    if (it % kDrainCheck == 0 || it == iters) {
      NCHK(cudaGetLastError());
      NCHK(cudaMemcpyAsync(&live, P.ctr + C_ACT + (int)(it & 1), 4, cudaMemcpyDeviceToHost, st));
      NCHK(cudaStreamSynchronize(st));
      cancelled = ctx->cancel.load() != 0;
    }
  }
  NCHK(cudaGetLastError());
  NCHK(cudaStreamSynchronize(st));
  unsigned long long hs[kStatWords];
  unsigned int ctrs[kCtrWords];
  NCHK(cudaMemcpy(hs, P.stats, sizeof(hs), cudaMemcpyDeviceToHost));
  NCHK(cudaMemcpy(ctrs, P.ctr, sizeof(ctrs), cudaMemcpyDeviceToHost));
#undef NCHK
  if (stats) {
    std::memset(stats, 0, sizeof(*stats));
    stats->samples = hs[0];
    stats->extend_rays = hs[1];
    stats->shadow_rays = hs[2];
    stats->shade_items = hs[3];
    stats->iterations = (uint64_t)it;
  }
  if (ctrs[C_ERR] != 0) return set_err(ctx, TR_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
  if (cancelled) return set_err(ctx, TR_ERR_CANCELLED, "render cancelled");
  if (ctrs[C_ACT + (int)(it & 1)] != 0)
    return set_err(ctx, TR_ERR_TIMEOUT, "wavefront did not drain within its iteration bound");
  return TR_OK;
}

}  // namespace trg

extern "C" tr_status tr_render_batch_dev(tr_ctx* ctx, const tr_batch_job* jobs, uint32_t n, tr_stats* stats) {
  if (!ctx || !jobs || n == 0 || n > (1u << 20)) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  std::vector<trg::JobSpec> spec(n);
  for (uint32_t k = 0; k < n; ++k) {
    if (!jobs[k].d_rgbw) return trg::set_err(ctx, TR_ERR_ARG, "batch job without a film");
    spec[k].scene = (int)jobs[k].scene;
    spec[k].cam = jobs[k].camera;
    spec[k].filter = jobs[k].filter;
    spec[k].prm = jobs[k].params;
    spec[k].film = jobs[k].d_rgbw;
    spec[k].fp64 = false;
  }
  return trg::render_jobs(ctx, spec.data(), (int)n, jobs[0].params.flags, stats);
}

extern "C" tr_status tr_autotune(tr_ctx* ctx, const tr_batch_job* jobs, uint32_t n, int32_t probe_spp,
                                  tr_tuning* best, double* best_ms) {
  if (!ctx || !jobs || n == 0 || !best || probe_spp <= 0) return TR_ERR_ARG;
  // the probe: the caller's jobs with at most probe_spp samples per pixel
  std::vector<tr_batch_job> probe(jobs, jobs + n);
  for (auto& j : probe) {
    j.params.spp = std::min(j.params.spp, probe_spp);
    j.params.flags = 0;
  }
  auto time_once = [&](const tr_tuning& t, double& ms) -> tr_status {
    tr_status s = tr_ctx_set_tuning(ctx, &t);
    if (s != TR_OK) return s;
    double v[3];
    for (int r = 0; r < 4; ++r) {  // one warm-up, median of three
      const auto t0 = std::chrono::steady_clock::now();
      s = tr_render_batch_dev(ctx, probe.data(), n, nullptr);
      if (s != TR_OK) return s;
      if (r) v[r - 1] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    std::sort(v, v + 3);
    ms = v[1];
    return TR_OK;
  };
  // coordinate descent over the discrete settings, the execution model first
  static const int kMode[] = {TR_RENDER_MODE_WAVEFRONT, TR_RENDER_MODE_PERSISTENT}, kBlocks[] = {0, 4, 6, 8},
                   kRefill[] = {12, 20, 28}, kShade[] = {8, 16, 32}, kGraph[] = {0, 4, 8, 16}, kWidth[] = {2, 4},
                   kBins[] = {0, 3, 4}, kTreelet[] = {0, 64, 256}, kCache[] = {0, 1}, kOrder[] = {0, 1, 2};
  struct Dim {
    int32_t tr_tuning::*field;
    const int* vals;
    int nv;
  };
  static const Dim kDims[] = {{&tr_tuning::render_mode, kMode, 2},        {&tr_tuning::trav_blocks_per_sm, kBlocks, 4},
                              {&tr_tuning::trav_refill_lanes, kRefill, 3}, {&tr_tuning::shade_blocks_per_sm, kShade, 3},
                              {&tr_tuning::graph_iterations, kGraph, 4},   {&tr_tuning::any_node_width, kWidth, 2},
                              {&tr_tuning::ray_bin_bits, kBins, 3},        {&tr_tuning::treelet_nodes, kTreelet, 3},
                              {&tr_tuning::occluder_cache, kCache, 2},    {&tr_tuning::any_hit_order, kOrder, 3}};
  tr_tuning cur = ctx->tune;
  double cur_ms = 0.0;
  tr_status s = time_once(cur, cur_ms);
  if (s != TR_OK) return s;
  for (int pass = 0; pass < 2; ++pass) {
    bool improved = false;
    for (const Dim& dim : kDims) {
      for (int k = 0; k < dim.nv; ++k) {
        tr_tuning t = cur;
        if (t.*dim.field == dim.vals[k]) continue;
        t.*dim.field = dim.vals[k];
        double ms = 0.0;
        s = time_once(t, ms);
        if (s != TR_OK) return s;
        if (ms < 0.98 * cur_ms) {  // keep only clear wins
          cur = t;
          cur_ms = ms;
          improved = true;
        }
      }
    }
    if (!improved) break;
  }
  s = tr_ctx_set_tuning(ctx, &cur);
  *best = cur;
  if (best_ms) *best_ms = cur_ms;
  return s;
}

extern "C" tr_status tr_render_guided_dev(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter,
                                          const tr_render_params* params, const tr_guide_params* guide,
                                          float* d_rgbw, double* d_rgbw64, tr_stats* stats) {
  if (!ctx || !cam || !filter || !params || !guide || ((d_rgbw == nullptr) == (d_rgbw64 == nullptr))) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  cudaError_t e;
  void* out = d_rgbw ? (void*)d_rgbw : (void*)d_rgbw64;
  if (((uintptr_t)out & 15u) != 0) return trg::set_err(ctx, TR_ERR_ARG, "film buffer must be 16-byte aligned");
  return trg::render_impl(ctx, cam, filter, params, out, d_rgbw64 != nullptr, stats, guide);
}

namespace trg {

// The light table's sampling distributions from its statistics: per
// (cell, light) group of nb bins, share / nb + (1 - share) * the bin's part
// of the group's recorded estimates (uniform where none), as a cumulative
// distribution ending at exactly 1.
__global__ void __launch_bounds__(128) k_lg_update(const float* __restrict__ acc, float* __restrict__ cdf,
                                                   size_t groups, int nb, float share) {
  for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < groups; g += (size_t)gridDim.x * blockDim.x) {
    const float* a = acc + g * nb;
    float* c = cdf + g * nb;
    double tot = 0.0;
    for (int b = 0; b < nb; ++b) tot += a[b];
    const double u = (double)share / nb;
    double run = 0.0;
    for (int b = 0; b < nb; ++b) {
      run += u + (tot > 0.0 ? (1.0 - share) * (double)a[b] / tot : (1.0 - share) / nb);
      c[b] = (float)run;
    }
    for (int b = 0; b < nb; ++b) c[b] = (float)((double)c[b] / run);
    c[nb - 1] = 1.0f;
  }
}

}  // namespace trg

extern "C" tr_status tr_guide_light_init(tr_ctx* ctx, const int32_t grid[3], int32_t bins) {
  if (!ctx || !grid || bins < 1 || bins > 16) return TR_ERR_ARG;
  if (!ctx->has_scene) return trg::set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (ctx->dsc.num_scenes != 1) return trg::set_err(ctx, TR_ERR_ARG, "the light table takes a single scene");
  long long cells = 1;
  for (int k = 0; k < 3; ++k) {
    if (grid[k] < 1 || grid[k] > 1024) return trg::set_err(ctx, TR_ERR_ARG, "light-table grid out of range");
    cells *= grid[k];
  }
  const int nl = std::max(ctx->dsc.max_lights, 1);
  const long long n = cells * nl * bins * bins;
  if (n > (1ll << 26)) return trg::set_err(ctx, TR_ERR_ARG, "light table above 2^26 entries");
  TR_DEVICE_SCOPE(ctx);
  TR_CUDA(ctx, ctx->d_lg_acc.reserve((size_t)n * 4));
  TR_CUDA(ctx, ctx->d_lg_cdf.reserve((size_t)n * 4));
  TR_CUDA(ctx, cudaMemsetAsync(ctx->d_lg_acc.p, 0, (size_t)n * 4, ctx->stream));
  for (int k = 0; k < 3; ++k) ctx->lg_grid[k] = grid[k];
  ctx->lg_bins = bins;
  ctx->lg_nl = nl;
  trg::k_lg_update<<<1024, 128, 0, ctx->stream>>>(ctx->d_lg_acc.as<float>(), ctx->d_lg_cdf.as<float>(),
                                                 (size_t)(n / (bins * bins)), bins * bins, 1.0f);
  TR_CUDA(ctx, cudaGetLastError());
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TR_OK;
}

extern "C" tr_status tr_guide_light_update(tr_ctx* ctx, float uniform_share) {
  if (!ctx || !(uniform_share > 0.0f && uniform_share <= 1.0f)) return TR_ERR_ARG;
  if (!ctx->d_lg_cdf.p || ctx->lg_bins <= 0) return trg::set_err(ctx, TR_ERR_STATE, "light table not initialised");
  TR_DEVICE_SCOPE(ctx);
  const int nb = ctx->lg_bins * ctx->lg_bins;
  const size_t groups = (size_t)ctx->lg_grid[0] * ctx->lg_grid[1] * ctx->lg_grid[2] * ctx->lg_nl;
  trg::k_lg_update<<<1024, 128, 0, ctx->stream>>>(ctx->d_lg_acc.as<float>(), ctx->d_lg_cdf.as<float>(), groups, nb,
                                                 uniform_share);
  TR_CUDA(ctx, cudaGetLastError());
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TR_OK;
}

extern "C" tr_status tr_guide_train_on_records(tr_ctx* ctx, int32_t steps, uint32_t batch, float lr, uint64_t seed,
                                               float* mean_loss) {
  if (!ctx || steps < 0 || batch == 0 || batch > (1u << 22) || !(lr > 0.0f)) return TR_ERR_ARG;
  if (!ctx->guide || !ctx->guide->params.p) return trg::set_err(ctx, TR_ERR_STATE, "guide model not initialised");
  if (!ctx->rb || ctx->rb->tb_count == 0) return trg::set_err(ctx, TR_ERR_STATE, "no training records");
  TR_DEVICE_SCOPE(ctx);
  cudaError_t e;
  trg::RenderBuffers* rb = ctx->rb;
  const float* in = rb->tb.as<float>();
  const float* dir = in + (size_t)rb->tb_cap * 7;
  const float* w = dir + (size_t)rb->tb_cap * 3;
  tr_status s = trg::guide_train_on(ctx, in, dir, w, rb->tb_count, steps, batch, lr, seed, mean_loss);
  if (s != TR_OK) return s;
  int ge = 0;
  e = cudaMemcpy(&ge, ctx->d_err.as<int>() + 2, 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return trg::cuda_fail(ctx, e, "guide error word");
  if (ge) {
    cudaMemset(ctx->d_err.as<int>() + 2, 0, 4);
    return trg::set_err(ctx, TR_ERR_TIMEOUT, "tensor-core MMA wait timed out");
  }
  return TR_OK;
}

extern "C" tr_status tr_render_dev_noalloc(tr_ctx* ctx, const tr_camera* cam, const tr_filter* filter,
                                           const tr_render_params* params, float* d_rgbw, tr_stats* stats) {
  if (!ctx || !cam || !filter || !params || !d_rgbw) return TR_ERR_ARG;
  if (((uintptr_t)d_rgbw & 15u) != 0) return trg::set_err(ctx, TR_ERR_ARG, "film buffer must be 16-byte aligned");
  TR_DEVICE_SCOPE(ctx);
  return trg::render_noalloc_impl(ctx, cam, filter, params, d_rgbw, stats);
}
