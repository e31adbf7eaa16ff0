// traverse.cuh -- BVH traversal and primitive tests on the device.
//
// Reference: BVHAccel::intersect_p / ::intersect (src/accelerator/bvh.cpp:112-185),
// Bounds3::intersect_p (src/utility/geometry.hpp:837-864),
// Triangle::intersect(_p) (src/shape/triangle.cpp:117-174),
// sphere::intersect(_p) + TransformedShape::to_local (src/shape/sphere.cpp:15-47,
// src/shape/transformed_shape.hpp:17-21), GeometricPrimitive::intersect_p
// (src/shape/geometry.cpp:49-60).
//
// Order and culling match the reference exactly on child-pair nodes:
//  * the reference pops a node, tests its box against the CURRENT ray.t_max,
//    and pushes the children near-last (near = second child when
//    dir_is_neg[split_axis]);
//  * a box test is "slab overlap and tMax > 0" (independent of t_max) and
//    "tMin < t_max". Here both children of a visited node are tested at once;
//    the near child is entered immediately (no t_max change can happen in
//    between in the reference), the far child is pushed with its tMin and
//    the tMin < t_max part is re-evaluated when it is popped.
// Triangle arithmetic: the two cross products run in double and round to
// float, the dot products in float, exactly as the reference (no FMA: this
// file is compiled with --fmad=false).
#pragma once

#include "scene_types.h"

namespace trg {

struct RayIn {
  f3 o, d;
  float t_min, t_max;
};

struct Hit {
  int prim;       // -1: miss
  float t_attr;   // the accepted primitive's own parameter (triangle t, local sphere t)
  float alpha, beta;
};

__device__ __forceinline__ float4 ldg4(const float4* p) { return __ldg(p); }

// The shared-memory treelet (DScene::treelet, staged by each block of a
// traversal kernel into its dynamic shared memory). Float4 k of treelet node j
// sits at 4 * j + (k ^ ((j >> 1) & 3)): eight lanes reading the same field of
// eight consecutive nodes then hit eight different bank groups (without the
// swizzle a 64-byte node stride leaves only two).
extern __shared__ float4 trav_smem[];

__device__ __forceinline__ int treelet_slot(int j, int k) { return 4 * j + (k ^ ((j >> 1) & 3)); }

// Copies the first n treelet nodes into shared memory; every thread of the
// block calls it once, before any traversal.
__device__ __forceinline__ void stage_treelet(const DScene& sc, int n) {
  const float4* src = reinterpret_cast<const float4*>(sc.treelet);
  for (int i = threadIdx.x; i < 4 * n; i += blockDim.x) trav_smem[treelet_slot(i >> 2, i & 3)] = __ldg(src + i);
  __syncthreads();
}

// Slab test with the reference's arithmetic. Returns the t_max-independent
// part ("pass"), and tmin for the "tMin < ray.t_max" part.
// Written without branches (the reference's early returns become flags;
// each conditional assignment is a select with the same NaN behaviour), so
// the lanes of a warp never diverge inside a box test. tmin is meaningful
// only when the test passes.
__device__ __forceinline__ bool box_pass(float lx, float ly, float lz, float hx, float hy, float hz, f3 o,
                                         f3 inv, bool n0, bool n1, bool n2, float& tmin) {
  float tMin = ((n0 ? hx : lx) - o.x) * inv.x;
  float tMax = slab_scale(((n0 ? lx : hx) - o.x) * inv.x);
  const float tyMin = ((n1 ? hy : ly) - o.y) * inv.y;
  const float tyMax = slab_scale(((n1 ? ly : hy) - o.y) * inv.y);
  const float tzMin = ((n2 ? hz : lz) - o.z) * inv.z;
  const float tzMax = slab_scale(((n2 ? lz : hz) - o.z) * inv.z);
  const bool miss_y = (tMin > tyMax) | (tyMin > tMax);
  tMin = tyMin > tMin ? tyMin : tMin;
  tMax = tyMax < tMax ? tyMax : tMax;
  const bool miss_z = (tMin > tzMax) | (tzMin > tMax);
  tMin = tzMin > tMin ? tzMin : tMin;
  tMax = tzMax < tMax ? tzMax : tMax;
  tmin = tMin;
  return !miss_y & !miss_z & (tMax > 0.0f);
}

// Möller-Trumbore as the reference writes it. A = s0.xyz, AB = s1.xyz, AC = s2.xyz.
__device__ __forceinline__ bool tri_test(float4 s0, float4 s1, float4 s2, f3 o, f3 d, float t_min, float t_max,
                                         float& t, float& alpha, float& beta) {
  const f3 A = mk3(s0.x, s0.y, s0.z), AB = mk3(s1.x, s1.y, s1.z), AC = mk3(s2.x, s2.y, s2.z);
  const f3 S1 = cross(d, AC);
  const float div = dot(S1, AB);
  if (!div) return false;
  const float inv_div = 1.0f / div;
  const f3 AO = o - A;
  alpha = dot(AO, S1) * inv_div;
  if (alpha < 0.0f) return false;
  const f3 S2 = cross(AO, AB);
  beta = dot(d, S2) * inv_div;
  if (beta < 0.0f || alpha + beta > 1.0f) return false;
  t = dot(AC, S2) * inv_div;
  if (t < t_min || t > t_max) return false;
  return true;
}

// Local ray of a TransformedShape: origin by the inverse point transform,
// direction by the inverse vector transform then the Ray constructor's
// double normalisation.
__device__ __forceinline__ void sphere_local(const DSphere& s, f3 o, f3 d, f3& lo, f3& ld) {
  lo = xform_point(s.inv, o);
  ld = normalize(xform_vec(s.inv, d));
}

// sphere::get_abc + the quadratic (src/shape/sphere.cpp:7-47). C widens to
// double in the reference; for float operands that equals the float
// difference (an inexact double difference needs an exponent gap > 29 bits,
// where both roundings give the larger operand).
__device__ __forceinline__ bool sphere_roots(f3 lo, f3 ld, float radius, float& t0, float& t1) {
  const float A = len2f(ld);
  const float B = 2.0f * dot(ld, lo);
  const float C = len2f(lo) - radius * radius;
  float delta = B * B - 4.0f * A * C;
  if (delta < 0.0f) return false;
  delta = sqrtf(delta);
  const float inv2A = 0.5f / A;
  t0 = (-B - delta) * inv2A;
  t1 = (-B + delta) * inv2A;
  return true;
}

// Boxes tested and leaf primitives tested by one traversal (the per-ray
// units of the traversal's algorithmic-bytes figure).
struct VisitCount {
  unsigned int boxes = 0, prims = 0;
  unsigned int cache_hits = 0;  // any-hit rays answered by a remembered occluder
};

template <bool ANY, bool COUNT = false>
struct Traversal {
  // Tests one leaf slot. Returns true when ANY and the ray is occluded.
  static __device__ __forceinline__ bool test_slot(const DScene& sc, int slot, f3 o, f3 d, float t_min,
                                                   float& t_max, Hit& h) {
    const float4 s0 = ldg4(sc.slots + 3 * slot);
    const float4 s1 = ldg4(sc.slots + 3 * slot + 1);
    const int kind = __float_as_int(s1.w);
    if (kind < 0) {
      const float4 s2 = ldg4(sc.slots + 3 * slot + 2);
      float t, a, b;
      if (tri_test(s0, s1, s2, o, d, t_min, t_max, t, a, b)) {
        if (ANY) return true;
        t_max = t;
        h.prim = __float_as_int(s0.w);
        h.t_attr = t;
        h.alpha = a;
        h.beta = b;
      }
    } else {
      const DSphere& s = sc.spheres[kind];
      f3 lo, ld;
      sphere_local(s, o, d, lo, ld);
      float t0, t1;
      if (!sphere_roots(lo, ld, s.radius, t0, t1)) return false;
      if (ANY) return (t_min <= t0 && t0 <= t_max) || (t_min <= t1 && t1 <= t_max);
      if (t_max < t0 || t1 < t_min) return false;
      const bool not_t0 = t0 < t_min;
      if (not_t0 && t1 > t_max) return false;
      // Sphere::intersect_p never writes its hit_t argument, so
      // GeometricPrimitive stores 0 into ray.t_max (src/shape/sphere.cpp:98-119,
      // src/shape/geometry.cpp:49-57).
      t_max = 0.0f;
      h.prim = __float_as_int(s0.w);
      h.t_attr = not_t0 ? t1 : t0;
      h.alpha = 0.0f;
      h.beta = 0.0f;
    }
    return false;
  }

};

// Any hit through a remembered occluder: slot s, tested after the box of its
// BVH leaf (stored in the leaf's parent node). The slab test passes a box
// whenever it passes a box inside it (rounding is monotone, a child's box
// lies in its parent's, and the NaN cases of a slab plane through the origin
// act like the parent's infinities), and the culling bound t_max is fixed for
// any hits; so a ray that passes the leaf's box passes every box above it,
// the reference's walk reaches the slot, and a hit there is the walk's answer
// (occluded). A miss here says nothing: the walk follows.
__device__ __forceinline__ bool occluded_by_slot(const DScene& sc, int scene, int s, f3 o, f3 d, float t_min,
                                                 float t_max) {
  const int lp = __ldg(sc.slot_leaf + s);
  float lx, ly, lz, hx, hy, hz;
  if (lp >= 0) {
    const float4* np = reinterpret_cast<const float4*>(sc.nodes + (lp >> 1));
    const float4 b = ldg4(np + 1);
    if (lp & 1) {
      const float4 c = ldg4(np + 2);
      lx = b.z; ly = b.w; lz = c.x; hx = c.y; hy = c.z; hz = c.w;
    } else {
      const float4 a = ldg4(np);
      lx = a.x; ly = a.y; lz = a.z; hx = a.w; hy = b.x; hz = b.y;
    }
  } else {
    const SceneRoot& R = sc.roots[scene];
    lx = R.lo[0]; ly = R.lo[1]; lz = R.lo[2]; hx = R.hi[0]; hy = R.hi[1]; hz = R.hi[2];
  }
  const f3 inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  float tmin;
  if (!box_pass(lx, ly, lz, hx, hy, hz, o, inv, inv.x < 0.0f, inv.y < 0.0f, inv.z < 0.0f, tmin) || !(tmin < t_max))
    return false;
  Hit h;
  float tm = t_max;
  return Traversal<true>::test_slot(sc, s, o, d, t_min, tm, h);
}

// ---------------------------------------------------------------------------
// Persistent traversal with dynamic fetch. Each lane runs the same per-ray
// algorithm as Traversal::run (same order, same culling, same tests), cut
// into steps so that a warp can keep its lanes busy: interior steps repeat
// while any lane of the warp is at an interior node, then the lanes at
// leaves test their primitives; when fewer than `refill` lanes still hold a
// ray, the finished lanes take new rays from the work queue (one atomic per
// warp). Every loop decision is warp-uniform; all 32 lanes stay in the loop
// until the queue is exhausted, so the kernel must be launched with whole
// warps and no lane may return early.

// The traversal stack, in (L1-cached) local memory: 8 bytes per entry, one
// 8-byte store per push. An entry holds the child reference shifted left by
// 5 with its primitive count in the low 5 bits (count 31 stands for "31 or
// more": the true count is then kept in a rarely touched second array) and
// the child's box entry t. Child references stay below 2^26 (checked on
// upload). A stack in shared memory was slower: shared memory takes its
// space from the L1 that serves the node and triangle reads.
constexpr int kStackBinary = 96;               // entries (a binary walk pushes at most one per level)
constexpr int kMaxDepth = kStackBinary - 4;      // the host rejects binary trees this many levels deep
constexpr int kStackWide = 96;                   // entries; the host keeps four-wide trees whose stack bound fits

template <bool ANY, bool COUNT, bool WIDE = false>
struct TravLane {
  static_assert(ANY || !WIDE, "closest-hit traversal keeps the binary order");
  static constexpr int kStack = WIDE ? kStackWide : kStackBinary;
  f3 o, d, inv;
  bool n0, n1, n2;
  float t_min, t_max;
  int cur, cnt, sp;  // current node: cnt 0 interior, > 0 leaf, -1 none (stack ran dry, a leaf is postponed)
  int pl, pc;        // postponed leaf (pc > 0), speculative traversal
  float path_t;      // largest box entry t on the path taken since the last pop
  Hit h;
  bool occluded, failed;
  int2 st[kStack];      // (ref << 5 | min(count, 31), t bits)
  int big_cnt[kStack];  // counts of 31 or more, by stack index

  __device__ __forceinline__ void push(int ref, int c, float t) {
    if (c >= 31) big_cnt[sp] = c;
    st[sp++] = make_int2((ref << 5) | min(c, 31), __float_as_int(t));
  }

  // Starts a ray in scene `scene` of the set; returns false when it misses
  // the root box (done at once).
  // tl: the block staged scene 0's treelet (its root is treelet node 0).
  __device__ __forceinline__ bool start(const DScene& sc, int scene, f3 o_, f3 d_, float tmin_, float tmax_,
                                        VisitCount& vc, bool tl) {
    o = o_;
    d = d_;
    t_min = tmin_;
    t_max = tmax_;
    h.prim = -1;
    occluded = false;
    failed = false;
    sp = 0;
    pc = 0;
    path_t = -INFINITY;
    const SceneRoot& R = sc.roots[scene];
    if (R.kind == 0) return false;
    if (COUNT) ++vc.boxes;
    inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    n0 = inv.x < 0.0f;
    n1 = inv.y < 0.0f;
    n2 = inv.z < 0.0f;
    float tmin;
    if (!box_pass(R.lo[0], R.lo[1], R.lo[2], R.hi[0], R.hi[1], R.hi[2], o, inv, n0, n1, n2, tmin) || !(tmin < t_max))
      return false;
    cur = WIDE && R.kind == 1 ? R.offset4 : R.offset;
    if (!WIDE && tl && scene == 0 && R.kind == 1) cur = kTreeletRef;
    cnt = R.kind == 2 ? R.count : 0;
    return true;
  }

  // Next entry from the stack whose box entry is still before t_max;
  // returns false when the traversal is over.
  __device__ __forceinline__ bool pop() {
    while (sp > 0) {
      const int2 e = st[--sp];
      if (__int_as_float(e.y) < t_max) {
        cur = e.x >> 5;
        cnt = e.x & 31;
        if (cnt == 31) cnt = big_cnt[sp];
        path_t = __int_as_float(e.y);
        return true;
      }
    }
    return false;
  }

  // One child-pair visit at interior node `cur`; returns false when done.
  __device__ __forceinline__ bool interior(const DScene& sc, int* err, VisitCount& vc) {
    float4 a, b, c, dd;
    if (cur & kTreeletRef) {
      const int j = cur & (kTreeletRef - 1);
      a = trav_smem[treelet_slot(j, 0)];
      b = trav_smem[treelet_slot(j, 1)];
      c = trav_smem[treelet_slot(j, 2)];
      dd = trav_smem[treelet_slot(j, 3)];
    } else {
      const float4* np = reinterpret_cast<const float4*>(sc.nodes + cur);
      a = ldg4(np);
      b = ldg4(np + 1);
      c = ldg4(np + 2);
      dd = ldg4(np + 3);
    }
    if (COUNT) vc.boxes += 2;
    float tl, tr;
    const bool hl = box_pass(a.x, a.y, a.z, a.w, b.x, b.y, o, inv, n0, n1, n2, tl) && tl < t_max;
    const bool hr = box_pass(b.z, b.w, c.x, c.y, c.z, c.w, o, inv, n0, n1, n2, tr) && tr < t_max;
    const int axis = __float_as_int(dd.w);
    bool second_near = axis == 0 ? n0 : (axis == 1 ? n1 : n2);
    if (ANY && !COUNT && sc.any_order != 0) {
      // any hit: the answer does not depend on the order, only the visits do
      // (the counting walk keeps the reference's visits)
      if (sc.any_order == 1) {
        second_near = !second_near;  // the far child first
      } else {  // the child with the larger box surface first
        const float lx = a.w - a.x, ly = b.x - a.y, lz = b.y - a.z;
        const float rx = c.y - b.z, ry = c.z - b.w, rz = c.w - c.x;
        second_near = rx * ry + ry * rz + rz * rx > lx * ly + ly * lz + lz * lx;
      }
    }
    const int lref = __float_as_int(dd.x), rref = __float_as_int(dd.y);
    const unsigned cc = (unsigned)__float_as_int(dd.z);
    const int lcnt = (int)(cc & 0xffffu), rcnt = (int)(cc >> 16);
    if (hl && hr) {
      if (sp >= kStack) {
        atomicOr(err, 1);
        h.prim = -1;
        occluded = false;
        failed = true;
        return false;
      }
      if (second_near) {
        push(lref, lcnt, tl);
        cur = rref;
        cnt = rcnt;
        path_t = fmaxf(path_t, tr);
      } else {
        push(rref, rcnt, tr);
        cur = lref;
        cnt = lcnt;
        path_t = fmaxf(path_t, tl);
      }
      return true;
    }
    if (hl) {
      cur = lref;
      cnt = lcnt;
      path_t = fmaxf(path_t, tl);
      return true;
    }
    if (hr) {
      cur = rref;
      cnt = rcnt;
      path_t = fmaxf(path_t, tr);
      return true;
    }
    return pop();
  }

  // Speculative traversal: the leaf just reached is postponed and the walk
  // goes on from the stack (with the t_max from before the leaf's tests).
  __device__ __forceinline__ void postpone() {
    pl = cur;
    pc = cnt;
    if (!pop()) cnt = -1;
  }

  // Tests the postponed leaf; returns false when the traversal is over.
  // Closest hit: the walk made since the postponement used a t_max that the
  // leaf may have lowered. Every box entry t on the current path (path_t is
  // their maximum, counted from the last pop) still below the new t_max means
  // the reference, testing the leaf first, takes the same path and pushes
  // the same entries; otherwise the reference would have culled a box on it:
  // the path is dropped and the next entry popped (entries pushed along it
  // are culled when popped, their boxes lying inside the dropped one).
  __device__ __forceinline__ bool postponed_leaf(const DScene& sc, VisitCount& vc) {
    for (int i = 0; i < pc; ++i) {
      if (COUNT) ++vc.prims;
      if (Traversal<ANY, COUNT>::test_slot(sc, pl + i, o, d, t_min, t_max, h)) {
        occluded = true;
        h.prim = pl + i;  // any hit: the occluding slot
        return false;
      }
    }
    pc = 0;
    if (!ANY && cnt >= 0 && !(path_t < t_max)) cnt = -1;
    if (cnt < 0) return pop();
    return true;
  }

  // One visit of four-wide node `cur` (any-hit only): the children whose
  // boxes pass are all taken, the nearest entered and the others pushed;
  // returns false when done.
  __device__ __forceinline__ bool interior4(const DScene& sc, int* err, VisitCount& vc) {
    const float4* np = reinterpret_cast<const float4*>(sc.nodes4 + cur);
    const float4 lx = ldg4(np), ly = ldg4(np + 1), lz = ldg4(np + 2);
    const float4 hx = ldg4(np + 3), hy = ldg4(np + 4), hz = ldg4(np + 5);
    const float4 rf = ldg4(np + 6), ct = ldg4(np + 7);
    const int refs[4] = {__float_as_int(rf.x), __float_as_int(rf.y), __float_as_int(rf.z), __float_as_int(rf.w)};
    const int cnts[4] = {__float_as_int(ct.x), __float_as_int(ct.y), __float_as_int(ct.z), __float_as_int(ct.w)};
    float t[4];
    bool hit[4];
    hit[0] = cnts[0] >= 0 && box_pass(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, o, inv, n0, n1, n2, t[0]) && t[0] < t_max;
    hit[1] = cnts[1] >= 0 && box_pass(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, o, inv, n0, n1, n2, t[1]) && t[1] < t_max;
    hit[2] = cnts[2] >= 0 && box_pass(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, o, inv, n0, n1, n2, t[2]) && t[2] < t_max;
    hit[3] = cnts[3] >= 0 && box_pass(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, o, inv, n0, n1, n2, t[3]) && t[3] < t_max;
    if (COUNT) vc.boxes += (cnts[0] >= 0) + (cnts[1] >= 0) + (cnts[2] >= 0) + (cnts[3] >= 0);
    int best = -1;
    float bt = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (hit[i] && (best < 0 || t[i] < bt)) {
        best = i;
        bt = t[i];
      }
    if (best < 0) return pop();
    const int npush = hit[0] + hit[1] + hit[2] + hit[3] - 1;
    if (sp + npush > kStack) {
      atomicOr(err, 1);
      h.prim = -1;
      occluded = false;
      failed = true;
      return false;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
      if (hit[i] && i != best) push(refs[i], cnts[i], t[i]);
    cur = best == 0 ? refs[0] : best == 1 ? refs[1] : best == 2 ? refs[2] : refs[3];
    cnt = best == 0 ? cnts[0] : best == 1 ? cnts[1] : best == 2 ? cnts[2] : cnts[3];
    return true;
  }

  // The primitives of leaf `cur`; returns false when done.
  __device__ __forceinline__ bool leaf(const DScene& sc, VisitCount& vc) {
    for (int i = 0; i < cnt; ++i) {
      if (COUNT) ++vc.prims;
      if (Traversal<ANY, COUNT>::test_slot(sc, cur + i, o, d, t_min, t_max, h)) {
        occluded = true;
        h.prim = cur + i;  // any hit: the occluding slot
        return false;
      }
    }
    return pop();
  }
};

// Job: unsigned count() const;
//      void load(unsigned i, f3& o, f3& d, float& t_min, float& t_max, int& scene);
//      int cached(unsigned i) const;  any hits: a slot to test first (occluded_by_slot), or -1
//      void store(unsigned i, const Hit& h, float t_max, bool occluded).
// For an occluded any-hit ray h.prim is the occluding slot.
// tl_n: treelet nodes to stage in shared memory (the launch gives the block
// at least tl_n * 64 bytes of dynamic shared memory; 0: none). The four-wide
// walk does not use the treelet.
template <bool ANY, bool COUNT, bool WIDE = false, class Job>
__device__ __forceinline__ void persistent_traverse(const DScene& sc, Job& job, unsigned int* fetch, int* err,
                                                    VisitCount& vc, int refill, int tl_n = 0) {
  const bool tl = !WIDE && tl_n > 0;
  if (tl) stage_treelet(sc, tl_n);
  const unsigned int n = job.count();
  const unsigned int lane = threadIdx.x & 31u;
  const unsigned int below = (1u << lane) - 1u;
  TravLane<ANY, COUNT, WIDE> L;
  unsigned int item = 0;
  bool live = false, exhausted = false;
  for (;;) {
    const unsigned int need = __ballot_sync(0xffffffffu, !live && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned int base = 0;
      if ((int)lane == leader) base = atomicAdd(fetch, (unsigned int)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (!live && !exhausted) {
        item = base + (unsigned int)__popc(need & below);
        if (item < n) {
          f3 o, d;
          float tmin, tmax;
          int scene;
          job.load(item, o, d, tmin, tmax, scene);
          const int cs = ANY ? job.cached(item) : -1;
          if (ANY && cs >= 0 && occluded_by_slot(sc, scene, cs, o, d, tmin, tmax)) {
            ++vc.cache_hits;
            L.h.prim = cs;
            job.store(item, L.h, tmax, true);
            live = false;
          } else {
            live = L.start(sc, scene, o, d, tmin, tmax, vc, tl);
            if (!live) job.store(item, L.h, L.t_max, false);
          }
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, live)) {
      if (__all_sync(0xffffffffu, exhausted)) break;
      continue;
    }
    if (COUNT) {
      // the reference's walk step for step (its box and primitive counts)
      for (;;) {
        while (__any_sync(0xffffffffu, live && L.cnt == 0)) {
          if (live && L.cnt == 0) {
            live = WIDE ? L.interior4(sc, err, vc) : L.interior(sc, err, vc);
            if (!live) job.store(item, L.h, L.t_max, L.occluded);
          }
        }
        if (live) {
          live = L.leaf(sc, vc);
          if (!live) job.store(item, L.h, L.t_max, L.occluded);
        }
        if (__popc(__ballot_sync(0xffffffffu, live)) < refill) break;
      }
    } else {
      // speculative while-while: interior steps go on while some lane has
      // not found a leaf; a lane holding a postponed leaf keeps walking
      // (and waits at a second leaf); then the postponed leaves are tested
      for (;;) {
        for (;;) {
          if (live && L.cnt > 0 && L.pc == 0) L.postpone();
          if (!__any_sync(0xffffffffu, live && L.pc == 0)) break;
          if (live && L.cnt == 0) {
            const bool more = WIDE ? L.interior4(sc, err, vc) : L.interior(sc, err, vc);
            if (!more) {
              if (L.failed || L.pc == 0) {
                live = false;
                job.store(item, L.h, L.t_max, L.occluded);
              } else {
                L.cnt = -1;
              }
            }
          }
        }
        if (live) {
          live = L.postponed_leaf(sc, vc);
          if (!live) job.store(item, L.h, L.t_max, L.occluded);
        }
        if (__popc(__ballot_sync(0xffffffffu, live)) < refill) break;
      }
    }
  }
}

}  // namespace trg
