// bvh_build.cpp -- host builder of the reference's binned-SAH BVH.
//
// The GPU traverses exactly the tree BVHAccel::build produces
// (src/accelerator/bvh.cpp:78-105, 191-306), because closest-hit ties
// (t == t_max is accepted) make the answer depend on the order primitives are
// tested in. This builder follows the same steps, with the same std
// algorithms from the same C++ library:
//  * node bounds; one primitive -> leaf;
//  * centroid bounds; degenerate along the widest axis -> leaf;
//  * two primitives -> std::nth_element at the midpoint;
//  * otherwise 12 buckets by 12 * offset (truncated, 12 -> 11), cost
//    1 + (nL * SA_L + nR * SA_R) / SA, first minimum by std::min_element,
//    std::partition by bucket when count > max_leaf_prims, else a leaf;
//  * the right subtree is built before the left one (GCC evaluates the two
//    recursive calls passed to init_interior right to left), which fixes
//    the leaf slot offsets;
//  * depth-first flattening, second child stored as an offset.
// It is compiled with -ffp-contract=off like every parity-critical unit.

#include <algorithm>
#include <cstring>
#include <vector>

#include "bvh_build.h"

namespace trg {

namespace {

struct Aabb {
  float lo[3], hi[3];
};

inline Aabb empty_box() {
  Aabb b;
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = kRealMax;
    b.hi[k] = -kRealMax;
  }
  return b;
}
inline void grow(Aabb& b, const float* lo, const float* hi) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = smin(b.lo[k], lo[k]);
    b.hi[k] = smax(b.hi[k], hi[k]);
  }
}
inline void grow_pt(Aabb& b, const float* p) { grow(b, p, p); }
inline float area(const Aabb& b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return 2 * (dx * dy + dx * dz + dy * dz);
}
inline int widest(const Aabb& b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  if (dx > dy && dx > dz) return 0;
  if (dy > dz) return 1;
  return 2;
}

struct Ref {
  uint32_t id;
  Aabb box;
  float c[3];
};

struct Node {
  Aabb box;
  int kids[2] = {-1, -1};
  int axis = 0;
  size_t first = 0, count = 0;
};

struct Build {
  std::vector<Ref>& refs;
  int max_leaf;
  std::vector<Node> nodes;
  std::vector<uint32_t> order;
  int max_depth = 0;

  int make_leaf(int id, size_t s, size_t e, const Aabb& box) {
    nodes[id].first = order.size();
    for (size_t i = s; i < e; ++i) order.push_back(refs[i].id);
    nodes[id].count = e - s;
    nodes[id].box = box;
    return id;
  }

  int run(size_t s, size_t e, int depth) {
    if (depth > max_depth) max_depth = depth;
    int id = (int)nodes.size();
    nodes.emplace_back();
    Aabb box = empty_box();
    for (size_t i = s; i < e; ++i) grow(box, refs[i].box.lo, refs[i].box.hi);
    const size_t n = e - s;
    if (n == 1) return make_leaf(id, s, e, box);
    Aabb cb = empty_box();
    for (size_t i = s; i < e; ++i) grow_pt(cb, refs[i].c);
    int mid = (int)((s + e) >> 1);
    const int dim = widest(cb);
    if (cb.hi[dim] == cb.lo[dim]) return make_leaf(id, s, e, box);
    const float clo = cb.lo[dim], chi = cb.hi[dim];
    auto bucket = [clo, chi, dim](const Ref& r) {
      float o = r.c[dim] - clo;
      if (chi > clo) o /= chi - clo;
      int b = (int)(12 * o);
      return b == 12 ? 11 : b;
    };
    if (n <= 2) {
      std::nth_element(&refs[s], &refs[mid], &refs[e - 1] + 1,
                       [dim](const Ref& a, const Ref& b) { return a.c[dim] < b.c[dim]; });
    } else {
      size_t cnt[12] = {0};
      Aabb bb[12];
      for (int k = 0; k < 12; ++k) bb[k] = empty_box();
      for (size_t i = s; i < e; ++i) {
        int b = bucket(refs[i]);
        cnt[b]++;
        grow(bb[b], refs[i].box.lo, refs[i].box.hi);
      }
      float cost[11];
      const float sa = area(box);
      for (int k = 0; k < 11; ++k) {
        Aabb l = empty_box(), r = empty_box();
        int nl = 0, nr = 0;
        for (int j = 0; j <= k; ++j) { grow(l, bb[j].lo, bb[j].hi); nl += (int)cnt[j]; }
        for (int j = k + 1; j < 12; ++j) { grow(r, bb[j].lo, bb[j].hi); nr += (int)cnt[j]; }
        cost[k] = 1 + (nl * area(l) + nr * area(r)) / sa;
      }
      const long best = std::min_element(cost, cost + 11) - cost;
      if (n > (size_t)max_leaf) {
        Ref* p = std::partition(&refs[s], &refs[e - 1] + 1, [&](const Ref& r) { return bucket(r) <= best; });
        mid = (int)(p - refs.data());
      } else {
        return make_leaf(id, s, e, box);
      }
    }
    const int right = run((size_t)mid, e, depth + 1);
    const int left = run(s, (size_t)mid, depth + 1);
    nodes[id].kids[0] = left;
    nodes[id].kids[1] = right;
    nodes[id].axis = dim;
    Aabb u = nodes[left].box;
    grow(u, nodes[right].box.lo, nodes[right].box.hi);
    nodes[id].box = u;
    nodes[id].count = 0;
    return id;
  }

  int flatten(int b, std::vector<tr_bvh_node32>& out) {
    const int off = (int)out.size();
    out.emplace_back();
    std::memset(&out[off], 0, sizeof(tr_bvh_node32));
    for (int k = 0; k < 3; ++k) {
      out[off].lo[k] = nodes[b].box.lo[k];
      out[off].hi[k] = nodes[b].box.hi[k];
    }
    if (nodes[b].count > 0) {
      out[off].count = (uint16_t)nodes[b].count;
      out[off].offset = (int32_t)nodes[b].first;
    } else {
      out[off].axis = (uint8_t)nodes[b].axis;
      flatten(nodes[b].kids[0], out);
      const int second = flatten(nodes[b].kids[1], out);
      out[off].offset = second;
    }
    return off;
  }
};

}  // namespace

BvhResult build_reference_bvh(const float* lo, const float* hi, size_t n, int max_leaf_prims) {
  BvhResult res;
  if (n == 0) return res;
  std::vector<Ref> refs(n);
  for (size_t i = 0; i < n; ++i) {
    Ref& r = refs[i];
    r.id = (uint32_t)i;
    for (int k = 0; k < 3; ++k) {
      r.box.lo[k] = lo[3 * i + k];
      r.box.hi[k] = hi[3 * i + k];
      // 0.5 * low + 0.5 * high: double scale rounded to float, float add (bvh.cpp:18)
      r.c[k] = (float)(0.5 * r.box.lo[k]) + (float)(0.5 * r.box.hi[k]);
    }
  }
  Build b{refs, max_leaf_prims, {}, {}, 0};
  b.nodes.reserve(2 * n);
  b.order.reserve(n);
  const int root = b.run(0, n, 0);
  b.flatten(root, res.nodes);
  res.order = std::move(b.order);
  res.depth = b.max_depth;
  return res;
}

}  // namespace trg
