// context.cu -- context, scene upload and ray-batch entry points of the C ABI.
//
// Scene upload does on the host what the reference does at construction time
// (src/shape/triangle.cpp:216-236, src/shape/sphere.cpp:83-92,
// src/material/phong.cpp:29-70, src/accelerator/bvh.cpp:78-105), then packs
// the device tables described in scene_types.h. Host arithmetic here is
// compiled with -ffp-contract=off so the precomputed values are the ones the
// reference computes.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <thread>
#include <atomic>
#include <cstring>
#include <string>
#include <vector>

#include "binning.cuh"
#include "bvh_build.h"
#include "context.h"
#include "mat_setup.cuh"
#include "traverse.cuh"

namespace trg {

tr_status set_err(tr_ctx* ctx, tr_status s, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return s;
}

tr_status cuda_fail(tr_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return set_err(ctx, TR_ERR_OOM, std::string(what) + ": " + cudaGetErrorString(e));
  }
  return set_err(ctx, TR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}


namespace {

const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

inline float as_float(int i) {
  float f;
  std::memcpy(&f, &i, 4);
  return f;
}

// A child of a four-wide node under construction.
struct Child4 {
  float lo[3], hi[3];
  int ref, cnt;
};

void node_children(const DNode& n, Child4& l, Child4& r) {
  const uint32_t cc = (uint32_t)n.d.z;
  l = Child4{{n.a.x, n.a.y, n.a.z}, {n.a.w, n.b.x, n.b.y}, n.d.x, (int)(cc & 0xffffu)};
  r = Child4{{n.b.z, n.b.w, n.c.x}, {n.c.y, n.c.z, n.c.w}, n.d.y, (int)(cc >> 16)};
}

float half_area(const Child4& c) {
  const float x = c.hi[0] - c.lo[0], y = c.hi[1] - c.lo[1], z = c.hi[2] - c.lo[2];
  return x * y + y * z + z * x;
}

// Collapses the child-pair tree below DNode `root` into four-wide nodes
// appended to `out` (the interior child of largest surface area is opened
// until four children or only leaves remain) and returns the root's index.
// `stack` receives a bound on the traversal stack its any-hit walk needs: a
// node pushes at most all its children but the one it enters, so the bound
// is (children - 1) plus the largest bound of an interior child.
int collapse4(const std::vector<DNode>& dn, int root, std::vector<DNode4>& out, int& stack) {
  Child4 ch[4];
  int k = 2;
  node_children(dn[root], ch[0], ch[1]);
  while (k < 4) {
    int best = -1;
    float area = -1.0f;
    for (int i = 0; i < k; ++i)
      if (ch[i].cnt == 0 && half_area(ch[i]) > area) {
        area = half_area(ch[i]);
        best = i;
      }
    if (best < 0) break;
    node_children(dn[ch[best].ref], ch[best], ch[k]);
    ++k;
  }
  const int idx = (int)out.size();
  out.emplace_back();
  int refs[4] = {0, 0, 0, 0}, cnts[4] = {-1, -1, -1, -1}, deepest = 0;
  for (int i = 0; i < k; ++i) {
    cnts[i] = ch[i].cnt;
    if (ch[i].cnt > 0) {
      refs[i] = ch[i].ref;
    } else {
      int sub = 0;
      refs[i] = collapse4(dn, ch[i].ref, out, sub);
      deepest = std::max(deepest, sub);
    }
  }
  stack = (k - 1) + deepest;
  float v[6][4] = {};
  for (int i = 0; i < k; ++i)
    for (int c = 0; c < 3; ++c) {
      v[c][i] = ch[i].lo[c];
      v[3 + c][i] = ch[i].hi[c];
    }
  DNode4& o = out[idx];
  float4* box = &o.lox;
  for (int r = 0; r < 6; ++r) box[r] = float4{v[r][0], v[r][1], v[r][2], v[r][3]};
  o.ref = int4{refs[0], refs[1], refs[2], refs[3]};
  o.cnt = int4{cnts[0], cnts[1], cnts[2], cnts[3]};
  return idx;
}

}  // namespace

// Builds DNodes + slots from hs.nodes/hs.order and uploads every table.
tr_status upload_device_tables(tr_ctx* ctx) {
  HostScene& hs = ctx->hs;
  if (hs.device_bvh) return upload_device_built(ctx);
  const size_t nn = hs.nodes.size();
  // validate the flattened tree: children strictly after their parent, leaf
  // ranges inside the slot array, depth bounded by the traversal stack
  std::vector<int> dix(nn, -1), depth(nn, 0);
  int ninterior = 0;
  for (size_t i = 0; i < nn; ++i) {
    const tr_bvh_node32& n = hs.nodes[i];
    if (n.count > 0) {
      if (n.offset < 0 || (size_t)n.offset + n.count > hs.order.size())
        return set_err(ctx, TR_ERR_ARG, "bvh leaf range outside the primitive order");
    } else {
      if (i + 1 >= nn || n.offset <= (int32_t)(i + 1) || (size_t)n.offset >= nn)
        return set_err(ctx, TR_ERR_ARG, "bvh interior node with invalid children");
      dix[i] = ninterior++;
    }
  }
  for (uint32_t p : hs.order)
    if (p >= hs.prims.size()) return set_err(ctx, TR_ERR_ARG, "bvh primitive order entry out of range");
  int maxd = 0;
  for (size_t i = 0; i < nn; ++i) {
    const tr_bvh_node32& n = hs.nodes[i];
    if (n.count == 0) {
      depth[i + 1] = std::max(depth[i + 1], depth[i] + 1);
      depth[n.offset] = std::max(depth[n.offset], depth[i] + 1);
    }
    maxd = std::max(maxd, depth[i]);
  }
  if (maxd >= kMaxDepth)
    return set_err(ctx, TR_ERR_UNSUPPORTED, "bvh deeper than the device traversal stack (" + std::to_string(kMaxDepth) + ")");
  if (hs.order.size() >= (1u << 26) || (size_t)ninterior >= (1u << 26))
    return set_err(ctx, TR_ERR_UNSUPPORTED, "more than 2^26 primitives or interior nodes in one upload");
  hs.depth = maxd;

  std::vector<DNode> dn(ninterior);
  for (size_t i = 0; i < nn; ++i) {
    const tr_bvh_node32& n = hs.nodes[i];
    if (n.count > 0) continue;
    const tr_bvh_node32& L = hs.nodes[i + 1];
    const tr_bvh_node32& R = hs.nodes[n.offset];
    DNode& d = dn[dix[i]];
    d.a = float4{L.lo[0], L.lo[1], L.lo[2], L.hi[0]};
    d.b = float4{L.hi[1], L.hi[2], R.lo[0], R.lo[1]};
    d.c = float4{R.lo[2], R.hi[0], R.hi[1], R.hi[2]};
    const int lref = L.count > 0 ? L.offset : dix[i + 1];
    const int rref = R.count > 0 ? R.offset : dix[n.offset];
    d.d = int4{lref, rref, (int)((uint32_t)L.count | ((uint32_t)R.count << 16)), (int)n.axis};
  }
  std::vector<float4> slots(3 * hs.order.size());
  for (size_t s = 0; s < hs.order.size(); ++s) {
    const uint32_t pid = hs.order[s];
    const DPrim& p = hs.prims[pid];
    if (p.kind == PRIM_TRIANGLE) {
      const f3 A = hs.A[p.shape], AB = hs.AB[p.shape], AC = hs.AC[p.shape];
      slots[3 * s] = float4{A.x, A.y, A.z, as_float((int)pid)};
      slots[3 * s + 1] = float4{AB.x, AB.y, AB.z, as_float(-1)};
      slots[3 * s + 2] = float4{AC.x, AC.y, AC.z, 0.0f};
    } else {
      slots[3 * s] = float4{0.0f, 0.0f, 0.0f, as_float((int)pid)};
      slots[3 * s + 1] = float4{0.0f, 0.0f, 0.0f, as_float(p.shape)};
      slots[3 * s + 2] = float4{0.0f, 0.0f, 0.0f, 0.0f};
    }
  }
  auto put = [&](DevBuf& b, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t e = b.reserve(bytes ? bytes : 16);
    if (e != cudaSuccess) return e;
    if (bytes) return cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    return cudaSuccess;
  };
  // where each slot's leaf box is stored (the occluder cache tests it)
  std::vector<int> slot_leaf(hs.order.size(), -1);
  for (size_t i = 0; i < nn; ++i) {
    const tr_bvh_node32& n = hs.nodes[i];
    if (n.count > 0) continue;
    const tr_bvh_node32* kids[2] = {&hs.nodes[i + 1], &hs.nodes[n.offset]};
    for (int side = 0; side < 2; ++side)
      if (kids[side]->count > 0)
        for (int s = 0; s < kids[side]->count; ++s) slot_leaf[(size_t)kids[side]->offset + s] = 2 * dix[i] + side;
  }
  TR_CUDA(ctx, put(ctx->d_nodes, dn.data(), dn.size() * sizeof(DNode)));
  TR_CUDA(ctx, put(ctx->d_slots, slots.data(), slots.size() * sizeof(float4)));
  TR_CUDA(ctx, put(ctx->d_slot_leaf, slot_leaf.data(), slot_leaf.size() * sizeof(int)));
  TR_CUDA(ctx, put(ctx->d_spheres, hs.spheres.data(), hs.spheres.size() * sizeof(DSphere)));
  TR_CUDA(ctx, put(ctx->d_prims, hs.prims.data(), hs.prims.size() * sizeof(DPrim)));
  TR_CUDA(ctx, put(ctx->d_tshade, hs.tshade.data(), hs.tshade.size() * sizeof(DTriShade)));
  TR_CUDA(ctx, put(ctx->d_mats, hs.mats.data(), hs.mats.size() * sizeof(DMat)));
  TR_CUDA(ctx, put(ctx->d_lights, hs.lights.data(), hs.lights.size() * sizeof(DLight)));

  // one root per scene of the set
  const size_t nsc = hs.scene_node.size();
  std::vector<SceneRoot> roots(nsc);
  int max_lights = 0;
  for (size_t k = 0; k < nsc; ++k) {
    SceneRoot& R = roots[k];
    std::memset(&R, 0, sizeof(R));
    const size_t first = hs.scene_node[k], end = k + 1 < nsc ? hs.scene_node[k + 1] : nn;
    R.light_base = (int)hs.scene_light[k];
    R.num_lights = (int)hs.scene_nlight[k];
    max_lights = std::max(max_lights, R.num_lights);
    if (first >= end) {
      R.kind = 0;
      continue;
    }
    const tr_bvh_node32& r = hs.nodes[first];
    for (int c = 0; c < 3; ++c) {
      R.lo[c] = r.lo[c];
      R.hi[c] = r.hi[c];
    }
    if (r.count > 0) {
      R.kind = 2;
      R.offset = r.offset;
      R.count = r.count;
    } else {
      R.kind = 1;
      R.offset = dix[first];
    }
  }
  // the four-wide any-hit tree of every scene, unless its stack bound is
  // above the traversal stack
  std::vector<DNode4> dn4;
  dn4.reserve(dn.size() / 2 + nsc);
  int stack4 = 0;
  for (size_t k = 0; k < nsc; ++k)
    if (roots[k].kind == 1) {
      int sub = 0;
      roots[k].offset4 = collapse4(dn, roots[k].offset, dn4, sub);
      stack4 = std::max(stack4, sub);
    }
  const bool wide = stack4 <= kStackWide;
  if (wide) TR_CUDA(ctx, put(ctx->d_nodes4, dn4.data(), dn4.size() * sizeof(DNode4)));
  ctx->any4_nodes = wide ? dn4.size() : 0;
  ctx->any4_stack = stack4;
  TR_CUDA(ctx, put(ctx->d_roots, roots.data(), roots.size() * sizeof(SceneRoot)));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  hs.root0 = nsc == 1 && roots[0].kind == 1 ? roots[0].offset : -1;
  hs.dnodes = std::move(dn);

  DScene& sc = ctx->dsc;
  sc.nodes = ctx->d_nodes.as<DNode>();
  sc.nodes4 = wide ? ctx->d_nodes4.as<DNode4>() : nullptr;
  sc.treelet = nullptr;
  sc.treelet_n = 0;
  sc.slots = ctx->d_slots.as<float4>();
  sc.slot_leaf = ctx->d_slot_leaf.as<int>();
  sc.spheres = ctx->d_spheres.as<DSphere>();
  sc.prims = ctx->d_prims.as<DPrim>();
  sc.tshade = ctx->d_tshade.as<DTriShade>();
  sc.mats = ctx->d_mats.as<DMat>();
  sc.lights = ctx->d_lights.as<DLight>();
  sc.roots = ctx->d_roots.as<SceneRoot>();
  sc.num_scenes = (int)nsc;
  sc.max_lights = max_lights;
  sc.any_order = ctx->tune.any_hit_order;
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
  es = upload_treelet(ctx);
  if (es != TR_OK) return es;
  ctx->has_scene = true;
  return TR_OK;
}

// A sphere around an area-light triangle as the triangle test sees it (A,
// A + AB, A + AC, in double), widened by 1e-3 of its radius and of the
// coordinates' scale: every point that test accepts lies well inside.
static void light_sphere(DLight& L) {
  const double A[3] = {L.A.x, L.A.y, L.A.z}, AB[3] = {L.AB.x, L.AB.y, L.AB.z}, AC[3] = {L.AC.x, L.AC.y, L.AC.z};
  double c[3], scale = 1.0, r2 = 0.0;
  for (int k = 0; k < 3; ++k) c[k] = A[k] + (AB[k] + AC[k]) / 3.0;
  float cf[3];
  for (int k = 0; k < 3; ++k) cf[k] = (float)c[k];
  for (int v = 0; v < 3; ++v) {
    double d2 = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double p = A[k] + (v == 1 ? AB[k] : v == 2 ? AC[k] : 0.0);
      scale = std::max(scale, std::fabs(p));
      const double e = p - (double)cf[k];
      d2 += e * e;
    }
    r2 = std::max(r2, d2);
  }
  for (int k = 0; k < 3; ++k) L.bs[k] = cf[k];
  L.bs[3] = (float)(std::sqrt(r2) * (1.0 + 1e-3) + 1e-3 * scale);
  L.bs_cn = (float)std::sqrt((double)cf[0] * cf[0] + (double)cf[1] * cf[1] + (double)cf[2] * cf[2]);
}

tr_status upload_treelet(tr_ctx* ctx) {
  DScene& sc = ctx->dsc;
  sc.treelet = nullptr;
  sc.treelet_n = 0;
  const HostScene& hs = ctx->hs;
  const int want = ctx->tune.treelet_nodes;
  if (want <= 0 || hs.root0 < 0 || hs.dnodes.size() >= (size_t)kTreeletRef) return TR_OK;
  // breadth first from the root: node `order[i]` becomes treelet node i
  std::vector<int> order{hs.root0};
  std::vector<int> at(hs.dnodes.size(), -1);
  at[hs.root0] = 0;
  for (size_t h = 0; h < order.size(); ++h) {
    const DNode& d = hs.dnodes[order[h]];
    const unsigned cc = (unsigned)d.d.z;
    const int child[2] = {d.d.x, d.d.y};
    const bool interior[2] = {(cc & 0xffffu) == 0, (cc >> 16) == 0};
    for (int c = 0; c < 2; ++c)
      if (interior[c] && (int)order.size() < want) {
        at[child[c]] = (int)order.size();
        order.push_back(child[c]);
      }
  }
  std::vector<DNode> tl(order.size());
  for (size_t i = 0; i < order.size(); ++i) {
    DNode d = hs.dnodes[order[i]];
    const unsigned cc = (unsigned)d.d.z;
    if ((cc & 0xffffu) == 0 && at[d.d.x] >= 0) d.d.x = kTreeletRef | at[d.d.x];
    if ((cc >> 16) == 0 && at[d.d.y] >= 0) d.d.y = kTreeletRef | at[d.d.y];
    tl[i] = d;
  }
  TR_CUDA(ctx, ctx->d_treelet.reserve(tl.size() * sizeof(DNode)));
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_treelet.p, tl.data(), tl.size() * sizeof(DNode), cudaMemcpyHostToDevice,
                               ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  sc.treelet = ctx->d_treelet.as<DNode>();
  sc.treelet_n = (int)tl.size();
  return TR_OK;
}

cudaError_t allow_dynamic_smem(const void* kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

tr_status upload_textures(tr_ctx* ctx) {
  const std::vector<HostScene::Tex>& tx = ctx->hs.textures;
  DScene& sc = ctx->dsc;
  sc.textures = nullptr;
  sc.msrc = nullptr;
  sc.has_textures = 0;
  for (const DMat& m : ctx->hs.mats)
    if (m.tex_any) sc.has_textures = 1;
  if (tx.empty()) return TR_OK;
  if (sc.has_textures) {
    // the factory arguments of every material, for the set-ups at hits with maps
    TR_CUDA(ctx, ctx->d_msrc.reserve(ctx->hs.msrc.size() * sizeof(tr_material)));
    TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_msrc.p, ctx->hs.msrc.data(), ctx->hs.msrc.size() * sizeof(tr_material),
                                 cudaMemcpyHostToDevice, ctx->stream));
    sc.msrc = ctx->d_msrc.as<tr_material>();
  }
  // one pool, 16 bytes per float texel and 4 per byte texel, every map 16-byte aligned
  size_t total = 0;
  std::vector<size_t> off(tx.size());
  for (size_t i = 0; i < tx.size(); ++i) {
    off[i] = total;
    const size_t bytes = tx[i].texels.empty() ? tx[i].texels8.size() : tx[i].texels.size() * sizeof(float);
    total += (bytes + 15) & ~size_t(15);
  }
  std::vector<uint8_t> pool(total, 0);
  for (size_t i = 0; i < tx.size(); ++i) {
    if (!tx[i].texels.empty()) std::memcpy(pool.data() + off[i], tx[i].texels.data(), tx[i].texels.size() * 4);
    else std::memcpy(pool.data() + off[i], tx[i].texels8.data(), tx[i].texels8.size());
  }
  TR_CUDA(ctx, ctx->d_tex_pool.reserve(total));
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_tex_pool.p, pool.data(), total, cudaMemcpyHostToDevice, ctx->stream));
  const uint8_t* base = ctx->d_tex_pool.as<uint8_t>();
  std::vector<DTex> recs(tx.size());
  for (size_t i = 0; i < tx.size(); ++i) {
    recs[i].texels = tx[i].texels.empty() ? nullptr : reinterpret_cast<const float4*>(base + off[i]);
    recs[i].texels8 = tx[i].texels8.empty() ? nullptr : reinterpret_cast<const uchar4*>(base + off[i]);
    recs[i].w = tx[i].w;
    recs[i].h = tx[i].h;
  }
  TR_CUDA(ctx, ctx->d_texs.reserve(recs.size() * sizeof(DTex)));
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_texs.p, recs.data(), recs.size() * sizeof(DTex), cudaMemcpyHostToDevice,
                               ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  sc.textures = ctx->d_texs.as<DTex>();
  return TR_OK;
}

tr_status upload_envs(tr_ctx* ctx) {
  const std::vector<EnvHost>& envs = ctx->hs.envs;
  DScene& sc = ctx->dsc;
  sc.envs = nullptr;
  sc.has_env = envs.empty() ? 0 : 1;
  if (envs.empty()) return TR_OK;
  // one pool of floats, every array starting on a 16-byte boundary
  size_t total = 0;
  auto take = [&](size_t n) {
    const size_t at = total;
    total += (n + 3) & ~size_t(3);
    return at;
  };
  struct Off { size_t tex, tex8, cf, cc, ci, mc; };
  std::vector<Off> off(envs.size());
  for (size_t i = 0; i < envs.size(); ++i) {
    const EnvHost& e = envs[i];
    off[i] = {take(e.texels.size()), take(e.texels8.size() / 4), take(e.cond_func.size()),
              take(e.cond_cdf.size()), take(e.cond_int.size()), take(e.marg_cdf.size())};
  }
  std::vector<float> pool(total, 0.0f);
  for (size_t i = 0; i < envs.size(); ++i) {
    const EnvHost& e = envs[i];
    std::copy(e.texels.begin(), e.texels.end(), pool.begin() + (ptrdiff_t)off[i].tex);
    if (!e.texels8.empty()) std::memcpy(pool.data() + off[i].tex8, e.texels8.data(), e.texels8.size());
    std::copy(e.cond_func.begin(), e.cond_func.end(), pool.begin() + (ptrdiff_t)off[i].cf);
    std::copy(e.cond_cdf.begin(), e.cond_cdf.end(), pool.begin() + (ptrdiff_t)off[i].cc);
    std::copy(e.cond_int.begin(), e.cond_int.end(), pool.begin() + (ptrdiff_t)off[i].ci);
    std::copy(e.marg_cdf.begin(), e.marg_cdf.end(), pool.begin() + (ptrdiff_t)off[i].mc);
  }
  TR_CUDA(ctx, ctx->d_env_pool.reserve(total * sizeof(float)));
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_env_pool.p, pool.data(), total * sizeof(float), cudaMemcpyHostToDevice,
                               ctx->stream));
  const float* base = ctx->d_env_pool.as<float>();
  std::vector<DEnv> recs(envs.size());
  for (size_t i = 0; i < envs.size(); ++i) {
    const EnvHost& e = envs[i];
    DEnv& r = recs[i];
    std::memset(&r, 0, sizeof(r));
    r.texels = e.texels.empty() ? nullptr : reinterpret_cast<const float4*>(base + off[i].tex);
    r.texels8 = e.texels8.empty() ? nullptr : reinterpret_cast<const uchar4*>(base + off[i].tex8);
    r.cond_func = base + off[i].cf;
    r.cond_cdf = base + off[i].cc;
    r.cond_int = base + off[i].ci;
    r.marg_cdf = base + off[i].mc;
    r.marg_int = e.marg_int;
    r.w = e.w;
    r.h = e.h;
    r.nu = e.nu;
    r.nv = e.nv;
    std::memcpy(r.to_light, e.to_light, sizeof(r.to_light));
    std::memcpy(r.to_world, e.to_world, sizeof(r.to_world));
    std::memcpy(r.center, e.center, sizeof(r.center));
    r.radius = e.radius;
  }
  TR_CUDA(ctx, ctx->d_envs.reserve(recs.size() * sizeof(DEnv)));
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_envs.p, recs.data(), recs.size() * sizeof(DEnv), cudaMemcpyHostToDevice,
                               ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  sc.envs = ctx->d_envs.as<DEnv>();
  return TR_OK;
}

// ------------------------------------------------------------ batch kernels
// Rays as two float4: (o.xyz, d.x), (d.y, d.z, t_min, t_max).
struct BatchJob {
  const float4* __restrict__ rays;
  unsigned int n;
  int32_t* prim;  // closest: prim id and t (prim, tout); any: hit flags (hit); all null: no output
  float* tout;
  uint8_t* hit;
  const int* perm;  // ray binning: work item i is ray perm[i] (null: ray i)
  __device__ __forceinline__ unsigned int count() const { return n; }
  __device__ __forceinline__ int cached(unsigned int) const { return -1; }
  __device__ __forceinline__ void load(unsigned int w, f3& o, f3& d, float& t_min, float& t_max, int& scene) const {
    scene = 0;
    const unsigned int i = perm ? (unsigned int)perm[w] : w;
    const float4 r0 = __ldg(rays + 2 * (size_t)i), r1 = __ldg(rays + 2 * (size_t)i + 1);
    o = mk3(r0.x, r0.y, r0.z);
    d = mk3(r0.w, r1.x, r1.y);
    t_min = r1.z;
    t_max = r1.w;
  }
  __device__ __forceinline__ void store(unsigned int w, const Hit& h, float t_max, bool occluded) const {
    const unsigned int i = perm ? (unsigned int)perm[w] : w;
    if (prim) {
      prim[i] = h.prim;
      tout[i] = t_max;
    } else if (hit) {
      hit[i] = occluded ? 1 : 0;
    }  // neither: a counting run without outputs
  }
};

// The caller's ray array as a source of ray binning (binning.cuh).
struct BatchSrc {
  const float4* rays;
  unsigned int n;
  __device__ __forceinline__ unsigned int count() const { return n; }
  __device__ __forceinline__ int item(unsigned int i) const { return (int)i; }
  __device__ __forceinline__ void ray(unsigned int i, f3& o, f3& d, int& scene) const {
    scene = 0;
    const float4 r0 = __ldg(rays + 2 * (size_t)i), r1 = __ldg(rays + 2 * (size_t)i + 1);
    o = mk3(r0.x, r0.y, r0.z);
    d = mk3(r0.w, r1.x, r1.y);
  }
};

template <bool ANY, bool WIDE = false>
__global__ void __launch_bounds__(128) k_trace_batch(DScene sc, BatchJob job, unsigned int* fetch, int* err,
                                                    int refill, int tl_n) {
  VisitCount vc;
  persistent_traverse<ANY, false, WIDE>(sc, job, fetch, err, vc, refill, tl_n);
}

// The same traversal counting boxes and primitives tested (all lanes leave
// the persistent loop together, so the warp reduction sees every lane).
template <bool ANY, bool WIDE = false>
__global__ void __launch_bounds__(128) k_trace_count(DScene sc, BatchJob job, unsigned int* fetch, int* err,
                                                    int refill, unsigned long long* counts, int tl_n) {
  VisitCount vc;
  persistent_traverse<ANY, true, WIDE>(sc, job, fetch, err, vc, refill, tl_n);
  const unsigned int b = __reduce_add_sync(0xffffffffu, vc.boxes), p = __reduce_add_sync(0xffffffffu, vc.prims);
  if ((threadIdx.x & 31u) == 0) {
    atomicAdd(counts, (unsigned long long)b);
    atomicAdd(counts + 1, (unsigned long long)p);
  }
}

int traversal_grid(const tr_ctx* ctx, const void* kernel, size_t smem) {
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess) {
    cudaGetLastError();
    sms = 1;
  }
  int per_sm = ctx->tune.trav_blocks_per_sm;
  if (per_sm <= 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 128, smem) != cudaSuccess || per_sm <= 0) {
      cudaGetLastError();
      per_sm = 4;
    }
  }
  return std::max(sms, 1) * per_sm;
}

// Launches the persistent traversal of `job` (counts: the counting kernel,
// which adds boxes and primitives tested there) on the context stream: the
// tuned grid, the shared-memory treelet for binary walks, and -- with
// ray_bin_bits -- the rays visited in binned order.
template <bool ANY, bool WIDE>
tr_status launch_trace(tr_ctx* ctx, BatchJob& job, unsigned long long* counts) {
  cudaStream_t st = ctx->stream;
  unsigned int* fetch = reinterpret_cast<unsigned int*>(ctx->d_err.as<int>() + 1);
  TR_CUDA(ctx, cudaMemsetAsync(fetch, 0, sizeof(int), st));  // work-fetch position
  const int bits = ctx->tune.ray_bin_bits;
  if (bits > 0) {
    const int nb = 1 << (3 + 3 * bits);
    TR_CUDA(ctx, ctx->d_perm.reserve((size_t)job.n * 4));
    TR_CUDA(ctx, ctx->d_bin_key.reserve((size_t)job.n * 4));
    TR_CUDA(ctx, ctx->d_bin_cnt.reserve((size_t)nb * 4));
    unsigned int* cnt = ctx->d_bin_cnt.as<unsigned int>();
    unsigned int* keys = ctx->d_bin_key.as<unsigned int>();
    int sms = 1;
    TR_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    const BatchSrc src{job.rays, job.n};
    TR_CUDA(ctx, cudaMemsetAsync(cnt, 0, (size_t)nb * 4, st));
    k_bin_count<<<sms * 8, 128, 0, st>>>(src, ctx->dsc, cnt, keys, bits);
    k_bin_scan<<<1, kBinScanThreads, 0, st>>>(cnt, nb);
    k_bin_scatter<<<sms * 8, 128, 0, st>>>(src, cnt, keys, ctx->d_perm.as<int>());
    job.perm = ctx->d_perm.as<int>();
  }
  const int tl = WIDE ? 0 : treelet_nodes(ctx);
  const size_t smem = (size_t)tl * sizeof(DNode);
  const void* k = counts ? (const void*)k_trace_count<ANY, WIDE> : (const void*)k_trace_batch<ANY, WIDE>;
  TR_CUDA(ctx, allow_dynamic_smem(k, smem));
  const int grid = traversal_grid(ctx, k, smem);
  if (counts)
    k_trace_count<ANY, WIDE><<<grid, 128, smem, st>>>(ctx->dsc, job, fetch, ctx->d_err.as<int>(),
                                                      ctx->tune.trav_refill_lanes, counts, tl);
  else
    k_trace_batch<ANY, WIDE><<<grid, 128, smem, st>>>(ctx->dsc, job, fetch, ctx->d_err.as<int>(),
                                                      ctx->tune.trav_refill_lanes, tl);
  TR_CUDA(ctx, cudaGetLastError());
  return TR_OK;
}

}  // namespace trg

using namespace trg;

extern "C" {

const char* tr_status_string(tr_status s) {
  switch (s) {
    case TR_OK: return "ok";
    case TR_ERR_ARG: return "invalid argument";
    case TR_ERR_OOM: return "out of memory";
    case TR_ERR_QUEUE_OVERFLOW: return "device queue overflow";
    case TR_ERR_TIMEOUT: return "device loop gave up";
    case TR_ERR_CUDA: return "CUDA error";
    case TR_ERR_STATE: return "call out of order";
    case TR_ERR_CANCELLED: return "cancelled";
    case TR_ERR_UNSUPPORTED: return "unsupported scene feature";
  }
  return "unknown status";
}

tr_status tr_make_ray(const float o[3], const float d[3], float t_min, float t_max, tr_ray* out) {
  if (!o || !d || !out) return TR_ERR_ARG;
  const f3 n = normalize(mk3(d[0], d[1], d[2]));
  out->o[0] = o[0]; out->o[1] = o[1]; out->o[2] = o[2];
  out->d[0] = n.x; out->d[1] = n.y; out->d[2] = n.z;
  out->t_min = t_min;
  out->t_max = t_max;
  return TR_OK;
}

tr_status tr_ctx_create(tr_ctx** out, int device) {
  if (!out) return TR_ERR_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return TR_ERR_CUDA;
  }
  trg::DeviceScope scope(device);
  if (scope.status != cudaSuccess) return TR_ERR_CUDA;
  tr_ctx* ctx = new tr_ctx();
  ctx->device = device;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return TR_ERR_CUDA;
  }
  if (ctx->d_err.reserve(64) != cudaSuccess || cudaMemset(ctx->d_err.p, 0, 64) != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return TR_ERR_OOM;
  }
  *out = ctx;
  return TR_OK;
}

void tr_ctx_destroy(tr_ctx* ctx) {
  if (!ctx) return;
  trg::DeviceScope scope(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  release_render(ctx);
  release_guide(ctx);
  for (DevBuf* b : {&ctx->d_nodes, &ctx->d_nodes4, &ctx->d_slots, &ctx->d_spheres, &ctx->d_prims, &ctx->d_tshade,
                    &ctx->d_mats, &ctx->d_lights, &ctx->d_roots, &ctx->d_rays, &ctx->d_out0, &ctx->d_out1,
                    &ctx->d_err, &ctx->d_env_pool, &ctx->d_envs, &ctx->d_tex_pool, &ctx->d_texs, &ctx->d_treelet,
                    &ctx->d_perm, &ctx->d_bin_key, &ctx->d_bin_cnt, &ctx->d_slot_leaf, &ctx->d_lg_acc,
                    &ctx->d_lg_cdf, &ctx->d_msrc})
    b->release();
  cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char* tr_ctx_last_error(const tr_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }
void* tr_ctx_stream(tr_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

tr_status tr_ctx_set_tuning(tr_ctx* ctx, const tr_tuning* t) {
  if (!ctx || !t) return TR_ERR_ARG;
  if (t->trav_refill_lanes < 1 || t->trav_refill_lanes > 32 || t->trav_blocks_per_sm < 0 ||
      t->trav_blocks_per_sm > 64 || t->shade_blocks_per_sm < 1 || t->shade_blocks_per_sm > 64 ||
      t->graph_iterations < 0 || t->graph_iterations > 64 || (t->any_node_width != 2 && t->any_node_width != 4) ||
      t->ray_bin_bits < 0 || t->ray_bin_bits > kBinBitsMax || t->treelet_nodes < 0 || t->treelet_nodes > kTreeletMax ||
      (t->occluder_cache != 0 && t->occluder_cache != 1) || t->render_mode < TR_RENDER_MODE_AUTO ||
      t->render_mode > TR_RENDER_MODE_PERSISTENT || t->any_hit_order < 0 || t->any_hit_order > 2)
    return set_err(ctx, TR_ERR_ARG, "tuning out of range");
  const bool restage = t->treelet_nodes != ctx->tune.treelet_nodes;
  ctx->tune = *t;
  ctx->dsc.any_order = t->any_hit_order;
  if (restage && ctx->has_scene) {
    TR_DEVICE_SCOPE(ctx);
    return upload_treelet(ctx);
  }
  return TR_OK;
}

tr_status tr_ctx_get_tuning(const tr_ctx* ctx, tr_tuning* t) {
  if (!ctx || !t) return TR_ERR_ARG;
  *t = ctx->tune;
  return TR_OK;
}

tr_status tr_synchronize(tr_ctx* ctx) {
  if (!ctx) return TR_ERR_ARG;
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return TR_OK;
}

// Host tables and reference BVH of one scene description.
static tr_status build_host_scene(tr_ctx* ctx, const tr_scene_desc* d, HostScene& hs, bool device_bvh) {
  if (d->num_vertices && (!d->positions || !d->normals || !d->uvs))
    return set_err(ctx, TR_ERR_ARG, "vertex arrays missing");
  if (d->num_triangles && !d->indices) return set_err(ctx, TR_ERR_ARG, "indices missing");
  if (d->num_spheres && (!d->sphere_radius || !d->sphere_to_world || !d->sphere_to_local))
    return set_err(ctx, TR_ERR_ARG, "sphere arrays missing");
  if (d->num_prims && (!d->prim_shape || !d->prim_material || !d->prim_emission))
    return set_err(ctx, TR_ERR_ARG, "primitive arrays missing");
  if (d->num_materials && !d->materials) return set_err(ctx, TR_ERR_ARG, "materials missing");
  if (d->num_lights && !d->light_prims) return set_err(ctx, TR_ERR_ARG, "light list missing");
  if (d->num_prims > 0x7fffffffu) return set_err(ctx, TR_ERR_ARG, "too many primitives");
  for (uint32_t i = 0; i < 3 * d->num_triangles; ++i)
    if (d->indices[i] < 0 || (uint32_t)d->indices[i] >= d->num_vertices)
      return set_err(ctx, TR_ERR_ARG, "triangle index out of range");
  for (uint32_t m = 0; m < d->num_materials; ++m)
    if (d->materials[m].kind != TR_MAT_PHONG && d->materials[m].kind != TR_MAT_DISNEY12 &&
        d->materials[m].kind != TR_MAT_GLASS && d->materials[m].kind != TR_MAT_METAL &&
        d->materials[m].kind != TR_MAT_DISNEY15)
      return set_err(ctx, TR_ERR_ARG, "unknown material kind");
  for (uint32_t s = 0; s < d->num_spheres; ++s)
    if (!(d->sphere_radius[s] > 0.0f)) return set_err(ctx, TR_ERR_ARG, "invalid sphere radius");  // sphere.cpp:88-90

  // Mesh vertices through the identity local_to_world, normals normalised
  // at creation (triangle.cpp:224-228) and again on first use (:182-184).
  std::vector<f3> P(d->num_vertices), N(d->num_vertices);
  for (uint32_t v = 0; v < d->num_vertices; ++v) {
    P[v] = xform_point(kIdentity, mk3(d->positions[3 * v], d->positions[3 * v + 1], d->positions[3 * v + 2]));
    N[v] = normalize(xform_normal_inv(kIdentity, mk3(d->normals[3 * v], d->normals[3 * v + 1], d->normals[3 * v + 2])));
  }
  const uint32_t nt = d->num_triangles, ns = d->num_spheres, np = d->num_prims;
  hs.A.resize(nt);
  hs.AB.resize(nt);
  hs.AC.resize(nt);
  hs.tshade.resize(nt);
  std::vector<f3> Bv(nt), Cv(nt);
  for (uint32_t t = 0; t < nt; ++t) {
    const int i0 = d->indices[3 * t], i1 = d->indices[3 * t + 1], i2 = d->indices[3 * t + 2];
    const f3 A = P[i0], B = P[i1], C = P[i2];
    hs.A[t] = A;
    Bv[t] = B;
    Cv[t] = C;
    const f3 AB = B - A, AC = C - A;
    hs.AB[t] = AB;
    hs.AC[t] = AC;
    const float* uA = d->uvs + 2 * i0;
    const float* uB = d->uvs + 2 * i1;
    const float* uC = d->uvs + 2 * i2;
    const float m00 = uB[0] - uA[0], m01 = uB[1] - uA[1], m10 = uC[0] - uA[0], m11 = uC[1] - uA[1];
    DTriShade& ts = hs.tshade[t];
    std::memset(&ts, 0, sizeof(ts));
    // geometry frame (triangle.cpp:193-198): constant per triangle
    const f3 gn = normalize(cross(AB, AC));
    f3 dpdu, dpdv;
    compute_ss_ts(AB, AC, m00, m01, m10, m11, gn, dpdu, dpdv);
    dpdu = cross(dpdv, gn);
    dpdv = cross(gn, dpdu);
    const Frame g = make_frame(dpdu, dpdv, gn);
    ts.gx = g.x;
    ts.gy = g.y;
    ts.gz = g.z;
    const f3 nA = normalize(N[i0]), nB = normalize(N[i1]), nC = normalize(N[i2]);
    ts.nA = nA;
    ts.dn1 = nB - nA;
    ts.dn2 = nC - nA;
    ts.uvA[0] = uA[0];
    ts.uvA[1] = uA[1];
    ts.duv1[0] = m00;
    ts.duv1[1] = m01;
    ts.duv2[0] = m10;
    ts.duv2[1] = m11;
    const float det = m00 * m11 - m01 * m10;
    ts.det_nonzero = det ? 1 : 0;
    if (det) {
      const float inv_det = 1.0f / det;
      ts.dndu0 = scale(ts.dn1, m11 * inv_det) - scale(ts.dn2, m01 * inv_det);
      ts.dndv0 = scale(ts.dn1, m10 * inv_det) - scale(ts.dn2, m00 * inv_det);
    }
  }
  hs.spheres.resize(ns);
  std::vector<float> sph_wr(ns);
  for (uint32_t s = 0; s < ns; ++s) {
    DSphere& S = hs.spheres[s];
    std::memset(&S, 0, sizeof(S));
    std::memcpy(S.m, d->sphere_to_world + 16 * s, 64);
    std::memcpy(S.inv, d->sphere_to_local + 16 * s, 64);
    S.radius = d->sphere_radius[s];
    const float ratio = (float)lengthd(xform_vec(S.m, mk3(1.0f, 0.0f, 0.0f)));  // transformed_shape.hpp:13-15
    sph_wr[s] = ratio * S.radius;
  }
  if (d->num_textures && !d->textures) return set_err(ctx, TR_ERR_ARG, "textures missing");
  for (uint32_t m = 0; m < d->num_materials; ++m) {
    const tr_material& tm = d->materials[m];
    if (tm.kind == TR_MAT_PHONG &&
        (tm.tex_ka > d->num_textures || tm.tex_kd > d->num_textures || tm.tex_ks > d->num_textures ||
         tm.tex_ns > d->num_textures))
      return set_err(ctx, TR_ERR_ARG, "material names a missing texture");
    bool maps = tm.kind == TR_MAT_PHONG && (tm.tex_kd | tm.tex_ks | tm.tex_ns);
    for (int k = 0; k < mapped_params(tm.kind); ++k) {
      if (tm.tex_param[k] > d->num_textures) return set_err(ctx, TR_ERR_ARG, "material names a missing texture");
      maps |= tm.tex_param[k] != 0;
    }
    DMat dm = derive_material(tm);
    dm.tex_any = maps ? 1 : 0;
    hs.mats.push_back(dm);
    tr_material src = tm;
    for (int k = mapped_params(tm.kind); k < 13; ++k) src.tex_param[k] = 0;
    hs.msrc.push_back(src);
  }
  for (uint32_t k = 0; k < d->num_textures; ++k) {
    const tr_texture& t = d->textures[k];
    if (t.width == 0 || t.height == 0 || t.width > 65536 || t.height > 65536 || (!t.texels == !t.texels8))
      return set_err(ctx, TR_ERR_ARG, "invalid texture " + std::to_string(k));
    HostScene::Tex x;
    x.w = (int)t.width;
    x.h = (int)t.height;
    const size_t n = (size_t)x.w * x.h;
    if (t.texels) {
      x.texels.resize(4 * n);
      for (size_t i = 0; i < n; ++i)
        for (int c = 0; c < 4; ++c) x.texels[4 * i + c] = c < 3 ? t.texels[3 * i + c] : 0.0f;
    } else {
      x.texels8.resize(4 * n);
      for (size_t i = 0; i < n; ++i)
        for (int c = 0; c < 4; ++c) x.texels8[4 * i + c] = c < 3 ? t.texels8[3 * i + c] : 0;
    }
    hs.textures.push_back(std::move(x));
  }
  hs.prims.resize(np);
  std::vector<float> lo(3 * (size_t)np), hi(3 * (size_t)np);
  for (uint32_t p = 0; p < np; ++p) {
    DPrim& pr = hs.prims[p];
    std::memset(&pr, 0, sizeof(pr));
    const int sh = d->prim_shape[p];
    if (sh >= 0) {
      if ((uint32_t)sh >= nt) return set_err(ctx, TR_ERR_ARG, "primitive names a missing triangle");
      pr.kind = PRIM_TRIANGLE;
      pr.shape = sh;
      // Triangle::world_bound: Union(Bounds3f(A, B), C)
      const f3 A = hs.A[sh], B = Bv[sh], C = Cv[sh];
      float l[3] = {smin(A.x, B.x), smin(A.y, B.y), smin(A.z, B.z)};
      float h[3] = {smax(A.x, B.x), smax(A.y, B.y), smax(A.z, B.z)};
      l[0] = smin(l[0], C.x); l[1] = smin(l[1], C.y); l[2] = smin(l[2], C.z);
      h[0] = smax(h[0], C.x); h[1] = smax(h[1], C.y); h[2] = smax(h[2], C.z);
      for (int k = 0; k < 3; ++k) { lo[3 * p + k] = l[k]; hi[3 * p + k] = h[k]; }
      pr.area = (float)(0.5 * lengthd(cross(B - A, C - A)));  // Triangle::surface_area
    } else {
      const uint32_t si = (uint32_t)(~sh);
      if (si >= ns) return set_err(ctx, TR_ERR_ARG, "primitive names a missing sphere");
      pr.kind = PRIM_SPHERE;
      pr.shape = (int)si;
      // Sphere::world_bound (sphere.cpp:121-127)
      const f3 o = xform_point(hs.spheres[si].m, mk3(0.0f, 0.0f, 0.0f));
      const float r = sph_wr[si] + kEps;
      lo[3 * p] = o.x - r; lo[3 * p + 1] = o.y - r; lo[3 * p + 2] = o.z - r;
      hi[3 * p] = o.x + r; hi[3 * p + 1] = o.y + r; hi[3 * p + 2] = o.z + r;
    }
    const int mi = d->prim_material[p];
    if (mi < 0 || (uint32_t)mi >= d->num_materials) return set_err(ctx, TR_ERR_ARG, "material index out of range");
    pr.material = mi;
    pr.emission = mk3(d->prim_emission[3 * p], d->prim_emission[3 * p + 1], d->prim_emission[3 * p + 2]);
    pr.emissive = !(pr.emission.x == 0.0f && pr.emission.y == 0.0f && pr.emission.z == 0.0f);
    if (pr.emissive && pr.kind == PRIM_SPHERE)
      return set_err(ctx, TR_ERR_UNSUPPORTED, "emissive spheres are outside the GPU path");
  }
  std::vector<uint8_t> listed(np, 0);
  for (uint32_t l = 0; l < d->num_lights; ++l) {
    const int p = d->light_prims[l];
    if (p < 0 || (uint32_t)p >= np) return set_err(ctx, TR_ERR_ARG, "light primitive out of range");
    const DPrim& pr = hs.prims[p];
    if (!pr.emissive) return set_err(ctx, TR_ERR_ARG, "light primitive is not emissive");
    listed[p] = 1;
    DLight L;
    std::memset(&L, 0, sizeof(L));
    L.A = hs.A[pr.shape];
    L.B = Bv[pr.shape];
    L.C = Cv[pr.shape];
    L.gz = hs.tshade[pr.shape].gz;
    L.emission = pr.emission;
    L.area_pdf = 1.0f / pr.area;
    L.extent = fabsf(L.A.x) + fabsf(L.A.y) + fabsf(L.A.z) + fabsf(L.B.x) + fabsf(L.B.y) + fabsf(L.B.z) + fabsf(L.C.x) +
               fabsf(L.C.y) + fabsf(L.C.z) + 1.0f;
    L.prim = p;
    L.env = -1;
    L.AB = hs.AB[pr.shape];
    L.AC = hs.AC[pr.shape];
    light_sphere(L);
    hs.lights.push_back(L);
  }
  if (d->env_texels || d->env_texels8) {
    // the environment light follows the area lights in scene.lights; its
    // bounding sphere is that of the tree's root box, the union of the
    // primitive boxes
    EnvHost env;
    std::string why;
    if (!build_env_tables(d, env, why)) return set_err(ctx, TR_ERR_ARG, why);
    float rlo[3] = {kRealMax, kRealMax, kRealMax}, rhi[3] = {-kRealMax, -kRealMax, -kRealMax};
    for (uint32_t p = 0; p < np; ++p)
      for (int k = 0; k < 3; ++k) {
        rlo[k] = smin(rlo[k], lo[3 * p + k]);
        rhi[k] = smax(rhi[k], hi[3 * p + k]);
      }
    env_bounding_sphere(env, rlo, rhi, np == 0);
    DLight L;
    std::memset(&L, 0, sizeof(L));
    L.prim = -1;
    L.env = 0;
    hs.lights.push_back(L);
    hs.envs.push_back(std::move(env));
  }
  if (device_bvh) {  // the tree is built on the device at upload
    hs.device_bvh = true;
    hs.blo = std::move(lo);
    hs.bhi = std::move(hi);
  } else {
    BvhResult bvh = build_reference_bvh(lo.data(), hi.data(), np, d->max_leaf_prims);
    hs.nodes = std::move(bvh.nodes);
    hs.order = std::move(bvh.order);
  }
  hs.scene_prim = {0};
  hs.scene_leaf = {(int)d->max_leaf_prims};
  uint8_t unlisted = 0;
  for (uint32_t p = 0; p < np; ++p) unlisted |= (uint8_t)(hs.prims[p].emissive && !listed[p]);
  hs.scene_unlisted = {unlisted};
  hs.scene_node = {0};
  hs.scene_light = {0};
  hs.scene_nlight = {(uint32_t)hs.lights.size()};
  return TR_OK;
}

// Concatenates scene `src` into `dst`, offsetting every index.
static void append_scene(HostScene& dst, const HostScene& src) {
  const uint32_t node_base = (uint32_t)dst.nodes.size(), order_base = (uint32_t)dst.order.size();
  const uint32_t prim_base = (uint32_t)dst.prims.size(), tri_base = (uint32_t)dst.tshade.size();
  const uint32_t sph_base = (uint32_t)dst.spheres.size(), mat_base = (uint32_t)dst.mats.size();
  const uint32_t light_base = (uint32_t)dst.lights.size();
  dst.scene_node.push_back(node_base);
  dst.scene_light.push_back(light_base);
  dst.scene_nlight.push_back((uint32_t)src.lights.size());
  dst.scene_prim.push_back(prim_base);
  dst.scene_leaf.insert(dst.scene_leaf.end(), src.scene_leaf.begin(), src.scene_leaf.end());
  dst.scene_unlisted.insert(dst.scene_unlisted.end(), src.scene_unlisted.begin(), src.scene_unlisted.end());
  dst.device_bvh = src.device_bvh;
  dst.blo.insert(dst.blo.end(), src.blo.begin(), src.blo.end());
  dst.bhi.insert(dst.bhi.end(), src.bhi.begin(), src.bhi.end());
  for (tr_bvh_node32 n : src.nodes) {
    n.offset += (int32_t)(n.count > 0 ? order_base : node_base);
    dst.nodes.push_back(n);
  }
  for (uint32_t o : src.order) dst.order.push_back(o + prim_base);
  for (DPrim p : src.prims) {
    p.shape += (int)(p.kind == PRIM_TRIANGLE ? tri_base : sph_base);
    p.material += (int)mat_base;
    dst.prims.push_back(p);
  }
  dst.tshade.insert(dst.tshade.end(), src.tshade.begin(), src.tshade.end());
  dst.spheres.insert(dst.spheres.end(), src.spheres.begin(), src.spheres.end());
  const int tex_base = (int)dst.textures.size();
  for (DMat m : src.mats) {
    if (m.kind == MAT_PHONG) {
      if (m.tex_kd) m.tex_kd += tex_base;
      if (m.tex_ks) m.tex_ks += tex_base;
      if (m.tex_ns) m.tex_ns += tex_base;
    }
    dst.mats.push_back(m);
  }
  for (tr_material m : src.msrc) {
    for (uint32_t& t : m.tex_param)
      if (t) t += (uint32_t)tex_base;
    dst.msrc.push_back(m);
  }
  dst.textures.insert(dst.textures.end(), src.textures.begin(), src.textures.end());
  const int env_base = (int)dst.envs.size();
  for (DLight l : src.lights) {
    if (l.env >= 0) l.env += env_base;
    else l.prim += (int)prim_base;
    dst.lights.push_back(l);
  }
  dst.envs.insert(dst.envs.end(), src.envs.begin(), src.envs.end());
  dst.A.insert(dst.A.end(), src.A.begin(), src.A.end());
  dst.AB.insert(dst.AB.end(), src.AB.begin(), src.AB.end());
  dst.AC.insert(dst.AC.end(), src.AC.begin(), src.AC.end());
}

tr_status tr_scene_upload(tr_ctx* ctx, const tr_scene_desc* d) {
  if (!ctx || !d) return TR_ERR_ARG;
  return tr_scene_set_upload(ctx, d, 1);
}

tr_status tr_scene_set_upload(tr_ctx* ctx, const tr_scene_desc* descs, uint32_t n) {
  if (!ctx || !descs || n == 0 || n > 65536) return TR_ERR_ARG;
  TR_DEVICE_SCOPE(ctx);
  ctx->has_scene = false;
  const bool device_bvh = ctx->bvh_builder == TR_BVH_DEVICE;
  // each scene's tables and tree on its own host thread
  std::vector<HostScene> parts(n);
  std::vector<tr_status> st(n, TR_OK);
  std::vector<std::string> msg(n);
  const unsigned int workers = std::max(1u, std::min(n, std::thread::hardware_concurrency()));
  std::atomic<uint32_t> next{0};
  auto work = [&]() {
    tr_ctx scratch;  // per-thread error sink
    for (uint32_t k; (k = next.fetch_add(1)) < n;) {
      st[k] = build_host_scene(&scratch, descs + k, parts[k], device_bvh);
      if (st[k] != TR_OK) msg[k] = scratch.err;
    }
  };
  std::vector<std::thread> pool;
  for (unsigned int w = 1; w < workers; ++w) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  for (uint32_t k = 0; k < n; ++k)
    if (st[k] != TR_OK) return set_err(ctx, st[k], "scene " + std::to_string(k) + ": " + msg[k]);
  HostScene hs;
  if (n == 1) {
    hs = std::move(parts[0]);
  } else {
    for (uint32_t k = 0; k < n; ++k) {
      append_scene(hs, parts[k]);
      HostScene().A.swap(parts[k].A);  // release as we go
    }
  }
  ctx->hs = std::move(hs);
  return upload_device_tables(ctx);
}

tr_status tr_ctx_set_bvh_builder(tr_ctx* ctx, int32_t builder) {
  if (!ctx || (builder != TR_BVH_REFERENCE && builder != TR_BVH_DEVICE)) return TR_ERR_ARG;
  ctx->bvh_builder = builder;
  return TR_OK;
}

tr_status tr_bvh_stats(const tr_ctx* ctx, int32_t* builder, int32_t* depth) {
  if (!ctx || !builder || !depth) return TR_ERR_ARG;
  if (!ctx->has_scene) return TR_ERR_STATE;
  *builder = ctx->hs.device_bvh ? TR_BVH_DEVICE : TR_BVH_REFERENCE;
  *depth = ctx->hs.depth;
  return TR_OK;
}

tr_status tr_bvh_info(tr_ctx* ctx, size_t* num_nodes, size_t* num_prims) {
  if (!ctx || !num_nodes || !num_prims) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (ctx->hs.device_bvh) return set_err(ctx, TR_ERR_STATE, "the BVH was built on the device (TR_BVH_DEVICE)");
  *num_nodes = ctx->hs.nodes.size();
  *num_prims = ctx->hs.order.size();
  return TR_OK;
}

tr_status tr_any_tree_info(const tr_ctx* ctx, uint64_t* num_nodes4, int32_t* stack_bound) {
  if (!ctx || !num_nodes4 || !stack_bound) return TR_ERR_ARG;
  *num_nodes4 = ctx->any4_nodes;
  *stack_bound = ctx->any4_stack;
  return TR_OK;
}

tr_status tr_bvh_export(tr_ctx* ctx, tr_bvh_node32* nodes, uint32_t* prim_order) {
  if (!ctx || !nodes || !prim_order) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (ctx->hs.device_bvh) return set_err(ctx, TR_ERR_STATE, "the BVH was built on the device (TR_BVH_DEVICE)");
  std::memcpy(nodes, ctx->hs.nodes.data(), ctx->hs.nodes.size() * sizeof(tr_bvh_node32));
  std::memcpy(prim_order, ctx->hs.order.data(), ctx->hs.order.size() * sizeof(uint32_t));
  return TR_OK;
}

tr_status tr_bvh_upload(tr_ctx* ctx, const tr_bvh_node32* nodes, size_t num_nodes, const uint32_t* prim_order,
                        size_t num_prims) {
  if (!ctx || (num_nodes && !nodes) || (num_prims && !prim_order)) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (ctx->hs.device_bvh) return set_err(ctx, TR_ERR_STATE, "the BVH was built on the device (TR_BVH_DEVICE)");
  if (ctx->hs.scene_node.size() != 1) return set_err(ctx, TR_ERR_STATE, "tr_bvh_upload replaces the tree of a single scene");
  TR_DEVICE_SCOPE(ctx);
  std::vector<tr_bvh_node32> keep_nodes = ctx->hs.nodes;
  std::vector<uint32_t> keep_order = ctx->hs.order;
  ctx->hs.nodes.assign(nodes, nodes + num_nodes);
  ctx->hs.order.assign(prim_order, prim_order + num_prims);
  ctx->has_scene = false;
  tr_status s = upload_device_tables(ctx);
  if (s != TR_OK) {
    ctx->hs.nodes = std::move(keep_nodes);
    ctx->hs.order = std::move(keep_order);
    std::string msg = ctx->err;
    tr_status s2 = upload_device_tables(ctx);
    ctx->err = msg;
    (void)s2;
  }
  return s;
}

static tr_status check_err_word(tr_ctx* ctx) {
  int e = 0;
  TR_CUDA(ctx, cudaMemcpyAsync(&e, ctx->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  TR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (e) {
    cudaMemsetAsync(ctx->d_err.p, 0, sizeof(int), ctx->stream);
    return set_err(ctx, TR_ERR_QUEUE_OVERFLOW, "traversal stack overflow");
  }
  return TR_OK;
}

tr_status tr_trace_closest_dev(tr_ctx* ctx, const tr_ray* d_rays, size_t n, int32_t* d_prim, float* d_t) {
  if (!ctx || (n && (!d_rays || !d_prim || !d_t))) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (n == 0) return TR_OK;
  if (n > 0x7fffffffull) return set_err(ctx, TR_ERR_ARG, "too many rays");
  if (((uintptr_t)d_rays & 15u) != 0) return set_err(ctx, TR_ERR_ARG, "ray buffer must be 16-byte aligned");
  TR_DEVICE_SCOPE(ctx);
  BatchJob job{reinterpret_cast<const float4*>(d_rays), (unsigned int)n, d_prim, d_t, nullptr, nullptr};
  return launch_trace<false, false>(ctx, job, nullptr);
}

tr_status tr_trace_any_dev(tr_ctx* ctx, const tr_ray* d_rays, size_t n, uint8_t* d_hit) {
  if (!ctx || (n && (!d_rays || !d_hit))) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (n == 0) return TR_OK;
  if (n > 0x7fffffffull) return set_err(ctx, TR_ERR_ARG, "too many rays");
  if (((uintptr_t)d_rays & 15u) != 0) return set_err(ctx, TR_ERR_ARG, "ray buffer must be 16-byte aligned");
  TR_DEVICE_SCOPE(ctx);
  BatchJob job{reinterpret_cast<const float4*>(d_rays), (unsigned int)n, nullptr, nullptr, d_hit, nullptr};
  if (any_wide(ctx)) return launch_trace<true, true>(ctx, job, nullptr);
  return launch_trace<true, false>(ctx, job, nullptr);
}

tr_status tr_trace_count_dev(tr_ctx* ctx, const tr_ray* d_rays, size_t n, int32_t any, uint64_t* boxes,
                             uint64_t* prims) {
  if (!ctx || !boxes || !prims || (n && !d_rays)) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (n > 0x7fffffffull) return set_err(ctx, TR_ERR_ARG, "too many rays");
  if (((uintptr_t)d_rays & 15u) != 0) return set_err(ctx, TR_ERR_ARG, "ray buffer must be 16-byte aligned");
  *boxes = *prims = 0;
  if (n == 0) return TR_OK;
  TR_DEVICE_SCOPE(ctx);
  // scratch: the words after the error word and the fetch position
  unsigned long long* counts = reinterpret_cast<unsigned long long*>(ctx->d_err.as<char>() + 16);
  TR_CUDA(ctx, cudaMemsetAsync(ctx->d_err.as<int>() + 1, 0, sizeof(int), ctx->stream));
  TR_CUDA(ctx, cudaMemsetAsync(counts, 0, 16, ctx->stream));
  BatchJob job{reinterpret_cast<const float4*>(d_rays), (unsigned int)n, nullptr, nullptr, nullptr, nullptr};
  tr_status ls;
  if (any && any_wide(ctx)) ls = launch_trace<true, true>(ctx, job, counts);
  else if (any) ls = launch_trace<true, false>(ctx, job, counts);
  else ls = launch_trace<false, false>(ctx, job, counts);
  if (ls != TR_OK) return ls;
  unsigned long long h[2];
  TR_CUDA(ctx, cudaMemcpyAsync(h, counts, 16, cudaMemcpyDeviceToHost, ctx->stream));
  tr_status s = check_err_word(ctx);
  *boxes = h[0];
  *prims = h[1];
  return s;
}

tr_status tr_trace_closest(tr_ctx* ctx, const tr_ray* rays, size_t n, int32_t* prim, float* t) {
  if (!ctx || (n && (!rays || !prim || !t))) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (n == 0) return TR_OK;
  TR_DEVICE_SCOPE(ctx);
  TR_CUDA(ctx, ctx->d_rays.reserve(n * sizeof(tr_ray)));
  TR_CUDA(ctx, ctx->d_out0.reserve(n * sizeof(int32_t)));
  TR_CUDA(ctx, ctx->d_out1.reserve(n * sizeof(float)));
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_rays.p, rays, n * sizeof(tr_ray), cudaMemcpyHostToDevice, ctx->stream));
  tr_status s = tr_trace_closest_dev(ctx, ctx->d_rays.as<tr_ray>(), n, ctx->d_out0.as<int32_t>(), ctx->d_out1.as<float>());
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaMemcpyAsync(prim, ctx->d_out0.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  TR_CUDA(ctx, cudaMemcpyAsync(t, ctx->d_out1.p, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  return check_err_word(ctx);
}

tr_status tr_trace_any(tr_ctx* ctx, const tr_ray* rays, size_t n, uint8_t* hit) {
  if (!ctx || (n && (!rays || !hit))) return TR_ERR_ARG;
  if (!ctx->has_scene) return set_err(ctx, TR_ERR_STATE, "no scene uploaded");
  if (n == 0) return TR_OK;
  TR_DEVICE_SCOPE(ctx);
  TR_CUDA(ctx, ctx->d_rays.reserve(n * sizeof(tr_ray)));
  TR_CUDA(ctx, ctx->d_out0.reserve(n));
  TR_CUDA(ctx, cudaMemcpyAsync(ctx->d_rays.p, rays, n * sizeof(tr_ray), cudaMemcpyHostToDevice, ctx->stream));
  tr_status s = tr_trace_any_dev(ctx, ctx->d_rays.as<tr_ray>(), n, ctx->d_out0.as<uint8_t>());
  if (s != TR_OK) return s;
  TR_CUDA(ctx, cudaMemcpyAsync(hit, ctx->d_out0.p, n, cudaMemcpyDeviceToHost, ctx->stream));
  return check_err_word(ctx);
}

tr_status tr_cancel(tr_ctx* ctx) {
  if (!ctx) return TR_ERR_ARG;
  ctx->cancel.store(1);
  return TR_OK;
}

}  // extern "C"
