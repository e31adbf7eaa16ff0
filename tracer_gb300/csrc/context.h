// context.h -- the tr_ctx object behind the C ABI (internal).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/tracer_gpu.h"
#include "env_light.h"
#include "scene_types.h"

namespace trg {
struct GuideModel;

// A device allocation that grows on demand and is freed with the context.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t reserve(size_t n) {
    if (n <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct HostScene {
  // what the device tables were built from (kept for export and re-upload)
  std::vector<tr_bvh_node32> nodes;
  std::vector<uint32_t> order;
  std::vector<DPrim> prims;
  std::vector<DTriShade> tshade;
  std::vector<DSphere> spheres;
  std::vector<DMat> mats;
  std::vector<DLight> lights;
  std::vector<f3> A, AB, AC;  // per triangle
  int depth = 0;
  // scene set: first node, first light and light count of every scene
  std::vector<uint32_t> scene_node, scene_light, scene_nlight;
  std::vector<uint32_t> scene_prim;  // first primitive of every scene
  std::vector<int> scene_leaf;       // max_leaf_prims of every scene
  // 1 for a scene with an emissive primitive outside its light list (its
  // MIS rays are all traced: the light list cannot tell which reach emission)
  std::vector<uint8_t> scene_unlisted;
  // TR_BVH_DEVICE: no host tree; the primitive bounds (3 floats each) for the device build
  bool device_bvh = false;
  std::vector<float> blo, bhi;
  // environment lights of the set (DLight::env indexes them)
  std::vector<EnvHost> envs;
  // image textures of the materials, 4 floats or 4 bytes per texel
  struct Tex {
    int w = 0, h = 0;
    std::vector<float> texels;
    std::vector<uint8_t> texels8;
  };
  std::vector<Tex> textures;
  // the child-pair nodes as uploaded and scene 0's root among them (-1: the
  // root is a leaf, or the tree was built on the device)
  std::vector<DNode> dnodes;
  int root0 = -1;
  // every material's factory arguments and maps (the device re-derives the
  // set-up of a material with maps at each of its hits)
  std::vector<tr_material> msrc;
};

struct RenderBuffers;  // render.cu

}  // namespace trg

struct tr_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  bool has_scene = false;
  trg::HostScene hs;
  trg::DScene dsc{};
  trg::DevBuf d_nodes, d_nodes4, d_slots, d_spheres, d_prims, d_tshade, d_mats, d_lights, d_roots;
  trg::DevBuf d_rays, d_out0, d_out1, d_err;
  trg::DevBuf d_env_pool, d_envs;  // environment lights: texels and tables, DEnv records
  trg::DevBuf d_tex_pool, d_texs;  // material textures: texels, DTex records
  trg::DevBuf d_treelet;           // the shared-memory treelet (DScene::treelet)
  trg::DevBuf d_slot_leaf;         // DScene::slot_leaf
  // learned light sampling: per (grid cell, light) the statistics and the
  // sampling distribution (cumulative) over bins x bins sample-square cells
  trg::DevBuf d_lg_acc, d_lg_cdf;
  trg::DevBuf d_msrc;  // DScene::msrc
  int lg_grid[3] = {0, 0, 0};
  int lg_bins = 0, lg_nl = 0;
  trg::DevBuf d_perm, d_bin_key, d_bin_cnt;  // ray binning of tr_trace_*: order, keys, bin counts
  std::atomic<int> cancel{0};
  trg::RenderBuffers* rb = nullptr;
  tr_tuning tune{20, 0, 32, 8, 2, 3, 0, 1, TR_RENDER_MODE_AUTO, 1};
  int bvh_builder = TR_BVH_REFERENCE;
  size_t any4_nodes = 0;  // four-wide any-hit tree of the uploaded set (0: not available)
  int any4_stack = 0;     // its traversal stack bound
  trg::GuideModel* guide = nullptr;
};

namespace trg {
tr_status cuda_fail(tr_ctx* ctx, cudaError_t e, const char* what);
tr_status set_err(tr_ctx* ctx, tr_status s, const std::string& msg);
tr_status upload_device_tables(tr_ctx* ctx);
tr_status upload_device_built(tr_ctx* ctx);  // bvh_gpu.cu: the TR_BVH_DEVICE path
// Uploads the set's environment lights and sets the scene's envs / has_env.
tr_status upload_envs(tr_ctx* ctx);
// Uploads the set's material textures and sets the scene's textures / has_textures.
tr_status upload_textures(tr_ctx* ctx);
// Grid of a persistent traversal kernel: SMs x resident blocks (tuned or as
// many as fit with `smem` bytes of dynamic shared memory per block).
int traversal_grid(const tr_ctx* ctx, const void* kernel, size_t smem = 0);
// Builds and uploads the shared-memory treelet for the tuned node count.
tr_status upload_treelet(tr_ctx* ctx);
// Nodes of the treelet the traversal kernels stage (0: none).
inline int treelet_nodes(const tr_ctx* ctx) { return ctx->tune.treelet_nodes > 0 ? ctx->dsc.treelet_n : 0; }
// Lets `kernel` take `bytes` of dynamic shared memory (above the 48 KiB default).
cudaError_t allow_dynamic_smem(const void* kernel, size_t bytes);
// Whether any-hit traversal walks the four-wide tree (tuning and scene allow it).
inline bool any_wide(const tr_ctx* ctx) { return ctx->tune.any_node_width == 4 && ctx->dsc.nodes4 != nullptr; }
void release_render(tr_ctx* ctx);
void release_guide(tr_ctx* ctx);
}  // namespace trg

namespace trg {
// Makes a device current for the duration of a C ABI call and gives the
// caller's current device back when the call returns.
struct DeviceScope {
  int prev = -1;
  cudaError_t status = cudaSuccess;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) {
      cudaGetLastError();
      prev = -1;
    }
    if (prev != dev) status = cudaSetDevice(dev);
  }
  ~DeviceScope() {
    int now = -1;
    if (prev >= 0 && cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
  }
  DeviceScope(const DeviceScope&) = delete;
  DeviceScope& operator=(const DeviceScope&) = delete;
};
}  // namespace trg

// The context's device for the rest of the enclosing C ABI function (the
// caller's device is restored on return); returns the error if it cannot be
// made current.
#define TR_DEVICE_SCOPE(ctx)                                                          \
  trg::DeviceScope dev_scope_((ctx)->device);                                         \
  do {                                                                                \
    if (dev_scope_.status != cudaSuccess) return trg::cuda_fail((ctx), dev_scope_.status, "cudaSetDevice"); \
  } while (0)

// Returns from the enclosing C ABI function with the context's error when a
// CUDA runtime call fails.
#define TR_CUDA(ctx, call)                                          \
  do {                                                              \
    cudaError_t e_ = (call);                                        \
    if (e_ != cudaSuccess) return trg::cuda_fail(ctx, e_, #call);   \
  } while (0)
