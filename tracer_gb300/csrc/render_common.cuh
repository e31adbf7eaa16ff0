// render_common.cuh -- what the wavefront kernels (render.cu) and the
// persistent render kernel (mega.cu) share: the job table of a render and the
// film update of PixelSamplerRenderer (src/renderer/pixel_sampler_renderer.cpp:60-94).
#pragma once

#include "shade.cuh"

namespace trg {

// PathTraceRenderer::max_specular_depth (src/renderer/path_trace_renderer.cpp:20):
// delta samples that do not count toward the path depth
constexpr int kMaxSpecularDepth = 20;

// P1.w holds the path depth (low 16 bits) and the count of delta samples
// that did not count toward it (high bits). The depth must stay below 2^16
// with the uncounted delta samples on top: larger max_depth is rejected.
constexpr int kMaxPathDepth = 0xffff - kMaxSpecularDepth;
__device__ __forceinline__ int path_depth(float w) { return __float_as_int(w) & 0xffff; }
__device__ __forceinline__ int spec_depth(float w) { return __float_as_int(w) >> 16; }

// One render of a batch: a scene of the set seen through a camera onto a
// film. Its path slots are slot_base .. slot_base + W * H - 1, one per pixel.
struct JobDev {
  Cam cam;
  int W, H, spp, min_depth, max_depth;
  unsigned int seed_base;
  int scene, slot_base;
  int light_base, nl;  // the scene's lights in DScene::lights
  int env;             // the scene's environment light in DScene::envs (its last light), or -1
  float filter_radius, filter_alpha, filter_exp;
  int fp64;
  float4* film;  // film sums (float4 per pixel, or 2 x double2)
};

// The job a path slot belongs to (slot bases ascend with the job index).
__device__ __forceinline__ const JobDev& job_of(const JobDev* jobs, int njobs, int slot) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].slot_base <= slot) lo = mid;
    else hi = mid - 1;
  }
  return jobs[lo];
}

// Film::Tile::add_sample (src/core/render.hpp:37-57). With radius <= 0.5 a
// sample reaches only its own pixel with non-zero weight (neighbours get
// exactly 0), so the slot owns its pixel and adds in sample order.
__device__ __forceinline__ void film_add(const JobDev& J, int slot, float px, float py, f3 L) {
  const int pix = slot - J.slot_base;
  const int x = pix % J.W, y = pix / J.W;
  if (J.filter_radius <= 0.5f) {
    const float ox = px - ((float)x + 0.5f), oy = py - ((float)y + 0.5f);  // exact for W, H < 2^23
    const float fw = gaussian(J.filter_alpha, ox, J.filter_exp) * gaussian(J.filter_alpha, oy, J.filter_exp);
    const f3 c = muls(muls(L, fw), 1.0f);
    if (J.fp64) {
      double2* a = reinterpret_cast<double2*>(J.film) + 2 * pix;
      double2 a0 = a[0], a1 = a[1];
      a0.x += c.x;
      a0.y += c.y;
      a1.x += c.z;
      a1.y += fw;
      a[0] = a0;
      a[1] = a1;
    } else {
      float4 a = J.film[pix];
      a.x += c.x;
      a.y += c.y;
      a.z += c.z;
      a.w += fw;
      J.film[pix] = a;
    }
    return;
  }
  // wider filters: scatter with atomics (order of additions not fixed)
  const float r = J.filter_radius;
  const float dx = px - 0.5f, dy = py - 0.5f;
  const int x0 = max((int)ceilf(dx - r), 0), y0 = max((int)ceilf(dy - r), 0);
  const int x1 = min((int)floorf(dx + r) + 1, J.W), y1 = min((int)floorf(dy + r) + 1, J.H);
  for (int yy = y0; yy < y1; ++yy)
    for (int xx = x0; xx < x1; ++xx) {
      const float ox = px - ((float)xx + 0.5f), oy = py - ((float)yy + 0.5f);
      const float fw = gaussian(J.filter_alpha, ox, J.filter_exp) * gaussian(J.filter_alpha, oy, J.filter_exp);
      const f3 c = muls(muls(L, fw), 1.0f);
      const int o = yy * J.W + xx;
      if (J.fp64) {
        double* a = reinterpret_cast<double*>(J.film) + 4 * o;
        atomicAdd(a, (double)c.x);
        atomicAdd(a + 1, (double)c.y);
        atomicAdd(a + 2, (double)c.z);
        atomicAdd(a + 3, (double)fw);
      } else {
        float* a = reinterpret_cast<float*>(J.film) + 4 * o;
        atomicAdd(a, c.x);
        atomicAdd(a + 1, c.y);
        atomicAdd(a + 2, c.z);
        atomicAdd(a + 3, fw);
      }
    }
}

}  // namespace trg
