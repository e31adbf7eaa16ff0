// render_common.cuh -- what the wavefront kernels (render.cu) and the
// persistent render kernel (mega.cu) share: the job table of a render and the
// film update of PixelSamplerRenderer (src/renderer/pixel_sampler_renderer.cpp:60-94).
#pragma once

#include "shade.cuh"
#include "traverse.cuh"

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
  float lsph[4];       // a sphere around the scene's area-light triangles with a margin (radius < 0: none)
  float lsph_cn;       // |centre|
  int mis_always;      // the scene has emissive primitives outside its light list: every MIS ray is traced
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

// Lights of a job tested before its MIS rays are traced (more: always traced).
constexpr int kMisLightTests = 32;

// Whether the MIS BSDF ray of a vertex (sample_bsdf,
// src/renderer/direct_illumination.cpp:144-198) can contribute, before it is
// traced. It contributes only when it leaves a scene with an environment
// light, or when its closest hit is an area light. That closest hit is a
// primitive the triangle test hits -- the walk tests the same slot data with
// the same arithmetic, and its culling only removes candidates -- so a ray
// that hits none of the job's emissive triangles, in a scene without an
// environment light, contributes the zero its traced closest hit would give,
// and is not traced.
// Whether a ray (d of unit length) may pass through a sphere (centre s, radius
// s[3], |centre| cn). The spheres hold every point the triangle test can
// accept with a margin far above that test's rounding; a false answer needs
// the ray to pass outside, or move away, by more than this test's own
// rounding (1e-5 of the distances).
__device__ __forceinline__ bool ray_may_pass(const float* s, float cn, f3 o, f3 d, float on) {
  const f3 v = mk3(s[0] - o.x, s[1] - o.y, s[2] - o.z);
  const float r = s[3] + 1e-5f * (on + cn);
  const float vv = dot(v, v), tca = dot(v, d);
  if (tca < 0.0f && vv > r * r) return false;
  const f3 w = v - scale(d, tca);
  return dot(w, w) <= r * r;
}

// The traversal's triangle test on an area light (out of line: it is rarely
// reached, and inlined it would weigh on the instruction cache of every
// shading kernel).
static __device__ __noinline__ bool light_tri_hit(const DLight& lt, f3 o, f3 d) {
  float t, a, b;
  return tri_test(make_float4(lt.A.x, lt.A.y, lt.A.z, 0.0f), make_float4(lt.AB.x, lt.AB.y, lt.AB.z, 0.0f),
                  make_float4(lt.AC.x, lt.AC.y, lt.AC.z, 0.0f), o, d, 0.0f, kRealMax, t, a, b);
}

__device__ __forceinline__ bool mis_may_hit_light(const DScene& sc, const JobDev& J, f3 o, f3 d) {
  if (J.env >= 0 || J.nl > kMisLightTests || J.mis_always) return true;
  if (J.lsph[3] < 0.0f) return false;
  const float on = sqrtf(dot(o, o));
  if (!ray_may_pass(J.lsph, J.lsph_cn, o, d, on)) return false;  // all lights
  for (int l = 0; l < J.nl; ++l) {
    const DLight& lt = sc.lights[J.light_base + l];
    // an area light emits on its front side only: a hit on its back gives the
    // zero that light_emit gives there (the contribution's own test, the same
    // normal and direction)
    if (!(dot(lt.gz, -d) > 0.0f)) continue;
    if (!ray_may_pass(lt.bs, lt.bs_cn, o, d, on)) continue;
    if (light_tri_hit(lt, o, d)) return true;
  }
  return false;
}

}  // namespace trg
