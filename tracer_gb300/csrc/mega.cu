// mega.cu -- the persistent render kernel: every camera sample of a render
// (or of a whole batch of renders) in ONE launch.
//
// PixelSamplerRenderer::render (src/renderer/pixel_sampler_renderer.cpp:24-109)
// calls PathTraceRenderer::eval_pixel_li (src/renderer/path_trace_renderer.cpp:27-210)
// once per camera sample, the samples of a pixel in order from one pcg32
// stream. Here a thread owns a pixel (a path slot) at a time and runs its
// samples one after another with the whole path state in registers; when the
// pixel's samples are done it claims the next unrendered pixel of any job
// (one atomic per warp). Each loop iteration processes one path vertex of
// every lane of a warp, in phases the 32 lanes go through together:
//
//   extend   closest hit of every lane's ray (warp-cooperative traversal)
//   vertex   emission, escape to the environment light, BSDF sample, the
//            light-sample draws, the MIS sample, throughput, Russian roulette
//   lights   for each light index: the light sample and its shadow ray
//   mis      closest hit of the MIS ray and its weighted emission
//   finish   direct lighting added, the sample's film update, the next sample
//
// The arithmetic, the order of random draws and the order of the sums are
// those of the wavefront kernels of render.cu (k_logic, k_material, k_glass,
// k_nee, mis_contribution), so a pixel gets the same film bit for bit either
// way; only the work is arranged for small renders, where the wavefront's
// ten launches per path vertex over a few thousand slots cannot fill the GPU.
// Guided rendering and instrumented renders (stage times, visit counts) use
// the wavefront.

#include <cuda_runtime.h>

#include "mega.h"
#include "traverse.cuh"

namespace trg {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// What a trace gives back: the hit record (any hit: the occluding slot in
// prim) and whether the ray is occluded.
struct Traced {
  Hit h;
  bool occluded;
};

// Closest hit (ANY = false) or occlusion (ANY = true) of every lane's ray,
// the 32 lanes walking together: the speculative while-while of
// persistent_traverse without its refill. Lanes with `active` false take no
// part in the walk; every lane of the warp must call it. Out of line: one
// copy serves the extension and the MIS ray; the walk's state is local to the
// call (registers, its stack in local memory).
template <bool ANY>
__device__ __noinline__ Traced warp_trace(const DScene& sc, bool active, int scene, f3 o, f3 d, float tmin,
                                          float tmax, int* err) {
  TravLane<ANY, false> L;
  VisitCount vc;
  bool live = active && L.start(sc, scene, o, d, tmin, tmax, vc, false);
  if (!active) {
    L.h.prim = -1;
    L.occluded = false;
  }
  for (;;) {
    for (;;) {
      if (live && L.cnt > 0 && L.pc == 0) L.postpone();
      if (!__any_sync(kFull, live && L.pc == 0)) break;
      if (live && L.cnt == 0) {
        const bool more = L.interior(sc, err, vc);
        if (!more) {
          if (L.failed || L.pc == 0) live = false;
          else L.cnt = -1;
        }
      }
    }
    if (live) live = L.postponed_leaf(sc, vc);
    if (!__any_sync(kFull, live)) break;
  }
  return Traced{L.h, L.occluded};
}

// Material dispatch limited to the kinds of the instantiation (the sampler
// out of line: one copy serves the path's and the MIS sample).
template <unsigned MASK>
__device__ __noinline__ BsdfSample m_sample(const Bsdf& b, int kind, f3 wo, float u, float v, float w) {
  if ((MASK & MK_DISNEY12) && kind == MAT_DISNEY12) return b.disney_sample(wo, u, v, w);
  if ((MASK & MK_METAL) && kind == MAT_METAL) return b.metal_sample(wo, u, v, w);
  if ((MASK & MK_DISNEY15) && kind == MAT_DISNEY15) return b.d15_sample(wo, u, v, w);
  return b.phong_sample_agg(wo, u, v, w);
}
template <unsigned MASK>
__device__ __forceinline__ f3 m_eval(const Bsdf& b, int kind, f3 wi, f3 wo) {
  if ((MASK & MK_DISNEY12) && kind == MAT_DISNEY12) return b.disney_eval(wi, wo);
  if ((MASK & MK_METAL) && kind == MAT_METAL) return b.metal_eval(wi, wo);
  if ((MASK & MK_DISNEY15) && kind == MAT_DISNEY15) return b.d15_eval(wi, wo);
  return b.phong_eval_agg(wi, wo);
}
template <unsigned MASK>
__device__ __forceinline__ float m_pdf(const Bsdf& b, int kind, f3 wi, f3 wo) {
  if ((MASK & MK_DISNEY12) && kind == MAT_DISNEY12) return b.disney_pdf(wi, wo);
  if ((MASK & MK_METAL) && kind == MAT_METAL) return b.metal_pdf(wi, wo);
  if ((MASK & MK_DISNEY15) && kind == MAT_DISNEY15) return b.d15_pdf(wi, wo);
  return b.phong_pdf_agg(wi, wo);
}

// The per-lane state of one pixel slot.
struct Path {
  int slot;  // -1: none
  const JobDev* J;
  unsigned long long st;
  int sample, depth, sdepth;
  bool spec;      // the ray continues a delta sample (emission it reaches counts)
  bool has_ray;   // a ray to extend this iteration
  f3 o, d, coef, L;
  float px, py;
  unsigned int finished;
};

// start_sample of render.cu: the slot's next camera sample, finishing samples
// that Russian roulette ends before their first vertex.
__device__ __forceinline__ bool start_sample(Path& p) {
  const JobDev& J = *p.J;
  const int pix = p.slot - J.slot_base;
  const int x = pix % J.W, y = pix / J.W;
  while (p.sample < J.spp) {
    const float fu = Pcg::next(p.st), fv = Pcg::next(p.st);
    const float lu = Pcg::next(p.st), lv = Pcg::next(p.st);
    const float px = (float)x + fu, py = (float)y + fv;
    f3 o, d;
    camera_ray(J.cam, px / (float)J.W, py / (float)J.H, lu, lv, o, d);
    f3 coef = mk3(1.0f, 1.0f, 1.0f);
    bool dead = false;
    if (0 > J.min_depth) {  // Russian roulette at depth 0
      if (Pcg::next(p.st) > 0.9f) dead = true;
      else coef = divs(coef, 0.9f);
    }
    if (!dead && !valid3(coef)) dead = true;
    if (dead) {
      film_add(J, p.slot, px, py, mk3(0.0f, 0.0f, 0.0f));
      ++p.finished;
      ++p.sample;
      continue;
    }
    p.o = o;
    p.d = d;
    p.coef = coef;
    p.L = mk3(0.0f, 0.0f, 0.0f);
    p.px = px;
    p.py = py;
    p.depth = 0;
    p.sdepth = 0;
    p.spec = false;
    return true;
  }
  return false;
}

// finish_sample of render.cu: the film update and the next sample.
__device__ __forceinline__ void finish_sample(Path& p) {
  f3 L = p.L;
  if (!valid3(L)) L = mk3(0.0f, 0.0f, 0.0f);  // eval_pixel_li returns {} (path_trace_renderer.cpp:204-209)
  film_add(*p.J, p.slot, p.px, p.py, L);
  ++p.finished;
  ++p.sample;
  p.has_ray = start_sample(p);
}

template <unsigned MASK>
__global__ void __launch_bounds__(kMegaThreads, 1) k_mega(MegaLaunch P) {
  const DScene& sc = P.sc;
  const int lane = (int)(threadIdx.x & 31u);
  Path p;
  p.slot = -1;
  p.has_ray = false;
  p.finished = 0;
  bool done = false;
  long long steps = 0, max_steps = 0;  // vertex bound of the current pixel
  float2 nu[kMegaLights];              // light-sample draws of the current vertex
  int oc[kMegaLights];                 // the slot that last blocked each light's shadow ray (-1: none)
  DMat tmat;                           // the Phong set-up at a hit with image maps
  unsigned long long n_ext = 0, n_sh = 0, n_vert = 0, n_hits = 0;
  for (;;) {
    // lanes without a ray claim pixels until they have one or none are left
    for (;;) {
      const bool want = !done && !p.has_ray;
      const unsigned need = __ballot_sync(kFull, want);
      if (!need) break;
      const int leader = __ffs(need) - 1;
      unsigned int base = 0;
      if (lane == leader) base = atomicAdd(P.fetch, (unsigned int)__popc(need));
      base = __shfl_sync(kFull, base, leader);
      if (want) {
        const unsigned int s = base + (unsigned int)__popc(need & ((1u << lane) - 1u));
        if (s < (unsigned int)P.nslots) {
          p.slot = (int)s;
          p.J = &job_of(P.jobs, P.njobs, p.slot);
          const int pix = p.slot - p.J->slot_base;
          const int x = pix % p.J->W, y = pix / p.J->W;
          p.st = Pcg::seed((int)(p.J->seed_base + (unsigned)y * (unsigned)p.J->W + (unsigned)x));
          p.sample = 0;
          for (int l = 0; l < kMegaLights; ++l) oc[l] = -1;
          steps = 0;
          max_steps = (long long)p.J->spp * ((long long)p.J->max_depth + 2 + ((MASK & MK_GLASS) ? kMaxSpecularDepth : 0));
          p.has_ray = start_sample(p);
        } else {
          done = true;
        }
      }
    }
    // the block goes through the phases together (one phase's code in the
    // instruction cache at a time); it ends when all its lanes are done
    if (!__syncthreads_or(!done)) break;

    // ---- extend: closest hit of the continuation or camera ray (k_extend)
    const int scene = p.has_ray ? p.J->scene : 0;
    const Traced ext = warp_trace<false>(sc, p.has_ray, scene, p.o, p.d, 0.0f, kRealMax, P.err);
    n_ext += p.has_ray;

    __syncthreads();
    // ---- vertex (k_logic, then k_material / k_glass)
    bool vertex = false, term = false, mis = false, mis_trace = false;
    bool ended = false;  // the sample ended at this hit without direct lighting
    int kind = 0, mcode = 0;
    Isect is;
    f3 coef_prev = mk3(0.0f, 0.0f, 0.0f);
    f3 mo = coef_prev, md = coef_prev, mf = coef_prev;
    float mpdf = 0.0f, mcos = 0.0f;
    unsigned int nee_mask = 0;
    if (p.has_ray) {
      ++n_vert;
      if (++steps > max_steps) {
        atomicOr(P.err, 2);
        p.has_ray = false;
        p.slot = -1;
      } else {
        const int pid = ext.h.prim;
        const float4 hit = make_float4(__int_as_float(pid), ext.h.t_attr, ext.h.alpha, ext.h.beta);
        if (pid < 0) {
          // a camera ray or one after a delta sample left the scene: the
          // environment light's radiance along it (path_trace_renderer.cpp:66-81)
          if ((MASK & MK_ENV) && (p.depth == 0 || p.spec) && p.J->env >= 0)
            p.L = p.L + mulc(p.coef, env_emit(sc.envs[p.J->env], p.d));
          ended = true;
        } else {
          const DPrim& pr = sc.prims[pid];
          if ((p.depth == 0 || p.spec) && pr.emissive) {
            // emission seen by the camera ray or after a delta sample
            const f3 gz = sc.tshade[pr.shape].gz;
            if (dot(gz, -p.d) > 0.0f) p.L = p.L + mulc(p.coef, pr.emission);
          }
          kind = sc.mats[pr.material].kind;
          make_isect(sc, hit, p.o, p.d, is);
          Bsdf bsdf;
          mcode = pr.material;
          bsdf.m = sc.mats + mcode;
          if ((MASK & MK_MAPS) && bsdf.m->tex_any) {  // image maps: the material at this hit's uv
            float u, v;
            hit_uv(sc, hit, p.o, p.d, u, v);
            material_at(sc, pr.material, u, v, &tmat);
            bsdf.m = &tmat;
            mcode = -1;
          }
          bsdf.g = is.g;
          bsdf.s = is.s;
          if ((MASK & MK_GLASS) && kind == MAT_GLASS) {
            // k_glass: a delta sample, no direct lighting
            const float u0 = Pcg::next(p.st);
            Pcg::skip<2>(p.st);  // the rest of sample3()
            const BsdfSample bs = bsdf.glass_sample(is.wo, u0);
            bool t = black(bs.f) || bs.pdf < kEps;
            if (!t) {
              const bool counted = p.sdepth >= kMaxSpecularDepth;
              if (!counted) ++p.sdepth;
              p.coef = mulc(p.coef, divs(muls(bs.f, abs_cos(is.g.z, bs.wi)), bs.pdf));
              t = !valid3(p.coef);
              if (!t) {
                if (counted) ++p.depth;
                if (p.depth >= p.J->max_depth) {
                  t = true;
                } else if (p.depth > p.J->min_depth) {
                  if (Pcg::next(p.st) > 0.9f) t = true;
                  else {
                    p.coef = divs(p.coef, 0.9f);
                    if (!valid3(p.coef)) t = true;
                  }
                }
              }
            }
            if (t) {
              ended = true;
            } else {
              p.o = is.eps_offset(bs.wi);
              p.d = normalize(normalize(bs.wi));
              p.spec = true;
            }
          } else {
            const float u0 = Pcg::next(p.st), u1 = Pcg::next(p.st), u2 = Pcg::next(p.st);
            const BsdfSample bs = m_sample<MASK>(bsdf, kind, is.wo, u0, u1, u2);
            if (black(bs.f) || bs.pdf < kEps) {
              ended = true;
            } else {
              vertex = true;
              // next-event estimation draws on every light (sample_area_light)
              const JobDev& J = *p.J;
              const float pos_mag = fabsf(is.pos.x) + fabsf(is.pos.y) + fabsf(is.pos.z);
              for (int l = 0; l < J.nl; ++l) {
                // a vertex well behind a light's plane gets nothing from it
                // (k_material's skip: its five draws only advance the stream)
                const DLight& lt = sc.lights[J.light_base + l];
                const float side = dot(lt.gz, is.pos - lt.A);
                const float tol = 1e-4f * (pos_mag + lt.extent);
                if (side < -tol) {
                  Pcg::skip<5>(p.st);
                  continue;
                }
                const float lu = Pcg::next(p.st), lv = Pcg::next(p.st);
                Pcg::skip<3>(p.st);
                nu[l] = make_float2(lu, lv);
                nee_mask |= 1u << l;
              }
              // the MIS BSDF ray (sample_bsdf, src/renderer/direct_illumination.cpp:144-155)
              const float v0 = Pcg::next(p.st), v1 = Pcg::next(p.st), v2 = Pcg::next(p.st);
              const BsdfSample ms = m_sample<MASK>(bsdf, kind, is.wo, v0, v1, v2);
              if (ms.valid()) {
                const f3 wi = normalize(ms.wi);
                mo = is.eps_offset(wi);
                md = normalize(wi);
                mpdf = ms.pdf;
                mcos = abs_cos(is.g.z, md);
                mf = ms.f;
                mis = true;
                mis_trace = mis_may_hit_light(sc, J, mo, md);
              }
              coef_prev = p.coef;
              p.coef = mulc(p.coef, divs(muls(bs.f, abs_cos(is.g.z, bs.wi)), bs.pdf));
              term = !valid3(p.coef);
              if (!term) {
                ++p.depth;
                if (p.depth >= J.max_depth) {
                  term = true;
                } else if (p.depth > J.min_depth) {
                  if (Pcg::next(p.st) > 0.9f) term = true;
                  else {
                    p.coef = divs(p.coef, 0.9f);
                    if (!valid3(p.coef)) term = true;
                  }
                }
              }
              if (!term) {
                p.o = is.eps_offset(bs.wi);
                p.d = normalize(normalize(bs.wi));
                p.spec = false;
              }
            }
          }
        }
      }
    }

    __syncthreads();
    // ---- lights: the light sample and its shadow ray per light (k_nee, k_shadow)
    f3 direct = mk3(0.0f, 0.0f, 0.0f);
    Bsdf bsdf;
    bsdf.m = mcode >= 0 ? sc.mats + mcode : &tmat;
    bsdf.g = is.g;
    bsdf.s = is.s;
    for (int l = 0; l < P.nl_max; ++l) {
      bool trace = false;
      f3 cc = mk3(0.0f, 0.0f, 0.0f), so = cc, sd = cc;
      float dist = 0.0f;
      if (vertex && ((nee_mask >> l) & 1u)) {
        const float2 uv = nu[l];
        const DLight& lt = sc.lights[p.J->light_base + l];
        if ((MASK & MK_ENV) && lt.env >= 0) {
          // sample_environment_light (src/renderer/direct_illumination.cpp:73-106)
          f3 Le, lpos;
          float lpdf;
          if (env_sample(sc.envs[lt.env], is.pos, uv.x, uv.y, Le, lpdf, lpos) && !black(Le)) {
            f3 to_light = lpos - is.pos;
            bool too_close;
            dist = dist_minus_eps(len2f(to_light), too_close);
            if (!too_close) {
              to_light = normalize(to_light);
              const f3 bf = m_eval<MASK>(bsdf, kind, to_light, is.wo);
              trace = !black(bf);
              if (trace) {
                const float bpdf = m_pdf<MASK>(bsdf, kind, to_light, is.wo);
                const f3 fl = muls(mulc(Le, bf), abs_cos(to_light, bsdf.g.z));
                const float w = power_heuristic(lpdf, bpdf);
                cc = mulc(coef_prev, divs(muls(fl, w), lpdf));
                so = is.pos;
                sd = normalize(to_light);
              }
            }
          }
        } else {
          // sample_area_light (src/renderer/direct_illumination.cpp:35-71) via
          // UniformSampleTriangle (src/shape/triangle.cpp:61-97)
          const float su0 = sqrtf(uv.x);
          const float bx = 1.0f - su0, by = uv.y * su0;
          const f3 lpos = scale(lt.A, bx) + scale(lt.B, by) + scale(lt.C, 1.0f - bx - by);
          const f3 sp2ref = is.pos - lpos;
          if (dot(lt.gz, sp2ref) > 0.0f) {
            const float dist2 = len2f(sp2ref);
            const float lpdf = area_to_solid_pdf(lt.area_pdf * dist2, dot(lt.gz, sp2ref), dist2);
            if (lpdf) {
              f3 to_light = lpos - is.pos;
              bool too_close;
              dist = dist_minus_eps(len2f(to_light), too_close);
              if (!too_close) {
                to_light = normalize(to_light);
                const f3 bf = m_eval<MASK>(bsdf, kind, to_light, is.wo);
                trace = !black(bf);
                if (trace) {
                  const float bpdf = m_pdf<MASK>(bsdf, kind, to_light, is.wo);
                  const f3 fl = muls(mulc(lt.emission, bf), abs_cos(to_light, bsdf.g.z));
                  const float w = power_heuristic(lpdf, bpdf);
                  cc = mulc(coef_prev, divs(muls(fl, w), lpdf));
                  so = is.pos;
                  sd = normalize(to_light);
                }
              }
            }
          }
        }
      }
      // the shadow ray: the remembered occluder first, then the walk
      bool blocked = false;
      bool walk = trace;
      if (trace && P.occluder_cache && sc.slot_leaf && oc[l] >= 0 &&
          occluded_by_slot(sc, p.J->scene, oc[l], so, sd, kEps, dist)) {
        blocked = true;
        walk = false;
        ++n_hits;
      }
      n_sh += trace;
      if (__any_sync(kFull, walk)) {
        const Traced sh = warp_trace<true>(sc, walk, walk ? p.J->scene : 0, so, sd, kEps, dist, P.err);
        if (walk && sh.occluded) {
          blocked = true;
          oc[l] = sh.h.prim;
        }
      }
      if (trace && !blocked) direct = direct + cc;
      // the block walks each light's shadow rays together: without this
      // barrier the warps interleave one light's walk with the next light's
      // sampling (86 against 101 Msamples/s on the Cornell box)
      __syncthreads();
    }

    __syncthreads();
    // ---- mis: the BSDF-sampled ray's emission, weighted against the light
    //      (mis_contribution of render.cu, direct_illumination.cpp:144-198)
    {
      // a ray that can reach no light is not traced: its closest hit would give zero
      Traced mh;
      mh.h.prim = -1;
      if (__any_sync(kFull, mis_trace))
        mh = warp_trace<false>(sc, mis_trace, mis_trace ? p.J->scene : 0, mo, md, 0.0f, kRealMax, P.err);
      n_ext += mis_trace;
      if (mis) {
        const int pid = mis_trace ? mh.h.prim : -1;
        f3 c = mk3(0.0f, 0.0f, 0.0f);
        if (pid < 0) {
          const int ei = p.J->env;
          if ((MASK & MK_ENV) && ei >= 0) {
            const DEnv& e = sc.envs[ei];
            const f3 Le = env_emit(e, md);
            if (!black(Le)) {
              const f3 f = muls(mulc(Le, mf), mcos);
              const float w = power_heuristic(mpdf, env_pdf(e, md));
              c = divs(muls(f, w), mpdf);
            }
          }
        } else {
          const DPrim& pr = sc.prims[pid];
          if (pr.emissive) {
            const f3 gz = sc.tshade[pr.shape].gz;
            if (dot(gz, -md) > 0.0f) {
              const f3 f = muls(mulc(pr.emission, mf), mcos);
              const f3 pos = mo + scale(md, mh.h.t_attr);
              const float lpdf = light_pdf_at(pr.area, mo, pos, gz);
              const float w = power_heuristic(mpdf, lpdf);
              c = divs(muls(f, w), mpdf);
            }
          }
        }
        direct = direct + mulc(coef_prev, c);
      }
    }

    // ---- finish: the vertex's direct lighting, then the path goes on or ends.
    // Samples that ended in the vertex phase finish here too (they draw no
    // more random numbers this iteration). With one inlined copy of the film
    // update and the camera-ray code instead of four, the kernel spills less
    // and ran 2.5% faster on the Cornell box.
    if (vertex) p.L = p.L + direct;
    if (ended || (vertex && term)) finish_sample(p);
    if (!done && !p.has_ray) p.slot = -1;  // the pixel's samples are done: claim another
  }
  // statistics (warp sums, one atomic per warp)
  const unsigned long long sums[5] = {p.finished, n_ext, n_sh, n_vert, n_hits};
  const int where[5] = {0, 1, 2, 3, 8};
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    unsigned long long v = sums[k];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(kFull, v, off);
    if (lane == 0 && v) atomicAdd(P.stats + where[k], v);
  }
}

constexpr unsigned kMaskPhong = MK_PHONG;
constexpr unsigned kMaskPD = MK_PHONG | MK_DISNEY12;
constexpr unsigned kMaskAll = MK_PHONG | MK_DISNEY12 | MK_GLASS | MK_METAL | MK_DISNEY15 | MK_ENV | MK_MAPS;

const void* kernel_of(unsigned mask) {
  if (mask == kMaskPhong) return (const void*)k_mega<kMaskPhong>;
  if (mask == kMaskPD) return (const void*)k_mega<kMaskPD>;
  return (const void*)k_mega<kMaskAll>;
}

}  // namespace

unsigned mega_kernel_mask(const DScene& sc, bool has_disney12) {
  if (sc.has_glass || sc.has_metal || sc.has_disney15 || sc.has_env || sc.has_textures) return kMaskAll;
  return has_disney12 ? kMaskPD : kMaskPhong;
}

cudaError_t launch_mega(const MegaLaunch& P, unsigned mask, int grid, int threads, cudaStream_t st) {
  if (mask == kMaskPhong) k_mega<kMaskPhong><<<grid, threads, 0, st>>>(P);
  else if (mask == kMaskPD) k_mega<kMaskPD><<<grid, threads, 0, st>>>(P);
  else k_mega<kMaskAll><<<grid, threads, 0, st>>>(P);
  return cudaGetLastError();
}

int mega_blocks_per_sm(unsigned mask) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel_of(mask), kMegaThreads, 0) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    n = 1;
  }
  return n;
}

}  // namespace trg
