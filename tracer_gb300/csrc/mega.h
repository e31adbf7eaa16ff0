// mega.h -- the persistent render kernel (mega.cu), launched by render.cu.
#pragma once

#include <cuda_runtime.h>

#include "render_common.cuh"

namespace trg {

// Material kinds (bit per MAT_* kind) and features one instantiation of the
// persistent kernel handles; the host picks the smallest that covers a set.
enum : unsigned {
  MK_PHONG = 1u << MAT_PHONG,
  MK_DISNEY12 = 1u << MAT_DISNEY12,
  MK_GLASS = 1u << MAT_GLASS,
  MK_METAL = 1u << MAT_METAL,
  MK_DISNEY15 = 1u << MAT_DISNEY15,
  MK_ENV = 1u << 8,   // an environment light
  MK_MAPS = 1u << 9,  // Phong image maps
};
// Lights of one scene the persistent kernel keeps per-thread state for
// (light-sample draws and remembered occluders); sets with more render with
// the wavefront.
constexpr int kMegaLights = 16;

struct MegaLaunch {
  DScene sc;
  const JobDev* jobs;
  int njobs, nslots;
  int nl_max;            // most lights of one job's scene (<= kMegaLights)
  int occluder_cache;    // remember each (slot, light)'s last occluder (tr_tuning.occluder_cache)
  unsigned int* fetch;   // next unclaimed path slot (zeroed by the host)
  int* err;              // bit 0: traversal stack overflow; bit 1: a slot ran past its vertex bound
  unsigned long long* stats;  // samples, extend rays, shadow rays, vertices, 4-7 unused, occluder hits (8)
};

// The smallest instantiation covering a scene set (MK_* bits).
unsigned mega_kernel_mask(const DScene& sc, bool has_disney12);
// Launches the persistent kernel of instantiation `mask` (grid blocks of
// `threads` threads, at most kMegaThreads, a multiple of 32) on `st`.
cudaError_t launch_mega(const MegaLaunch& P, unsigned mask, int grid, int threads, cudaStream_t st);
// Resident blocks per SM of that instantiation.
int mega_blocks_per_sm(unsigned mask);
constexpr int kMegaThreads = 512;

}  // namespace trg
