// env_light.h -- host-side tables of the environment light (the reference's
// IBL over an HDR texture, src/light/environment_light.cpp:14-84): the texels
// as float4 and the luminance distribution of its sampling routine, built
// once per upload with the reference's float/double arithmetic so that the
// device samples and weights directions from the same tables.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tracer_gpu.h"

namespace trg {

struct EnvHost {
  int w = 0, h = 0;              // texture size
  int nu = 0, nv = 0;            // distribution grid: min(w, 360) x min(h, 180)
  std::vector<float> texels;     // 4 per texel (r, g, b, 0), texel (x, y) at 4 * (x + y * w)
  std::vector<uint8_t> texels8;  // an 8-bit map instead: 4 bytes per texel (r, g, b, 0)
  std::vector<float> cond_func;  // nv rows of nu: the conditional densities p(u | v) before normalisation
  std::vector<float> cond_cdf;   // nv rows of nu + 1
  std::vector<float> cond_int;   // nv: each row's integral (the marginal's function)
  std::vector<float> marg_cdf;   // nv + 1
  float marg_int = 0.0f;
  float to_light[9], to_world[9];  // rotation/scale parts of world_to_light and its inverse, row-major
  float center[3] = {0.0f, 0.0f, 0.0f};
  float radius = 0.0f;           // bounding sphere of the scene's root box (EnvironmentLight::preprocess)
};

// Validates the description's environment map and fills `env` (all but the
// bounding sphere). Returns false with `err` set on invalid input.
bool build_env_tables(const tr_scene_desc* d, EnvHost& env, std::string& err);

// EnvironmentLight::preprocess (src/core/light.hpp:93-95) over the root box
// lo/hi of the scene's tree (empty = the default box).
void env_bounding_sphere(EnvHost& env, const float lo[3], const float hi[3], bool empty);

}  // namespace trg
