// env_light.cu -- host-side tables of the environment light: the IBL
// constructor's luminance distribution (src/light/environment_light.cpp:20-81)
// over Distribution2D / Distribution1D (src/utility/distribution.hpp:12-111),
// and EnvironmentLight::preprocess (src/core/light.hpp:93-95). Host code only
// (compiled without contraction, like the reference); the device reads the
// resulting tables.
#include <algorithm>
#include <cmath>

#include "env_light.h"
#include "env_tex.cuh"

namespace trg {
namespace {

// Distribution1D's constructor: cdf[i + 1] = cdf[i] + f[i] / n, then
// normalised by the integral (or uniform when it is zero).
float build_1d(const float* f, int n, float* cdf) {
  cdf[0] = 0.0f;
  for (int i = 0; i < n; i++) cdf[i + 1] = cdf[i] + f[i] / n;
  const float integral = cdf[n];
  if (!integral) {
    for (int i = 1; i < n + 1; i++) cdf[i] = (float)i / n;
  } else {
    for (int i = 1; i < n + 1; i++) cdf[i] /= integral;
  }
  return integral;
}

}  // namespace

bool build_env_tables(const tr_scene_desc* d, EnvHost& env, std::string& err) {
  if (!d->env_texels && !d->env_texels8) return true;
  if (d->env_width == 0 || d->env_height == 0 || d->env_width > 65536 || d->env_height > 65536) {
    err = "environment map size out of range";
    return false;
  }
  if (!d->env_to_light || !d->env_to_world) {
    err = "environment light transform missing";
    return false;
  }
  const int w = (int)d->env_width, h = (int)d->env_height;
  env.w = w;
  env.h = h;
  if (d->env_texels) {
    env.texels.resize(4 * (size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
      env.texels[4 * i] = d->env_texels[3 * i];
      env.texels[4 * i + 1] = d->env_texels[3 * i + 1];
      env.texels[4 * i + 2] = d->env_texels[3 * i + 2];
      env.texels[4 * i + 3] = 0.0f;
    }
  } else {
    env.texels8.resize(4 * (size_t)w * h);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
      env.texels8[4 * i] = d->env_texels8[3 * i];
      env.texels8[4 * i + 1] = d->env_texels8[3 * i + 1];
      env.texels8[4 * i + 2] = d->env_texels8[3 * i + 2];
      env.texels8[4 * i + 3] = 0;
    }
  }
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      env.to_light[3 * r + c] = d->env_to_light[4 * r + c];
      env.to_world[3 * r + c] = d->env_to_world[4 * r + c];
    }
  const float4* tex = reinterpret_cast<const float4*>(env.texels.data());
  const uchar4* tex8 = reinterpret_cast<const uchar4*>(env.texels8.data());
  const bool ldr = !env.texels8.empty();
  // luminance x solid angle per cell of the (at most) 360 x 180 grid; each
  // cell sums the luminance of the texel centres it covers plus a one-texel
  // border
  const int nw = std::min(w, 360), nh = std::min(h, 180);
  env.nu = nw;
  env.nv = nh;
  env.cond_func.assign((size_t)nw * nh, 0.0f);
  for (int y = 0; y < nh; ++y) {
    const float y0 = (float)y / nh, y1 = (float)(y + 1) / nh;
    const float sy0 = y0 * h, sy1 = y1 * h;
    const int yb = std::max(0, (int)(std::floor(sy0) - 1.0f));
    const int ye = std::min(h - 1, (int)(std::floor(sy1) + 1.0f));
    for (int x = 0; x < nw; ++x) {
      const float x0 = (float)x / nw, x1 = (float)(x + 1) / nw;
      const float sx0 = x0 * w, sx1 = x1 * w;
      const int xb = std::max(0, (int)(std::floor(sx0) - 1.0f));
      const int xe = std::min(w - 1, (int)(std::floor(sx1) + 1.0f));
      float lum = 0.0f;
      for (int sy = yb; sy <= ye; ++sy)
        for (int sx = xb; sx <= xe; ++sx) {
          const float su = (float)(sx + 0.5) / w, sv = (float)(sy + 0.5) / h;
          const f3 c = ldr ? env_tex_eval8(tex8, w, h, su, sv) : env_tex_eval(tex, w, h, su, sv);
          lum += 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z;
        }
      // d_omega = sin(theta) d_theta d_phi over the cell, the sine in double
      const float a = 2.0f * kPi * (x1 - x0) * kPi * (y1 - y0);
      const float area = (float)std::fabs((double)a * std::sin((double)kPi * 0.5 * (double)(y1 + y0)));
      env.cond_func[(size_t)x + (size_t)y * nw] = lum * area;
    }
  }
  env.cond_cdf.resize((size_t)nh * (nw + 1));
  env.cond_int.resize(nh);
  for (int y = 0; y < nh; ++y)
    env.cond_int[y] = build_1d(&env.cond_func[(size_t)y * nw], nw, &env.cond_cdf[(size_t)y * (nw + 1)]);
  env.marg_cdf.resize(nh + 1);
  env.marg_int = build_1d(env.cond_int.data(), nh, env.marg_cdf.data());
  return true;
}

void env_bounding_sphere(EnvHost& env, const float lo[3], const float hi[3], bool empty) {
  if (empty) {  // Bounds3f(): low = max, high = lowest
    env.center[0] = env.center[1] = env.center[2] = 0.0f;
    env.radius = 0.0f;
    return;
  }
  // (low + high) / 2 via the double reciprocal; inside(center, box) ? distance(center, high) : 0
  bool inside = true;
  for (int k = 0; k < 3; ++k) {
    env.center[k] = (float)(0.5 * (double)(lo[k] + hi[k]));
    inside = inside && env.center[k] >= lo[k] && env.center[k] <= hi[k];
  }
  const f3 dv = mk3(env.center[0] - hi[0], env.center[1] - hi[1], env.center[2] - hi[2]);
  env.radius = inside ? (float)lengthd(dv) : 0.0f;
}

}  // namespace trg
