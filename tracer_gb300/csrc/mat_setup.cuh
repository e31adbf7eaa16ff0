// mat_setup.cuh -- a material's per-shading set-up from its factory
// arguments, on the host (constant materials, once at upload) and on the
// device (materials with image maps, at every hit, after the maps are
// evaluated at the hit's uv).
#pragma once

#include "../../include/tracer_gpu.h"
#include "scene_types.h"

namespace trg {

// Color3::lum (src/core/spectrum.hpp:94-96)
TR_HD float mat_lum(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

TR_HD DMat derive_material(const tr_material& m) {
  DMat d{};
  if (m.kind == TR_MAT_PHONG) {
    d.kind = MAT_PHONG;
    d.kd_c = mk3(m.kd[0], m.kd[1], m.kd[2]);
    d.ks_c = mk3(m.ks[0], m.ks[1], m.ks[2]);
    d.ns_c = m.ns;
    d.tex_kd = (int)m.tex_kd;
    d.tex_ks = (int)m.tex_ks;
    d.tex_ns = (int)m.tex_ns;
    phong_setup(d, d.kd_c, d.ks_c, d.ns_c);  // the constants; a hit with maps sets up again
  } else if (m.kind == TR_MAT_METAL) {
    // create_metal(color, eta, k) hands over to Metal(color, k, eta), whose
    // shading builds PaintedConductorFresnelPoint(color, 1, eta, k) with
    // parameters (eta_outside, eta_inside, k, paint): eta_outside = color,
    // eta_inside = 1, conductor k = the caller's k, paint = the caller's eta
    d.kind = MAT_METAL;
    d.base = mk3(m.color[0], m.color[1], m.color[2]);
    d.albedo = d.base;  // AggregateBSDF<1>(..., color)
    float e2[3], ek2[3];
    for (int c = 0; c < 3; ++c) {
      e2[c] = 1.0f / m.color[c];
      e2[c] *= e2[c];
      ek2[c] = m.k[c] / m.color[c];
      ek2[c] *= ek2[c];
    }
    d.f_eta2 = mk3(e2[0], e2[1], e2[2]);
    d.f_etak2 = mk3(ek2[0], ek2[1], ek2[2]);
    d.f_paint = mk3(m.eta[0], m.eta[1], m.eta[2]);
    d.roughness = m.roughness;
    d.anisotropic = m.anisotropic;
    // GGXMicrofacetReflectionBXDF (src/material/bxdf/microfacet_refl_bxdf.cpp:6-11)
    const float aspect = m.anisotropic > 0.0f ? sqrtf(1.0f - 0.9f * m.anisotropic) : 1.0f;
    d.ax = smax(0.001f, m.roughness * m.roughness / aspect);
    d.ay = smax(0.001f, m.roughness * m.roughness * aspect);
  } else if (m.kind == TR_MAT_DISNEY15) {
    // Disney::shading and DisneyBSDF's constructor (src/material/disney.cpp:341-392,616-651)
    d.kind = MAT_DISNEY15;
    d.base = mk3(m.base_color[0], m.base_color[1], m.base_color[2]);
    d.albedo = d.base;  // get_albedo(): C_
    d.metallic = m.metallic;
    d.roughness = m.roughness;
    d.specular_tint = m.specular_tint;
    d.anisotropic = m.anisotropic;
    d.sheen = m.sheen;
    d.sheen_tint = m.sheen_tint;
    d.clearcoat = m.clearcoat;
    d.spec_scale = mk3(m.specular_scale[0], m.specular_scale[1], m.specular_scale[2]);
    d.transmission = m.transmission;
    const float l = mat_lum(d.base);  // to_tint
    d.c_tint = l > 0.0f ? mk3(d.base.x / l, d.base.y / l, d.base.z / l) : mk3(1.0f, 1.0f, 1.0f);
    d.ior = smax(1.01f, m.ior);
    const float aspect = m.anisotropic > 0.0f ? sqrtf(1.0f - 0.9f * m.anisotropic) : 1.0f;
    d.ax = smax(0.001f, m.roughness * m.roughness / aspect);
    d.ay = smax(0.001f, m.roughness * m.roughness * aspect);
    const float tr = m.transmission_roughness;
    d.trans_ax = smax(0.001f, tr * tr / aspect);
    d.trans_ay = smax(0.001f, tr * tr * aspect);
    float cr = (1.0f - m.clearcoat_gloss) * 0.1f + m.clearcoat_gloss * 0.0f;  // mix(0.1, 0, gloss)
    cr *= cr;
    d.cc_rough = smax(cr, 0.0001f);
    float A = mat_lum(d.base) * (1.0f - d.metallic);
    A = A < 0.3f ? 0.3f : (0.7f < A ? 0.7f : A);
    const float B = 1.0f - A;
    d.w_diff15 = A * (1.0f - d.transmission);
    d.w_trans = A * d.transmission;
    d.w_spec15 = B * 2.0f / (2.0f + d.clearcoat);
    d.w_cc = B * d.clearcoat / (2.0f + d.clearcoat);
  } else if (m.kind == TR_MAT_GLASS) {
    d.kind = MAT_GLASS;
    d.kr = mk3(m.kr[0], m.kr[1], m.kr[2]);
    d.kt_sqrt = mk3(sqrtf(m.kt[0]), sqrtf(m.kt[1]), sqrtf(m.kt[2]));  // Glass::shading
    d.ior = m.ior;
    d.albedo = mk3(0.5f * (d.kr.x + d.kt_sqrt.x), 0.5f * (d.kr.y + d.kt_sqrt.y), 0.5f * (d.kr.z + d.kt_sqrt.z));
  } else {
    d.kind = MAT_DISNEY12;
    d.base = mk3(m.base_color[0], m.base_color[1], m.base_color[2]);
    d.albedo = d.base;
    d.subsurface = m.subsurface;
    d.metallic = m.metallic;
    d.specular_s = m.specular;
    d.specular_tint = m.specular_tint;
    d.roughness = m.roughness;
    d.anisotropic = m.anisotropic;
    d.sheen = m.sheen;
    d.sheen_tint = m.sheen_tint;
    d.clearcoat = m.clearcoat;
    d.clearcoat_gloss = m.clearcoat_gloss;
    // DisneyBRDF's per-call constants (src/material/disney_brdf.cpp:81-83,142-151,188-193)
    const float aspect = (float)sqrt(1.0 - (double)m.anisotropic * 0.9);
    d.ax = smax(0.001f, m.roughness * m.roughness / aspect);
    d.ay = smax(0.001f, m.roughness * m.roughness * aspect);
    d.p_diffuse = smin(0.8f, 1.0f - m.metallic);
    d.p_spec_sample = (float)(1.0 / (1.0 + 0.5 * (double)m.clearcoat) * (double)(1.0f - d.p_diffuse));
    d.p_spec_pdf = (float)(1.0 / (1.0 + 0.5 * (double)m.clearcoat));
  }
  return d;
}


// The image maps of a material at texture coordinates (u, v): every mapped
// factory argument of tr_material.tex_param (Phong's own maps are set up by
// phong_at) replaced by the map's value there -- a colour, or the red
// channel for scalar arguments (Texture2D::evaluate / evaluate_s as the
// materials' shading calls them: src/material/glass.cpp:117-140,
// src/material/metal.cpp:33-56, src/material/disney.cpp:604-639,
// src/material/disney_brdf.cpp:278-302). Eval: f3 (int texture index, u, v).
template <class Eval>
TR_HD void apply_maps(tr_material& m, const Eval& eval) {
  auto col = [&](int i, float* dst) {
    if (m.tex_param[i]) {
      const f3 c = eval((int)m.tex_param[i] - 1);
      dst[0] = c.x;
      dst[1] = c.y;
      dst[2] = c.z;
    }
  };
  auto scl = [&](int i, float& dst) {
    if (m.tex_param[i]) dst = eval((int)m.tex_param[i] - 1).x;
  };
  if (m.kind == TR_MAT_GLASS) {
    col(0, m.kr);
    col(1, m.kt);
    scl(2, m.ior);
  } else if (m.kind == TR_MAT_METAL) {
    col(0, m.color);
    col(1, m.eta);
    col(2, m.k);
    scl(3, m.roughness);
    scl(4, m.anisotropic);
  } else if (m.kind == TR_MAT_DISNEY15) {
    col(0, m.base_color);
    scl(1, m.metallic);
    scl(2, m.roughness);
    scl(3, m.transmission);
    scl(4, m.transmission_roughness);
    scl(5, m.ior);
    col(6, m.specular_scale);
    scl(7, m.specular_tint);
    scl(8, m.anisotropic);
    scl(9, m.sheen);
    scl(10, m.sheen_tint);
    scl(11, m.clearcoat);
    scl(12, m.clearcoat_gloss);
  } else if (m.kind == TR_MAT_DISNEY12) {
    col(0, m.base_color);
    scl(1, m.subsurface);
    scl(2, m.metallic);
    scl(3, m.specular);
    scl(4, m.specular_tint);
    scl(5, m.roughness);
    scl(6, m.anisotropic);
    scl(7, m.sheen);
    scl(8, m.sheen_tint);
    scl(9, m.clearcoat);
    scl(10, m.clearcoat_gloss);
  }
}

// Factory arguments of a material kind that tex_param maps.
TR_HD int mapped_params(int kind) {
  return kind == TR_MAT_GLASS ? 3 : kind == TR_MAT_METAL ? 5 : kind == TR_MAT_DISNEY15 ? 13
         : kind == TR_MAT_DISNEY12 ? 11 : 0;
}

}  // namespace trg
