// shade.cuh -- per-vertex shading on the device: sampler, camera, hit
// records, BSDFs (Phong aggregate and Disney12), area lights, film filter.
//
// Each function restates one reference function (cited) with its exact
// float/double arithmetic; this file is compiled with --fmad=false.
// Transcendentals (sinf, cosf, atan2f, powf, logf, expf) are CUDA's: they may
// differ from glibc in the last bit, so paths that pass through them can
// diverge from the CPU reference after the first such difference; ray
// arithmetic (traversal, frames, normalisation) is exact.
#pragma once

#include "env_tex.cuh"
#include "mat_setup.cuh"
#include "scene_types.h"

namespace trg {

// ----------------------------------------------------------------- sampler
// pcg32 (setseq XSH-RR 64/32, default stream, output of the previous state)
// behind SimpleUniformSampler and std::uniform_real_distribution<float>
// (src/core/sampler.hpp:30-86): u = float(x) / 2^32, clamped below 1.
struct Pcg {
  static constexpr unsigned long long kMul = 6364136223846793005ULL;
  static constexpr unsigned long long kInc = 1442695040888963407ULL;
  static __device__ __forceinline__ unsigned long long seed(int s) {
    return ((unsigned long long)(long long)s + kInc) * kMul + kInc;
  }
  static __device__ __forceinline__ float next(unsigned long long& st) {
    const unsigned long long old = st;
    st = old * kMul + kInc;
    const unsigned xs = (unsigned)(((old >> 18u) ^ old) >> 27u);
    const unsigned rot = (unsigned)(old >> 59u);
    const unsigned x = (xs >> rot) | (xs << ((32u - rot) & 31u));
    float u = __uint2float_rn(x) * 2.3283064365386963e-10f;
    return u >= 1.0f ? 0.99999994f : u;
  }
  // Jump-ahead of the LCG state by n draws: s_n = mul_n * s + inc_n.
  static __host__ __device__ constexpr unsigned long long jump_mul(int n) {
    unsigned long long r = 1;
    for (int i = 0; i < n; ++i) r *= kMul;
    return r;
  }
  static __host__ __device__ constexpr unsigned long long jump_inc(int n) {
    unsigned long long r = 0;
    for (int i = 0; i < n; ++i) r = r * kMul + kInc;
    return r;
  }
  // Advances the state past N draws whose values are not used.
  template <int N>
  static __device__ __forceinline__ void skip(unsigned long long& st) {
    constexpr unsigned long long m = jump_mul(N), c = jump_inc(N);
    st = st * m + c;
  }
};

// ---------------------------------------------------------------- sampling
// ConcentricSampleDisk (src/core/sampling.cpp:8-22)
__device__ __forceinline__ void concentric_disk(float u, float v, float& ox, float& oy) {
  const float x = u * 2.0f - 1.0f, y = v * 2.0f - 1.0f;
  if (x == 0.0f && y == 0.0f) {
    ox = 0.0f;
    oy = 0.0f;
    return;
  }
  float theta, r;
  if (fabsf(x) > fabsf(y)) {
    r = x;
    theta = kPiOver4 * (y / x);
  } else {
    r = y;
    theta = kPiOver2 - kPiOver4 * (x / y);
  }
  float st, ct;
  sincosf(theta, &st, &ct);
  ox = r * ct;
  oy = r * st;
}
// CosineSampleHemisphere (src/core/sampling.cpp:24-28)
__device__ __forceinline__ f3 cosine_hemisphere(float u, float v) {
  float dx, dy;
  concentric_disk(u, v, dx, dy);
  const float z = sqrtf(smax(0.0f, 1.0f - dx * dx - dy * dy));
  return mk3(dx, dy, z);
}
__device__ __forceinline__ float cosine_pdf(float c) { return c * kInvPi; }
// PowerHeuristic (src/core/sampling.hpp:230-233)
__device__ __forceinline__ float power_heuristic(float fp, float gp) { return (fp * fp) / (fp * fp + gp * gp); }

// Spectrum helpers (src/core/spectrum.hpp)
__device__ __forceinline__ f3 mulc(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ f3 muls(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ f3 divs(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ f3 adds(f3 a, float s) { return mk3(a.x + s, a.y + s, a.z + s); }
__device__ __forceinline__ bool black(f3 c) { return c.x == 0.0f && c.y == 0.0f && c.z == 0.0f; }
__device__ __forceinline__ bool finite3(f3 c) { return isfinite(c.x) && isfinite(c.y) && isfinite(c.z); }
__device__ __forceinline__ bool valid3(f3 c) { return c.x >= 0.0f && c.y >= 0.0f && c.z >= 0.0f && finite3(c); }
__device__ __forceinline__ float lum(f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
// mix(l, r, f) = (1 - f) * l + f * r (src/utility/geometry.hpp:989-993)
__device__ __forceinline__ f3 mix3(f3 l, f3 r, float f) { return muls(l, 1.0f - f) + muls(r, f); }
__device__ __forceinline__ float mixf(float l, float r, float f) { return (1.0f - f) * l + f * r; }

// ---------------------------------------------------------------- surface
struct Isect {
  f3 pos, wo;
  Frame g, s;
  int prim;
  // SurfacePoint::eps_offset (src/core/intersection.hpp:19-23)
  __device__ __forceinline__ f3 eps_offset(f3 dir) const {
    if (dot(g.z, dir) > 0.0f) return pos + scale(g.z, kEps);
    return pos - scale(g.z, kEps);
  }
};

// Triangle::intersect_p hit record (src/shape/triangle.cpp:175-213); the
// geometry frame and compute_ss_ts of the normals are per-triangle constants.
__device__ __forceinline__ void triangle_isect(const DTriShade& ts, f3 o, f3 d, float t, float alpha, float beta,
                                               Isect& is) {
  is.wo = -d;
  is.pos = o + scale(d, t);
  is.g.x = ts.gx;
  is.g.y = ts.gy;
  is.g.z = ts.gz;
  const f3 sn = ts.nA + scale(ts.dn1, alpha) + scale(ts.dn2, beta);
  f3 dndu, dndv;
  if (ts.det_nonzero) {
    dndu = ts.dndu0;
    dndv = ts.dndv0;
  } else {
    coordinate(sn, dndu, dndv);
  }
  if (len2f(dndu) < kEps || len2f(dndv) < kEps) coordinate(sn, dndu, dndv);
  dndu = cross(dndv, sn);
  dndv = cross(sn, dndu);
  is.s = make_frame(dndu, dndv, sn);
}

// Sphere::intersect_p hit record + TransformedShape::to_world
// (src/shape/sphere.cpp:48-78,98-119; src/shape/transformed_shape.hpp:31-44).
// The (u, v) coordinates are not formed: constant textures never read them.
__device__ __forceinline__ void sphere_isect(const DSphere& S, f3 o, f3 d, float t, Isect& is) {
  const f3 lo = xform_point(S.inv, o);
  const f3 ld = normalize(xform_vec(S.inv, d));
  const f3 p = lo + scale(ld, t);
  f3 ex, ey, ez = normalize(p);
  if (fabsf(ez.z - 1.0f) < kEps) {
    ex = mk3(1.0f, 0.0f, 0.0f);
    ey = mk3(0.0f, 1.0f, 0.0f);
    ez = mk3(0.0f, 0.0f, 1.0f);
  } else if (fabsf(ez.z + 1.0f) < kEps) {
    ex = mk3(0.0f, 1.0f, 0.0f);
    ey = mk3(1.0f, 0.0f, 0.0f);
    ez = mk3(0.0f, 0.0f, -1.0f);
  } else {
    ex = cross(mk3(0.0f, 0.0f, 1.0f), ez);
    ey = cross(ez, ex);
  }
  const Frame c = make_frame(ex, ey, ez);
  is.pos = xform_point(S.m, p);
  is.g = make_frame(xform_vec(S.m, c.x), xform_vec(S.m, c.y), xform_vec(S.m, c.z));
  is.s = is.g;
  is.wo = xform_vec(S.m, -ld);
}

// The hit's uv, formed only for materials with image maps: the barycentric
// blend of Triangle::intersect_p (src/shape/triangle.cpp:186) or
// sphere::local_geometry_uv_and_coord (src/shape/sphere.cpp:48-56) at the
// local hit point.
static __device__ __noinline__ void hit_uv(const DScene& sc, const float4 hit, f3 o, f3 d, float& u, float& v) {
  const DPrim& p = sc.prims[__float_as_int(hit.x)];
  if (p.kind == PRIM_TRIANGLE) {
    const DTriShade& ts = sc.tshade[p.shape];
    u = ts.uvA[0] + hit.z * ts.duv1[0] + hit.w * ts.duv2[0];
    v = ts.uvA[1] + hit.z * ts.duv1[1] + hit.w * ts.duv2[1];
    return;
  }
  const DSphere& S = sc.spheres[p.shape];
  const f3 lo = xform_point(S.inv, o);
  const f3 ld = normalize(xform_vec(S.inv, d));
  const f3 q = lo + scale(ld, hit.y);
  float phi = (!q.x && !q.y) ? 0.0f : atan2f(q.y, q.x);
  if (phi < 0.0f) phi += 2.0f * kPi;
  float st = q.z / S.radius;
  st = st < -1.0f ? -1.0f : (1.0f < st ? 1.0f : st);
  u = 0.5f * kInvPi * phi;
  v = kInvPi * asinf(st) + 0.5f;
}

// Texture2D::evaluate of an image texture (HDR or 8-bit) at (u, v).
__device__ __forceinline__ f3 tex_eval(const DTex& t, float u, float v) {
  return t.texels8 ? env_tex_eval8(t.texels8, t.w, t.h, u, v) : env_tex_eval(t.texels, t.w, t.h, u, v);
}

// Phong::shading with maps: kd, ks and ns (its red channel) at the hit's uv,
// then the same set-up as for constants, written to `out`.
static __device__ __noinline__ void phong_at(const DScene& sc, const DMat& m, float u, float v, DMat* out) {
  const f3 kd = m.tex_kd ? tex_eval(sc.textures[m.tex_kd - 1], u, v) : m.kd_c;
  const f3 ks = m.tex_ks ? tex_eval(sc.textures[m.tex_ks - 1], u, v) : m.ks_c;
  const float ns = m.tex_ns ? tex_eval(sc.textures[m.tex_ns - 1], u, v).x : m.ns_c;
  DMat d;
  d.kind = MAT_PHONG;
  phong_setup(d, kd, ks, ns);
  out->kind = d.kind;
  out->ns = d.ns;
  out->w_diffuse = d.w_diffuse;
  out->w_specular = d.w_specular;
  out->diffuse_coef = d.diffuse_coef;
  out->specular = d.specular;
  out->albedo = d.albedo;
}

// The set-up of a material with image maps at a hit's (u, v): Phong's maps
// through phong_at; the other kinds' mapped arguments evaluated from
// DScene::msrc, then the same set-up as for constants (derive_material).
static __device__ __noinline__ void material_at(const DScene& sc, int mi, float u, float v, DMat* out) {
  const DMat& m = sc.mats[mi];
  if (m.kind == MAT_PHONG) {
    phong_at(sc, m, u, v, out);
    return;
  }
  tr_material src = sc.msrc[mi];
  apply_maps(src, [&](int t) { return tex_eval(sc.textures[t], u, v); });
  *out = derive_material(src);
  out->tex_any = 0;
}

__device__ __forceinline__ void make_isect(const DScene& sc, const float4 hit, f3 o, f3 d, Isect& is) {
  const int pid = __float_as_int(hit.x);
  const DPrim& p = sc.prims[pid];
  is.prim = pid;
  if (p.kind == PRIM_TRIANGLE)
    triangle_isect(sc.tshade[p.shape], o, d, hit.y, hit.z, hit.w, is);
  else
    sphere_isect(sc.spheres[p.shape], o, d, hit.y, is);
}

// ------------------------------------------------------------------- BSDFs
struct BsdfSample {
  f3 wi, f;
  float pdf;
  bool delta = false;  // BSDFSampleResult::is_delta
  __device__ __forceinline__ bool valid() const { return pdf > 0.0f && !black(f); }  // core/bsdf.hpp:21-23
};

// ConductorFresnelPoint::evaluate (src/material/utility/fresnel_point.hpp:47-66), one channel
__device__ __forceinline__ float conductor_fresnel(float eta_2, float eta_k_2, float cos_theta_i) {
  if (cos_theta_i <= 0.0f) return 0.0f;
  const float cos2 = cos_theta_i * cos_theta_i;
  const float sin2 = fmaxf(0.0f, 1.0f - cos2);
  const float t0 = eta_2 - eta_k_2 - sin2;
  const float a2b2 = sqrtf(t0 * t0 + 4.0f * eta_2 * eta_k_2);
  const float t1 = a2b2 + cos2;
  const float a = sqrtf(0.5f * (a2b2 + t0));
  const float t2 = 2.0f * cos_theta_i * a;
  const float rs = (t1 - t2) / (t1 + t2);
  const float t3 = cos2 * a2b2 + sin2 * sin2;
  const float t4 = t2 * sin2;
  const float rp = rs * (t3 - t4) / (t3 + t4);
  return 0.5f * (rp + rs);
}

// dielectric_fresnel (src/utility/reflection.hpp:16-40)
__device__ __forceinline__ float dielectric_fresnel(float eta_i, float eta_o, float cos_theta_i) {
  if (cos_theta_i < 0.0f) {
    const float t = eta_i;
    eta_i = eta_o;
    eta_o = t;
    cos_theta_i = -cos_theta_i;
  }
  const float sin_theta_i = sqrtf(fmaxf(0.0f, 1.0f - cos_theta_i * cos_theta_i));
  const float sin_theta_t = eta_o / eta_i * sin_theta_i;
  if (sin_theta_t >= 1.0f) return 1.0f;
  const float cos_theta_t = sqrtf(fmaxf(0.0f, 1.0f - sin_theta_t * sin_theta_t));
  const float para = (eta_i * cos_theta_i - eta_o * cos_theta_t) / (eta_i * cos_theta_i + eta_o * cos_theta_t);
  const float perp = (eta_o * cos_theta_i - eta_i * cos_theta_t) / (eta_o * cos_theta_i + eta_i * cos_theta_t);
  return 0.5f * (para * para + perp * perp);
}

// microfacet helpers (src/material/utility/microfacet.cpp:7-134, microfacet.hpp:10-14)
__device__ __forceinline__ float sqr(float x) { return x * x; }
__device__ __forceinline__ float one_minus_5(float x) {
  const float t = 1.0f - x;
  const float t2 = t * t;
  return t2 * t2 * t;
}
__device__ __forceinline__ float compute_alpha(float sp, float cp, float ax, float ay) {
  return sqr(cp / ax) + sqr(sp / ay);
}
__device__ __forceinline__ float anisotropic_gtr2(float sp, float cp, float st, float ct, float ax, float ay) {
  const float A = compute_alpha(sp, cp, ax, ay);
  const float RD = sqr(st) * A + sqr(ct);
  return 1.0f / (kPi * ax * ay * sqr(RD));
}
__device__ __forceinline__ float gtr1(float st, float ct, float alpha) {
  if (alpha >= 1.0f) return kInvPi;
  const float U = sqr(alpha) - 1.0f;
  const float LD = 2.0f * kPi * logf(alpha);
  const float RD = sqr(alpha * ct) + sqr(st);
  return U / (LD * RD);
}
__device__ __forceinline__ float smith_aniso_gtr2(float cos_phi, float sin_phi, float ax, float ay, float tan_theta) {
  const float t = sqr(ax * cos_phi) + sqr(ay * sin_phi);
  const float sq = 1.0f + t * sqr(tan_theta);
  const float lambda = -0.5f + 0.5f * sqrtf(sq);
  return 1.0f / (1.0f + lambda);
}
__device__ __forceinline__ float smith_gtr2(float tan_theta, float alpha) {
  if (!tan_theta) return 1.0f;
  const float root = alpha * tan_theta;
  return 2.0f / (1.0f + sqrtf(1.0f + root * root));
}
__device__ __forceinline__ f3 sample_aniso_gtr2(float ax, float ay, float u, float v) {
  float s2, c2;
  sincosf(2.0f * kPi * u, &s2, &c2);
  float sp = ay * s2;
  float cp = ax * c2;
  const float nor = 1.0f / sqrtf(sqr(sp) + sqr(cp));
  sp *= nor;
  cp *= nor;
  const float A = compute_alpha(sp, cp, ax, ay);
  const float ct = sqrtf(A * (1.0f - v) / ((1.0f - A) * v + A));
  const float st = sqrtf(smax(0.0f, 1.0f - sqr(ct)));
  return normalize(mk3(st * cp, st * sp, ct));
}
__device__ __forceinline__ float local_cos_to_sin(float c) { return sqrtf(smax(0.0f, 1.0f - c * c)); }
__device__ __forceinline__ f3 sample_gtr1(float alpha, float u, float v) {
  const float phi = 2.0f * kPi * u;
  const float ct = sqrtf((powf(alpha, 2.0f - 2.0f * v) - 1.0f) / (sqr(alpha) - 1.0f));
  const float st = local_cos_to_sin(ct);
  float sphi, cphi;
  sincosf(phi, &sphi, &cphi);
  return normalize(mk3(st * cphi, st * sphi, ct));
}
// local_phi / local_tan_theta (src/utility/geometry.hpp:912-928)
__device__ __forceinline__ float local_phi(f3 w) {
  if (!w.y && !w.x) return 0.0f;
  const float r = atan2f(w.y, w.x);
  return r < 0.0f ? (r + 2.0f * kPi) : r;
}
__device__ __forceinline__ float local_tan_theta(f3 w) {
  const float t = 1.0f - w.z * w.z;
  if (t <= 0.0f) return 0.0f;
  return sqrtf(t) / w.z;
}
// reflect (src/utility/reflection.hpp:12-14)
__device__ __forceinline__ f3 reflect(f3 w, f3 n) { return scale(n, 2.0f * dot(w, n)) - w; }

// PhongSpecularBXDF (src/material/bxdf/phong_specular_bxdf.cpp:10-71)
__device__ __forceinline__ float powcos_pdf(float e, float c) { return (e + 1.0f) * kInv2Pi * powf(c, e); }
__device__ __forceinline__ f3 phong_eval(const DMat& m, f3 lwi, f3 lwo) {
  if (lwi.z <= 0.0f || lwo.z <= 0.0f) return mk3(0.0f, 0.0f, 0.0f);
  const f3 ideal = reflect(lwo, mk3(0.0f, 0.0f, 1.0f));
  const float c = cos_x(ideal, lwi);
  if (c <= 0.0f) return mk3(0.0f, 0.0f, 0.0f);
  return muls(m.specular, powcos_pdf(m.ns, c));
}
__device__ __forceinline__ float phong_pdf(const DMat& m, f3 lwi, f3 lwo) {
  if (lwi.z <= 0.0f || lwo.z <= 0.0f) return 0.0f;
  const f3 ideal = reflect(lwo, mk3(0.0f, 0.0f, 1.0f));
  const float c = cosv(lwi, ideal);
  if (c <= 0.0f) return 0.0f;
  return powcos_pdf(m.ns, c);
}
__device__ __forceinline__ bool phong_sample(const DMat& m, f3 lwo, float u, float v, f3& lwi_out, f3& f,
                                             float& pdf) {
  if (lwo.z <= 0.0f) return false;
  const f3 ideal = normalize(reflect(lwo, mk3(0.0f, 0.0f, 1.0f)));
  const float ct = powf(u, 1.0f / (m.ns + 1.0f));
  const float st = sqrtf(smax(0.0f, 1.0f - ct * ct));
  const float phi = 2.0f * kPi * v;
  float sphi, cphi;
  sincosf(phi, &sphi, &cphi);
  const f3 local = normalize(mk3(st * cphi, st * sphi, ct));
  const f3 lwi = normalize(to_global(frame_from_z(ideal), local));
  if (lwi.z <= 0.0f) return false;
  pdf = powcos_pdf(m.ns, local.z);
  f = phong_eval(m, lwi, lwo);
  lwi_out = lwi;
  return pdf > 0.0f;
}
// DiffuseBXDF (src/material/bxdf/diffuse_bxdf.cpp:14-38)
__device__ __forceinline__ f3 diffuse_eval(const DMat& m, f3 lwi, f3 lwo) {
  if (lwi.z <= 0.0f || lwo.z <= 0.0f) return mk3(0.0f, 0.0f, 0.0f);
  return m.diffuse_coef;
}
__device__ __forceinline__ float diffuse_pdf(f3 lwi, f3 lwo) {
  if (lwi.z <= 0.0f || lwo.z <= 0.0f) return 0.0f;
  return cosine_pdf(lwi.z);
}

static __device__ inline float disney_fd90_d(float L, float r) {
  return (float)(0.5 + 2.0 * (double)L * (double)L * (double)r);
}
static __device__ inline float disney_ss_d(float Fss, float S) {
  return (float)(1.25 * ((double)Fss * (1.0 / (double)S - 0.5) + 0.5));
}

// Fd90 = 0.5 + 2. * LdotH * LdotH * roughness, evaluated in double by the
// reference (src/material/disney_brdf.cpp:120); certified float-float form.
__device__ __forceinline__ float disney_fd90(float L, float r) {
  if (L == 0.0f || r == 0.0f) return 0.5f;
  if (in_range(L) && in_range(r)) {
    const float th = L * L, tl = ffma(L, L, -th);
    const float a = th * r;
    if (in_range(a)) {
      const float al = ffma(th, r, -a) + tl * r;
      float e;
      const float s0 = two_sum(0.5f, 2.0f * a, e);
      const float w = e + 2.0f * al;
      float res;
      const float y = two_sum(s0, w, res);
      if (rounds_to(y, res, 5.6843419e-14f * (2.0f * fabsf(a) + 1.0f))) return y;  // 2^-44
    }
  }
  return disney_fd90_d(L, r);
}
// ss = 1.25 * (Fss * (1.0 / (NdotL + NdotV) - 0.5) + 0.5) in double
// (src/material/disney_brdf.cpp:125); certified float-float form.
__device__ __forceinline__ float disney_ss(float Fss, float S) {
  if (in_range(S) && (Fss == 0.0f || in_range(Fss))) {
    const float i0 = 1.0f / S;
    const float i1 = i0 * ffma(-i0, S, 1.0f);
    float e;
    const float t = two_sum(i0, -0.5f, e);
    const float tw = e + i1;
    const float ph = Fss * t;
    const float pl = ffma(Fss, t, -ph) + Fss * tw;
    float e2;
    const float q = two_sum(ph, 0.5f, e2);
    const float ql = e2 + pl;
    const float qh2 = q * 1.25f;
    const float ql2 = ffma(q, 1.25f, -qh2) + ql * 1.25f;
    float res;
    const float y = two_sum(qh2, ql2, res);
    const float err = 2.2737368e-13f * (1.0f + fabsf(Fss) * (fabsf(i0) + 1.0f));  // 2^-42
    if (rounds_to(y, res, err)) return y;
  }
  return disney_ss_d(Fss, S);
}

// normal_correct_factor (src/utility/coordinate.hpp:43-52)
__device__ __forceinline__ float normal_correct(const Frame& g, const Frame& s, f3 wi) {
  const float dem = fabsf(cosv(g.z, wi));
  return dem < kEps ? 1.0f : fabsf(cosv(s.z, wi)) / dem;
}

struct Bsdf {
  const DMat* m;
  Frame g, s;

  // LocalBSDF black-fringe handling (src/core/bsdf.hpp:55-91)
  __device__ __forceinline__ bool fringe(f3 w) const { return pos_hemi(g, w) ^ pos_hemi(s, w); }
  __device__ __forceinline__ f3 eval_fringe(f3 wi, f3 wo) const {
    if (pos_hemi(g, wi) & pos_hemi(g, wo)) return muls(m->albedo, kInvPi);
    return mk3(0.0f, 0.0f, 0.0f);
  }
  __device__ __forceinline__ BsdfSample sample_fringe(f3 wo, float u, float v) const {
    BsdfSample r;
    r.pdf = 0.0f;
    r.f = mk3(0.0f, 0.0f, 0.0f);
    r.wi = r.f;
    if (!pos_hemi(g, wo)) return r;
    const f3 lwi = cosine_hemisphere(u, v);
    const float pdf = cosine_pdf(lwi.z);
    if (pdf < kEps) return r;
    const f3 wi = normalize(to_global(g, lwi));
    const float nc = normal_correct(g, s, wi);
    r.wi = wi;
    r.f = muls(muls(m->albedo, kInvPi), nc);
    r.pdf = pdf;
    return r;
  }
  __device__ __forceinline__ float pdf_fringe(f3 wi, f3 wo) const {
    if (pos_hemi(g, wi) ^ pos_hemi(g, wo)) return 0.0f;
    return cosine_pdf(normalize(to_local(g, wi)).z);
  }

  // ---- AggregateBSDF<2> of Phong (src/material/aggregate_bsdf.hpp:36-118)
  __device__ f3 phong_eval_agg(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return eval_fringe(wi, wo);
    const f3 lwi = normalize(to_local(s, wi)), lwo = normalize(to_local(s, wo));
    if (!lwi.z || !lwo.z) return mk3(0.0f, 0.0f, 0.0f);
    f3 r = mk3(0.0f, 0.0f, 0.0f);
    r = r + diffuse_eval(*m, lwi, lwo);
    r = r + phong_eval(*m, lwi, lwo);
    return r;
  }
  __device__ float phong_pdf_agg(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return pdf_fringe(wi, wo);
    const f3 lwi = normalize(to_local(s, wi)), lwo = normalize(to_local(s, wo));
    if (!lwi.z || !lwo.z) return 0.0f;
    float ws = 0.0f, pdf = 0.0f;
    ws += m->w_diffuse;
    pdf += m->w_diffuse * diffuse_pdf(lwi, lwo);
    ws += m->w_specular;
    pdf += m->w_specular * phong_pdf(*m, lwi, lwo);
    return ws > 0.0f ? pdf / ws : 0.0f;
  }
  __device__ BsdfSample phong_sample_agg(f3 wo, float u, float v, float w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BsdfSample out;
    out.pdf = 0.0f;
    out.f = mk3(0.0f, 0.0f, 0.0f);
    out.wi = out.f;
    const f3 lwo = normalize(to_local(s, wo));
    if (!lwo.z) return out;
    float ws = 0.0f;
    ws += m->w_diffuse;
    ws += m->w_specular;
    float sel = (u - 0.001f) * ws;
    const float w0 = m->w_diffuse, w1 = m->w_specular;
    int which = -1;
    float weight = 0.0f;
    if (sel <= w0) {
      which = 0;
      weight = w0;
    } else {
      sel -= w0;
      if (sel <= w1) {
        which = 1;
        weight = w1;
      }
    }
    if (which < 0) return out;
    f3 lwi, f;
    float pdf;
    if (which == 0) {
      if (lwo.z <= 0.0f) return out;
      lwi = cosine_hemisphere(v, w);
      pdf = cosine_pdf(lwi.z);
      if (pdf < 0.001f) return out;
      f = m->diffuse_coef;
    } else {
      if (!phong_sample(*m, lwo, v, w, lwi, f, pdf)) return out;
    }
    lwi = normalize(lwi);
    pdf *= weight;
    if (which != 0) {
      f = f + diffuse_eval(*m, lwi, lwo);
      pdf += diffuse_pdf(lwi, lwo) * w0;
    }
    if (which != 1) {
      f = f + phong_eval(*m, lwi, lwo);
      pdf += phong_pdf(*m, lwi, lwo) * w1;
    }
    const f3 wi = to_global(s, lwi);
    const float nc = normal_correct(g, s, wi);
    out.wi = wi;
    out.f = muls(f, nc);
    out.pdf = pdf;
    return out;
  }

  // ---- DisneyBRDF (src/material/disney_brdf.cpp:56-227); its quirks are kept:
  // the diffuse draw is overwritten by the specular branch, p_specular differs
  // between sample and pdf, the pdf mixes with (1 - pdf_diffuse), clearcoat's
  // pdf passes (sin_phi, cos_phi, gloss) to gtr1, and the Smith term gets
  // (sin_phi, cos_phi) in its (cos_phi, sin_phi) slots.
  __device__ __forceinline__ void alphas(float& ax, float& ay) const {
    ax = m->ax;  // per-material constants computed at upload
    ay = m->ay;
  }
  __device__ f3 disney_eval(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return eval_fringe(wi, wo);
    const f3 lwi = normalize(to_local(s, wi));
    const f3 lwo = normalize(to_local(s, wo));
    if (lwi.z < kEps || lwo.z < kEps) return mk3(0.0f, 0.0f, 0.0f);
    const float NdotL = lwi.z, NdotV = lwo.z;
    const f3 H = normalize(lwi + lwo);
    const float LdotH = dot(lwi, H);
    const f3 bc = m->base;
    const float l = lum(bc);
    const f3 Ctint = l > 0.0f ? divs(bc, l) : mk3(1.0f, 1.0f, 1.0f);
    const f3 one = mk3(1.0f, 1.0f, 1.0f);
    const f3 Cspec0 = mix3(muls(mix3(one, Ctint, m->specular_tint), m->specular_s * 0.08f), bc, m->metallic);
    const f3 Csheen = mix3(one, Ctint, m->sheen_tint);
    float ax, ay;
    alphas(ax, ay);
    const float phi_h = local_phi(H);
    float sph, cph;
    sincosf(phi_h, &sph, &cph);
    const float Ds = anisotropic_gtr2(sph, cph, local_cos_to_sin(H.z), H.z, ax, ay);
    const float FH = one_minus_5(LdotH);
    const f3 Fs = mix3(Cspec0, one, FH);
    float spi, cpi, spo, cpo;
    sincosf(local_phi(lwi), &spi, &cpi);
    float Gs = smith_aniso_gtr2(spi, cpi, ax, ay, local_tan_theta(lwi));
    sincosf(local_phi(lwo), &spo, &cpo);
    Gs *= smith_aniso_gtr2(spo, cpo, ax, ay, local_tan_theta(lwo));
    const float Dr = gtr1(local_cos_to_sin(H.z), H.z, mixf(0.1f, 0.001f, m->clearcoat_gloss));
    const float Fr = mixf(0.04f, 1.0f, FH);
    const float Gr = smith_gtr2(local_tan_theta(lwi), 0.25f) * smith_gtr2(local_tan_theta(lwo), 0.25f);
    f3 fd = mk3(0.0f, 0.0f, 0.0f);
    fd = fd + divs(adds(muls(muls(Fs, Ds), Gs), 0.25f * m->clearcoat * Gr * Fr * Dr), 4.0f * NdotL * NdotV);
    if (m->metallic < 1.0f) {
      const float FL = one_minus_5(NdotL), FV = one_minus_5(NdotV);
      const float Fd90 = disney_fd90(LdotH, m->roughness);
      const float Fd = mixf(1.0f, Fd90, FL) * mixf(1.0f, Fd90, FV);
      const float Fss90 = LdotH * LdotH * m->roughness;
      const float Fss = mixf(1.0f, Fss90, FL) * mixf(1.0f, Fss90, FV);
      const float ss = disney_ss(Fss, NdotL + NdotV);
      const f3 Fsheen = muls(Csheen, FH * m->sheen);
      fd = fd + muls(muls(muls(bc, kInvPi), mixf(Fd, ss, m->subsurface)) + Fsheen, 1.0f - m->metallic);
    }
    return muls(fd, normal_correct(g, s, wi));
  }
  __device__ float disney_pdf(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return pdf_fringe(wi, wo);
    const float p_diffuse = m->p_diffuse;
    const float p_specular = m->p_spec_pdf;
    float ax, ay;
    alphas(ax, ay);
    const f3 lwi = normalize(to_local(s, wi));
    const f3 lwo = normalize(to_local(s, wo));
    if (lwi.z < kEps) return 0.0f;
    const f3 H = normalize(lwi + lwo);
    const float pdf_diffuse = cosine_pdf(lwi.z);
    float sph, cph;
    sincosf(local_phi(H), &sph, &cph);
    const float pdf_spec = anisotropic_gtr2(sph, cph, local_cos_to_sin(H.z), H.z, ax, ay) * H.z / (4.0f * dot(lwi, H));
    const float pdf_cc = gtr1(sph, cph, m->clearcoat_gloss) * H.z / (4.0f * dot(lwi, H));
    const float pdf = p_diffuse * pdf_diffuse + (1.0f - pdf_diffuse) * (p_specular * pdf_spec + (1.0f - p_specular) * pdf_cc);
    if (!isfinite(pdf)) return 0.0f;
    return pdf;
  }
  __device__ BsdfSample disney_sample(f3 wo, float u, float v, float w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BsdfSample r;
    r.pdf = 0.0f;
    r.f = mk3(0.0f, 0.0f, 0.0f);
    r.wi = r.f;
    const float p_diffuse = m->p_diffuse;
    const float p_specular = m->p_spec_sample;
    const f3 lwo = normalize(to_local(s, wo));
    f3 lwi = mk3(0.0f, 0.0f, 0.0f);
    float sel = u;
    float ax, ay;
    alphas(ax, ay);
    if (sel < p_diffuse) lwi = cosine_hemisphere(v, w);
    sel -= p_diffuse;
    if (sel < p_specular) {
      const f3 lwh = sample_aniso_gtr2(ax, ay, v, w);
      if (lwh.z > 0.0f) {
        lwi = normalize(scale(lwh, 2.0f * dot(lwo, lwh)) - lwo);
        if (lwi.z <= 0.0f) lwi = mk3(0.0f, 0.0f, 0.0f);
      }
    } else {
      const f3 lwh = sample_gtr1(m->clearcoat_gloss, v, w);
      if (lwh.z > 0.0f) {
        lwi = normalize(scale(lwh, 2.0f * dot(lwo, lwh)) - lwo);
        if (lwi.z <= 0.0f) lwi = mk3(0.0f, 0.0f, 0.0f);
      }
    }
    if (all_zero(lwi)) return r;
    r.wi = to_global(s, lwi);
    r.f = disney_eval(r.wi, wo);
    r.pdf = disney_pdf(r.wi, wo);
    return r;
  }

  // ---- GlassBSDF (src/material/glass.cpp:11-99) with DielectricFresnelPoint(ior, 1) and
  // TransportMode::Radiance: a delta BSDF (eval and pdf 0); u picks reflection with the
  // Fresnel probability, else refraction (refract_dir, src/utility/reflection.hpp:43-51)
  __device__ BsdfSample glass_sample(f3 wo, float u) const {
    BsdfSample out;
    out.pdf = 0.0f;
    out.f = mk3(0.0f, 0.0f, 0.0f);
    out.wi = out.f;
    const f3 lwo = normalize(to_local(s, wo));
    const f3 nor = lwo.z > 0.0f ? mk3(0.0f, 0.0f, 1.0f) : mk3(0.0f, 0.0f, -1.0f);
    const float fr = dielectric_fresnel(m->ior, 1.0f, lwo.z);
    if (u < fr) {
      const f3 lwi = mk3(-lwo.x, -lwo.y, lwo.z);
      const f3 wi = to_global(s, lwi);
      const float q = fr / fabsf(lwi.z);
      out.wi = wi;
      out.f = muls(mk3(m->kr.x * q, m->kr.y * q, m->kr.z * q), normal_correct(g, s, wi));
      out.pdf = fr;
      out.delta = true;
      return out;
    }
    const float eta_i = lwo.z > 0.0f ? 1.0f : m->ior, eta_t = lwo.z > 0.0f ? m->ior : 1.0f;
    const float eta = eta_i / eta_t;
    const float cos_i = fabsf(lwo.z);
    const float sin_i2 = fmaxf(0.0f, 1.0f - cos_i * cos_i);
    const float sin_t2 = eta * eta * sin_i2;
    if (sin_t2 >= 1.0f) return out;  // total internal reflection: no sample
    const float cos_t = sqrtf(1.0f - sin_t2);
    const f3 lwi = normalize(scale(nor, eta * cos_i - cos_t) - scale(lwo, eta));
    const f3 wi = to_global(s, lwi);
    const float corr = eta * eta, az = fabsf(lwi.z);
    const f3 f = mk3(((corr * m->kt_sqrt.x) * (1.0f - fr)) / az, ((corr * m->kt_sqrt.y) * (1.0f - fr)) / az,
                     ((corr * m->kt_sqrt.z) * (1.0f - fr)) / az);
    out.wi = wi;
    out.f = muls(f, normal_correct(g, s, wi));
    out.pdf = 1.0f - fr;
    out.delta = true;
    return out;
  }

  // ---- Metal: AggregateBSDF<1> (src/material/aggregate_bsdf.hpp:36-118) of one
  // GGXMicrofacetReflectionBXDF (src/material/bxdf/microfacet_refl_bxdf.cpp:13-78), weight 1
  __device__ void ggx(f3 lwi, f3 lwo, f3* eval, float* pdf) const {
    const float cos_theta_i = lwi.z, cos_theta_o = lwo.z;
    const f3 lwh = normalize(lwi + lwo);
    const float cos_theta_d = dot(lwi, lwh);
    float sin_phi_h, cos_phi_h, sin_phi_i, cos_phi_i, sin_phi_o, cos_phi_o;
    sincosf(local_phi(lwh), &sin_phi_h, &cos_phi_h);
    const float cos_theta_h = lwh.z;
    float sin_theta_h = sqrtf(1.0f - cos_theta_h * cos_theta_h);
    sin_theta_h = 0.0f < sin_theta_h ? sin_theta_h : 0.0f;  // std::max<real>(0, x)
    const float D = anisotropic_gtr2(sin_phi_h, cos_phi_h, sin_theta_h, cos_theta_h, m->ax, m->ay);
    sincosf(local_phi(lwi), &sin_phi_i, &cos_phi_i);
    sincosf(local_phi(lwo), &sin_phi_o, &cos_phi_o);
    const float Gi = smith_aniso_gtr2(cos_phi_i, sin_phi_i, m->ax, m->ay, local_tan_theta(lwi));
    const float Go = smith_aniso_gtr2(cos_phi_o, sin_phi_o, m->ax, m->ay, local_tan_theta(lwo));
    if (eval) {
      const float G = Gi * Go;
      const float den = fabsf(4.0f * cos_theta_i * cos_theta_o);
      const float Fr = m->f_paint.x * conductor_fresnel(m->f_eta2.x, m->f_etak2.x, cos_theta_d);
      const float Fg = m->f_paint.y * conductor_fresnel(m->f_eta2.y, m->f_etak2.y, cos_theta_d);
      const float Fb = m->f_paint.z * conductor_fresnel(m->f_eta2.z, m->f_etak2.z, cos_theta_d);
      *eval = mk3(Fr * D * G / den, Fg * D * G / den, Fb * D * G / den);
    }
    if (pdf) *pdf = Go * D / (4.0f * cos_theta_o);
  }
  // microfacet::sample_anisotropic_gtr2_with_visible_normal (src/material/utility/microfacet.cpp:58-80)
  __device__ f3 sample_vndf(f3 ve, float u, float v) const { return sample_vndf_a(ve, u, v, m->ax, m->ay); }
  static __device__ f3 sample_vndf_a(f3 ve, float u, float v, float ax, float ay) {
    const f3 vh = normalize(mk3(ax * ve.x, ay * ve.y, ve.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const f3 t1 = lensq > kEps ? divd(mk3(-vh.y, vh.x, 0.0f), (double)sqrtf(lensq)) : mk3(1.0f, 0.0f, 0.0f);
    const f3 t2 = cross(vh, t1);
    const float r = sqrtf(u);
    float sp, cp;
    sincosf(2.0f * kPi * v, &sp, &cp);
    const float t_1 = r * cp;
    const float t_2a = r * sp;
    const float sh = 0.5f * (1.0f + vh.z);
    const float t_2 = (1.0f - sh) * sqrtf(1.0f - t_1 * t_1) + sh * t_2a;
    const float q = 1.0f - t_1 * t_1 - t_2 * t_2;
    const f3 nh = scale(t1, t_1) + scale(t2, t_2) + scale(vh, sqrtf(0.0f < q ? q : 0.0f));
    return normalize(mk3(ax * nh.x, ay * nh.y, 0.0f < nh.z ? nh.z : 0.0f));
  }
  __device__ f3 metal_eval(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return eval_fringe(wi, wo);
    const f3 lwi = normalize(to_local(s, wi)), lwo = normalize(to_local(s, wo));
    if (!lwi.z || !lwo.z) return mk3(0.0f, 0.0f, 0.0f);
    f3 r = mk3(0.0f, 0.0f, 0.0f);
    if (!(lwi.z <= 0.0f || lwo.z <= 0.0f)) {
      f3 e;
      ggx(lwi, lwo, &e, nullptr);
      r = r + e;
    }
    return r;
  }
  __device__ float metal_pdf(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return pdf_fringe(wi, wo);
    const f3 lwi = normalize(to_local(s, wi)), lwo = normalize(to_local(s, wo));
    if (!lwi.z || !lwo.z) return 0.0f;
    float p = 0.0f;
    if (!(lwi.z <= 0.0f || lwo.z <= 0.0f)) ggx(lwi, lwo, nullptr, &p);
    return (1.0f * p) / 1.0f;
  }
  __device__ BsdfSample metal_sample(f3 wo, float u, float v, float w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BsdfSample out;
    out.pdf = 0.0f;
    out.f = mk3(0.0f, 0.0f, 0.0f);
    out.wi = out.f;
    const f3 lwo = normalize(to_local(s, wo));
    if (!lwo.z) return out;
    if (!((u - 0.001f) * 1.0f <= 1.0f)) return out;
    if (lwo.z <= 0.0f) return out;
    const f3 lwh = normalize(sample_vndf(lwo, v, w));
    if (lwh.z <= 0.0f) return out;
    const f3 lwi0 = normalize(scale(lwh, 2.0f * dot(lwo, lwh)) - lwo);
    if (lwi0.z <= 0.0f) return out;
    f3 f;
    float pdf = 0.0f;
    ggx(lwi0, lwo, &f, &pdf);
    if (!(pdf > 0.0f)) return out;  // BXDFSampleResult::is_valid
    const f3 lwi = normalize(lwi0);
    const f3 wi = to_global(s, lwi);
    out.wi = wi;
    out.f = muls(f, normal_correct(g, s, wi));
    out.pdf = pdf * 1.0f;
    return out;
  }

  // ---- DisneyBSDF, the 2015 model (src/material/disney.cpp:14-537), radiance transport
  static __device__ __forceinline__ float d15_D(f3 lwh, float ax, float ay) {
    float sp, cp;
    sincosf(local_phi(lwh), &sp, &cp);
    return anisotropic_gtr2(sp, cp, local_cos_to_sin(lwh.z), lwh.z, ax, ay);
  }
  static __device__ __forceinline__ float d15_G1(f3 lw, float ax, float ay) {
    float sp, cp;
    sincosf(local_phi(lw), &sp, &cp);
    return smith_aniso_gtr2(cp, sp, ax, ay, local_tan_theta(lw));
  }
  __device__ f3 d15_f_transmission(f3 lwi, f3 lwo) const {
    const float eta = lwo.z > 0.0f ? m->ior : 1.0f / m->ior;
    f3 lwh = normalize(lwo + scale(lwi, eta));
    if (lwh.z < 0.0f) lwh = -lwh;
    const float cd = dot(lwo, lwh);
    const float F = dielectric_fresnel(m->ior, 1.0f, cd);
    const float D = d15_D(lwh, m->trans_ax, m->trans_ay);
    const float G = d15_G1(lwi, m->trans_ax, m->trans_ay) * d15_G1(lwo, m->trans_ax, m->trans_ay);
    const float sdem = cd + eta * dot(lwi, lwh);
    const float corr = 1.0f / eta;
    const float val = (1.0f - F) * D * G * eta * eta * dot(lwi, lwh) * dot(lwo, lwh) * corr * corr /
                      (lwi.z * lwo.z * sdem * sdem);
    const float k = (1.0f - m->metallic) * (lwo.z > 0.0f ? m->transmission : 1.0f);
    const float av = fabsf(val);
    return mk3(k * sqrtf(m->base.x) * av, k * sqrtf(m->base.y) * av, k * sqrtf(m->base.z) * av);
  }
  __device__ f3 d15_f_inner_reflection(f3 lwi, f3 lwo) const {
    const f3 lwh = -normalize(lwi + lwo);
    const float F = dielectric_fresnel(m->ior, 1.0f, dot(lwo, lwh));
    const float D = d15_D(lwh, m->trans_ax, m->trans_ay);
    const float G = d15_G1(lwi, m->trans_ax, m->trans_ay) * d15_G1(lwo, m->trans_ax, m->trans_ay);
    return muls(muls(m->base, m->transmission), fabsf(F * D * G / (4.0f * lwi.z * lwo.z)));
  }
  __device__ f3 d15_f_specular(f3 lwi, f3 lwo) const {
    const f3 lwh = normalize(lwi + lwo);
    const float cd = dot(lwi, lwh);
    const f3 one = mk3(1.0f, 1.0f, 1.0f);
    const f3 Cspec = mix3(mix3(one, m->c_tint, m->specular_tint), m->base, m->metallic);
    const f3 diel = muls(Cspec, dielectric_fresnel(m->ior, 1.0f, cd));
    const f3 cond = Cspec + muls(one - Cspec, one_minus_5(cd));
    const f3 F = mix3(mulc(m->spec_scale, diel), cond, m->metallic);
    const float D = d15_D(lwh, m->ax, m->ay);
    const float G = d15_G1(lwi, m->ax, m->ay) * d15_G1(lwo, m->ax, m->ay);
    return divs(muls(muls(F, D), G), fabsf(4.0f * lwi.z * lwo.z));
  }
  __device__ float d15_pdf_transmission(f3 lwi, f3 lwo) const {
    const float eta = lwo.z > 0.0f ? m->ior : 1.0f / m->ior;
    f3 lwh = normalize(lwo + scale(lwi, eta));
    if (lwh.z < 0.0f) lwh = -lwh;
    if (((lwo.z > 0.0f) != (dot(lwh, lwo) > 0.0f)) || ((lwi.z > 0.0f) != (dot(lwh, lwi) > 0.0f))) return 0.0f;
    const float sdem = dot(lwo, lwh) + eta * dot(lwi, lwh);
    const float dwh_to_dwi = eta * eta * dot(lwi, lwh) / (sdem * sdem);
    const float D = d15_D(lwh, m->trans_ax, m->trans_ay);
    return fabsf(dot(lwi, lwh) * D * dwh_to_dwi);
  }
  __device__ float d15_pdf_inner_reflection(f3 lwi, f3 lwo) const {
    const f3 lwh = -normalize(lwi + lwo);
    const float D = d15_D(lwh, m->trans_ax, m->trans_ay);
    return fabsf(lwh.z * D / (4.0f * dot(lwi, lwh)));
  }
  __device__ f3 d15_eval(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return eval_fringe(wi, wo);
    const f3 lwi = normalize(to_local(s, wi)), lwo = normalize(to_local(s, wo));
    if (fabsf(lwi.z) < kEps || fabsf(lwo.z) < kEps) return mk3(0.0f, 0.0f, 0.0f);
    if (lwi.z * lwo.z < 0.0f) {
      if (m->transmission == 0.0f) return mk3(0.0f, 0.0f, 0.0f);
      return muls(d15_f_transmission(lwi, lwo), normal_correct(g, s, wi));
    }
    if (lwi.z < 0.0f && lwo.z < 0.0f) {
      if (m->transmission == 0.0f) return mk3(0.0f, 0.0f, 0.0f);
      return muls(d15_f_inner_reflection(lwi, lwo), normal_correct(g, s, wi));
    }
    const f3 lwh = normalize(lwi + lwo);
    const float cd = dot(lwi, lwh);
    f3 diffuse = mk3(0.0f, 0.0f, 0.0f), sheen = diffuse, clearcoat = diffuse;
    if (m->metallic < 1.0f) {
      // f_diffuse: Lambert with the retro-reflection term
      const float FL = one_minus_5(lwi.z), FV = one_minus_5(lwo.z);
      const float RR = 2.0f * m->roughness * cd * cd;
      const f3 lam = divs(m->base, kPi);
      const f3 retro = muls(muls(divs(m->base, kPi), RR), FL + FV + FL * FV * (RR - 1.0f));
      diffuse = muls(muls(lam, 1.0f - 0.5f * FL), 1.0f - 0.5f * FV) + retro;
      if (m->sheen > 0.0f)
        sheen = muls(muls(mix3(mk3(1.0f, 1.0f, 1.0f), m->c_tint, m->sheen_tint), 4.0f * m->sheen), one_minus_5(cd));
    }
    const f3 specular = d15_f_specular(lwi, lwo);
    if (m->clearcoat > 0.0f) {
      const float ch = lwh.z, sh = local_cos_to_sin(ch);
      const float D = gtr1(sh, ch, m->cc_rough);
      const float F = 0.04f + (1.0f - 0.04f) * one_minus_5(cd);
      const float G = smith_gtr2(local_tan_theta(lwi), 0.25f) * smith_gtr2(local_tan_theta(lwo), 0.25f);
      const float c = m->clearcoat * D * F * G / fabsf(4.0f * lwi.z * lwo.z);
      clearcoat = mk3(c, c, c);
    }
    const f3 ret = muls(diffuse + sheen, (1.0f - m->metallic) * (1.0f - m->transmission)) + specular + clearcoat;
    return muls(ret, normal_correct(g, s, wi));
  }
  __device__ float d15_pdf(f3 wi, f3 wo) const {
    if (fringe(wi) | fringe(wo)) return pdf_fringe(wi, wo);
    const f3 lwi = normalize(to_local(s, wi)), lwo = normalize(to_local(s, wo));
    if (fabsf(lwi.z) < kEps || fabsf(lwo.z) < kEps) return 0.0f;
    if (lwo.z < 0.0f) {
      if (m->transmission == 0.0f) return 0.0f;
      float F = dielectric_fresnel(m->ior, 1.0f, lwo.z);
      F = F < 0.1f ? 0.1f : (0.9f < F ? 0.9f : F);
      if (lwi.z > 0.0f) return (1.0f - F) * d15_pdf_transmission(lwi, lwo);
      return F * d15_pdf_inner_reflection(lwi, lwo);
    }
    if (lwi.z < 0.0f) return m->w_trans * d15_pdf_transmission(lwi, lwo);
    // pdf_specular_clearcoat (disney.cpp:250-281): sin(phi_o) from cos(phi_o)
    const f3 lwh = normalize(lwi + lwo);
    const float ch = lwh.z, sh = local_cos_to_sin(ch);
    const float cd = dot(lwi, lwh);
    const float cos_phi_o = cosf(local_phi(lwo));
    const float sin_phi_o = local_cos_to_sin(cos_phi_o);
    const float ps = smith_aniso_gtr2(cos_phi_o, sin_phi_o, m->ax, m->ay, local_tan_theta(lwo)) *
                     d15_D(lwh, m->ax, m->ay) / (4.0f * lwo.z);
    const float pc = ch * gtr1(sh, ch, m->cc_rough) / (4.0f * cd);
    return m->w_diff15 * cosine_pdf(lwi.z) + m->w_spec15 * ps + m->w_cc * pc;
  }
  __device__ BsdfSample d15_sample(f3 wo, float u, float v, float w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BsdfSample out;
    out.pdf = 0.0f;
    out.f = mk3(0.0f, 0.0f, 0.0f);
    out.wi = out.f;
    const f3 lwo = normalize(to_local(s, wo));
    if (fabsf(lwo.z) < kEps) return out;
    if (lwo.z < 0.0f && m->transmission == 0.0f) return out;
    // the lobe choice (disney.cpp:471-488): the second test is not inside the
    // first one's else, so a diffuse draw is always replaced by one of the
    // other three lobes (the cosine sample has no side effects and is skipped)
    float sel = u;
    if (!(sel < m->w_diff15)) sel -= m->w_diff15;
    f3 lwi = mk3(0.0f, 0.0f, 0.0f);
    if (sel < m->w_trans) {
      const f3 lwh = sample_aniso_gtr2(m->trans_ax, m->trans_ay, v, w);
      if (lwh.z > 0.0f && (lwo.z > 0.0f) == (dot(lwh, lwo) > 0.0f)) {
        // refract_dir (src/utility/reflection.hpp:43-51) about the facet normal
        const float eta = lwo.z > 0.0f ? 1.0f / m->ior : m->ior;
        const f3 owh = dot(lwh, lwo) > 0.0f ? lwh : -lwh;
        const float ci = fabsf(lwo.z);
        const float st2 = eta * eta * fmaxf(0.0f, 1.0f - ci * ci);
        if (st2 < 1.0f) {
          const f3 t = normalize(scale(owh, eta * ci - sqrtf(1.0f - st2)) - scale(lwo, eta));
          if (!(t.z * lwo.z > 0.0f || ((t.z > 0.0f) != (dot(lwh, t) > 0.0f)))) lwi = t;
        }
      }
    } else if (sel -= m->w_trans, sel < m->w_spec15) {
      const f3 lwh = normalize(sample_vndf_a(lwo, v, w, m->ax, m->ay));
      if (lwh.z > 0.0f) {
        const f3 t = normalize(scale(lwh, 2.0f * dot(lwo, lwh)) - lwo);
        if (t.z > 0.0f) lwi = t;
      }
    } else {
      const f3 lwh = sample_gtr1(m->cc_rough, v, w);
      if (lwh.z > 0.0f) {
        const f3 t = normalize(scale(lwh, 2.0f * dot(lwo, lwh)) - lwo);
        if (t.z > 0.0f) lwi = t;
      }
    }
    if (lwi.x == 0.0f && lwi.y == 0.0f && lwi.z == 0.0f) return out;
    out.wi = to_global(s, lwi);
    out.f = d15_eval(out.wi, wo);
    out.pdf = d15_pdf(out.wi, wo);
    return out;
  }

  __device__ __forceinline__ f3 eval(f3 wi, f3 wo) const {
    if (m->kind == MAT_GLASS) return mk3(0.0f, 0.0f, 0.0f);
    if (m->kind == MAT_METAL) return metal_eval(wi, wo);
    if (m->kind == MAT_DISNEY15) return d15_eval(wi, wo);
    return m->kind == MAT_PHONG ? phong_eval_agg(wi, wo) : disney_eval(wi, wo);
  }
  __device__ __forceinline__ float pdf(f3 wi, f3 wo) const {
    if (m->kind == MAT_GLASS) return 0.0f;
    if (m->kind == MAT_METAL) return metal_pdf(wi, wo);
    if (m->kind == MAT_DISNEY15) return d15_pdf(wi, wo);
    return m->kind == MAT_PHONG ? phong_pdf_agg(wi, wo) : disney_pdf(wi, wo);
  }
  __device__ __forceinline__ BsdfSample sample(f3 wo, float u, float v, float w) const {
    if (m->kind == MAT_GLASS) return glass_sample(wo, u);
    if (m->kind == MAT_METAL) return metal_sample(wo, u, v, w);
    if (m->kind == MAT_DISNEY15) return d15_sample(wo, u, v, w);
    return m->kind == MAT_PHONG ? phong_sample_agg(wo, u, v, w) : disney_sample(wo, u, v, w);
  }
};

// ------------------------------------------------------------------ lights
// DiffuseLight::pdf (src/light/diffuse_light.cpp:31-42)
__device__ __forceinline__ float light_pdf_at(float area, f3 ref, f3 pos, f3 n) {
  if (dot(n, ref - pos) <= 0.0f) return 0.0f;
  const f3 p2ref = ref - pos;
  const float dist2 = len2f(p2ref);
  const float abscos = fabsf(cos_x(n, p2ref));
  area *= abscos;
  return dist2 / area;
}

// ------------------------------------------------------- environment light
// The vector part of a Transform (src/utility/transform.hpp:89-95), 3 x 3 row-major.
__device__ __forceinline__ f3 rot3(const float* m, f3 v) {
  return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
             m[6] * v.x + m[7] * v.y + m[8] * v.z);
}
__device__ __forceinline__ float clamp_pm1(float z) { return z < -1.0f ? -1.0f : (1.0f < z ? 1.0f : z); }
__device__ __forceinline__ float clamp01(float x) { return x < 0.0f ? 0.0f : (1.0f < x ? 1.0f : x); }

// IBL::light_emit (src/light/environment_light.cpp:172-182): the map at
// (phi / 2pi, theta / pi) of the direction in light space.
__device__ __forceinline__ f3 env_emit(const DEnv& e, f3 d) {
  f3 dir = normalize(d);
  dir = normalize(rot3(e.to_light, dir));
  const float phi = local_phi(dir);
  const float theta = acosf(clamp_pm1(dir.z));
  const float u = clamp01(phi / (2.0f * kPi)), v = clamp01(theta * kInvPi);
  return e.texels8 ? env_tex_eval8(e.texels8, e.w, e.h, u, v) : env_tex_eval(e.texels, e.w, e.h, u, v);
}

// Distribution1D::sample_continuous (src/utility/distribution.hpp:37-55):
// the cell is the last index whose cdf is not above u (std::lower_bound over
// the reversed cdf), the offset inside it linear.
__device__ __forceinline__ float dist1d_sample(const float* __restrict__ func, const float* __restrict__ cdf, int n,
                                               float func_int, float u, float& pdf, int& off) {
  int lo = 0, hi = n + 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (cdf[mid] > u) hi = mid;
    else lo = mid + 1;
  }
  int offset = lo - 1;
  offset = offset < 0 ? 0 : (offset > n - 1 ? n - 1 : offset);
  off = offset;
  float du = u - cdf[offset];
  if (cdf[offset + 1] - cdf[offset] > 0.0f) du /= cdf[offset + 1] - cdf[offset];
  pdf = func_int > 0.0f ? func[offset] / func_int : 0.0f;
  return ((float)offset + du) / (float)n;
}

// IBL::sample_li (src/light/environment_light.cpp:88-116) through
// Distribution2D::sample_continuous (src/utility/distribution.hpp:95-102).
// Returns false where the reference returns an empty sample.
__device__ __forceinline__ bool env_sample(const DEnv& e, f3 ref, float u, float v, f3& radiance, float& pdf,
                                           f3& pos) {
  float p0, p1;
  int iv, iu;
  const float d1 = dist1d_sample(e.cond_int, e.marg_cdf, e.nv, e.marg_int, v, p1, iv);
  const float d0 = dist1d_sample(e.cond_func + (size_t)iv * e.nu, e.cond_cdf + (size_t)iv * (e.nu + 1), e.nu,
                                 e.cond_int[iv], u, p0, iu);
  const float map_pdf = p0 * p1;
  if (map_pdf == 0.0f) return false;
  const float theta = d1 * kPi, phi = d0 * 2.0f * kPi;
  const float cos_theta = cosf(theta), sin_theta = sinf(theta);
  const float sin_phi = sinf(phi), cos_phi = cosf(phi);
  f3 wi = mk3(sin_theta * cos_phi, sin_theta * sin_phi, cos_theta);
  wi = normalize(rot3(e.to_world, wi));
  if (sin_theta == 0.0f) return false;
  pdf = map_pdf / (2.0f * kPi * kPi * sin_theta);
  radiance = env_emit(e, wi);
  pos = ref + scale(wi, 2.0f * e.radius);
  return true;
}

// The density env_sample draws direction d with, per solid angle:
// func(u, v) / marginal integral / (2 pi^2 sin theta). (IBL::pdf below is
// the reference's weight, which multiplies by the integral instead; the
// guided estimator's MIS weights need the density itself.)
__device__ __forceinline__ float env_sample_density(const DEnv& e, f3 d) {
  const f3 wi = normalize(rot3(e.to_light, d));
  const float theta = acosf(clamp_pm1(wi.z));
  const float sin_theta = sinf(theta);
  if (!(sin_theta > 0.0f) || !(e.marg_int > 0.0f)) return 0.0f;
  const float phi = local_phi(wi);
  int iu = (int)(phi * kInv2Pi * (float)e.nu), iv = (int)(theta * kInvPi * (float)e.nv);
  iu = iu < 0 ? 0 : (iu > e.nu - 1 ? e.nu - 1 : iu);
  iv = iv < 0 ? 0 : (iv > e.nv - 1 ? e.nv - 1 : iv);
  return e.cond_func[(size_t)iv * e.nu + iu] / e.marg_int / (2.0f * kPi * kPi * sin_theta);
}

// IBL::pdf (src/light/environment_light.cpp:184-191) with Distribution2D::pdf
// (src/utility/distribution.hpp:103-107), which multiplies the conditional's
// function by the marginal integral.
__device__ __forceinline__ float env_pdf(const DEnv& e, f3 d) {
  const f3 wi = rot3(e.to_light, d);
  const float theta = acosf(clamp_pm1(wi.z));
  float phi = atan2f(wi.y, wi.x);
  phi = phi < 0.0f ? phi + 2.0f * kPi : phi;
  const float sin_theta = sinf(theta);
  if (sin_theta == 0.0f) return 0.0f;
  int iu = (int)(phi * kInv2Pi * (float)e.nu), iv = (int)(theta * kInvPi * (float)e.nv);
  iu = iu < 0 ? 0 : (iu > e.nu - 1 ? e.nu - 1 : iu);
  iv = iv < 0 ? 0 : (iv > e.nv - 1 ? e.nv - 1 : iv);
  return e.cond_func[(size_t)iv * e.nu + iu] * e.marg_int / (2.0f * kPi * kPi * sin_theta);
}

// ------------------------------------------------------------------ camera
struct Cam {
  float m[16];  // camera_to_world
  float film_w, film_h, focal, lens_radius;
};
// ThinLensCamera::generate_ray (src/camera/thin_lens_camera.cpp:40-59)
__device__ __forceinline__ void camera_ray(const Cam& c, float fx, float fy, float lu, float lv, f3& o, f3& d) {
  const f3 film = mk3((0.5f - fx) * c.film_w, (0.5f - fy) * c.film_h, c.focal);
  float dx, dy;
  concentric_disk(lu, lv, dx, dy);
  const f3 lens = mk3(c.lens_radius * dx, c.lens_radius * dy, 0.0f);
  o = xform_point(c.m, lens);
  d = xform_vec(c.m, normalize(film - lens));
}

// GaussianFilter::eval term (src/filter/gaussian_filter.cpp:20-30)
__device__ __forceinline__ float gaussian(float alpha, float d, float expv) {
  return smax(0.0f, expf(-alpha * d * d) - expv);
}

}  // namespace trg
