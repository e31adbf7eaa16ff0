// tracer_oracle.cpp -- CPU restatement of Tracer's unidirectional path-tracing
// hot path. TEST INFRASTRUCTURE ONLY: the tests check the GPU path's results
// against it, and it is the "port" CPU baseline. Nothing in the product links
// or calls it.
//
// Parity is pinned: tests/test_oracle_vs_reference.py compares every entry
// point here with the reference's own sources compiled by oracle/Makefile
// (target `ref`), and tests/golden/ holds fixtures made by that build.
//
// Every function restates one reference function; the citation is
// file:line relative to the reference project root. The arithmetic follows
// the reference operation by operation, including its float/double mixing:
//  * length_squared() sums in float and widens to double; length() is a
//    double sqrt; operator/ multiplies by a double reciprocal and rounds to
//    float (src/utility/geometry.hpp:429-445);
//  * cross() is evaluated in double and rounded (src/utility/geometry.hpp:584-589);
//  * the slab test scales tMax by the double constant 1 + 1e-7
//    (src/utility/geometry.hpp:848-859).
// Build with -ffp-contract=off (oracle/Makefile) so no multiply-add fuses.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

#include "tracer_gpu.h"

namespace orc {

typedef float real;
// common.hpp:47-73
const real kEps = real(3e-4);
const real kPi = real(3.141592653589793238462643383);
const real kInvPi = 1 / kPi;
const real kInv2Pi = 1 / (2 * kPi);
const real kPiOver2 = kPi / 2;
const real kPiOver4 = kPi / 4;
const real kRealMax = std::numeric_limits<real>::max();
const real kRealLowest = std::numeric_limits<real>::lowest();

// ---------------------------------------------------------------- vectors
struct V3 {
  real x = 0, y = 0, z = 0;
  V3() {}
  V3(real a, real b, real c) : x(a), y(b), z(c) {}
  explicit V3(real v) : x(v), y(v), z(v) {}
  real operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
// Vector3<T>::operator*(U s) with U = float: s * x in float (geometry.hpp:418-421).
inline V3 mulf(V3 v, real s) { return V3(s * v.x, s * v.y, s * v.z); }
inline bool all_zero(V3 v) { return !v.x && !v.y && !v.z; }  // geometry.hpp:411-413

// geometry.hpp:444 length_squared(): float sum, returned as double.
inline real len2f(V3 v) { return v.x * v.x + v.y * v.y + v.z * v.z; }
inline double length(V3 v) { return std::sqrt((double)len2f(v)); }
// geometry.hpp:429-433 operator/(U f): double reciprocal, double product, float result.
inline V3 divd(V3 v, double f) {
  double inv = (double)1 / f;
  return V3((real)(v.x * inv), (real)(v.y * inv), (real)(v.z * inv));
}
// geometry.hpp:570-572
inline V3 normalize(V3 v) { return divd(v, length(v)); }
// geometry.hpp:584-590
inline V3 cross(V3 a, V3 b) {
  double ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
  return V3((real)((ay * bz) - (az * by)), (real)((az * bx) - (ax * bz)), (real)((ax * by) - (ay * bx)));
}
// geometry.hpp:866-884
inline real dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// geometry.hpp:943-949
inline real cosv(V3 a, V3 b) { return dot(a, b) / (length(a) * length(b)); }
inline real abs_cos(V3 a, V3 b) { return std::abs(cosv(a, b)); }
// geometry.hpp:887-894
inline void coordinate(V3 v1, V3& v2, V3& v3) {
  if (std::abs(v1.x) > std::abs(v1.y))
    v2 = divd(V3(-v1.z, 0, v1.x), std::sqrt(v1.x * v1.x + v1.z * v1.z));
  else
    v2 = divd(V3(0, v1.z, -v1.y), std::sqrt(v1.y * v1.y + v1.z * v1.z));
  v3 = cross(v1, v2);
}
// geometry.hpp:912-932
inline real local_phi(V3 w) {
  if (!w.y && !w.x) return 0;
  real r = std::atan2(w.y, w.x);
  return r < 0 ? (r + 2 * kPi) : r;
}
inline real local_tan_theta(V3 w) {
  const real t = 1 - w.z * w.z;
  if (t <= 0) return 0;
  return std::sqrt(t) / w.z;
}
inline real local_cos_to_sin(real c) { return std::sqrt(std::max<real>(0, 1 - c * c)); }

// Spectrum (core/spectrum.hpp:13-161) as three floats.
struct Sp {
  real r = 0, g = 0, b = 0;
  Sp() {}
  Sp(real a, real b_, real c) : r(a), g(b_), b(c) {}
  explicit Sp(real v) : r(v), g(v), b(v) {}
  bool black() const { return r == 0 && g == 0 && b == 0; }
  bool finite() const { return std::isfinite(r) && std::isfinite(g) && std::isfinite(b); }
  bool valid() const { return r >= 0 && g >= 0 && b >= 0 && finite(); }
  real lum() const { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }
};
inline Sp operator+(Sp a, Sp b) { return Sp(a.r + b.r, a.g + b.g, a.b + b.b); }
inline Sp operator*(Sp a, Sp b) { return Sp(a.r * b.r, a.g * b.g, a.b * b.b); }
inline Sp operator*(Sp a, real s) { return Sp(a.r * s, a.g * s, a.b * s); }
inline Sp operator/(Sp a, real s) { return Sp(a.r / s, a.g / s, a.b / s); }
inline Sp operator+(Sp a, real s) { return Sp(a.r + s, a.g + s, a.b + s); }
inline void operator+=(Sp& a, Sp b) { a = a + b; }
inline Sp operator-(Sp a, Sp b) { return Sp(a.r - b.r, a.g - b.g, a.b - b.b); }
// geometry.hpp:989-993 mix() with a Spectrum pair and a float factor
inline Sp mix(Sp l, Sp r, real f) { return l * (1 - f) + r * f; }
inline real mixf(real l, real r, real f) { return (1 - f) * l + f * r; }

// --------------------------------------------------------- Coord frames
// utility/coordinate.hpp:15-116
struct Coord {
  V3 x{1, 0, 0}, y{0, 1, 0}, z{0, 0, 1};
  Coord() {}
  Coord(V3 a, V3 b, V3 c) : x(normalize(a)), y(normalize(b)), z(normalize(c)) {}
  static Coord from_z(V3 zz) {
    V3 nz = normalize(zz), ny;
    if (std::abs(nz.x) > std::abs(nz.y))
      ny = normalize(V3(-nz.z, 0, nz.x));
    else
      ny = normalize(V3(0, nz.z, -nz.y));
    return Coord(cross(ny, nz), ny, nz);
  }
  V3 to_local(V3 v) const { return V3(dot(x, v), dot(y, v), dot(z, v)); }
  V3 to_global(V3 v) const { return mulf(x, v.x) + mulf(y, v.y) + mulf(z, v.z); }
  bool pos_hemi(V3 v) const { return dot(v, z) > 0; }
};
// coordinate.hpp:43-52
inline real normal_correct_factor(const Coord& g, const Coord& s, V3 wi) {
  real dem = std::abs(cosv(g.z, wi));
  return dem < kEps ? 1 : std::abs(cosv(s.z, wi)) / dem;
}
// coordinate.hpp:54-68
inline void compute_ss_ts(V3 AB, V3 AC, real abx, real aby, real acx, real acy, V3 n, V3& ss, V3& ts) {
  const real m00 = abx, m01 = aby, m10 = acx, m11 = acy;
  const real det = m00 * m11 - m01 * m10;
  if (det) {
    const real inv_det = 1 / det;
    ss = mulf(AB, m11 * inv_det) - mulf(AC, m01 * inv_det);
    ts = mulf(AB, m10 * inv_det) - mulf(AC, m00 * inv_det);
  } else {
    coordinate(n, ss, ts);
  }
}

// --------------------------------------------------------------- sampler
// pcg32 = setseq XSH-RR 64/32 with the default stream, output of the previous
// state (dep/pcg_random.hpp), as used by SimpleUniformSampler
// (core/sampler.hpp:30-41). Seeding: state = bump(seed + inc).
struct Pcg32 {
  static constexpr uint64_t kMul = 6364136223846793005ULL;
  static constexpr uint64_t kInc = 1442695040888963407ULL;
  uint64_t s;
  explicit Pcg32(uint64_t seed) { s = (seed + kInc) * kMul + kInc; }
  uint32_t next() {
    uint64_t old = s;
    s = old * kMul + kInc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
};
// std::uniform_real_distribution<float>(0,1) over a 32-bit engine in
// libstdc++: one draw, float(x) / 2^32, clamped below 1.
struct Sampler {
  Pcg32 rng;
  explicit Sampler(int seed) : rng((uint64_t)(int64_t)seed) {}
  real u() {
    real v = (real)rng.next() / 4294967296.0f;
    if (v >= 1) v = std::nextafter(1.0f, 0.0f);
    return v;
  }
};

// --------------------------------------------------------------- sampling
// core/sampling.cpp:8-22
inline void concentric_disk(real u, real v, real& ox, real& oy) {
  real x = u * 2 - 1, y = v * 2 - 1;
  if (x == 0 && y == 0) { ox = 0; oy = 0; return; }
  real theta, r;
  if (std::abs(x) > std::abs(y)) {
    r = x;
    theta = kPiOver4 * (y / x);
  } else {
    r = y;
    theta = kPiOver2 - kPiOver4 * (x / y);
  }
  ox = r * std::cos(theta);
  oy = r * std::sin(theta);
}
// core/sampling.cpp:24-28
inline V3 cosine_hemisphere(real u, real v) {
  real dx, dy;
  concentric_disk(u, v, dx, dy);
  real z = std::sqrt(std::max<real>(0, 1 - dx * dx - dy * dy));
  return V3(dx, dy, z);
}
inline real cosine_pdf(real c) { return c * kInvPi; }  // sampling.hpp:228
// sampling.hpp:230-233
inline real power_heuristic(real fp, real gp) {
  real f = 1 * fp, g = 1 * gp;
  return (f * f) / (f * f + g * g);
}

// ------------------------------------------------------------------ scene
struct Tri {
  V3 A, B, C;       // world positions
  V3 nA, nB, nC;    // normalised vertex normals
  real uA[2], uB[2], uC[2];
};
struct Sphere {
  real radius, world_radius;
  real m[16], inv[16];  // local_to_world and inverse, row-major
  bool linear_identity;
};
struct Mat {
  int kind;
  // Phong::shading derived values (material/phong.cpp:29-70)
  Sp diffuse_coef;   // albedo / PI_r of the DiffuseBXDF
  Sp specular;       // normalised ks
  real ns, w_diffuse, w_specular;
  Sp albedo;         // diffuse + specular (AggregateBSDF albedo)
  // Disney12 parameters (material/disney_brdf.cpp:278-302)
  Sp base;
  real subsurface, metallic, specular_s, specular_tint, roughness, anisotropic, sheen, sheen_tint,
      clearcoat, clearcoat_gloss;
  // Glass::shading (material/glass.cpp:117-140): reflect colour, sqrt of the
  // transmit colour, index of refraction
  Sp kr, kt_sqrt;
  real ior;
  // Metal::shading (material/metal.cpp:33-56): the painted conductor Fresnel
  // as constructed there. create_metal(color, eta, k, ...) hands its
  // arguments to Metal(color, k, eta, ...), so Metal's k is the caller's eta
  // and its eta the caller's k; shading then builds
  // PaintedConductorFresnelPoint(color, 1, eta, k), whose parameters are
  // (eta_outside, eta_inside, k, paint). Net: eta_outside = color,
  // eta_inside = 1, conductor k = the caller's k, paint = the caller's eta.
  // GGX alphas (bxdf/microfacet_refl_bxdf.cpp:6-11); base holds the colour.
  Sp f_eta2, f_etak2, f_paint;
  real ax_m, ay_m;
  // DisneyBSDF's constructor (material/disney.cpp:341-392), with base,
  // metallic, roughness, specular_tint, anisotropic, sheen, sheen_tint and
  // clearcoat above: tint colour, specular scale, transmission, IOR, the
  // alphas, clearcoat roughness and the four sampling weights
  Sp c_tint, spec_scale;
  real transmission, ior15, ax15, ay15, trans_ax, trans_ay, cc_rough, w_diff, w_trans, w_spec, w_cc;
  // Phong maps (0: the constants; k: the scene's textures[k - 1]) and the constants
  int tex_ka = 0, tex_kd = 0, tex_ks = 0, tex_ns = 0;
  Sp kd_c, ks_c;
  real ns_c = 1;
  // another kind with image maps (tr_material.tex_param): set up again at each hit
  bool maps = false;
};
struct Prim {
  int kind;  // 0 triangle, 1 sphere
  int shape;
  int material;
  Sp emission;
  bool light;
};

// Point transform (utility/transform.hpp:70-81)
inline V3 xform_point(const real* m, V3 p) {
  real x = p.x, y = p.y, z = p.z;
  real xp = m[0] * x + m[1] * y + m[2] * z + m[3];
  real yp = m[4] * x + m[5] * y + m[6] * z + m[7];
  real zp = m[8] * x + m[9] * y + m[10] * z + m[11];
  real wp = m[12] * x + m[13] * y + m[14] * z + m[15];
  if (wp == 1) return V3(xp, yp, zp);
  double inv = (double)1 / wp;  // Point3::operator/ (geometry.hpp:289-293)
  return V3((real)(inv * xp), (real)(inv * yp), (real)(inv * zp));
}
// Vector transform (utility/transform.hpp:89-95)
inline V3 xform_vec(const real* m, V3 v) {
  real x = v.x, y = v.y, z = v.z;
  return V3(m[0] * x + m[1] * y + m[2] * z, m[4] * x + m[5] * y + m[6] * z, m[8] * x + m[9] * y + m[10] * z);
}
// Normal transform with the inverse, transposed (utility/transform.hpp:82-88)
inline V3 xform_normal(const real* inv, V3 n) {
  real x = n.x, y = n.y, z = n.z;
  return V3(inv[0] * x + inv[4] * y + inv[8] * z, inv[1] * x + inv[5] * y + inv[9] * z,
            inv[2] * x + inv[6] * y + inv[10] * z);
}

struct Bounds {
  V3 lo{kRealMax, kRealMax, kRealMax}, hi{kRealLowest, kRealLowest, kRealLowest};
};
inline real smin(real a, real b) { return (b < a) ? b : a; }  // std::min
inline real smax(real a, real b) { return (a < b) ? b : a; }  // std::max
inline V3 vmin(V3 a, V3 b) { return V3(smin(a.x, b.x), smin(a.y, b.y), smin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return V3(smax(a.x, b.x), smax(a.y, b.y), smax(a.z, b.z)); }
inline Bounds unite(const Bounds& b, V3 p) { Bounds r; r.lo = vmin(b.lo, p); r.hi = vmax(b.hi, p); return r; }
inline Bounds unite(const Bounds& a, const Bounds& b) { Bounds r; r.lo = vmin(a.lo, b.lo); r.hi = vmax(a.hi, b.hi); return r; }
inline real surface_area(const Bounds& b) {
  V3 d = b.hi - b.lo;
  return 2 * (d.x * d.y + d.x * d.z + d.y * d.z);
}
inline int max_extent(const Bounds& b) {
  V3 d = b.hi - b.lo;
  if (d.x > d.y && d.x > d.z) return 0;
  if (d.y > d.z) return 1;
  return 2;
}

struct Node {  // LinearBVHNode (accelerator/bvh.cpp:51-64)
  Bounds b;
  int32_t offset;
  uint16_t count;
  uint8_t axis;
};

struct Camera {
  real m[16];  // camera_to_world.m
  real focal_distance, lens_radius, film_w, film_h;
};

// ------------------------------------------------------ environment light
// Distribution1D (utility/distribution.hpp:12-79): piecewise-constant density
// over [0, 1) with n cells.
struct Dist1D {
  std::vector<real> func, cdf;
  real func_int = 0;
  Dist1D() = default;
  Dist1D(const real* f, int n) : func(f, f + n), cdf(n + 1, 0) {
    for (int i = 0; i < n; i++) cdf[i + 1] = cdf[i] + func[i] / n;
    func_int = cdf[n];
    if (!func_int) {
      for (int i = 1; i < n + 1; i++) cdf[i] = real(i) / n;
    } else {
      for (int i = 1; i < n + 1; i++) cdf[i] /= func_int;
    }
  }
  int count() const { return (int)func.size(); }
  // std::lower_bound over the reversed cdf with std::greater: the last index
  // i whose cdf[i] is not above u (cdf is non-decreasing)
  int last_not_above(real u) const {
    int lo = 0, hi = (int)cdf.size();  // answer + 1 lies in [lo, hi]
    while (lo < hi) {
      const int mid = (lo + hi) / 2;
      if (cdf[mid] > u) hi = mid;
      else lo = mid + 1;
    }
    return lo - 1;
  }
  real sample_continuous(real u, real* pdf, int* off = nullptr) const {
    int offset = std::clamp<int>(last_not_above(u), 0, (int)cdf.size() - 2);
    if (off) *off = offset;
    real du = u - cdf[offset];
    if (offset + 1 < (int)cdf.size() && cdf[offset + 1] - cdf[offset] > 0) du /= cdf[offset + 1] - cdf[offset];
    if (pdf) *pdf = (func_int > 0) ? func[offset] / func_int : 0;
    return (offset + du) / count();
  }
};
// Distribution2D (utility/distribution.hpp:81-111); its pdf multiplies by
// the marginal integral, as the reference does.
struct Dist2D {
  std::vector<Dist1D> cond;
  Dist1D marg;
  void build(const real* data, int nu, int nv) {
    cond.clear();
    for (int v = 0; v < nv; v++) cond.emplace_back(&data[v * nu], nu);
    std::vector<real> mf;
    for (int v = 0; v < nv; v++) mf.push_back(cond[v].func_int);
    marg = Dist1D(mf.data(), nv);
  }
  void sample_continuous(real u, real v, float* pdf, real& d0, real& d1) const {
    float pdfs[2];
    int iv;
    d1 = marg.sample_continuous(v, &pdfs[1], &iv);
    d0 = cond[iv].sample_continuous(u, &pdfs[0]);
    *pdf = pdfs[0] * pdfs[1];
  }
  real pdf(real u, real v) const {
    const int nu = cond[0].count(), nv = marg.count();
    const int iu = std::clamp<int>((int)(u * nu), 0, nu - 1);
    const int iv = std::clamp<int>((int)(v * nv), 0, nv - 1);
    return cond[iv].func[iu] * marg.func_int;
  }
};
// IBL over an HDRTexture2D (light/environment_light.cpp:14-193,
// texture/hdr_texture.cpp:9-37, core/texture.hpp:57-95)
// HDRTexture2D / ImageTexture2D behind Texture2D::evaluate
struct Tex {
  int w = 0, h = 0;
  std::vector<real> tex;      // 3 per texel, texel (x, y) at 3 * (x + y * w)
  std::vector<uint8_t> tex8;  // an 8-bit map (ImageTexture2D) instead, same layout
  Sp texel(int x, int y) const {
    const real* t = &tex[3 * ((size_t)x + (size_t)y * w)];
    return Sp(t[0], t[1], t[2]);
  }
  // Point3f * double (geometry.hpp:268-271): double product rounded to float
  static Sp scaled(Sp c, double f) { return Sp((real)(f * c.r), (real)(f * c.g), (real)(f * c.b)); }
  // Texture2D::evaluate with the repeat wrap, LinearSampler::Sample2D (utility/sampler.hpp:16-29)
  // Point3<uint8_t>: each product with a double truncates to a byte, sums are bytes
  struct B3 {
    uint8_t x, y, z;
  };
  B3 texel8(int x, int y) const {
    const uint8_t* t = &tex8[3 * ((size_t)x + (size_t)y * w)];
    return B3{t[0], t[1], t[2]};
  }
  static B3 scaled8(B3 c, double f) { return B3{(uint8_t)(f * c.x), (uint8_t)(f * c.y), (uint8_t)(f * c.z)}; }
  static B3 add8(B3 a, B3 b) { return B3{(uint8_t)(a.x + b.x), (uint8_t)(a.y + b.y), (uint8_t)(a.z + b.z)}; }
  Sp eval(real u_in, real v_in) const {
    const real uw = std::clamp<real>(u_in - std::floor(u_in), 0, 1);
    const real vw = std::clamp<real>(v_in - std::floor(v_in), 0, 1);
    double u = std::clamp((double)uw, 0.0, 1.0) * (w - 1);
    double v = std::clamp((double)vw, 0.0, 1.0) * (h - 1);
    const int u0 = std::clamp(static_cast<int>(u), 0, w - 1), u1 = std::clamp(u0 + 1, 0, w - 1);
    const int v0 = std::clamp(static_cast<int>(v), 0, h - 1), v1 = std::clamp(v0 + 1, 0, h - 1);
    const double du = u - u0, dv = v - v0;
    if (!tex8.empty()) {
      // ImageTexture2D::evaluate_impl (texture/image_texture2d.cpp:26-30): bytes / 255
      const B3 c = add8(scaled8(add8(scaled8(texel8(u0, v0), 1.0 - du), scaled8(texel8(u1, v0), du)), 1.0 - dv),
                        scaled8(add8(scaled8(texel8(u0, v1), 1.0 - du), scaled8(texel8(u1, v1), du)), dv));
      return Sp(c.x / real(255.0), c.y / real(255.0), c.z / real(255.0));
    }
    return scaled(scaled(texel(u0, v0), 1.0 - du) + scaled(texel(u1, v0), du), 1.0 - dv) +
           scaled(scaled(texel(u0, v1), 1.0 - du) + scaled(texel(u1, v1), du), dv);
  }
};
struct Env : Tex {
  real to_light[16], to_world[16];
  Dist2D dist;
  V3 center;
  real radius = 1;
  // the IBL constructor's sampling density: luminance times solid angle per
  // cell of a grid of at most 360 x 180 (environment_light.cpp:39-81)
  void build_distribution() {
    const int nw = std::min(w, 360), nh = std::min(h, 180);
    std::vector<real> img((size_t)nw * nh, 0);
    for (int y = 0; y < nh; ++y) {
      const real y0 = static_cast<real>(y) / nh, y1 = static_cast<real>(y + 1) / nh;
      const real sy0 = y0 * h, sy1 = y1 * h;
      const int yb = std::max<int>(0, (int)(std::floor(sy0) - 1));
      const int ye = std::min<int>(h - 1, (int)(std::floor(sy1) + 1));
      for (int x = 0; x < nw; ++x) {
        const real x0 = static_cast<real>(x) / nw, x1 = static_cast<real>(x + 1) / nw;
        const real sx0 = x0 * w, sx1 = x1 * w;
        const int xb = std::max<int>(0, (int)(std::floor(sx0) - 1));
        const int xe = std::min<int>(w - 1, (int)(std::floor(sx1) + 1));
        real lum = 0;
        for (int sy = yb; sy <= ye; ++sy)
          for (int sx = xb; sx <= xe; ++sx) {
            const real su = static_cast<real>(sx + 0.5) / w;
            const real sv = static_cast<real>(sy + 0.5) / h;
            lum += eval(su, sv).lum();
          }
        const real area = (real)std::abs(2 * kPi * (x1 - x0) * kPi * (y1 - y0) * std::sin(kPi * 0.5 * (y1 + y0)));
        img[(size_t)x + (size_t)y * nw] = lum * area;
      }
    }
    dist.build(img.data(), nw, nh);
  }
  // IBL::light_emit (environment_light.cpp:172-182)
  Sp emit(V3 d) const {
    V3 dir = normalize(d);
    dir = normalize(xform_vec(to_light, dir));
    const real phi = local_phi(dir);
    const real theta = std::acos(std::clamp<real>(dir.z, -1, 1));
    const real u = std::clamp<real>(phi / (2 * kPi), 0, 1);
    const real v = std::clamp<real>(theta * kInvPi, 0, 1);
    return eval(u, v);
  }
  // IBL::pdf (environment_light.cpp:184-191)
  real pdf(V3 d) const {
    const V3 wi = xform_vec(to_light, d);
    const real theta = std::acos(std::clamp<real>(wi.z, -1, 1));
    real phi = std::atan2(wi.y, wi.x);
    phi = (phi < 0) ? (phi + 2 * kPi) : phi;
    const real sin_theta = std::sin(theta);
    if (sin_theta == 0) return 0;
    return dist.pdf(phi * kInv2Pi, theta * kInvPi) / (2 * kPi * kPi * sin_theta);
  }
};

struct Scene {
  std::vector<Tri> tris;
  std::vector<Sphere> spheres;
  std::vector<Mat> mats;
  std::vector<tr_material> msrc;  // the materials' factory arguments and maps
  std::vector<Prim> prims;
  std::vector<int> lights;       // primitive ids in scene.lights order
  std::unique_ptr<Env> env;      // environment light (after the area lights in scene.lights)
  std::vector<Tex> textures;     // image textures of the materials
  std::vector<Node> nodes;
  std::vector<int> order;        // leaf slot -> primitive id
  int max_leaf = 1;
  Camera cam;
  real filter_radius = 0.5f, filter_alpha = 2, filter_exp = 0;
};

// ------------------------------------------------------------ shapes: bounds
// shape/triangle.cpp:47-52
inline Bounds tri_bound(const Tri& t) {
  Bounds b;
  b.lo = V3(smin(t.A.x, t.B.x), smin(t.A.y, t.B.y), smin(t.A.z, t.B.z));
  b.hi = V3(smax(t.A.x, t.B.x), smax(t.A.y, t.B.y), smax(t.A.z, t.B.z));
  return unite(b, t.C);
}
// shape/sphere.cpp:121-127
inline Bounds sphere_bound(const Sphere& s) {
  V3 o = xform_point(s.m, V3(0, 0, 0));
  Bounds b;
  b.lo = o - V3(s.world_radius + kEps);
  b.hi = o + V3(s.world_radius + kEps);
  return b;
}
inline Bounds prim_bound(const Scene& sc, int p) {
  const Prim& pr = sc.prims[p];
  return pr.kind == 0 ? tri_bound(sc.tris[pr.shape]) : sphere_bound(sc.spheres[pr.shape]);
}

// ------------------------------------------------------------- BVH build
// accelerator/bvh.cpp:15-23
struct PrimInfo {
  size_t index;
  Bounds b;
  V3 c;
};
struct BuildNode {
  Bounds b;
  int left = -1, right = -1, axis = 0;
  size_t first = 0, count = 0;
};

struct Builder {
  Scene& sc;
  std::vector<PrimInfo>& info;
  std::vector<BuildNode> nodes;
  std::vector<int> ordered;
  int max_leaf;

  // accelerator/bvh.cpp:191-288
  int build(size_t start, size_t end) {
    int id = (int)nodes.size();
    nodes.emplace_back();
    Bounds bounds;
    for (size_t i = start; i < end; ++i) bounds = unite(bounds, info[i].b);
    size_t n = end - start;
    auto leaf = [&]() {
      size_t first = ordered.size();
      for (size_t i = start; i < end; ++i) ordered.push_back((int)info[i].index);
      nodes[id].first = first;
      nodes[id].count = n;
      nodes[id].b = bounds;
    };
    if (n == 1) {
      leaf();
      return id;
    }
    Bounds cb;
    for (size_t i = start; i < end; ++i) cb = unite(cb, info[i].c);
    int mid = (int)((start + end) >> 1);
    int dim = max_extent(cb);
    if (cb.hi[dim] == cb.lo[dim]) {
      leaf();
      return id;
    }
    // Bounds3::offset(p)[dim] (geometry.hpp:745-751), then the bucket index
    auto bucket_of = [&](V3 c) {
      real o = c[dim] - cb.lo[dim];
      if (cb.hi[dim] > cb.lo[dim]) o /= cb.hi[dim] - cb.lo[dim];
      int b = (int)(12 * o);
      if (b == 12) b = 11;
      return b;
    };
    if (n <= 2) {
      std::nth_element(&info[start], &info[mid], &info[end - 1] + 1,
                       [dim](const PrimInfo& a, const PrimInfo& b) { return a.c[dim] < b.c[dim]; });
    } else {
      size_t cnt[12] = {0};
      Bounds bb[12];
      for (size_t i = start; i < end; ++i) {
        int b = bucket_of(info[i].c);
        cnt[b]++;
        bb[b] = unite(bb[b], info[i].b);
      }
      real cost[11];
      for (int i = 0; i < 11; ++i) {
        Bounds lb, rb;
        int lc = 0, rc = 0;
        for (int j = 0; j <= i; ++j) { lb = unite(lb, bb[j]); lc += (int)cnt[j]; }
        for (int j = i + 1; j < 12; ++j) { rb = unite(rb, bb[j]); rc += (int)cnt[j]; }
        cost[i] = 1 + (lc * surface_area(lb) + rc * surface_area(rb)) / surface_area(bounds);
      }
      long minb = std::min_element(cost, cost + 11) - cost;
      if (n > (size_t)max_leaf) {
        PrimInfo* pm = std::partition(&info[start], &info[end - 1] + 1,
                                      [&](const PrimInfo& pi) { return bucket_of(pi.c) <= minb; });
        mid = (int)(pm - &info[0]);
      } else {
        leaf();
        return id;
      }
    }
    // The reference passes both recursive calls as arguments of
    // init_interior (bvh.cpp:283-284); GCC evaluates them right to left, so
    // the right subtree claims its leaf slots first.
    int r = build((size_t)mid, end);
    int l = build(start, (size_t)mid);
    nodes[id].left = l;
    nodes[id].right = r;
    nodes[id].axis = dim;
    nodes[id].b = unite(nodes[l].b, nodes[r].b);
    nodes[id].count = 0;
    return id;
  }
  // accelerator/bvh.cpp:290-306
  int flatten(int b, std::vector<Node>& out) {
    int off = (int)out.size();
    out.emplace_back();
    out[off].b = nodes[b].b;
    if (nodes[b].count > 0) {
      out[off].count = (uint16_t)nodes[b].count;
      out[off].offset = (int32_t)nodes[b].first;
      out[off].axis = 0;
    } else {
      out[off].axis = (uint8_t)nodes[b].axis;
      out[off].count = 0;
      flatten(nodes[b].left, out);
      out[off].offset = flatten(nodes[b].right, out);
    }
    return off;
  }
};

// accelerator/bvh.cpp:78-105
void build_bvh(Scene& sc) {
  sc.nodes.clear();
  sc.order.clear();
  size_t n = sc.prims.size();
  if (!n) return;
  std::vector<PrimInfo> info(n);
  for (size_t i = 0; i < n; ++i) {
    info[i].index = i;
    info[i].b = prim_bound(sc, (int)i);
    // 0.5 * low + 0.5 * high: double scale, float point, float add
    V3 a((real)(0.5 * info[i].b.lo.x), (real)(0.5 * info[i].b.lo.y), (real)(0.5 * info[i].b.lo.z));
    V3 b((real)(0.5 * info[i].b.hi.x), (real)(0.5 * info[i].b.hi.y), (real)(0.5 * info[i].b.hi.z));
    info[i].c = a + b;
  }
  Builder bl{sc, info, {}, {}, sc.max_leaf};
  bl.nodes.reserve(2 * n);
  int root = bl.build(0, n);
  bl.flatten(root, sc.nodes);
  sc.order = bl.ordered;
}

// ------------------------------------------------------------- traversal
struct Ray {
  V3 o, d;
  real t_min = 0, t_max = kRealMax;
};
// Ray(o, d, t_min, t_max) normalises d (geometry.hpp:791-793)
inline Ray make_ray(V3 o, V3 d, real tmin = 0, real tmax = kRealMax) {
  Ray r;
  r.o = o;
  r.d = normalize(d);
  r.t_min = tmin;
  r.t_max = tmax;
  return r;
}

// geometry.hpp:837-864
inline bool box_hit(const Bounds& b, const Ray& r, V3 inv, const int neg[3]) {
  const V3* bs[2] = {&b.lo, &b.hi};
  real tMin = ((*bs[neg[0]]).x - r.o.x) * inv.x;
  real tMax = ((*bs[1 - neg[0]]).x - r.o.x) * inv.x;
  real tyMin = ((*bs[neg[1]]).y - r.o.y) * inv.y;
  real tyMax = ((*bs[1 - neg[1]]).y - r.o.y) * inv.y;
  tMax *= 1 + 0.0000001;
  tyMax *= 1 + 0.0000001;
  if (tMin > tyMax || tyMin > tMax) return false;
  if (tyMin > tMin) tMin = tyMin;
  if (tyMax < tMax) tMax = tyMax;
  real tzMin = ((*bs[neg[2]]).z - r.o.z) * inv.z;
  real tzMax = ((*bs[1 - neg[2]]).z - r.o.z) * inv.z;
  tzMax *= 1 + 0.0000001;
  if (tMin > tzMax || tzMin > tMax) return false;
  if (tzMin > tMin) tMin = tzMin;
  if (tzMax < tMax) tMax = tzMax;
  return (tMin < r.t_max) && (tMax > 0);
}

// Möller-Trumbore core shared by Triangle::intersect and ::intersect_p
// (shape/triangle.cpp:117-143, 145-174). Returns true and t on acceptance.
inline bool tri_test(const Tri& T, const Ray& r, real& t, real& alpha, real& beta) {
  const V3 AB = T.B - T.A;
  const V3 AC = T.C - T.A;
  V3 s1 = cross(r.d, AC);
  real div = dot(s1, AB);
  if (!div) return false;
  real inv_div = 1 / div;
  const V3 AO = r.o - T.A;
  alpha = dot(AO, s1) * inv_div;
  if (alpha < 0) return false;
  V3 s2 = cross(AO, AB);
  beta = dot(r.d, s2) * inv_div;
  if (beta < 0 || alpha + beta > 1) return false;
  t = dot(AC, s2) * inv_div;
  if (t < r.t_min || t > r.t_max) return false;
  return true;
}

// TransformedShape::to_local (shape/transformed_shape.hpp:17-21)
inline Ray sphere_local_ray(const Sphere& s, const Ray& wr) {
  return make_ray(xform_point(s.inv, wr.o), xform_vec(s.inv, wr.d), wr.t_min, wr.t_max);
}
// sphere::get_abc (shape/sphere.cpp:7-13); C widens to double as written
inline void sphere_abc(real radius_square, const Ray& r, real& A, real& B, real& C) {
  A = (real)(double)len2f(r.d);
  B = 2 * dot(r.d, r.o);
  C = (real)((double)len2f(r.o) - radius_square);
}
// sphere::intersect_p (shape/sphere.cpp:28-47), local ray
inline bool sphere_test_p(const Ray& r, real radius, real& t) {
  real A, B, C;
  sphere_abc(radius * radius, r, A, B, C);
  real delta = B * B - 4 * A * C;
  if (delta < 0) return false;
  delta = std::sqrt(delta);
  real inv2A = real(0.5) / A;
  real t0 = (-B - delta) * inv2A;
  real t1 = (-B + delta) * inv2A;
  if (r.t_max < t0 || t1 < r.t_min) return false;
  bool not_t0 = t0 < r.t_min;
  if (not_t0 && t1 > r.t_max) return false;
  t = not_t0 ? t1 : t0;
  return true;
}
// sphere::intersect (shape/sphere.cpp:15-27)
inline bool sphere_test_any(const Ray& r, real radius) {
  real A, B, C;
  sphere_abc(radius * radius, r, A, B, C);
  real delta = B * B - 4 * A * C;
  if (delta < 0) return false;
  delta = std::sqrt(delta);
  const real inv2A = real(0.5) / A;
  const real t0 = (-B - delta) * inv2A;
  const real t1 = (-B + delta) * inv2A;
  return (r.t_min <= t0 && t0 <= r.t_max) || (r.t_min <= t1 && t1 <= r.t_max);
}

struct Counters {
  uint64_t nodes = 0, prims = 0;
};

// BVHAccel::intersect_p (accelerator/bvh.cpp:149-185) with the
// GeometricPrimitive t_max update (shape/geometry.cpp:49-60). Returns the
// primitive id or -1; ray.t_max holds what the reference leaves there.
// Sphere::intersect_p never writes its hit_t argument (shape/sphere.cpp:98-119),
// so after a sphere hit GeometricPrimitive stores the initial 0.0 into
// ray.t_max: the first sphere hit in traversal order ends the search for
// everything not at t <= 0. *hit_t receives the accepted primitive's own
// parameter (the local sphere t for spheres), which the hit record uses.
int closest_hit(const Scene& sc, Ray& ray, Counters* cnt, real* hit_t = nullptr) {
  if (sc.nodes.empty()) return -1;
  V3 inv((real)(1.0 / ray.d.x), (real)(1.0 / ray.d.y), (real)(1.0 / ray.d.z));
  int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
  int hit = -1;
  std::vector<size_t> stack;
  stack.reserve(64);
  stack.push_back(0);
  while (!stack.empty()) {
    size_t ni = stack.back();
    stack.pop_back();
    const Node& nd = sc.nodes[ni];
    if (cnt) cnt->nodes++;
    if (!box_hit(nd.b, ray, inv, neg)) continue;
    if (nd.count > 0) {
      for (int i = 0; i < nd.count; ++i) {
        int p = sc.order[nd.offset + i];
        const Prim& pr = sc.prims[p];
        if (cnt) cnt->prims++;
        real t;
        if (pr.kind == 0) {
          real a, b;
          if (tri_test(sc.tris[pr.shape], ray, t, a, b)) { ray.t_max = t; hit = p; if (hit_t) *hit_t = t; }
        } else {
          const Sphere& s = sc.spheres[pr.shape];
          Ray lr = sphere_local_ray(s, ray);
          if (sphere_test_p(lr, s.radius, t)) { ray.t_max = 0; hit = p; if (hit_t) *hit_t = t; }
        }
      }
    } else {
      if (neg[nd.axis]) {
        stack.push_back(ni + 1);
        stack.push_back((size_t)nd.offset);
      } else {
        stack.push_back((size_t)nd.offset);
        stack.push_back(ni + 1);
      }
    }
  }
  return hit;
}

// BVHAccel::intersect (accelerator/bvh.cpp:112-147)
bool any_hit(const Scene& sc, const Ray& ray, Counters* cnt) {
  if (sc.nodes.empty()) return false;
  V3 inv((real)(1.0 / ray.d.x), (real)(1.0 / ray.d.y), (real)(1.0 / ray.d.z));
  int neg[3] = {inv.x < 0, inv.y < 0, inv.z < 0};
  std::vector<size_t> stack;
  stack.reserve(64);
  stack.push_back(0);
  while (!stack.empty()) {
    size_t ni = stack.back();
    stack.pop_back();
    const Node& nd = sc.nodes[ni];
    if (cnt) cnt->nodes++;
    if (!box_hit(nd.b, ray, inv, neg)) continue;
    if (nd.count > 0) {
      for (int i = 0; i < nd.count; ++i) {
        int p = sc.order[nd.offset + i];
        const Prim& pr = sc.prims[p];
        if (cnt) cnt->prims++;
        if (pr.kind == 0) {
          real t, a, b;
          if (tri_test(sc.tris[pr.shape], ray, t, a, b)) return true;
        } else {
          const Sphere& s = sc.spheres[pr.shape];
          if (sphere_test_any(sphere_local_ray(s, ray), s.radius)) return true;
        }
      }
    } else {
      if (neg[nd.axis]) {
        stack.push_back(ni + 1);
        stack.push_back((size_t)nd.offset);
      } else {
        stack.push_back((size_t)nd.offset);
        stack.push_back(ni + 1);
      }
    }
  }
  return false;
}

// ------------------------------------------------------ surface interaction
struct Isect {  // SurfaceIntersection (core/intersection.hpp:13-43)
  V3 pos;
  real uv[2];
  Coord g, s;
  V3 wo;
  int prim = -1;
  // SurfacePoint::eps_offset (intersection.hpp:19-23)
  V3 eps_offset(V3 dir) const {
    if (dot(g.z, dir) > 0) return pos + mulf(g.z, kEps);
    return pos - mulf(g.z, kEps);
  }
};

// Triangle::intersect_p hit record (shape/triangle.cpp:175-213)
void tri_attributes(const Tri& T, const Ray& r, real t, real alpha, real beta, Isect& is) {
  const V3 AB = T.B - T.A, AC = T.C - T.A;
  is.uv[0] = T.uA[0] + alpha * (T.uB[0] - T.uA[0]) + beta * (T.uC[0] - T.uA[0]);
  is.uv[1] = T.uA[1] + alpha * (T.uB[1] - T.uA[1]) + beta * (T.uC[1] - T.uA[1]);
  is.wo = -r.d;
  is.pos = r.o + mulf(r.d, t);
  V3 gn = normalize(cross(AB, AC));
  V3 dpdu, dpdv;
  compute_ss_ts(AB, AC, T.uB[0] - T.uA[0], T.uB[1] - T.uA[1], T.uC[0] - T.uA[0], T.uC[1] - T.uA[1], gn,
                dpdu, dpdv);
  dpdu = cross(dpdv, gn);
  dpdv = cross(gn, dpdu);
  is.g = Coord(dpdu, dpdv, gn);
  V3 sn = T.nA + mulf(T.nB - T.nA, alpha) + mulf(T.nC - T.nA, beta);
  V3 dndu, dndv;
  compute_ss_ts(T.nB - T.nA, T.nC - T.nA, T.uB[0] - T.uA[0], T.uB[1] - T.uA[1], T.uC[0] - T.uA[0],
                T.uC[1] - T.uA[1], sn, dndu, dndv);
  if ((real)(double)len2f(dndu) < kEps || (real)(double)len2f(dndv) < kEps) coordinate(sn, dndu, dndv);
  dndu = cross(dndv, sn);
  dndv = cross(sn, dndu);
  is.s = Coord(dndu, dndv, sn);
}

// sphere::local_geometry_uv_and_coord (shape/sphere.cpp:48-78)
void sphere_local_geometry(V3 p, real radius, real uv[2], Coord& c) {
  real phi = (!p.x && !p.y) ? real(0) : std::atan2(p.y, p.x);
  if (phi < 0) phi += 2 * kPi;
  const real sin_theta = std::clamp<real>(p.z / radius, -1, 1);
  const real theta = std::asin(sin_theta);
  uv[0] = real(0.5) * kInvPi * phi;
  uv[1] = kInvPi * theta + real(0.5);
  V3 ex, ey, ez = normalize(p);
  if (std::abs(ez.z - 1) < kEps) {
    ex = V3(1, 0, 0); ey = V3(0, 1, 0); ez = V3(0, 0, 1);
  } else if (std::abs(ez.z + 1) < kEps) {
    ex = V3(0, 1, 0); ey = V3(1, 0, 0); ez = V3(0, 0, -1);
  } else {
    ex = cross(V3(0, 0, 1), ez);
    ey = cross(ez, ex);
  }
  c = Coord(ex, ey, ez);
}

// Sphere::intersect_p hit record + to_world (shape/sphere.cpp:98-119,
// transformed_shape.hpp:31-44)
void sphere_attributes(const Sphere& s, const Ray& wr, real t, Isect& is) {
  Ray lr = sphere_local_ray(s, wr);
  V3 pos = lr.o + mulf(lr.d, t);
  Coord c;
  sphere_local_geometry(pos, s.radius, is.uv, c);
  is.pos = xform_point(s.m, pos);
  is.g = Coord(xform_vec(s.m, c.x), xform_vec(s.m, c.y), xform_vec(s.m, c.z));
  is.s = is.g;
  is.wo = xform_vec(s.m, -lr.d);
}

// Scene::intersect_p with the hit record of the closest primitive
bool intersect_p(const Scene& sc, Ray& ray, Isect& is, Counters* cnt) {
  Ray r0 = ray;
  real hit_t = 0;
  int p = closest_hit(sc, ray, cnt, &hit_t);
  if (p < 0) return false;
  const Prim& pr = sc.prims[p];
  is.prim = p;
  if (pr.kind == 0) {
    // re-run the accepted test on the original ray to recover alpha, beta
    // (t_max only gates acceptance; alpha, beta, t do not depend on it)
    Ray rr = r0;
    rr.t_max = hit_t;
    real t, a, b;
    tri_test(sc.tris[pr.shape], rr, t, a, b);
    tri_attributes(sc.tris[pr.shape], r0, t, a, b, is);
  } else {
    sphere_attributes(sc.spheres[pr.shape], r0, hit_t, is);
  }
  return true;
}

// --------------------------------------------------------------- BSDFs
struct BSDFSample {
  V3 wi;
  Sp f;
  real pdf = 0;
  bool delta = false;
  bool valid() const { return pdf > 0 && !f.black(); }  // core/bsdf.hpp:21-23
};

// ConductorFresnelPoint::evaluate (material/utility/fresnel_point.hpp:47-66), per channel
inline real conductor_fresnel(real eta_2, real eta_k_2, real cos_theta_i) {
  if (cos_theta_i <= 0) return 0;
  const real cos2 = cos_theta_i * cos_theta_i;
  const real sin2 = std::max(real(0), 1 - cos2);
  const real t0 = eta_2 - eta_k_2 - sin2;
  const real a2b2 = std::sqrt(t0 * t0 + real(4) * eta_2 * eta_k_2);
  const real t1 = a2b2 + cos2;
  const real a = std::sqrt(real(0.5) * (a2b2 + t0));
  const real t2 = 2 * cos_theta_i * a;
  const real rs = (t1 - t2) / (t1 + t2);
  const real t3 = cos2 * a2b2 + sin2 * sin2;
  const real t4 = t2 * sin2;
  const real rp = rs * (t3 - t4) / (t3 + t4);
  return real(0.5) * (rp + rs);
}

// dielectric_fresnel (utility/reflection.hpp:16-40)
inline real dielectric_fresnel(real eta_i, real eta_o, real cos_theta_i) {
  if (cos_theta_i < 0) {
    std::swap(eta_i, eta_o);
    cos_theta_i = -cos_theta_i;
  }
  const real sin_theta_i = std::sqrt(std::max(real(0), 1 - cos_theta_i * cos_theta_i));
  const real sin_theta_t = eta_o / eta_i * sin_theta_i;
  if (sin_theta_t >= 1) return 1;
  const real cos_theta_t = std::sqrt(std::max(real(0), 1 - sin_theta_t * sin_theta_t));
  const real para = (eta_i * cos_theta_i - eta_o * cos_theta_t) / (eta_i * cos_theta_i + eta_o * cos_theta_t);
  const real perp = (eta_o * cos_theta_i - eta_i * cos_theta_t) / (eta_o * cos_theta_i + eta_i * cos_theta_t);
  return real(0.5) * (para * para + perp * perp);
}
// refract_dir (utility/reflection.hpp:43-51); false: total internal reflection
inline bool refract_dir(V3 lwo, V3 n, real eta, V3& out) {
  const real cos_theta_i = std::abs(lwo.z);
  const real sin_theta_i_2 = std::max(real(0), 1 - cos_theta_i * cos_theta_i);
  const real sin_theta_t_2 = eta * eta * sin_theta_i_2;
  if (sin_theta_t_2 >= 1) return false;
  const real cos_theta_t = std::sqrt(1 - sin_theta_t_2);
  out = mulf(n, eta * cos_theta_i - cos_theta_t) - mulf(lwo, eta);
  return true;
}

// microfacet helpers (material/utility/microfacet.cpp:7-134, microfacet.hpp:10-14)
inline real sqr(real x) { return x * x; }
inline real one_minus_5(real x) { real t = 1 - x; real t2 = t * t; return t2 * t2 * t; }
inline real compute_alpha(real s, real c, real ax, real ay) { return sqr(c / ax) + sqr(s / ay); }
inline real anisotropic_gtr2(real sp, real cp, real st, real ct, real ax, real ay) {
  const real A = compute_alpha(sp, cp, ax, ay);
  const real RD = sqr(st) * A + sqr(ct);
  return 1 / (kPi * ax * ay * sqr(RD));
}
inline real gtr1(real st, real ct, real alpha) {
  if (alpha >= 1) return kInvPi;
  const real U = sqr(alpha) - 1;
  const real LD = 2 * kPi * std::log(alpha);
  const real RD = sqr(alpha * ct) + sqr(st);
  return U / (LD * RD);
}
inline real smith_anisotropic_gtr2(real cos_phi, real sin_phi, real ax, real ay, real tan_theta) {
  const real t = sqr(ax * cos_phi) + sqr(ay * sin_phi);
  const real sq = 1 + t * sqr(tan_theta);
  const real lambda = -real(0.5) + real(0.5) * std::sqrt(sq);
  return 1 / (1 + lambda);
}
inline real smith_gtr2(real tan_theta, real alpha) {
  if (!tan_theta) return 1;
  const real root = alpha * tan_theta;
  return 2 / (1 + std::sqrt(1 + root * root));
}
inline V3 sample_anisotropic_gtr2(real ax, real ay, real u, real v) {
  real sp = ay * std::sin(2 * kPi * u);
  real cp = ax * std::cos(2 * kPi * u);
  const real nor = 1 / std::sqrt(sqr(sp) + sqr(cp));
  sp *= nor;
  cp *= nor;
  const real A = compute_alpha(sp, cp, ax, ay);
  const real ct = std::sqrt(A * (1 - v) / ((1 - A) * v + A));
  const real st = std::sqrt(std::max<real>(0, 1 - sqr(ct)));
  return normalize(V3(st * cp, st * sp, ct));
}
inline V3 sample_gtr1(real alpha, real u, real v) {
  const real phi = 2 * kPi * u;
  const real ct = std::sqrt((std::pow(alpha, 2 - 2 * v) - 1) / (sqr(alpha) - 1));
  const real st = local_cos_to_sin(ct);
  return normalize(V3(st * std::cos(phi), st * std::sin(phi), ct));
}
// utility/reflection.hpp:12-14
inline V3 reflect(V3 w, V3 n) { return mulf(n, 2 * dot(w, n)) - w; }

// Phong specular lobe (material/bxdf/phong_specular_bxdf.cpp:10-71)
inline real powcos_pdf(real e, real c) { return (e + 1) * kInv2Pi * std::pow(c, e); }
inline Sp phong_eval(const Mat& m, V3 lwi, V3 lwo) {
  if (lwi.z <= 0 || lwo.z <= 0) return Sp();
  const V3 ideal = reflect(lwo, V3(0, 0, 1));
  const real c = dot(ideal, lwi) / (length(lwi) * length(ideal));
  if (c <= 0) return Sp();
  return m.specular * powcos_pdf(m.ns, c);
}
inline real phong_pdf(const Mat& m, V3 lwi, V3 lwo) {
  if (lwi.z <= 0 || lwo.z <= 0) return 0;
  const V3 ideal = reflect(lwo, V3(0, 0, 1));
  const real c = cosv(lwi, ideal);
  if (c <= 0) return 0;
  return powcos_pdf(m.ns, c);
}
inline bool phong_sample(const Mat& m, V3 lwo, real u, real v, V3& lwi_out, Sp& f, real& pdf) {
  if (lwo.z <= 0) return false;
  const V3 ideal = normalize(reflect(lwo, V3(0, 0, 1)));
  const real ct = std::pow(u, 1 / (m.ns + 1));
  const real st = std::sqrt(std::max<real>(0, 1 - ct * ct));
  const real phi = 2 * kPi * v;
  V3 local = normalize(V3(st * std::cos(phi), st * std::sin(phi), ct));
  V3 lwi = normalize(Coord::from_z(ideal).to_global(local));
  if (lwi.z <= 0) return false;
  pdf = powcos_pdf(m.ns, local.z);
  f = phong_eval(m, lwi, lwo);
  lwi_out = lwi;
  return pdf > 0;
}
// DiffuseBXDF (material/bxdf/diffuse_bxdf.cpp:14-38)
inline Sp diffuse_eval(const Mat& m, V3 lwi, V3 lwo) {
  if (lwi.z <= 0 || lwo.z <= 0) return Sp();
  return m.diffuse_coef;
}
inline real diffuse_pdf(V3 lwi, V3 lwo) {
  if (lwi.z <= 0 || lwo.z <= 0) return 0;
  return cosine_pdf(lwi.z);
}

struct BSDF {
  const Mat* m;
  Coord g, s;

  // LocalBSDF black-fringe helpers (core/bsdf.hpp:55-91)
  bool fringe(V3 w) const { return g.pos_hemi(w) ^ s.pos_hemi(w); }
  bool fringe(V3 a, V3 b) const { return fringe(a) | fringe(b); }
  Sp albedo() const { return m->kind == TR_MAT_PHONG ? m->albedo : m->base; }
  Sp eval_fringe(V3 wi, V3 wo) const {
    if (g.pos_hemi(wi) & g.pos_hemi(wo)) return albedo() * kInvPi;
    return Sp(0);
  }
  BSDFSample sample_fringe(V3 wo, real u, real v) const {
    BSDFSample r;
    if (!g.pos_hemi(wo)) return r;
    V3 lwi = cosine_hemisphere(u, v);
    real pdf = cosine_pdf(lwi.z);
    if (pdf < kEps) return r;
    V3 wi = normalize(g.to_global(lwi));
    real nc = normal_correct_factor(g, s, wi);
    r.wi = wi;
    r.f = albedo() * kInvPi * nc;
    r.pdf = pdf;
    return r;
  }
  real pdf_fringe(V3 wi, V3 wo) const {
    if (g.pos_hemi(wi) ^ g.pos_hemi(wo)) return 0;
    return cosine_pdf(normalize(g.to_local(wi)).z);
  }

  // ---- AggregateBSDF<2> of Phong (material/aggregate_bsdf.hpp:36-118)
  Sp phong_agg_eval(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return eval_fringe(wi, wo);
    V3 lwi = normalize(s.to_local(wi)), lwo = normalize(s.to_local(wo));
    if (!lwi.z || !lwo.z) return Sp();
    Sp r;
    r += diffuse_eval(*m, lwi, lwo);
    r += phong_eval(*m, lwi, lwo);
    return r;
  }
  BSDFSample phong_agg_sample(V3 wo, real u, real v, real w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BSDFSample out;
    const V3 lwo = normalize(s.to_local(wo));
    if (!lwo.z) return out;
    real ws = 0;
    ws += m->w_diffuse;
    ws += m->w_specular;
    real sel = (u - real(0.001)) * ws;
    int which = -1;
    real weight = 0;
    const real wts[2] = {m->w_diffuse, m->w_specular};
    for (int i = 0; i < 2; ++i) {
      if (sel <= wts[i]) { which = i; weight = wts[i]; break; }
      sel -= wts[i];
    }
    if (which < 0) return out;
    V3 lwi;
    Sp f;
    real pdf;
    if (which == 0) {
      if (lwo.z <= 0) return out;
      lwi = cosine_hemisphere(v, w);
      pdf = cosine_pdf(lwi.z);
      if (pdf < real(0.001)) return out;
      f = m->diffuse_coef;
    } else {
      if (!phong_sample(*m, lwo, v, w, lwi, f, pdf)) return out;
    }
    lwi = normalize(lwi);
    pdf *= weight;
    if (which != 0) { f += diffuse_eval(*m, lwi, lwo); pdf += diffuse_pdf(lwi, lwo) * wts[0]; }
    if (which != 1) { f += phong_eval(*m, lwi, lwo); pdf += phong_pdf(*m, lwi, lwo) * wts[1]; }
    V3 wi = s.to_global(lwi);
    real nc = normal_correct_factor(g, s, wi);
    out.wi = wi;
    out.f = f * nc;
    out.pdf = pdf;
    return out;
  }
  real phong_agg_pdf(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return pdf_fringe(wi, wo);
    V3 lwi = normalize(s.to_local(wi)), lwo = normalize(s.to_local(wo));
    if (!lwi.z || !lwo.z) return 0;
    real ws = 0, pdf = 0;
    ws += m->w_diffuse;
    pdf += m->w_diffuse * diffuse_pdf(lwi, lwo);
    ws += m->w_specular;
    pdf += m->w_specular * phong_pdf(*m, lwi, lwo);
    return ws > 0 ? pdf / ws : 0;
  }

  // ---- DisneyBRDF (material/disney_brdf.cpp:56-227)
  void disney_alphas(real& ax, real& ay) const {
    real aspect = (real)std::sqrt(1 - m->anisotropic * 0.9);
    ax = std::max<real>(0.001, m->roughness * m->roughness / aspect);
    ay = std::max<real>(0.001, m->roughness * m->roughness * aspect);
  }
  Sp disney_eval(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return eval_fringe(wi, wo);
    const V3 lwi = normalize(s.to_local(wi));
    const V3 lwo = normalize(s.to_local(wo));
    if (lwi.z < kEps || lwo.z < kEps) return Sp();
    const real NdotL = lwi.z, NdotV = lwo.z;
    const V3 H = normalize(lwi + lwo);
    const real LdotH = dot(lwi, H);
    const Sp& bc = m->base;
    real lum = bc.lum();
    Sp Ctint = lum > 0 ? bc / lum : Sp(1);
    Sp Cspec0 = mix(mix(Sp(1), Ctint, m->specular_tint) * (m->specular_s * 0.08f), bc, m->metallic);
    Sp Csheen = mix(Sp(1), Ctint, m->sheen_tint);
    Sp fd;
    real ax, ay;
    disney_alphas(ax, ay);
    real phi_h = local_phi(H);
    real sph = std::sin(phi_h), cph = std::cos(phi_h);
    real Ds = anisotropic_gtr2(sph, cph, local_cos_to_sin(H.z), H.z, ax, ay);
    real FH = one_minus_5(LdotH);
    Sp Fs = mix(Cspec0, Sp(1), FH);
    real phi_i = local_phi(lwi);
    real spi = std::sin(phi_i), cpi = std::cos(phi_i);
    real Gs = smith_anisotropic_gtr2(spi, cpi, ax, ay, local_tan_theta(lwi));
    real phi_o = local_phi(lwo);
    real spo = std::sin(phi_o), cpo = std::cos(phi_o);
    Gs *= smith_anisotropic_gtr2(spo, cpo, ax, ay, local_tan_theta(lwo));
    real Dr = gtr1(local_cos_to_sin(H.z), H.z, mixf(0.1f, 0.001f, m->clearcoat_gloss));
    real Fr = mixf(0.04f, 1.0f, FH);
    real Gr = smith_gtr2(local_tan_theta(lwi), 0.25f) * smith_gtr2(local_tan_theta(lwo), 0.25f);
    fd += ((Fs * Ds) * Gs + 0.25f * m->clearcoat * Gr * Fr * Dr) / (4 * NdotL * NdotV);
    if (m->metallic < 1) {
      real FL = one_minus_5(NdotL), FV = one_minus_5(NdotV);
      real Fd90 = (real)(0.5 + 2. * LdotH * LdotH * m->roughness);
      real Fd = mixf(1, Fd90, FL) * mixf(1, Fd90, FV);
      real Fss90 = LdotH * LdotH * m->roughness;
      real Fss = mixf(1, Fss90, FL) * mixf(1, Fss90, FV);
      real ss = (real)(1.25 * (Fss * (1.0 / (NdotL + NdotV) - 0.5) + 0.5));
      Sp Fsheen = Csheen * (FH * m->sheen);
      fd += ((bc * kInvPi) * mixf(Fd, ss, m->subsurface) + Fsheen) * (1 - m->metallic);
    }
    return fd * normal_correct_factor(g, s, wi);
  }
  real disney_pdf(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return pdf_fringe(wi, wo);
    real p_diffuse = std::min<real>(0.8, 1 - m->metallic);
    real p_specular = (real)(1.0 / (1.0 + 0.5 * m->clearcoat));
    real ax, ay;
    disney_alphas(ax, ay);
    const V3 lwi = normalize(s.to_local(wi));
    const V3 lwo = normalize(s.to_local(wo));
    if (lwi.z < kEps) return 0;
    const V3 H = normalize(lwi + lwo);
    real pdf_diffuse = cosine_pdf(lwi.z);
    real phi_h = local_phi(H);
    real sph = std::sin(phi_h), cph = std::cos(phi_h);
    real pdf_spec = anisotropic_gtr2(sph, cph, local_cos_to_sin(H.z), H.z, ax, ay) * H.z / (4 * dot(lwi, H));
    real pdf_cc = gtr1(sph, cph, m->clearcoat_gloss) * H.z / (4 * dot(lwi, H));
    real pdf = p_diffuse * pdf_diffuse + (1 - pdf_diffuse) * (p_specular * pdf_spec + (1 - p_specular) * pdf_cc);
    if (!std::isfinite(pdf)) return 0;
    return pdf;
  }
  BSDFSample disney_sample(V3 wo, real u, real v, real w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BSDFSample r;
    real p_diffuse = std::min<real>(0.8, 1 - m->metallic);
    real p_specular = (real)(1.0 / (1.0 + 0.5 * m->clearcoat) * (1 - p_diffuse));
    const V3 lwo = normalize(s.to_local(wo));
    V3 lwi;
    real sel = u;
    real ax, ay;
    disney_alphas(ax, ay);
    if (sel < p_diffuse) lwi = cosine_hemisphere(v, w);
    sel -= p_diffuse;
    if (sel < p_specular) {
      const V3 lwh = sample_anisotropic_gtr2(ax, ay, v, w);
      if (lwh.z > 0) {
        lwi = normalize(mulf(lwh, 2 * dot(lwo, lwh)) - lwo);
        if (lwi.z <= 0) lwi = V3();
      }
    } else {
      const V3 lwh = sample_gtr1(m->clearcoat_gloss, v, w);
      if (lwh.z > 0) {
        lwi = normalize(mulf(lwh, 2 * dot(lwo, lwh)) - lwo);
        if (lwi.z <= 0) lwi = V3();
      }
    }
    if (all_zero(lwi)) return r;
    r.wi = s.to_global(lwi);
    r.f = disney_eval(r.wi, wo);
    r.pdf = disney_pdf(r.wi, wo);
    return r;
  }

  // GlassBSDF::sample (material/glass.cpp:29-80), DielectricFresnelPoint(ior, 1),
  // TransportMode::Radiance; eval and pdf are 0 (a delta BSDF)
  BSDFSample glass_sample(V3 wo, real u) const {
    BSDFSample out;
    const V3 lwo = normalize(s.to_local(wo));
    const V3 nor = lwo.z > 0 ? V3(0, 0, 1) : V3(0, 0, -1);
    const real fr = dielectric_fresnel(m->ior, 1, lwo.z);
    if (u < fr) {
      const V3 lwi(-lwo.x, -lwo.y, lwo.z);
      const V3 wi = s.to_global(lwi);
      const real q = fr / std::abs(lwi.z);
      const Sp f(m->kr.r * q, m->kr.g * q, m->kr.b * q);
      out.wi = wi;
      out.f = f * normal_correct_factor(g, s, wi);
      out.pdf = fr;
      out.delta = true;
      return out;
    }
    const real eta_i = lwo.z > 0 ? real(1) : m->ior, eta_t = lwo.z > 0 ? m->ior : real(1);
    const real eta = eta_i / eta_t;
    V3 t;
    if (!refract_dir(lwo, nor, eta, t)) return out;
    const V3 lwi = normalize(t);
    const V3 wi = s.to_global(lwi);
    const real corr = eta * eta, az = std::abs(lwi.z);
    const Sp f(((corr * m->kt_sqrt.r) * (1 - fr)) / az, ((corr * m->kt_sqrt.g) * (1 - fr)) / az,
               ((corr * m->kt_sqrt.b) * (1 - fr)) / az);
    out.wi = wi;
    out.f = f * normal_correct_factor(g, s, wi);
    out.pdf = 1 - fr;
    out.delta = true;
    return out;
  }
  // ---- Metal: AggregateBSDF<1> (material/aggregate_bsdf.hpp:36-118) of one
  // GGXMicrofacetReflectionBXDF (bxdf/microfacet_refl_bxdf.cpp:13-78), weight 1
  void ggx(V3 lwi, V3 lwo, Sp* eval, real* pdf) const {
    const real cos_theta_i = lwi.z, cos_theta_o = lwo.z;
    const V3 lwh = normalize(lwi + lwo);
    const real cos_theta_d = dot(lwi, lwh);
    const real phi_h = local_phi(lwh);
    const real sin_phi_h = std::sin(phi_h), cos_phi_h = std::cos(phi_h);
    const real cos_theta_h = lwh.z;
    const real sin_theta_h = std::max<real>(0, std::sqrt(1 - cos_theta_h * cos_theta_h));
    const real D = anisotropic_gtr2(sin_phi_h, cos_phi_h, sin_theta_h, cos_theta_h, m->ax_m, m->ay_m);
    const real phi_i = local_phi(lwi), phi_o = local_phi(lwo);
    const real sin_phi_i = std::sin(phi_i), cos_phi_i = std::cos(phi_i);
    const real sin_phi_o = std::sin(phi_o), cos_phi_o = std::cos(phi_o);
    const real tan_theta_i = local_tan_theta(lwi), tan_theta_o = local_tan_theta(lwo);
    const real Gi = smith_anisotropic_gtr2(cos_phi_i, sin_phi_i, m->ax_m, m->ay_m, tan_theta_i);
    const real Go = smith_anisotropic_gtr2(cos_phi_o, sin_phi_o, m->ax_m, m->ay_m, tan_theta_o);
    if (eval) {
      const real G = Gi * Go;
      const real den = std::abs(4 * cos_theta_i * cos_theta_o);
      Sp F;
      F.r = m->f_paint.r * conductor_fresnel(m->f_eta2.r, m->f_etak2.r, cos_theta_d);
      F.g = m->f_paint.g * conductor_fresnel(m->f_eta2.g, m->f_etak2.g, cos_theta_d);
      F.b = m->f_paint.b * conductor_fresnel(m->f_eta2.b, m->f_etak2.b, cos_theta_d);
      *eval = Sp(F.r * D * G / den, F.g * D * G / den, F.b * D * G / den);
    }
    if (pdf) *pdf = Go * D / (4 * cos_theta_o);
  }
  // microfacet::sample_anisotropic_gtr2_with_visible_normal (utility/microfacet.cpp:58-80)
  V3 sample_vndf(V3 ve, real u, real v) const {
    const real ax = m->ax_m, ay = m->ay_m;
    const V3 vh = normalize(V3(ax * ve.x, ay * ve.y, ve.z));
    const real lensq = vh.x * vh.x + vh.y * vh.y;
    const V3 t1 = lensq > kEps ? divd(V3(-vh.y, vh.x, 0), std::sqrt(lensq)) : V3(1, 0, 0);
    const V3 t2 = cross(vh, t1);
    const real r = std::sqrt(u);
    const real phi = 2 * kPi * v;
    const real t_1 = r * std::cos(phi);
    const real _t_2 = r * std::sin(phi);
    const real sh = real(0.5) * (1 + vh.z);
    const real t_2 = (1 - sh) * std::sqrt(1 - t_1 * t_1) + sh * _t_2;
    const V3 nh = mulf(t1, t_1) + mulf(t2, t_2) + mulf(vh, std::sqrt(std::max(real(0), 1 - t_1 * t_1 - t_2 * t_2)));
    return normalize(V3(ax * nh.x, ay * nh.y, std::max(real(0), nh.z)));
  }
  Sp metal_eval(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return eval_fringe(wi, wo);
    const V3 lwi = normalize(s.to_local(wi)), lwo = normalize(s.to_local(wo));
    if (!lwi.z || !lwo.z) return Sp();
    Sp r;
    if (!(lwi.z <= 0 || lwo.z <= 0)) {
      Sp e;
      ggx(lwi, lwo, &e, nullptr);
      r += e;
    }
    return r;
  }
  real metal_pdf(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return pdf_fringe(wi, wo);
    const V3 lwi = normalize(s.to_local(wi)), lwo = normalize(s.to_local(wo));
    if (!lwi.z || !lwo.z) return 0;
    real weight_sum = 0, pdf = 0;
    weight_sum += 1;
    real p = 0;
    if (!(lwi.z <= 0 || lwo.z <= 0)) ggx(lwi, lwo, nullptr, &p);
    pdf += 1 * p;
    return weight_sum > 0 ? pdf / weight_sum : 0;
  }
  BSDFSample metal_sample(V3 wo, real u, real v, real w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BSDFSample out;
    const V3 lwo = normalize(s.to_local(wo));
    if (!lwo.z) return out;
    const real comp_sel = (u - real(0.001)) * 1;
    if (!(comp_sel <= 1)) return out;
    // GGXMicrofacetReflectionBXDF::sample with (v, w)
    if (lwo.z <= 0) return out;
    const V3 lwh = normalize(sample_vndf(lwo, v, w));
    if (lwh.z <= 0) return out;
    const V3 lwi0 = normalize(mulf(lwh, 2 * dot(lwo, lwh)) - lwo);
    if (lwi0.z <= 0) return out;
    Sp f;
    real pdf = 0;
    ggx(lwi0, lwo, &f, &pdf);
    if (!(pdf > 0)) return out;  // BXDFSampleResult::is_valid (material/bxdf/bxdf.hpp:17-19)
    const V3 lwi = normalize(lwi0);
    pdf *= 1;
    const V3 wi = s.to_global(lwi);
    out.wi = wi;
    out.f = f * normal_correct_factor(g, s, wi);
    out.pdf = pdf;
    return out;
  }

  // ---- DisneyBSDF, the 2015 model (material/disney.cpp:14-537), radiance transport
  static real gtr2_D(V3 lwh, real ax, real ay) {
    const real phi_h = local_phi(lwh);
    return anisotropic_gtr2(std::sin(phi_h), std::cos(phi_h), local_cos_to_sin(lwh.z), lwh.z, ax, ay);
  }
  static real smith_G(V3 lw, real ax, real ay) {
    const real phi = local_phi(lw);
    return smith_anisotropic_gtr2(std::cos(phi), std::sin(phi), ax, ay, local_tan_theta(lw));
  }
  static real schlick1(real R0, real c) { return R0 + (1 - R0) * one_minus_5(c); }
  Sp d15_f_transmission(V3 lwi, V3 lwo) const {
    const real cos_theta_i = lwi.z, cos_theta_o = lwo.z;
    const real eta = cos_theta_o > 0 ? m->ior15 : 1 / m->ior15;
    V3 lwh = normalize(lwo + mulf(lwi, eta));
    if (lwh.z < 0) lwh = -lwh;
    const real cos_theta_d = dot(lwo, lwh);
    const real F = dielectric_fresnel(m->ior15, 1, cos_theta_d);
    const real D = gtr2_D(lwh, m->trans_ax, m->trans_ay);
    const real G = smith_G(lwi, m->trans_ax, m->trans_ay) * smith_G(lwo, m->trans_ax, m->trans_ay);
    const real sdem = cos_theta_d + eta * dot(lwi, lwh);
    const real corr = 1 / eta;
    const Sp sqrtC(std::sqrt(m->base.r), std::sqrt(m->base.g), std::sqrt(m->base.b));
    const real val = (1 - F) * D * G * eta * eta * dot(lwi, lwh) * dot(lwo, lwh) * corr * corr /
                     (cos_theta_i * cos_theta_o * sdem * sdem);
    const real trans_factor = cos_theta_o > 0 ? m->transmission : 1;
    return sqrtC * ((1 - m->metallic) * trans_factor) * std::abs(val);
  }
  Sp d15_f_inner_reflection(V3 lwi, V3 lwo) const {
    const V3 lwh = -normalize(lwi + lwo);
    const real cos_theta_d = dot(lwo, lwh);
    const real F = dielectric_fresnel(m->ior15, 1, cos_theta_d);
    const real D = gtr2_D(lwh, m->trans_ax, m->trans_ay);
    const real G = smith_G(lwi, m->trans_ax, m->trans_ay) * smith_G(lwo, m->trans_ax, m->trans_ay);
    return m->base * m->transmission * std::abs(F * D * G / (4 * lwi.z * lwo.z));
  }
  Sp d15_f_diffuse(real ci, real co, real cd) const {
    const Sp f_lambert = m->base / kPi;
    const real FL = one_minus_5(ci), FV = one_minus_5(co);
    const real RR = 2 * m->roughness * cd * cd;
    const Sp retro = m->base / kPi * RR * (FL + FV + FL * FV * (RR - 1));
    return f_lambert * (1 - real(0.5) * FL) * (1 - real(0.5) * FV) + retro;
  }
  Sp d15_f_sheen(real cd) const {
    return mix(Sp(1), m->c_tint, m->sheen_tint) * (4 * m->sheen) * one_minus_5(cd);
  }
  Sp d15_f_specular(V3 lwi, V3 lwo) const {
    const V3 lwh = normalize(lwi + lwo);
    const real cd = dot(lwi, lwh);
    const Sp Cspec = mix(mix(Sp(1), m->c_tint, m->specular_tint), m->base, m->metallic);
    const Sp dielectric = Cspec * dielectric_fresnel(m->ior15, 1, cd);
    const Sp conductor = Cspec + (Sp(1) - Cspec) * one_minus_5(cd);
    const Sp F = mix(m->spec_scale * dielectric, conductor, m->metallic);
    const real D = gtr2_D(lwh, m->ax15, m->ay15);
    const real G = smith_G(lwi, m->ax15, m->ay15) * smith_G(lwo, m->ax15, m->ay15);
    return F * D * G / std::abs(4 * lwi.z * lwo.z);
  }
  real d15_pdf_transmission(V3 lwi, V3 lwo) const {
    const real eta = lwo.z > 0 ? m->ior15 : 1 / m->ior15;
    V3 lwh = normalize(lwo + mulf(lwi, eta));
    if (lwh.z < 0) lwh = -lwh;
    if (((lwo.z > 0) != (dot(lwh, lwo) > 0)) || ((lwi.z > 0) != (dot(lwh, lwi) > 0))) return 0;
    const real sdem = dot(lwo, lwh) + eta * dot(lwi, lwh);
    const real dwh_to_dwi = eta * eta * dot(lwi, lwh) / (sdem * sdem);
    const real D = gtr2_D(lwh, m->trans_ax, m->trans_ay);
    return std::abs(dot(lwi, lwh) * D * dwh_to_dwi);
  }
  real d15_pdf_inner_reflection(V3 lwi, V3 lwo) const {
    const V3 lwh = -normalize(lwi + lwo);
    const real D = gtr2_D(lwh, m->trans_ax, m->trans_ay);
    return std::abs(lwh.z * D / (4 * dot(lwi, lwh)));
  }
  void d15_pdf_spec_cc(V3 lwi, V3 lwo, real& ps, real& pc) const {
    const V3 lwh = normalize(lwi + lwo);
    const real cos_theta_h = lwh.z, sin_theta_h = local_cos_to_sin(cos_theta_h);
    const real cd = dot(lwi, lwh);
    const real cos_phi_o = std::cos(local_phi(lwo));
    const real sin_phi_o = local_cos_to_sin(cos_phi_o);
    const real spec_D = gtr2_D(lwh, m->ax15, m->ay15);
    ps = smith_anisotropic_gtr2(cos_phi_o, sin_phi_o, m->ax15, m->ay15, local_tan_theta(lwo)) * spec_D / (4 * lwo.z);
    pc = cos_theta_h * gtr1(sin_theta_h, cos_theta_h, m->cc_rough) / (4 * cd);
  }
  Sp d15_eval(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return eval_fringe(wi, wo);
    const V3 lwi = normalize(s.to_local(wi)), lwo = normalize(s.to_local(wo));
    if (std::abs(lwi.z) < kEps || std::abs(lwo.z) < kEps) return Sp();
    if (lwi.z * lwo.z < 0) {
      if (m->transmission == 0) return Sp();
      return d15_f_transmission(lwi, lwo) * normal_correct_factor(g, s, wi);
    }
    if (lwi.z < 0 && lwo.z < 0) {
      if (m->transmission == 0) return Sp();
      return d15_f_inner_reflection(lwi, lwo) * normal_correct_factor(g, s, wi);
    }
    const V3 lwh = normalize(lwi + lwo);
    const real cd = dot(lwi, lwh);
    Sp diffuse, sheen;
    if (m->metallic < 1) {
      diffuse = d15_f_diffuse(lwi.z, lwo.z, cd);
      if (m->sheen > 0) sheen = d15_f_sheen(cd);
    }
    const Sp specular = d15_f_specular(lwi, lwo);
    Sp clearcoat;
    if (m->clearcoat > 0) {
      const real ch = lwh.z, sh = local_cos_to_sin(ch);
      const real D = gtr1(sh, ch, m->cc_rough);
      const real F = schlick1(real(0.04), cd);
      const real G = smith_gtr2(local_tan_theta(lwi), real(0.25)) * smith_gtr2(local_tan_theta(lwo), real(0.25));
      clearcoat = Sp(m->clearcoat * D * F * G / std::abs(4 * lwi.z * lwo.z));
    }
    const Sp ret = (diffuse + sheen) * ((1 - m->metallic) * (1 - m->transmission)) + specular + clearcoat;
    return ret * normal_correct_factor(g, s, wi);
  }
  real d15_pdf(V3 wi, V3 wo) const {
    if (fringe(wi, wo)) return pdf_fringe(wi, wo);
    const V3 lwi = normalize(s.to_local(wi)), lwo = normalize(s.to_local(wo));
    if (std::abs(lwi.z) < kEps || std::abs(lwo.z) < kEps) return 0;
    if (lwo.z < 0) {
      if (m->transmission == 0) return 0;
      real macro_F = std::clamp<real>(dielectric_fresnel(m->ior15, 1, lwo.z), real(0.1), real(0.9));
      if (lwi.z > 0) return (1 - macro_F) * d15_pdf_transmission(lwi, lwo);
      return macro_F * d15_pdf_inner_reflection(lwi, lwo);
    }
    if (lwi.z < 0) return m->w_trans * d15_pdf_transmission(lwi, lwo);
    const real diffuse = cosine_pdf(lwi.z);
    real ps, pc;
    d15_pdf_spec_cc(lwi, lwo, ps, pc);
    return m->w_diff * diffuse + m->w_spec * ps + m->w_cc * pc;
  }
  BSDFSample d15_sample(V3 wo, real u, real v, real w) const {
    if (fringe(wo)) return sample_fringe(wo, u, v);
    BSDFSample out;
    const V3 lwo = normalize(s.to_local(wo));
    if (std::abs(lwo.z) < kEps) return out;
    if (lwo.z < 0 && m->transmission == 0) return out;
    // the lobe choice (disney.cpp:471-488): the second test is not inside the
    // first one's else, so a diffuse draw is always replaced by one of the
    // other three lobes (the cosine sample has no side effects and is skipped)
    real sel = u;
    V3 lwi(0, 0, 0);
    if (!(sel < m->w_diff)) sel -= m->w_diff;
    {
      if (sel < m->w_trans) {
        // sample_transmission (disney.cpp:286-306)
        const V3 lwh = sample_anisotropic_gtr2(m->trans_ax, m->trans_ay, v, w);
        if (lwh.z > 0 && (lwo.z > 0) == (dot(lwh, lwo) > 0)) {
          const real eta = lwo.z > 0 ? 1 / m->ior15 : m->ior15;
          const V3 owh = dot(lwh, lwo) > 0 ? lwh : -lwh;
          V3 t;
          if (refract_dir(lwo, owh, eta, t)) {
            const V3 tn = normalize(t);
            if (!(tn.z * lwo.z > 0 || ((tn.z > 0) != (dot(lwh, tn) > 0)))) lwi = tn;
          }
        }
      } else {
        sel -= m->w_trans;
        if (sel < m->w_spec) {
          // sample_specular (disney.cpp:322-333)
          const V3 lwh = normalize(sample_vndf15(lwo, v, w));
          if (lwh.z > 0) {
            const V3 t = normalize(mulf(lwh, 2 * dot(lwo, lwh)) - lwo);
            if (t.z > 0) lwi = t;
          }
        } else {
          // sample_clearcoat (disney.cpp:334-344)
          const V3 lwh = sample_gtr1(m->cc_rough, v, w);
          if (lwh.z > 0) {
            const V3 t = normalize(mulf(lwh, 2 * dot(lwo, lwh)) - lwo);
            if (t.z > 0) lwi = t;
          }
        }
      }
    }
    if (!lwi.x && !lwi.y && !lwi.z) return out;
    const V3 wi = s.to_global(lwi);
    out.wi = wi;
    out.f = d15_eval(wi, wo);
    out.pdf = d15_pdf(wi, wo);
    return out;
  }
  // microfacet::sample_anisotropic_gtr2_with_visible_normal with the 2015 alphas
  V3 sample_vndf15(V3 ve, real u, real v) const {
    const real ax = m->ax15, ay = m->ay15;
    const V3 vh = normalize(V3(ax * ve.x, ay * ve.y, ve.z));
    const real lensq = vh.x * vh.x + vh.y * vh.y;
    const V3 t1 = lensq > kEps ? divd(V3(-vh.y, vh.x, 0), std::sqrt(lensq)) : V3(1, 0, 0);
    const V3 t2 = cross(vh, t1);
    const real r = std::sqrt(u);
    const real phi = 2 * kPi * v;
    const real t_1 = r * std::cos(phi);
    const real _t_2 = r * std::sin(phi);
    const real sh = real(0.5) * (1 + vh.z);
    const real t_2 = (1 - sh) * std::sqrt(1 - t_1 * t_1) + sh * _t_2;
    const V3 nh = mulf(t1, t_1) + mulf(t2, t_2) + mulf(vh, std::sqrt(std::max(real(0), 1 - t_1 * t_1 - t_2 * t_2)));
    return normalize(V3(ax * nh.x, ay * nh.y, std::max(real(0), nh.z)));
  }

  Sp eval(V3 wi, V3 wo) const {
    if (m->kind == TR_MAT_DISNEY15) return d15_eval(wi, wo);
    if (m->kind == TR_MAT_METAL) return metal_eval(wi, wo);
    return m->kind == TR_MAT_PHONG ? phong_agg_eval(wi, wo) : (m->kind == TR_MAT_DISNEY12 ? disney_eval(wi, wo) : Sp());
  }
  real pdf(V3 wi, V3 wo) const {
    if (m->kind == TR_MAT_DISNEY15) return d15_pdf(wi, wo);
    if (m->kind == TR_MAT_METAL) return metal_pdf(wi, wo);
    return m->kind == TR_MAT_PHONG ? phong_agg_pdf(wi, wo) : (m->kind == TR_MAT_DISNEY12 ? disney_pdf(wi, wo) : 0);
  }
  BSDFSample sample(V3 wo, real u, real v, real w) const {
    if (m->kind == TR_MAT_GLASS) return glass_sample(wo, u);
    if (m->kind == TR_MAT_METAL) return metal_sample(wo, u, v, w);
    if (m->kind == TR_MAT_DISNEY15) return d15_sample(wo, u, v, w);
    return m->kind == TR_MAT_PHONG ? phong_agg_sample(wo, u, v, w) : disney_sample(wo, u, v, w);
  }
};

// --------------------------------------------------------------- lights
// Triangle::surface_area (shape/triangle.cpp:54-59)
inline real tri_area(const Tri& T) { return (real)(0.5 * length(cross(T.B - T.A, T.C - T.A))); }

struct LightSample {
  V3 pos;
  Sp radiance;
  real pdf = 0;
};
// DiffuseLight::sample_li over Triangle::sample (light/diffuse_light.cpp:44-60,
// shape/triangle.cpp:61-97, core/sampling.hpp:235-238)
LightSample light_sample_li(const Scene& sc, int prim, V3 ref, real u, real v) {
  LightSample out;
  const Prim& pr = sc.prims[prim];
  const Tri& T = sc.tris[pr.shape];
  real su0 = std::sqrt(u);
  real bx = 1 - su0, by = v * su0;
  const V3 AB = T.B - T.A, AC = T.C - T.A;
  V3 pos = mulf(T.A, bx) + mulf(T.B, by) + mulf(T.C, (1 - bx - by));
  V3 gn = normalize(cross(AB, AC));
  V3 dpdu, dpdv;
  compute_ss_ts(AB, AC, T.uB[0] - T.uA[0], T.uB[1] - T.uA[1], T.uC[0] - T.uA[0], T.uC[1] - T.uA[1], gn, dpdu,
                dpdv);
  Coord gc(dpdu, dpdv, gn);
  real area_pdf = 1 / tri_area(T);
  if (dot(gc.z, ref - pos) <= 0) return out;
  V3 sp2ref = ref - pos;
  real dist2 = len2f(sp2ref);
  out.pdf = (real)(area_pdf * dist2 / std::abs(dot(gc.z, sp2ref) / length(sp2ref)));
  out.pos = pos;
  out.radiance = pr.emission;
  return out;
}
// DiffuseLight::pdf (light/diffuse_light.cpp:31-42)
real light_pdf(const Scene& sc, int prim, V3 ref, V3 pos, V3 n) {
  if (dot(n, ref - pos) <= 0) return 0;
  real area = tri_area(sc.tris[sc.prims[prim].shape]);
  const V3 p2ref = ref - pos;
  real dist2 = len2f(p2ref);
  real abscos = (real)std::abs(dot(n, p2ref) / (length(n) * length(p2ref)));
  area *= abscos;
  return dist2 / area;
}
// DiffuseLight::light_emit (light/diffuse_light.cpp:22-24)
inline Sp light_emit(const Scene& sc, int prim, const Isect& is, V3 w) {
  return dot(is.g.z, w) > 0 ? sc.prims[prim].emission : Sp(0);
}

// IBL::sample_li (light/environment_light.cpp:88-116): a direction from the
// luminance distribution, its radiance and a point 2 world radii away.
LightSample env_sample_li(const Env& env, V3 ref, real u, real v) {
  LightSample out;
  float map_pdf;
  real su, sv;
  env.dist.sample_continuous(u, v, &map_pdf, su, sv);
  if (map_pdf == 0) return out;
  const real theta = sv * kPi, phi = su * 2 * kPi;
  const real cos_theta = std::cos(theta), sin_theta = std::sin(theta);
  const real sin_phi = std::sin(phi), cos_phi = std::cos(phi);
  V3 wi(sin_theta * cos_phi, sin_theta * sin_phi, cos_theta);
  wi = normalize(xform_vec(env.to_world, wi));
  if (sin_theta == 0) return out;
  out.pdf = map_pdf / (2 * kPi * kPi * sin_theta);
  out.radiance = env.emit(wi);
  out.pos = ref + mulf(wi, 2 * env.radius);
  return out;
}

// Phong::shading's set-up (material/phong.cpp:29-70) from kd, ks and ns.
inline void phong_setup(Mat& m, Sp diffuse, Sp spec, real ns) {
  real dem = 1;
  dem = std::max(dem, diffuse.r + spec.r);
  dem = std::max(dem, diffuse.g + spec.g);
  dem = std::max(dem, diffuse.b + spec.b);
  diffuse = diffuse / dem;
  spec = spec / dem;
  real dl = diffuse.lum(), sl = spec.lum();
  real wd = (dl + sl > kEps) ? dl / (dl + sl) : real(0.5);
  m.w_diffuse = wd;
  m.w_specular = 1 - wd;
  m.albedo = diffuse + spec;
  m.diffuse_coef = diffuse / kPi;
  m.specular = spec;
  m.ns = ns;
  m.base = diffuse;
}
// A material's set-up from its factory arguments (the shading functions'
// per-hit work that depends on the arguments only; see Mat).
static Mat make_mat(const tr_material& src) {
  Mat m;
  m.kind = src.kind;
  if (src.kind == TR_MAT_PHONG) {
    m.kd_c = Sp(src.kd[0], src.kd[1], src.kd[2]);
    m.ks_c = Sp(src.ks[0], src.ks[1], src.ks[2]);
    m.ns_c = src.ns;
    m.tex_ka = (int)src.tex_ka;
    m.tex_kd = (int)src.tex_kd;
    m.tex_ks = (int)src.tex_ks;
    m.tex_ns = (int)src.tex_ns;
    phong_setup(m, m.kd_c, m.ks_c, m.ns_c);
  } else if (src.kind == TR_MAT_METAL) {
    m.base = Sp(src.color[0], src.color[1], src.color[2]);
    for (int c = 0; c < 3; ++c) {
      // ConductorFresnelPoint(eta_outside = color, eta_inside = 1, k = the caller's k)
      real e2 = real(1) / src.color[c];
      e2 *= e2;
      real ek2 = src.k[c] / src.color[c];
      ek2 *= ek2;
      (c == 0 ? m.f_eta2.r : c == 1 ? m.f_eta2.g : m.f_eta2.b) = e2;
      (c == 0 ? m.f_etak2.r : c == 1 ? m.f_etak2.g : m.f_etak2.b) = ek2;
      (c == 0 ? m.f_paint.r : c == 1 ? m.f_paint.g : m.f_paint.b) = src.eta[c];
    }
    const real aspect = src.anisotropic > 0 ? std::sqrt(1 - real(0.9) * src.anisotropic) : real(1);
    m.ax_m = std::max(real(0.001), src.roughness * src.roughness / aspect);
    m.ay_m = std::max(real(0.001), src.roughness * src.roughness * aspect);
  } else if (src.kind == TR_MAT_DISNEY15) {
    // Disney::shading + DisneyBSDF's constructor (material/disney.cpp:341-392,616-651)
    m.base = Sp(src.base_color[0], src.base_color[1], src.base_color[2]);
    m.metallic = src.metallic; m.roughness = src.roughness; m.specular_tint = src.specular_tint;
    m.anisotropic = src.anisotropic; m.sheen = src.sheen; m.sheen_tint = src.sheen_tint;
    m.clearcoat = src.clearcoat;
    m.spec_scale = Sp(src.specular_scale[0], src.specular_scale[1], src.specular_scale[2]);
    m.transmission = src.transmission;
    const real lum = m.base.lum();
    m.c_tint = lum > 0 ? m.base / lum : Sp(1);
    m.ior15 = std::max(real(1.01), src.ior);
    const real aspect = src.anisotropic > 0 ? std::sqrt(1 - real(0.9) * src.anisotropic) : real(1);
    m.ax15 = std::max(real(0.001), src.roughness * src.roughness / aspect);
    m.ay15 = std::max(real(0.001), src.roughness * src.roughness * aspect);
    const real tr = src.transmission_roughness;
    m.trans_ax = std::max(real(0.001), tr * tr / aspect);
    m.trans_ay = std::max(real(0.001), tr * tr * aspect);
    real cr = mixf(real(0.1), real(0), src.clearcoat_gloss);
    cr *= cr;
    m.cc_rough = std::max(cr, real(0.0001));
    const real A = std::clamp(m.base.lum() * (1 - m.metallic), real(0.3), real(0.7));
    const real B = 1 - A;
    m.w_diff = A * (1 - m.transmission);
    m.w_trans = A * m.transmission;
    m.w_spec = B * 2 / (2 + m.clearcoat);
    m.w_cc = B * m.clearcoat / (2 + m.clearcoat);
  } else if (src.kind == TR_MAT_GLASS) {
    m.kr = Sp(src.kr[0], src.kr[1], src.kr[2]);
    m.kt_sqrt = Sp(std::sqrt(src.kt[0]), std::sqrt(src.kt[1]), std::sqrt(src.kt[2]));
    m.ior = src.ior;
  } else {
    m.base = Sp(src.base_color[0], src.base_color[1], src.base_color[2]);
    m.subsurface = src.subsurface; m.metallic = src.metallic; m.specular_s = src.specular;
    m.specular_tint = src.specular_tint; m.roughness = src.roughness; m.anisotropic = src.anisotropic;
    m.sheen = src.sheen; m.sheen_tint = src.sheen_tint; m.clearcoat = src.clearcoat;
    m.clearcoat_gloss = src.clearcoat_gloss;
  }

  return m;
}


// Factory arguments a kind's tex_param maps: glass (kr, kt, ior), metal
// (color, eta, k, roughness, anisotropic), Disney 2015 (13), Disney 2012 (11).
inline int mapped_args(int kind) {
  switch (kind) {
    case TR_MAT_GLASS: return 3;
    case TR_MAT_METAL: return 5;
    case TR_MAT_DISNEY15: return 13;
    case TR_MAT_DISNEY12: return 11;
    default: return 0;
  }
}

// The factory arguments at a hit: every mapped argument replaced by its map
// at the hit's uv -- Texture2D::evaluate for colours, evaluate_s (the red
// channel) for scalars, as Glass::shading, Metal::shading, Disney::shading and
// Disney12::shading call them (material/glass.cpp:117-140, metal.cpp:33-56,
// disney.cpp:604-639, disney_brdf.cpp:278-302).
inline tr_material mapped_args_at(const Scene& sc, tr_material m, const Isect& is) {
  auto col = [&](int i, float* dst) {
    if (!m.tex_param[i]) return;
    const Sp c = sc.textures[m.tex_param[i] - 1].eval(is.uv[0], is.uv[1]);
    dst[0] = c.r; dst[1] = c.g; dst[2] = c.b;
  };
  auto scl = [&](int i, float& dst) {
    if (m.tex_param[i]) dst = sc.textures[m.tex_param[i] - 1].eval(is.uv[0], is.uv[1]).r;
  };
  switch (m.kind) {
    case TR_MAT_GLASS:
      col(0, m.kr); col(1, m.kt); scl(2, m.ior);
      break;
    case TR_MAT_METAL:
      col(0, m.color); col(1, m.eta); col(2, m.k); scl(3, m.roughness); scl(4, m.anisotropic);
      break;
    case TR_MAT_DISNEY15:
      col(0, m.base_color); scl(1, m.metallic); scl(2, m.roughness); scl(3, m.transmission);
      scl(4, m.transmission_roughness); scl(5, m.ior); col(6, m.specular_scale); scl(7, m.specular_tint);
      scl(8, m.anisotropic); scl(9, m.sheen); scl(10, m.sheen_tint); scl(11, m.clearcoat);
      scl(12, m.clearcoat_gloss);
      break;
    case TR_MAT_DISNEY12:
      col(0, m.base_color); scl(1, m.subsurface); scl(2, m.metallic); scl(3, m.specular);
      scl(4, m.specular_tint); scl(5, m.roughness); scl(6, m.anisotropic); scl(7, m.sheen);
      scl(8, m.sheen_tint); scl(9, m.clearcoat); scl(10, m.clearcoat_gloss);
      break;
  }
  return m;
}

// The material at a hit: a material with image maps evaluates them at the
// hit's uv and sets up again -- Phong from its own maps (Texture2D::evaluate,
// evaluate_s), the other kinds through their mapped factory arguments.
inline const Mat& material_at(const Scene& sc, int mi, const Isect& is, Mat& scratch) {
  const Mat& m = sc.mats[mi];
  if (m.maps) {
    scratch = make_mat(mapped_args_at(sc, sc.msrc[mi], is));
    return scratch;
  }
  if (m.kind != TR_MAT_PHONG || !(m.tex_kd | m.tex_ks | m.tex_ns)) return m;
  scratch = m;
  const Sp kd = m.tex_kd ? sc.textures[m.tex_kd - 1].eval(is.uv[0], is.uv[1]) : m.kd_c;
  const Sp ks = m.tex_ks ? sc.textures[m.tex_ks - 1].eval(is.uv[0], is.uv[1]) : m.ks_c;
  const real ns = m.tex_ns ? sc.textures[m.tex_ns - 1].eval(is.uv[0], is.uv[1]).r : m.ns_c;
  phong_setup(scratch, kd, ks, ns);
  return scratch;
}

// ---------------------------------------------------------- ray recording
struct RayLog {
  std::vector<tr_ray> closest, any;
  std::vector<int32_t> closest_prim;
  std::vector<float> closest_t;
  std::vector<uint8_t> any_hit;
};
inline tr_ray to_tr(const Ray& r) {
  tr_ray t;
  t.o[0] = r.o.x; t.o[1] = r.o.y; t.o[2] = r.o.z;
  t.d[0] = r.d.x; t.d[1] = r.d.y; t.d[2] = r.d.z;
  t.t_min = r.t_min; t.t_max = r.t_max;
  return t;
}

struct Tracer {
  const Scene& sc;
  RayLog* log;
  Counters* cnt;
  bool trace_p(Ray& r, Isect& is) {
    tr_ray in = to_tr(r);
    bool h = intersect_p(sc, r, is, cnt);
    if (log) {
      log->closest.push_back(in);
      log->closest_prim.push_back(h ? is.prim : -1);
      log->closest_t.push_back(r.t_max);
    }
    return h;
  }
  bool trace_any(const Ray& r) {
    bool h = any_hit(sc, r, cnt);
    if (log) {
      log->any.push_back(to_tr(r));
      log->any_hit.push_back(h ? 1 : 0);
    }
    return h;
  }
};

// ---------------------------------------------------------- integrator
// sample_area_light (renderer/direct_illumination.cpp:35-71)
Sp sample_area_light(Tracer& tr, int light, const Isect& is, const BSDF& bsdf, Sampler& smp) {
  const real u = smp.u(), v = smp.u();
  smp.u(); smp.u(); smp.u();
  LightSample ls = light_sample_li(tr.sc, light, is.pos, u, v);
  if (ls.radiance.black() || !ls.pdf) return Sp();
  V3 to_light = ls.pos - is.pos;
  double dist = length(to_light) - kEps;
  if (dist <= kEps) return Sp();
  to_light = normalize(to_light);
  const Ray shadow = make_ray(is.pos, to_light, kEps, (real)dist);
  if (tr.trace_any(shadow)) return Sp();
  const Sp bf = bsdf.eval(to_light, is.wo);
  if (bf.black()) return Sp();
  const real bpdf = bsdf.pdf(to_light, is.wo);
  const Sp f = ((Sp(1) * ls.radiance) * bf) * abs_cos(to_light, is.g.z);
  float weight = power_heuristic(ls.pdf, bpdf);
  return (f * weight) / ls.pdf;
}
// sample_environment_light (renderer/direct_illumination.cpp:73-106)
Sp sample_env_light(Tracer& tr, const Isect& is, const BSDF& bsdf, Sampler& smp) {
  const real u = smp.u(), v = smp.u();
  smp.u(); smp.u(); smp.u();
  LightSample ls = env_sample_li(*tr.sc.env, is.pos, u, v);
  if (ls.radiance.black()) return Sp();
  V3 to_light = ls.pos - is.pos;
  double dist = length(to_light) - kEps;
  if (dist <= kEps) return Sp();
  to_light = normalize(to_light);
  const Ray shadow = make_ray(is.pos, to_light, kEps, (real)dist);
  if (tr.trace_any(shadow)) return Sp();
  const Sp bf = bsdf.eval(to_light, is.wo);
  if (bf.black()) return Sp();
  const real bpdf = bsdf.pdf(to_light, is.wo);
  const Sp f = (ls.radiance * bf) * abs_cos(to_light, is.g.z);
  float weight = power_heuristic(ls.pdf, bpdf);
  return (f * weight) / ls.pdf;
}
// sample_bsdf (renderer/direct_illumination.cpp:144-198)
Sp sample_bsdf_mis(Tracer& tr, const Isect& is, const BSDF& bsdf, Sampler& smp) {
  const real u = smp.u(), v = smp.u(), w = smp.u();
  BSDFSample bs = bsdf.sample(is.wo, u, v, w);
  if (!bs.valid()) return Sp();
  bs.wi = normalize(bs.wi);
  Ray ray = make_ray(is.eps_offset(bs.wi), bs.wi);
  Isect t;
  if (!tr.trace_p(ray, t)) {
    // the environment light's share (direct_illumination.cpp:156-174)
    if (!tr.sc.env) return Sp();
    const Sp Le = tr.sc.env->emit(ray.d);
    if (Le.black()) return Sp();
    const Sp f = (Le * bs.f) * abs_cos(is.g.z, ray.d);
    if (bs.delta) return f / bs.pdf;
    const real lpdf = tr.sc.env->pdf(ray.d);
    const real weight = power_heuristic(bs.pdf, lpdf);
    return (f * weight) / bs.pdf;
  }
  const Prim& pr = tr.sc.prims[t.prim];
  if (!pr.light) return Sp();
  Sp Le = light_emit(tr.sc, t.prim, t, t.wo);
  if (Le.black()) return Sp();
  Sp f = ((Sp(1) * Le) * bs.f) * abs_cos(is.g.z, ray.d);
  real lpdf = light_pdf(tr.sc, t.prim, ray.o, t.pos, t.g.z);
  real weight = power_heuristic(bs.pdf, lpdf);
  return (f * weight) / bs.pdf;
}

// PathTraceRenderer::eval_pixel_li (renderer/path_trace_renderer.cpp:27-210)
// for vacuum media. A ray that leaves the scene at depth 0 or after a delta
// sample adds the environment light's radiance (:66-81). A delta sample gets no direct
// lighting, the emission its ray reaches counts, and up to
// max_specular_depth (20, path_trace_renderer.cpp:20) of them do not count
// toward the depth (:131-139).
Sp eval_li(Tracer& tr, Ray ray, Sampler& smp, int min_depth, int max_depth) {
  const Scene& sc = tr.sc;
  Sp coef(1), L(0);
  bool specular = false;
  for (int depth = 0, s_depth = 0; depth < max_depth; ++depth) {
    if (depth > min_depth) {
      if (smp.u() > 0.9) break;
      coef = coef / (real)0.9;  // Color3::operator/=(T) with T = float
    }
    if (!coef.valid()) break;
    Isect is;
    bool found = tr.trace_p(ray, is);
    if ((depth == 0 || specular) && found && sc.prims[is.prim].light) L += coef * light_emit(sc, is.prim, is, -ray.d);
    if ((depth == 0 || specular) && !found && sc.env) L += coef * sc.env->emit(ray.d);
    if (!found) break;
    Mat hit_mat;
    BSDF bsdf{&material_at(sc, sc.prims[is.prim].material, is, hit_mat), is.g, is.s};
    const real u = smp.u(), v = smp.u(), w = smp.u();
    BSDFSample bs = bsdf.sample(is.wo, u, v, w);
    if (bs.f.black() || bs.pdf < kEps) break;
    specular = bs.delta;
    if (specular && s_depth < 20) {
      s_depth++;
      depth--;
    }
    if (!specular) {
      Sp direct;
      for (int li : sc.lights) direct += coef * sample_area_light(tr, li, is, bsdf, smp);
      if (sc.env) direct += coef * sample_env_light(tr, is, bsdf, smp);
      direct += coef * sample_bsdf_mis(tr, is, bsdf, smp);
      L += direct * (real(1) / 1);
    }
    coef = coef * ((bs.f * abs_cos(is.g.z, bs.wi)) / bs.pdf);
    if (!coef.valid()) break;
    ray = make_ray(is.eps_offset(bs.wi), normalize(bs.wi));
  }
  if (!L.valid()) return Sp();
  return L;
}

// ThinLensCamera (camera/thin_lens_camera.cpp:23-59) + look_at (utility/transform.cpp:96-124)
void setup_camera(Camera& c, const tr_camera& p) {
  V3 pos(p.pos[0], p.pos[1], p.pos[2]), target(p.target[0], p.target[1], p.target[2]);
  V3 up(p.up[0], p.up[1], p.up[2]);
  V3 dir = normalize(target - pos);
  V3 right = normalize(cross(normalize(up), dir));
  V3 new_up = cross(dir, right);
  real m[16] = {right.x, new_up.x, dir.x, pos.x, right.y, new_up.y, dir.y, pos.y,
                right.z, new_up.z, dir.z, pos.z, 0, 0, 0, 1};
  std::memcpy(c.m, m, sizeof(m));
  c.focal_distance = p.focal_dist;
  c.lens_radius = p.lens_radius;
  c.film_h = (real)(2 * p.focal_dist * std::tan(p.fov * 0.5));
  c.film_w = p.film_aspect * c.film_h;
}
Ray generate_ray(const Camera& c, real fx, real fy, real lu, real lv) {
  V3 film((real(0.5) - fx) * c.film_w, (real(0.5) - fy) * c.film_h, c.focal_distance);
  real dx, dy;
  concentric_disk(lu, lv, dx, dy);
  V3 lens(c.lens_radius * dx, c.lens_radius * dy, 0);
  Ray r;
  r.o = xform_point(c.m, lens);
  r.d = xform_vec(c.m, normalize(film - lens));
  return r;
}

// GaussianFilter (filter/gaussian_filter.cpp:9-31)
inline real gaussian(real alpha, real d, real expv) { return std::max((real)0, real(std::exp(-alpha * d * d) - expv)); }

struct TilePx {
  Sp c;
  real w = 0;
};

// Film::Tile::add_sample (core/render.hpp:37-57) into a per-pixel tile
struct PixelTile {
  int x0, y0, x1, y1;  // tile pixel bounds [x0,x1) x [y0,y1)
  TilePx px[64];
};

void pixel_tile_bounds(const Scene& sc, int W, int H, int x, int y, PixelTile& t) {
  // Film::get_film_tile (core/render.hpp:79-88)
  real r = sc.filter_radius;
  int lx = (int)std::ceil((real)x - 0.5f - r), ly = (int)std::ceil((real)y - 0.5f - r);
  int hx = (int)std::floor((real)(x + 1) - 0.5f + r) + 1, hy = (int)std::floor((real)(y + 1) - 0.5f + r) + 1;
  t.x0 = std::max(lx, 0); t.y0 = std::max(ly, 0);
  t.x1 = std::min(hx, W); t.y1 = std::min(hy, H);
}

void add_sample(const Scene& sc, PixelTile& t, real px, real py, Sp L) {
  real r = sc.filter_radius;
  real dx = px - 0.5f, dy = py - 0.5f;
  int p0x = (int)std::ceil(dx - r), p0y = (int)std::ceil(dy - r);
  int p1x = (int)std::floor(dx + r) + 1, p1y = (int)std::floor(dy + r) + 1;
  p0x = std::max(p0x, t.x0); p0y = std::max(p0y, t.y0);
  p1x = std::min(p1x, t.x1); p1y = std::min(p1y, t.y1);
  int tw = t.x1 - t.x0;
  for (int y = p0y; y < p1y; ++y)
    for (int x = p0x; x < p1x; ++x) {
      real ox = px - (real)(x + 0.5), oy = py - (real)(y + 0.5);
      real fw = gaussian(sc.filter_alpha, ox, sc.filter_exp) * gaussian(sc.filter_alpha, oy, sc.filter_exp);
      TilePx& p = t.px[(x - t.x0) + (y - t.y0) * tw];
      p.c += (L * fw) * 1.0f;
      p.w += fw;
    }
}

template <class F>
void parallel_for(int n, int threads, F&& f) {
  if (threads <= 1) {
    for (int i = 0; i < n; ++i) f(i, 0);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&, t] {
      for (;;) {
        int i = next++;
        if (i >= n) return;
        f(i, t);
      }
    });
  for (auto& th : pool) th.join();
}

}  // namespace orc

using namespace orc;

extern "C" {

// Builds the scene the way the reference factories do (shape/triangle.cpp:216-236,
// shape/sphere.cpp:83-92, material/phong.cpp:29-70) and the BVH.
void* orc_scene_create(const tr_scene_desc* d) {
  auto* sc = new Scene();
  sc->max_leaf = d->max_leaf_prims;
  const real I[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
  std::vector<V3> P(d->num_vertices), N(d->num_vertices);
  for (uint32_t v = 0; v < d->num_vertices; ++v) {
    // local_to_world is the identity Transform(): apply it like the reference
    P[v] = xform_point(I, V3(d->positions[3 * v], d->positions[3 * v + 1], d->positions[3 * v + 2]));
    V3 n = xform_normal(I, V3(d->normals[3 * v], d->normals[3 * v + 1], d->normals[3 * v + 2]));
    N[v] = normalize(n);
  }
  sc->tris.resize(d->num_triangles);
  for (uint32_t t = 0; t < d->num_triangles; ++t) {
    Tri& T = sc->tris[t];
    int i0 = d->indices[3 * t], i1 = d->indices[3 * t + 1], i2 = d->indices[3 * t + 2];
    T.A = P[i0]; T.B = P[i1]; T.C = P[i2];
    // Triangle::intersect_p/sample normalise the stored normals again on use
    // (shape/triangle.cpp:73-75,182-184)
    T.nA = normalize(N[i0]); T.nB = normalize(N[i1]); T.nC = normalize(N[i2]);
    T.uA[0] = d->uvs[2 * i0]; T.uA[1] = d->uvs[2 * i0 + 1];
    T.uB[0] = d->uvs[2 * i1]; T.uB[1] = d->uvs[2 * i1 + 1];
    T.uC[0] = d->uvs[2 * i2]; T.uC[1] = d->uvs[2 * i2 + 1];
  }
  sc->spheres.resize(d->num_spheres);
  for (uint32_t s = 0; s < d->num_spheres; ++s) {
    Sphere& S = sc->spheres[s];
    S.radius = d->sphere_radius[s];
    std::memcpy(S.m, d->sphere_to_world + 16 * s, 64);
    std::memcpy(S.inv, d->sphere_to_local + 16 * s, 64);
    real ratio = (real)length(xform_vec(S.m, V3(1, 0, 0)));
    S.world_radius = ratio * S.radius;
  }
  sc->mats.resize(d->num_materials);
  sc->msrc.assign(d->materials, d->materials + d->num_materials);
  for (uint32_t i = 0; i < d->num_materials; ++i) {
    sc->mats[i] = make_mat(d->materials[i]);
    const tr_material& src = d->materials[i];
    for (int k = 0; k < mapped_args(src.kind); ++k) sc->mats[i].maps |= src.tex_param[k] != 0;
  }
  sc->prims.resize(d->num_prims);
  for (uint32_t p = 0; p < d->num_prims; ++p) {
    Prim& pr = sc->prims[p];
    int sh = d->prim_shape[p];
    pr.kind = sh >= 0 ? 0 : 1;
    pr.shape = sh >= 0 ? sh : ~sh;
    pr.material = d->prim_material[p];
    pr.emission = Sp(d->prim_emission[3 * p], d->prim_emission[3 * p + 1], d->prim_emission[3 * p + 2]);
    pr.light = !pr.emission.black();
  }
  for (uint32_t l = 0; l < d->num_lights; ++l) sc->lights.push_back(d->light_prims[l]);
  for (uint32_t k = 0; k < d->num_textures; ++k) {
    const tr_texture& t = d->textures[k];
    Tex x;
    x.w = (int)t.width;
    x.h = (int)t.height;
    if (t.texels) x.tex.assign(t.texels, t.texels + 3 * (size_t)x.w * x.h);
    else x.tex8.assign(t.texels8, t.texels8 + 3 * (size_t)x.w * x.h);
    sc->textures.push_back(std::move(x));
  }
  build_bvh(*sc);
  if ((d->env_texels || d->env_texels8) && d->env_width > 0 && d->env_height > 0) {
    auto env = std::make_unique<Env>();
    env->w = (int)d->env_width;
    env->h = (int)d->env_height;
    if (d->env_texels) env->tex.assign(d->env_texels, d->env_texels + 3 * (size_t)env->w * env->h);
    else env->tex8.assign(d->env_texels8, d->env_texels8 + 3 * (size_t)env->w * env->h);
    std::memcpy(env->to_light, d->env_to_light, 64);
    std::memcpy(env->to_world, d->env_to_world, 64);
    env->build_distribution();
    // EnvironmentLight::preprocess over the tree's root box (core/light.hpp:93-95,
    // Bounds3::bounding_sphere, geometry.hpp:752-755)
    // (an empty tree's default box gives centre 0 and radius 0)
    env->radius = 0;
    if (!sc->nodes.empty()) {
      const Bounds& b = sc->nodes[0].b;
      const V3 sum = b.lo + b.hi;
      env->center = V3((real)(0.5 * sum.x), (real)(0.5 * sum.y), (real)(0.5 * sum.z));
      const bool inside = env->center.x >= b.lo.x && env->center.x <= b.hi.x && env->center.y >= b.lo.y &&
                          env->center.y <= b.hi.y && env->center.z >= b.lo.z && env->center.z <= b.hi.z;
      env->radius = inside ? (real)length(env->center - b.hi) : 0;
    }
    sc->env = std::move(env);
  }
  return sc;
}

void orc_scene_destroy(void* h) { delete static_cast<Scene*>(h); }

void orc_set_camera(void* h, const tr_camera* c, const tr_filter* f) {
  Scene* sc = static_cast<Scene*>(h);
  setup_camera(sc->cam, *c);
  sc->filter_radius = f->radius;
  sc->filter_alpha = f->alpha;
  sc->filter_exp = std::exp(-f->alpha * f->radius * f->radius);
}

size_t orc_bvh_num_nodes(void* h) { return static_cast<Scene*>(h)->nodes.size(); }

void orc_bvh_export(void* h, tr_bvh_node32* nodes, uint32_t* order) {
  Scene* sc = static_cast<Scene*>(h);
  for (size_t i = 0; i < sc->nodes.size(); ++i) {
    const Node& n = sc->nodes[i];
    tr_bvh_node32& o = nodes[i];
    o.lo[0] = n.b.lo.x; o.lo[1] = n.b.lo.y; o.lo[2] = n.b.lo.z;
    o.hi[0] = n.b.hi.x; o.hi[1] = n.b.hi.y; o.hi[2] = n.b.hi.z;
    o.offset = n.offset; o.count = n.count; o.axis = n.axis; o.pad = 0;
  }
  for (size_t i = 0; i < sc->order.size(); ++i) order[i] = (uint32_t)sc->order[i];
}

void orc_make_ray(const float* o, const float* d, float t_min, float t_max, tr_ray* out) {
  *out = to_tr(make_ray(V3(o[0], o[1], o[2]), V3(d[0], d[1], d[2]), t_min, t_max));
}

// Closest hit per ray; nodes/prims (optional) receive per-ray visit counts.
void orc_trace_closest(void* h, const tr_ray* rays, size_t n, int32_t* prim, float* t, uint32_t* nodes,
                       uint32_t* prims, int threads) {
  Scene* sc = static_cast<Scene*>(h);
  const size_t chunk = 4096;
  parallel_for((int)((n + chunk - 1) / chunk), threads, [&](int c, int) {
    for (size_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) {
      Ray r;
      r.o = V3(rays[i].o[0], rays[i].o[1], rays[i].o[2]);
      r.d = V3(rays[i].d[0], rays[i].d[1], rays[i].d[2]);
      r.t_min = rays[i].t_min;
      r.t_max = rays[i].t_max;
      Counters cnt;
      prim[i] = closest_hit(*sc, r, &cnt);
      t[i] = r.t_max;
      if (nodes) nodes[i] = (uint32_t)cnt.nodes;
      if (prims) prims[i] = (uint32_t)cnt.prims;
    }
  });
}

void orc_trace_any(void* h, const tr_ray* rays, size_t n, uint8_t* hit, uint32_t* nodes, uint32_t* prims,
                   int threads) {
  Scene* sc = static_cast<Scene*>(h);
  const size_t chunk = 4096;
  parallel_for((int)((n + chunk - 1) / chunk), threads, [&](int c, int) {
    for (size_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) {
      Ray r;
      r.o = V3(rays[i].o[0], rays[i].o[1], rays[i].o[2]);
      r.d = V3(rays[i].d[0], rays[i].d[1], rays[i].d[2]);
      r.t_min = rays[i].t_min;
      r.t_max = rays[i].t_max;
      Counters cnt;
      hit[i] = any_hit(*sc, r, &cnt) ? 1 : 0;
      if (nodes) nodes[i] = (uint32_t)cnt.nodes;
      if (prims) prims[i] = (uint32_t)cnt.prims;
    }
  });
}

// Per-pixel-seeded render over rows [row0, row1) (the whole film when
// row1 <= row0). rgbw (float) or rgbw64 (double accumulation of the same
// per-sample values) receive color sums and weights for all W*H pixels;
// rows outside the range stay untouched. Returns the number of samples.
uint64_t orc_render(void* h, const tr_render_params* p, int row0, int row1, float* rgbw, double* rgbw64,
                    int threads) {
  Scene* sc = static_cast<Scene*>(h);
  const int W = p->width, H = p->height;
  if (row1 <= row0) { row0 = 0; row1 = H; }
  const int nrows = row1 - row0;
  std::vector<std::vector<PixelTile>> tiles(nrows);
  std::vector<std::vector<Sp>> sums64;  // unused placeholder for symmetry
  std::vector<double> acc64;
  if (rgbw64) acc64.assign((size_t)W * H * 4, 0.0);
  std::vector<std::vector<double>> row64(rgbw64 ? nrows : 0);
  parallel_for(nrows, threads, [&](int ri, int) {
    int y = row0 + ri;
    Tracer tr{*sc, nullptr, nullptr};
    tiles[ri].resize(W);
    if (rgbw64) row64[ri].assign((size_t)W * 4, 0.0);
    for (int x = 0; x < W; ++x) {
      PixelTile& tile = tiles[ri][x];
      pixel_tile_bounds(*sc, W, H, x, y, tile);
      std::memset(tile.px, 0, sizeof(tile.px));
      Sampler smp((int)(p->seed_base + (uint32_t)y * (uint32_t)W + (uint32_t)x));
      for (int i = 0; i < p->spp; ++i) {
        const real fu = smp.u(), fv = smp.u();
        const real lu = smp.u(), lv = smp.u();
        const real pxf = x + fu, pyf = y + fv;
        Ray ray = generate_ray(sc->cam, pxf / W, pyf / H, lu, lv);
        Sp L = eval_li(tr, ray, smp, p->min_depth, p->max_depth);
        if (std::isfinite(L.r) && std::isfinite(L.g) && std::isfinite(L.b)) {
          add_sample(*sc, tile, pxf, pyf, L);
          if (rgbw64 && sc->filter_radius <= 0.5f) {
            // same per-sample terms, summed in double (own pixel only at r <= 0.5)
            real ox = pxf - (real)(x + 0.5), oy = pyf - (real)(y + 0.5);
            real fw = gaussian(sc->filter_alpha, ox, sc->filter_exp) * gaussian(sc->filter_alpha, oy, sc->filter_exp);
            Sp c = (L * fw) * 1.0f;
            double* a = &row64[ri][4 * x];
            a[0] += c.r; a[1] += c.g; a[2] += c.b; a[3] += fw;
          }
        }
      }
    }
  });
  if (rgbw) {
    std::vector<Sp> color((size_t)W * H);
    std::vector<real> weight((size_t)W * H, 0);
    for (int i = 0; i < W * H; ++i) {
      color[i] = Sp(rgbw[4 * i], rgbw[4 * i + 1], rgbw[4 * i + 2]);
      weight[i] = rgbw[4 * i + 3];
    }
    for (int ri = 0; ri < nrows; ++ri)
      for (int x = 0; x < W; ++x) {
        const PixelTile& t = tiles[ri][x];
        int tw = t.x1 - t.x0;
        for (int yy = t.y0; yy < t.y1; ++yy)
          for (int xx = t.x0; xx < t.x1; ++xx) {
            const TilePx& tp = t.px[(xx - t.x0) + (yy - t.y0) * tw];
            color[xx + yy * W] += tp.c;
            weight[xx + yy * W] += tp.w;
          }
      }
    for (int i = 0; i < W * H; ++i) {
      rgbw[4 * i] = color[i].r; rgbw[4 * i + 1] = color[i].g; rgbw[4 * i + 2] = color[i].b;
      rgbw[4 * i + 3] = weight[i];
    }
  }
  if (rgbw64)
    for (int ri = 0; ri < nrows; ++ri)
      for (int k = 0; k < W * 4; ++k) rgbw64[(size_t)(row0 + ri) * W * 4 + k] += row64[ri][k];
  return (uint64_t)nrows * W * p->spp;
}

// Per-pixel-seeded render of an arbitrary set of rows (in parallel); rgbw
// receives the rows' own filtered sums (radius <= 0.5: each sample reaches
// only its pixel), in the order given. Returns the number of samples.
uint64_t orc_render_rows(void* h, const tr_render_params* p, const int* rows, int nrows, float* rgbw,
                         int threads) {
  Scene* sc = static_cast<Scene*>(h);
  const int W = p->width, H = p->height;
  parallel_for(nrows, threads, [&](int ri, int) {
    const int y = rows[ri];
    Tracer tr{*sc, nullptr, nullptr};
    for (int x = 0; x < W; ++x) {
      PixelTile tile;
      pixel_tile_bounds(*sc, W, H, x, y, tile);
      std::memset(tile.px, 0, sizeof(tile.px));
      Sampler smp((int)(p->seed_base + (uint32_t)y * (uint32_t)W + (uint32_t)x));
      for (int i = 0; i < p->spp; ++i) {
        const real fu = smp.u(), fv = smp.u();
        const real lu = smp.u(), lv = smp.u();
        const real pxf = x + fu, pyf = y + fv;
        Ray ray = generate_ray(sc->cam, pxf / W, pyf / H, lu, lv);
        Sp L = eval_li(tr, ray, smp, p->min_depth, p->max_depth);
        if (std::isfinite(L.r) && std::isfinite(L.g) && std::isfinite(L.b)) add_sample(*sc, tile, pxf, pyf, L);
      }
      const TilePx& own = tile.px[(x - tile.x0) + (y - tile.y0) * (tile.x1 - tile.x0)];
      float* o = rgbw + 4 * ((size_t)ri * W + x);
      o[0] = own.c.r; o[1] = own.c.g; o[2] = own.c.b; o[3] = own.w;
    }
  });
  return (uint64_t)nrows * W * p->spp;
}

// Renders pixels [pix0, pix1) in row-major order on one thread and records
// every closest-hit and any-hit query with its result (the ray-replay log).
// Returns the number of closest rays; call orc_log_fetch to copy them out.
static RayLog g_log;
size_t orc_render_log(void* h, const tr_render_params* p, int pix0, int pix1, size_t* n_any) {
  Scene* sc = static_cast<Scene*>(h);
  g_log = RayLog();
  Tracer tr{*sc, &g_log, nullptr};
  const int W = p->width, H = p->height;
  for (int pi = pix0; pi < pix1; ++pi) {
    int x = pi % W, y = pi / W;
    Sampler smp((int)(p->seed_base + (uint32_t)y * (uint32_t)W + (uint32_t)x));
    for (int i = 0; i < p->spp; ++i) {
      const real fu = smp.u(), fv = smp.u();
      const real lu = smp.u(), lv = smp.u();
      Ray ray = generate_ray(sc->cam, (x + fu) / W, (y + fv) / H, lu, lv);
      eval_li(tr, ray, smp, p->min_depth, p->max_depth);
    }
  }
  *n_any = g_log.any.size();
  return g_log.closest.size();
}
void orc_log_fetch(tr_ray* closest, int32_t* prim, float* t, tr_ray* any, uint8_t* hit) {
  std::memcpy(closest, g_log.closest.data(), g_log.closest.size() * sizeof(tr_ray));
  std::memcpy(prim, g_log.closest_prim.data(), g_log.closest_prim.size() * 4);
  std::memcpy(t, g_log.closest_t.data(), g_log.closest_t.size() * 4);
  std::memcpy(any, g_log.any.data(), g_log.any.size() * sizeof(tr_ray));
  std::memcpy(hit, g_log.any_hit.data(), g_log.any_hit.size());
}

// Unit entry points for kernel-level parity tests.
void orc_cross(const float* a, const float* b, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    V3 r = cross(V3(a[3 * i], a[3 * i + 1], a[3 * i + 2]), V3(b[3 * i], b[3 * i + 1], b[3 * i + 2]));
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
  }
}
void orc_normalize(const float* a, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    V3 r = normalize(V3(a[3 * i], a[3 * i + 1], a[3 * i + 2]));
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
  }
}
void orc_slab_scale(const float* x, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    real v = x[i];
    v *= 1 + 0.0000001;
    out[i] = v;
  }
}
void orc_pcg_uniform(int seed, float* out, size_t n) {
  Sampler s(seed);
  for (size_t i = 0; i < n; ++i) out[i] = s.u();
}


// ---- output path (test restatement)
// Film::write_render_target (src/core/render.hpp:105-115): sum / weight per
// channel where the weight is positive, else 0. film: r, g, b, w per pixel.
void orc_post_resolve(const float* film, size_t n, float* rgb) {
  for (size_t i = 0; i < n; ++i) {
    const float w = film[4 * i + 3];
    for (int c = 0; c < 3; ++c) rgb[3 * i + c] = w > 0.0f ? film[4 * i + c] / w : 0.0f;
  }
}
// ACESToneMapper::process (src/post_processor/aces.cpp:9-43): per channel
// clamp(x (2.51 x + 0.03) / (x (2.43 x + 0.59) + 0.14), 0, 1), x = c * exposure;
// a negative exposure is replaced by 1.
void orc_post_aces(float* rgb, size_t n3, float exposure) {
  if (exposure < 0.0f) exposure = 1.0f;
  for (size_t i = 0; i < n3; ++i) {
    const float x = rgb[i] * exposure;
    const float v = (x * (2.51f * x + 0.03f)) / (x * (2.43f * x + 0.59f) + 0.14f);
    rgb[i] = v < 0.0f ? 0.0f : (1.0f < v ? 1.0f : v);
  }
}
// GammaCorrector::process (src/post_processor/gamma.cpp:26-38): pow(c, gamma)
// per channel; gamma <= 0 is replaced by 1.
void orc_post_gamma(float* rgb, size_t n3, float gamma) {
  if (gamma <= 0.0f) gamma = 1.0f;
  for (size_t i = 0; i < n3; ++i) rgb[i] = std::pow(rgb[i], gamma);
}
// The demo driver's 8-bit image (src/main.hpp:171-178): clamp<int>(pow(c,
// inv_gamma) * 255, 0, 255), the float converted to int by truncation
// (NaN and out-of-range values: 0 below, 255 above, as a saturating
// conversion gives).
void orc_post_rgb8(const float* rgb, size_t n3, float inv_gamma, uint8_t* out) {
  for (size_t i = 0; i < n3; ++i) {
    const float v = std::pow(rgb[i], inv_gamma) * 255;
    int iv = v != v ? 0 : (v >= 2147483647.0f ? 2147483647 : (v <= -2147483648.0f ? (-2147483647 - 1) : (int)v));
    out[i] = (uint8_t)(iv < 0 ? 0 : (iv > 255 ? 255 : iv));
  }
}
// Radiance RGBE (G. Ward, "Real Pixels", Graphics Gems II): the largest
// channel v = m 2^e with m in [0.5, 1) sets the shared exponent e + 128 and
// each channel becomes floor(c * m * 256 / v); v < 1e-32 encodes as zeros.
void orc_post_rgbe(const float* rgb, size_t n, uint8_t* out) {
  for (size_t i = 0; i < n; ++i) {
    const float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
    float v = r;
    if (g > v) v = g;
    if (b > v) v = b;
    uint8_t* o = out + 4 * i;
    if (!(v >= 1e-32f)) {
      o[0] = o[1] = o[2] = o[3] = 0;
      continue;
    }
    int e;
    const float m = std::frexp(v, &e);
    const float s = m * 256.0f / v;
    const float c[3] = {r * s, g * s, b * s};
    for (int k = 0; k < 3; ++k) o[k] = (uint8_t)(c[k] > 0.0f ? (c[k] < 255.0f ? (int)c[k] : 255) : 0);
    o[3] = (uint8_t)(e + 128);
  }
}

}  // extern "C"
