// scene_types.h -- device-resident scene layout (HBM), shared by host upload
// code and kernels.
//
// Layout decisions (one scene, read-only during a render):
//  * DNode: the reference's binary BVH re-packed as child pairs. One 64-byte
//    record per interior node holds both children's boxes, child references
//    and the split axis, so a visit is four 16-byte vector loads and two box
//    tests. Traversal keeps the reference's order and culling exactly (see
//    traverse.cuh).
//  * DNode4: the same tree collapsed to four-wide nodes for any-hit rays,
//    whose result does not depend on the visiting order.
//  * Slots: primitives in BVH leaf order, three float4 (48 bytes) each.
//    Triangle: (A, id) (B-A, -1) (C-A, 0) -- B-A and C-A are the float
//    differences the reference computes on every test. Sphere: (0, id)
//    (0, sphere index) (0).
//  * Per-primitive, per-triangle, per-sphere, per-material and per-light
//    tables indexed by the scene description's ids, holding only values
//    the reference would recompute identically on every hit (constant
//    frames, material-derived weights).
#pragma once

#include <stdint.h>

#include "exact32.cuh"

#if !defined(__CUDACC__)
struct alignas(16) float4 {
  float x, y, z, w;
};
struct alignas(16) int4 {
  int x, y, z, w;
};
#endif

struct tr_material;  // the C ABI's material record (tracer_gpu.h)

namespace trg {

// Launch-tuning limits (tr_tuning): ray-binning grid bits per axis, and the
// child-pair nodes of the shared-memory treelet.
constexpr int kBinBitsMax = 5;
constexpr int kTreeletMax = 1024;
// A child reference with this bit set names a node of the shared-memory
// treelet (its index in the low bits) instead of a DNode in global memory.
constexpr int kTreeletRef = 1 << 25;

struct alignas(16) DNode {
  float4 a;  // L.lo.x L.lo.y L.lo.z L.hi.x
  float4 b;  // L.hi.y L.hi.z R.lo.x R.lo.y
  float4 c;  // R.lo.z R.hi.x R.hi.y R.hi.z
  int4 d;    // L.ref, R.ref, L.count | R.count << 16, axis. count > 0: ref is a
             // leaf's first slot; count == 0: ref is the child's DNode index.
};
static_assert(sizeof(DNode) == 64, "DNode must be 64 bytes");

// Any-hit tree: the binary tree collapsed to up to four children per node
// (128 bytes, boxes as structure of arrays). cnt > 0: ref is a leaf's first
// slot; cnt == 0: ref is a DNode4 index; cnt < 0: no child.
struct alignas(16) DNode4 {
  float4 lox, loy, loz, hix, hiy, hiz;
  int4 ref, cnt;
};
static_assert(sizeof(DNode4) == 128, "DNode4 must be 128 bytes");

struct DSphere {
  float inv[16];  // world_to_local (row-major)
  float m[16];    // local_to_world
  float radius;
  int pad[3];
};

enum { PRIM_TRIANGLE = 0, PRIM_SPHERE = 1 };

struct DPrim {
  int kind;
  int shape;     // triangle or sphere index
  int material;
  int emissive;  // 1 if the emission is not black (GeometricPrimitive owns a DiffuseLight)
  f3 emission;
  float area;    // Triangle::surface_area() of emissive triangles
};

struct DTriShade {
  f3 gx, gy, gz;  // geometry frame: constant per triangle (src/shape/triangle.cpp:193-198)
  f3 nA, dn1, dn2;  // normalised vertex normal A, nB - nA, nC - nA
  f3 dndu0, dndv0;  // compute_ss_ts(nB-nA, nC-nA, uv...) when its determinant != 0
  int det_nonzero;
  float uvA[2], duv1[2], duv2[2];  // uvA, uvB - uvA, uvC - uvA (the hit's uv, triangle.cpp:186)
  int pad;
};

// An image texture (HDRTexture2D or ImageTexture2D): w x h texels, texel
// (x, y) at x + y * w; exactly one of the two pointers is set.
struct DTex {
  const float4* texels;
  const uchar4* texels8;
  int w, h;
};

enum { MAT_PHONG = 0, MAT_DISNEY12 = 1, MAT_GLASS = 2, MAT_METAL = 3, MAT_DISNEY15 = 4 };
constexpr int kMatKinds = 5;
// kinds with light sampling: Phong, Disney12, metal, Disney15 (glass is a delta BSDF)
constexpr int kNeeKinds = 4;

// Phong: the AggregateBSDF<2> that Phong::shading builds (src/material/phong.cpp:29-70)
// Disney12: the eleven parameters (src/material/disney_brdf.cpp:278-302)
// Glass: GlassBSDF's colours and index of refraction
struct DMat {
  int kind;
  float ns, w_diffuse, w_specular;
  // Disney12 per-material constants the reference recomputes on every call
  // (src/material/disney_brdf.cpp:81-83,142-151,188-193)
  float ax, ay, p_diffuse, p_spec_sample, p_spec_pdf;
  f3 diffuse_coef;  // albedo / PI of DiffuseBXDF
  f3 specular;      // PhongSpecularBXDF colour
  f3 albedo;        // LocalBSDF::get_albedo(): diffuse + specular, or Disney base colour
  float subsurface, metallic, specular_s, specular_tint, roughness, anisotropic;
  float sheen, sheen_tint, clearcoat, clearcoat_gloss;
  f3 base;
  // Glass (src/material/glass.cpp:117-140): reflect colour, sqrt(transmit colour), ior
  f3 kr, kt_sqrt;
  float ior;
  // Metal (src/material/metal.cpp:33-56): painted conductor Fresnel constants
  // (squared ratios and paint, per channel); ax, ay above hold its GGX alphas
  f3 f_eta2, f_etak2, f_paint;
  // Disney15 (src/material/disney.cpp:341-392): tint colour, specular scale,
  // transmission, the transmission alphas, clearcoat roughness and the lobe
  // weights; base, metallic, roughness, specular_tint, sheen, sheen_tint and
  // clearcoat above, ax, ay its specular alphas, ior its IOR (at least 1.01)
  f3 c_tint, spec_scale;
  float transmission, trans_ax, trans_ay, cc_rough, w_diff15, w_trans, w_spec15, w_cc;
  // Phong maps (0: the constants below; k: DScene::textures[k - 1]) and the constants
  int tex_kd, tex_ks, tex_ns;
  f3 kd_c, ks_c;
  float ns_c;
  // some argument of the material is an image map: a hit sets the material
  // up from DScene::msrc at its uv (0 in such per-hit set-ups)
  int tex_any;
};

// Phong::shading's set-up (src/material/phong.cpp:29-70): kd and ks scaled
// down so that no channel sums above 1, lobe weights by luminance.
TR_HD void phong_setup(DMat& d, f3 diffuse, f3 spec, float ns) {
  float dem = 1.0f;
  dem = (dem < diffuse.x + spec.x) ? diffuse.x + spec.x : dem;
  dem = (dem < diffuse.y + spec.y) ? diffuse.y + spec.y : dem;
  dem = (dem < diffuse.z + spec.z) ? diffuse.z + spec.z : dem;
  diffuse = mk3(diffuse.x / dem, diffuse.y / dem, diffuse.z / dem);
  spec = mk3(spec.x / dem, spec.y / dem, spec.z / dem);
  const float dl = 0.2126f * diffuse.x + 0.7152f * diffuse.y + 0.0722f * diffuse.z;
  const float sl = 0.2126f * spec.x + 0.7152f * spec.y + 0.0722f * spec.z;
  const float wd = (dl + sl > kEps) ? dl / (dl + sl) : 0.5f;
  d.w_diffuse = wd;
  d.w_specular = 1.0f - wd;
  d.albedo = diffuse + spec;
  d.diffuse_coef = mk3(diffuse.x / kPi, diffuse.y / kPi, diffuse.z / kPi);
  d.specular = spec;
  d.ns = ns;
}

// A diffuse area light on a triangle (src/light/diffuse_light.cpp:44-60)
struct DLight {
  f3 A, B, C;
  f3 gz;          // geometry normal of sampled points
  f3 emission;
  float area_pdf; // 1 / surface_area()
  int prim;
  float extent;   // sum of |coordinates| of A, B, C plus 1 (scale of the back-side margin)
  int env;        // >= 0: the environment light DScene::envs[env] (prim is -1), else -1
  f3 AB, AC;      // the triangle's edges as its traversal slot holds them (B - A, C - A)
  float bs[4];    // a sphere around the triangle with a margin (centre, radius)
  float bs_cn;    // |centre|
};

// Environment light of one scene: the reference's IBL over an HDR texture
// (src/light/environment_light.cpp:14-193). Tables built on the host with
// the reference's arithmetic: the texels, the Distribution2D of its
// luminance (rows of the conditional p(u | v), the marginal over v), the
// rotation parts of world_to_light and its inverse, and the scene's
// bounding sphere.
struct DEnv {
  const float4* texels;     // w x h, texel (x, y) at x + y * w
  const uchar4* texels8;    // an 8-bit map instead (texels is then null)
  const float* cond_func;   // nv x nu
  const float* cond_cdf;    // nv x (nu + 1)
  const float* cond_int;    // nv (the marginal's function)
  const float* marg_cdf;    // nv + 1
  float marg_int;
  int w, h, nu, nv;
  float to_light[9], to_world[9];
  float center[3], radius;
};

// Root of one scene of the uploaded set: its tree and its lights.
struct SceneRoot {
  int kind;    // 0 empty, 1 interior (DNode `offset`), 2 leaf (slots offset .. offset + count)
  int offset, count;
  int light_base, num_lights;  // the scene's lights in DScene::lights
  float lo[3], hi[3];          // root box
  int offset4;                 // kind 1: the root's DNode4 index
};

// The device tables of a scene set: every scene's nodes, slots, primitives,
// materials and lights concatenated, indices already offset.
struct DScene {
  const DNode* nodes;
  const DNode4* nodes4;  // null when the any-hit tree is not available
  const float4* slots;
  const DSphere* spheres;
  const DPrim* prims;
  const DTriShade* tshade;
  const DMat* mats;
  const DLight* lights;
  const SceneRoot* roots;
  int num_scenes;
  int max_lights;  // most lights of one scene
  int has_glass;   // some material is a delta BSDF (glass)
  int has_metal;   // some material is metal
  int has_disney15;  // some material is the 2015 Disney BSDF
  const DEnv* envs;  // environment lights of the set (DLight::env indexes them)
  int has_env;       // some scene has an environment light
  const DTex* textures;  // image textures of the set's materials
  int has_textures;      // some material has an image map
  // Top of scene 0's child-pair tree, breadth first from the root, for
  // staging in shared memory (single-scene sets only): copies of DNodes whose
  // references to other treelet nodes are kTreeletRef | treelet index.
  const DNode* treelet;
  int treelet_n;  // nodes in it (0: none)
  // Per slot: 2 * (its leaf's parent DNode) + (1 if the leaf is the right
  // child); -1 where the leaf is a scene's root. Null for device-built trees.
  const int* slot_leaf;
  // The materials' factory arguments and maps, by material index (only for
  // sets with image maps; null otherwise)
  const tr_material* msrc;
  // Binary any-hit walks: the child entered first when both pass
  // (tr_tuning.any_hit_order: 0 near, 1 far, 2 larger box surface).
  int any_order;
};

}  // namespace trg
