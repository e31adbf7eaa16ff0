// tracer_gb300.hpp -- C++ host API of the GB300 path tracer.
//
// The scene-building and renderer interface of Tracer (reference
// src/factory/*.hpp, src/core/renderer.hpp, src/core/scene.hpp), kept name
// for name and argument for argument for the parts the path-tracing hot path
// uses, so a program written against the reference's factories builds its
// scene the same way and selects the GPU renderer with
// create_gpu_pt_renderer beside the reference's create_pt_renderer
// (src/factory/renderer.hpp:12-21).
//
// Underneath, every object records the flat description the C ABI
// (tracer_gpu.h) uploads: world-space triangle and sphere tables, materials,
// emissive primitives and the light list. Construction errors throw, as in
// the reference (src/shape/sphere.cpp:88-90); render errors throw TracerError
// carrying the C ABI's status.
//
// Constant textures and image maps (HDR or 8-bit) as material arguments; the
// vacuum medium only.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "tracer_gpu.h"

namespace tracer {

using real = float;
template <class T>
using RC = std::shared_ptr<T>;
template <class T>
using Box = std::unique_ptr<T>;
template <class T>
using Span = std::vector<T>;

class TracerError : public std::runtime_error {
 public:
  TracerError(tr_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  tr_status status;
};

// ---- values (src/core/spectrum.hpp, src/utility/geometry.hpp) ----

struct Spectrum {
  real r = 0, g = 0, b = 0;
  Spectrum() = default;
  explicit Spectrum(real v) : r(v), g(v), b(v) {}
  Spectrum(real r_, real g_, real b_) : r(r_), g(g_), b(b_) {}
  bool is_black() const { return r == 0 && g == 0 && b == 0; }
  explicit operator bool() const { return !is_black(); }
};

struct Point2f {
  real x = 0, y = 0;
};
struct Point2i {
  int x = 0, y = 0;
};
struct Point3f {
  real x = 0, y = 0, z = 0;
};
struct Vector3f {
  real x = 0, y = 0, z = 0;
};
struct Normal3f {
  real x = 0, y = 0, z = 0;
};

// ---- transforms (src/utility/transform.hpp, transform.cpp) ----

struct Matrix4x4 {
  real m[4][4];
  Matrix4x4();  // identity
  Matrix4x4(real t00, real t01, real t02, real t03, real t10, real t11, real t12, real t13, real t20, real t21,
            real t22, real t23, real t30, real t31, real t32, real t33);
  static Matrix4x4 mul(const Matrix4x4& a, const Matrix4x4& b);
};
Matrix4x4 transpose(const Matrix4x4& m);
Matrix4x4 inverse(const Matrix4x4& m);  // throws std::runtime_error when singular

class Transform {
 public:
  Transform() = default;
  explicit Transform(const Matrix4x4& m);
  Transform(const Matrix4x4& m, const Matrix4x4& inv_m) : m_(m), inv_(inv_m) {}
  Point3f operator()(const Point3f& p) const;
  Vector3f operator()(const Vector3f& v) const;
  Normal3f operator()(const Normal3f& n) const;  // by the inverse transpose
  const Matrix4x4& matrix() const { return m_; }
  const Matrix4x4& inverse_matrix() const { return inv_; }
  friend Transform inverse(const Transform& t) { return Transform(t.inv_, t.m_); }
  friend Transform operator*(const Transform& a, const Transform& b);

 private:
  Matrix4x4 m_, inv_;
};
Transform translate(const Vector3f& delta);
Transform scale(real x, real y, real z);
Transform rotate_x(real theta);  // radians
Transform rotate_y(real theta);
Transform rotate_z(real theta);

// ---- meshes (src/utility/mesh_load.hpp:15-89) ----

struct vertex_t {
  Point3f pos;
  Normal3f n;
  Point2f uv;
};
struct mesh_t {
  std::string name;
  std::vector<vertex_t> vertices;
  std::vector<int> indices;
  std::vector<int> materials;
};
// A Wavefront MTL material (src/utility/mesh_load.hpp:27-79): colours and
// scalars as written, texture maps by file name.
struct material_t {
  std::string name;
  real ambient[3] = {0, 0, 0}, diffuse[3] = {0, 0, 0}, specular[3] = {0, 0, 0}, transmittance[3] = {0, 0, 0},
       emission[3] = {0, 0, 0};
  real shininess = 1, ior = 1, dissolve = 1;
  int illum = 0;
  std::string map_ka, map_kd, map_ks, map_ns, map_bump, disp, map_d, refl;
  real roughness = 0, metallic = 0, sheen = 0, clearcoat_thickness = 0, clearcoat_roughness = 0;
  std::string map_pr, map_pm, map_ps, map_ke, norm;
};
struct model_t {
  std::string name;
  std::vector<mesh_t> mesh;
  std::vector<material_t> material;
};
// load_model_from_file (src/utility/mesh_load.cpp:25-113), read by a
// project-written Wavefront OBJ/MTL parser: one mesh per object/group with
// faces, polygons fan-triangulated, vertices deduplicated by (position,
// normal, uv) in first-use order, normals normalised, the material id of
// every triangle (-1 without usemtl); mtllib files relative to the OBJ.
// Faces need vertex normals, as the reference reads them unchecked.
// Throws TracerError on a missing file or a malformed line.
model_t load_model_from_file(const std::string& path);

// ---- scene objects ----

class Texture2D {
 public:
  virtual ~Texture2D() = default;
  virtual Spectrum evaluate(const Point2f& uv) const = 0;
  real evaluate_s(const Point2f& uv) const { return evaluate(uv).r; }  // core/texture.hpp:74-83
};
RC<Texture2D> create_constant_texture2d(const Spectrum& constant);

class Shape {
 public:
  virtual ~Shape() = default;
};
RC<Shape> create_sphere(real radius, const Transform& local_to_world);
std::vector<RC<Shape>> create_triangle_mesh(const mesh_t& mesh, const Transform& local_to_world);

class Material {
 public:
  explicit Material(const tr_material& m) : rec(m) {}
  tr_material rec;
  // image maps of the factory's arguments in their order (Phong: ka, kd, ks,
  // ns; the other kinds as tr_material.tex_param lists them); null where the
  // argument is a constant
  RC<const Texture2D> maps[13];
};
RC<Material> create_phong_material(RC<const Texture2D> map_ka, RC<const Texture2D> map_kd,
                                   RC<const Texture2D> map_ks, RC<const Texture2D> map_ns);
RC<Material> create_disney_brdf(RC<const Texture2D> base_color, RC<const Texture2D> subsurface,
                                RC<const Texture2D> metallic, RC<const Texture2D> specular,
                                RC<const Texture2D> specular_tint, RC<const Texture2D> roughness,
                                RC<const Texture2D> anisotropic, RC<const Texture2D> sheen,
                                RC<const Texture2D> sheen_tint, RC<const Texture2D> clearcoat,
                                RC<const Texture2D> clearcoat_gloss);
// create_glass (src/factory/material.hpp:13-17, src/material/glass.cpp:145-154)
RC<Material> create_glass(RC<const Texture2D> map_kr, RC<const Texture2D> map_kt, RC<const Texture2D> map_ior);
// create_disney, the 2015 Disney BSDF (src/factory/material.hpp:37-53,
// src/material/disney.cpp:541-677), with no normal mapper and no BSSRDF
RC<Material> create_disney(RC<const Texture2D> base_color, RC<const Texture2D> metallic,
                           RC<const Texture2D> roughness, RC<const Texture2D> transmission,
                           RC<const Texture2D> transmission_roughness, RC<const Texture2D> ior,
                           RC<const Texture2D> specular_scale, RC<const Texture2D> specular_tint,
                           RC<const Texture2D> anisotropic, RC<const Texture2D> sheen,
                           RC<const Texture2D> sheen_tint, RC<const Texture2D> clearcoat,
                           RC<const Texture2D> clearcoat_gloss);
// create_metal (src/factory/material.hpp:90-96, src/material/metal.cpp:68-76) with
// no normal mapper; the painted conductor Fresnel is built as the reference
// builds it from (color, eta, k)
RC<Material> create_metal(RC<const Texture2D> color, RC<const Texture2D> eta, RC<const Texture2D> k,
                          RC<const Texture2D> roughness, RC<const Texture2D> anisotropic);

class Medium {
 public:
  virtual ~Medium() = default;
};
RC<Medium> create_vacuum();
struct MediumInterface {
  MediumInterface() = default;
  explicit MediumInterface(RC<const Medium> m) : inside(m), outside(m) {}
  MediumInterface(RC<const Medium> in, RC<const Medium> out) : inside(std::move(in)), outside(std::move(out)) {}
  RC<const Medium> inside, outside;
};

class Light {
 public:
  virtual ~Light() = default;
};
class AreaLight : public Light {};
// An environment light: create_ibl_light (src/factory/light.hpp:12-14).
class EnvironmentLight : public Light {
 public:
  virtual ~EnvironmentLight() = default;
};

class Primitive {
 public:
  virtual ~Primitive() = default;
  virtual const AreaLight* as_area_light() const noexcept = 0;
};
RC<Primitive> create_geometric_primitive(const RC<Shape>& shape, const RC<Material>& material,
                                         const MediumInterface& mi, const Spectrum& emission);

class Aggregate {
 public:
  virtual ~Aggregate() = default;
  virtual void build(std::vector<RC<Primitive>> primitives) = 0;
};
RC<Aggregate> create_bvh_accel(int max_leaf_primitives);

class Camera {
 public:
  explicit Camera(const tr_camera& c) : rec(c) {}
  tr_camera rec;
};
RC<Camera> create_thin_lens_camera(real film_aspect, const Point3f& cam_pos, const Point3f& target,
                                   const Vector3f& up, real fov, real lens_radius, real focal_dist);

class Filter {
 public:
  explicit Filter(const tr_filter& f) : rec(f) {}
  real radius() const { return rec.radius; }
  tr_filter rec;
};
RC<Filter> create_gaussin_filter(real radius, real alpha);

// Flat scene as uploaded (owned arrays; tr_scene_desc points into them).
struct SceneDesc {
  std::vector<float> positions, normals, uvs;
  std::vector<int32_t> indices;
  std::vector<float> sphere_radius, sphere_to_world, sphere_to_local;
  std::vector<tr_material> materials;
  std::vector<int32_t> prim_shape, prim_material;
  std::vector<float> prim_emission;
  std::vector<int32_t> light_prims;
  int32_t max_leaf_prims = 1;
  uint32_t env_width = 0, env_height = 0;  // environment map (0 x 0: none)
  std::vector<float> env_texels, env_to_light, env_to_world;
  std::vector<uint8_t> env_texels8;  // an 8-bit map instead of env_texels
  struct TextureData {
    uint32_t width = 0, height = 0;
    std::vector<float> texels;     // 3 per texel (HDR)
    std::vector<uint8_t> texels8;  // or 3 bytes per texel (8-bit)
  };
  std::vector<TextureData> textures;  // the materials' image maps (tr_material::tex_* - 1)
  tr_scene_desc view() const;

 private:
  mutable std::vector<tr_texture> texture_recs_;
};

class Scene {
 public:
  virtual ~Scene() = default;
  virtual void set_camera(RC<const Camera> camera) = 0;
  virtual RC<const Camera> get_camera() const noexcept = 0;
  virtual void prepare_to_render() = 0;
  Span<const Light*> lights;
  // src/core/scene.hpp:31; when set, it is also the last entry of `lights`
  // (as src/main.cpp:59-67 arranges)
  RC<EnvironmentLight> environment_light;
  // GPU-path additions: the description prepare_to_render() assembled and a
  // counter that changes whenever it is rebuilt.
  virtual const SceneDesc& desc() const = 0;
  virtual uint64_t revision() const noexcept = 0;
};
RC<Scene> create_general_scene(const RC<Aggregate>& accel);

// ---- film and renderers (src/core/render.hpp, src/core/renderer.hpp) ----

template <class T>
class Image2D {
 public:
  Image2D() = default;
  Image2D(int w, int h) : w_(w), h_(h), data_((size_t)w * h) {}
  int width() const { return w_; }
  int height() const { return h_; }
  T& at(int x, int y) { return data_[(size_t)y * w_ + x]; }
  const T& at(int x, int y) const { return data_[(size_t)y * w_ + x]; }
  T* get_data() { return data_.data(); }

 private:
  int w_ = 0, h_ = 0;
  std::vector<T> data_;
};

using Color3f = Point3f;

// create_hdr_texture2d (src/factory/texture.hpp:16, src/texture/hdr_texture.cpp:9-37):
// bilinear lookups of a linear-RGB image, texel (x, y) at
// (u, v) = (x / (width - 1), y / (height - 1)), coordinates wrapped by repeat.
RC<Texture2D> create_hdr_texture2d(const RC<Image2D<Color3f>>& image);
// create_ibl_light (src/light/environment_light.cpp:196-203): the texture
// (an HDR, 8-bit image or constant texture) over the sphere of directions,
// (u, v) = (phi / 2pi, theta / pi) in the light space of world_to_light.
RC<EnvironmentLight> create_ibl_light(RC<const Texture2D> tex, const Transform& world_to_light);

struct RenderTarget {
  Image2D<Spectrum> color;
};

// ---- image files (src/utility/image_file.hpp:12-45), read and written by
// project code in place of the reference's stb dependency ----

struct Color3b {
  uint8_t x = 0, y = 0, z = 0;
};
// Radiance HDR: the header, "-Y height +X width", RGBE scanlines (row 0 first).
void write_image_to_hdr(const Image2D<Spectrum>& image, const std::string& filename);
// 8-bit RGB PNG (row 0 first).
void write_image_to_png(const Image2D<Color3b>& image, const std::string& filename);
// An 8-bit PNG (grey, RGB, palette or RGBA; not interlaced), rows flipped
// so that the file's last row is row 0, as load_image_from_file
// (src/utility/image_file.cpp:26-58) loads it; grey+alpha is refused.
RC<Image2D<Color3b>> load_image_from_file(const std::string& filename);
// create_image_texture2d (src/texture/image_texture2d.cpp:9-37): bilinear
// lookups in byte arithmetic (each weighted texel truncated to a byte), / 255.
RC<Texture2D> create_image_texture2d(const RC<Image2D<Color3b>>& image);
// A Radiance HDR file (flat or run-length scanlines, "-Y height +X width"),
// row 0 = the first scanline, RGBE decoded as byte * 2^(exponent - 136).
RC<Image2D<Color3f>> load_hdr_from_file(const std::string& filename);
// create_texture2d_from_file (src/utility/image_file.cpp:168-178): ".hdr"
// files become HDR textures, ".png" files image textures. JPEG has no reader
// here and throws TracerError(TR_ERR_UNSUPPORTED); other extensions throw
// TR_ERR_ARG, as the reference throws for them.
RC<const Texture2D> create_texture2d_from_file(const std::string& filename);
// The textures of an MTL material (src/utility/image_file.hpp:23-45).
struct MaterialTexture {
  RC<Texture2D> map_ka, map_kd, map_ks, map_kt, ior, map_ns, map_bump, disp, map_d, refl;
  RC<Texture2D> map_pr, map_pm, map_ps, map_ke, norm;
  bool has_emission = false;
  bool as_glass = false;
};
// create_texture_from_file (src/utility/image_file.cpp:136-166): a constant
// texture of the MTL value where no map is named, else the map file scaled
// by the value (1 where the value is black); emission flags has_emission; an
// ior above 1 makes the material glass with kt = ks (1 where ks is black).
MaterialTexture create_texture_from_file(const material_t& material);

class Film {
 public:
  Film(const Point2i& res, const RC<Filter>& filter) : resolution(res), filter(filter) {}
  int width() const { return resolution.x; }
  int height() const { return resolution.y; }
  const RC<Filter>& get_filter() const { return filter; }

 private:
  Point2i resolution;
  RC<Filter> filter;
};

class Renderer {
 public:
  virtual ~Renderer() = default;
  virtual RenderTarget render(const Scene& scene, Film film) = 0;
};

// PTRendererParams (src/factory/renderer.hpp:12-19) for the GPU: the device
// replaces worker_count/task_tile_size; seed_base fixes the per-pixel pcg32
// seeds ((int32)(seed_base + y * width + x)).
struct GPUPTRendererParams {
  int device = 0;
  int spp = 1;
  int min_depth = 3;
  int max_depth = 10;
  int direct_light_sample_num = 1;
  uint32_t seed_base = 0;
  bool fp64_film = false;  // accumulate the film sums in double
};

// The GPU renderer; render() returns sum / weight per pixel like
// Film::write_render_target (src/core/render.hpp:104-115). The raw sums of
// the last render and its statistics stay readable for checks.
class GpuPathTraceRenderer : public Renderer {
 public:
  virtual const std::vector<double>& film_sums() const = 0;  // W*H*4: r, g, b, weight
  virtual tr_stats last_stats() const = 0;
};
RC<GpuPathTraceRenderer> create_gpu_pt_renderer(const GPUPTRendererParams& params);

}  // namespace tracer
