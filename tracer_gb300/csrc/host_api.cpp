// host_api.cpp -- the C++ scene/factory/renderer API of tracer_gb300.hpp.
//
// Objects record the flat scene description; create_gpu_pt_renderer's
// render() uploads it through the C ABI and renders on the GPU. Transform
// arithmetic is the reference's float arithmetic in the same operation order
// (src/utility/transform.hpp:70-96, transform.cpp:127-177), so world-space
// vertices equal the ones the reference's create_triangle_mesh stores
// (src/shape/triangle.cpp:216-236).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <utility>

#include "tracer_gb300.hpp"

namespace tracer {

// ---------------------------------------------------------------- transforms

Matrix4x4::Matrix4x4() {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) m[i][j] = i == j ? 1.0f : 0.0f;
}

Matrix4x4::Matrix4x4(real t00, real t01, real t02, real t03, real t10, real t11, real t12, real t13, real t20,
                     real t21, real t22, real t23, real t30, real t31, real t32, real t33) {
  const real v[16] = {t00, t01, t02, t03, t10, t11, t12, t13, t20, t21, t22, t23, t30, t31, t32, t33};
  std::memcpy(m, v, sizeof(v));
}

Matrix4x4 Matrix4x4::mul(const Matrix4x4& a, const Matrix4x4& b) {
  Matrix4x4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
  return r;
}

Matrix4x4 transpose(const Matrix4x4& a) {
  Matrix4x4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i][j] = a.m[j][i];
  return r;
}

// Gauss-Jordan elimination with partial pivoting, in double.
Matrix4x4 inverse(const Matrix4x4& a) {
  double w[4][8];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      w[i][j] = a.m[i][j];
      w[i][j + 4] = i == j ? 1.0 : 0.0;
    }
  for (int c = 0; c < 4; ++c) {
    int p = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(w[r][c]) > std::fabs(w[p][c])) p = r;
    if (w[p][c] == 0.0) throw std::runtime_error("singular matrix in inverse");
    if (p != c)
      for (int j = 0; j < 8; ++j) std::swap(w[p][j], w[c][j]);
    const double s = 1.0 / w[c][c];
    for (int j = 0; j < 8; ++j) w[c][j] *= s;
    for (int r = 0; r < 4; ++r) {
      if (r == c || w[r][c] == 0.0) continue;
      const double f = w[r][c];
      for (int j = 0; j < 8; ++j) w[r][j] -= f * w[c][j];
    }
  }
  Matrix4x4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i][j] = (real)w[i][j + 4];
  return r;
}

Transform::Transform(const Matrix4x4& m) : m_(m), inv_(inverse(m)) {}

Point3f Transform::operator()(const Point3f& p) const {
  const auto& m = m_.m;
  const real x = p.x, y = p.y, z = p.z;
  const real xp = m[0][0] * x + m[0][1] * y + m[0][2] * z + m[0][3];
  const real yp = m[1][0] * x + m[1][1] * y + m[1][2] * z + m[1][3];
  const real zp = m[2][0] * x + m[2][1] * y + m[2][2] * z + m[2][3];
  const real wp = m[3][0] * x + m[3][1] * y + m[3][2] * z + m[3][3];
  if (wp == 1) return {xp, yp, zp};
  const double inv = 1.0 / wp;  // Point3::operator/ multiplies by a double reciprocal
  return {(real)(inv * xp), (real)(inv * yp), (real)(inv * zp)};
}

Vector3f Transform::operator()(const Vector3f& v) const {
  const auto& m = m_.m;
  return {m[0][0] * v.x + m[0][1] * v.y + m[0][2] * v.z, m[1][0] * v.x + m[1][1] * v.y + m[1][2] * v.z,
          m[2][0] * v.x + m[2][1] * v.y + m[2][2] * v.z};
}

Normal3f Transform::operator()(const Normal3f& n) const {
  const auto& m = inv_.m;
  return {m[0][0] * n.x + m[1][0] * n.y + m[2][0] * n.z, m[0][1] * n.x + m[1][1] * n.y + m[2][1] * n.z,
          m[0][2] * n.x + m[1][2] * n.y + m[2][2] * n.z};
}

Transform operator*(const Transform& a, const Transform& b) {
  return Transform(Matrix4x4::mul(a.m_, b.m_), Matrix4x4::mul(b.inv_, a.inv_));
}

Transform translate(const Vector3f& d) {
  return Transform(Matrix4x4(1, 0, 0, d.x, 0, 1, 0, d.y, 0, 0, 1, d.z, 0, 0, 0, 1),
                   Matrix4x4(1, 0, 0, -d.x, 0, 1, 0, -d.y, 0, 0, 1, -d.z, 0, 0, 0, 1));
}

Transform scale(real x, real y, real z) {
  return Transform(Matrix4x4(x, 0, 0, 0, 0, y, 0, 0, 0, 0, z, 0, 0, 0, 0, 1),
                   Matrix4x4((real)(1.0 / x), 0, 0, 0, 0, (real)(1.0 / y), 0, 0, 0, 0, (real)(1.0 / z), 0, 0, 0,
                             0, 1));
}

Transform rotate_x(real theta) {
  const real s = std::sin(theta), c = std::cos(theta);
  const Matrix4x4 m(1, 0, 0, 0, 0, c, -s, 0, 0, s, c, 0, 0, 0, 0, 1);
  return Transform(m, transpose(m));
}

Transform rotate_y(real theta) {
  const real s = std::sin(theta), c = std::cos(theta);
  const Matrix4x4 m(c, 0, s, 0, 0, 1, 0, 0, -s, 0, c, 0, 0, 0, 0, 1);
  return Transform(m, transpose(m));
}

Transform rotate_z(real theta) {
  const real s = std::sin(theta), c = std::cos(theta);
  const Matrix4x4 m(c, -s, 0, 0, s, c, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1);
  return Transform(m, transpose(m));
}

// ---------------------------------------------------------------- textures

namespace {

class ConstantTexture : public Texture2D {
 public:
  explicit ConstantTexture(const Spectrum& c) : c_(c) {}
  Spectrum evaluate(const Point2f&) const override { return c_; }

 private:
  Spectrum c_;
};

Spectrum tex(const RC<const Texture2D>& t, const char* what) {
  if (!t) throw std::invalid_argument(std::string("null texture: ") + what);
  if (!dynamic_cast<const ConstantTexture*>(t.get()))
    throw TracerError(TR_ERR_UNSUPPORTED, std::string("texture kind outside the GPU path: ") + what);
  return t->evaluate(Point2f{});
}

// ---------------------------------------------------------------- shapes

struct MeshData {
  std::vector<Point3f> p;
  std::vector<Normal3f> n;
  std::vector<Point2f> uv;
  std::vector<int> indices;
};

class TriangleShape : public Shape {
 public:
  TriangleShape(RC<const MeshData> m, int i) : mesh(std::move(m)), index(i) {}
  RC<const MeshData> mesh;
  int index;
};

class SphereShape : public Shape {
 public:
  SphereShape(real r, const Transform& t) : radius(r), local_to_world(t) {}
  real radius;
  Transform local_to_world;
};

class VacuumMedium : public Medium {};

class DiffuseAreaLight : public AreaLight {
 public:
  explicit DiffuseAreaLight(const Primitive* p) : prim(p) {}
  const Primitive* prim;
};

class GeometricPrimitive : public Primitive {
 public:
  GeometricPrimitive(RC<Shape> s, RC<Material> m, const Spectrum& e)
      : shape(std::move(s)), material(std::move(m)), emission(e), light(this) {}
  // only emitting primitives are area lights (src/shape/geometry.cpp:31-41,66-68)
  const AreaLight* as_area_light() const noexcept override { return emission ? &light : nullptr; }
  RC<Shape> shape;
  RC<Material> material;
  Spectrum emission;
  DiffuseAreaLight light;
};

class BvhAggregate : public Aggregate {
 public:
  explicit BvhAggregate(int max_leaf) : max_leaf_prims(max_leaf) {}
  void build(std::vector<RC<Primitive>> primitives) override {
    prims = std::move(primitives);
    ++built;
  }
  int max_leaf_prims;
  std::vector<RC<Primitive>> prims;
  uint64_t built = 0;
};

// Normal3::normalize (src/utility/geometry.hpp:492-515): float sum of squares
// widened to double, double reciprocal of the double sqrt, products rounded.
Normal3f normalize_ref(const Normal3f& n) {
  const float s = n.x * n.x + n.y * n.y + n.z * n.z;
  const double inv = 1.0 / std::sqrt((double)s);
  return {(float)(n.x * inv), (float)(n.y * inv), (float)(n.z * inv)};
}

// The reference normalises mesh normals on creation and again, in place, on
// every hit (src/shape/triangle.cpp:216-236, :178-211), so a normal settles
// on a fixed point of normalize during a render; start from that point.
Normal3f settled_normal(const Normal3f& n) {
  Normal3f v = normalize_ref(n);
  for (int i = 0; i < 8; ++i) {
    const Normal3f w = normalize_ref(v);
    if (w.x == v.x && w.y == v.y && w.z == v.z) break;
    v = w;
  }
  return v;
}

void put_matrix(std::vector<float>& out, const Matrix4x4& m) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out.push_back(m.m[i][j]);
}

// HDRTexture2D (src/texture/hdr_texture.cpp:9-37) behind Texture2D::evaluate
// with the repeat wrap (src/core/texture.hpp:57-95) and LinearSampler::Sample2D
// (src/utility/sampler.hpp:16-29).
class HdrTexture : public Texture2D {
 public:
  explicit HdrTexture(RC<Image2D<Color3f>> img) : img_(std::move(img)) {}
  Spectrum evaluate(const Point2f& uv) const override {
    auto wrap = [](real x) { return std::clamp<real>(x - std::floor(x), 0, 1); };
    const int w = img_->width(), h = img_->height();
    const double u = std::clamp((double)wrap(uv.x), 0.0, 1.0) * (w - 1);
    const double v = std::clamp((double)wrap(uv.y), 0.0, 1.0) * (h - 1);
    const int u0 = std::clamp((int)u, 0, w - 1), u1 = std::clamp(u0 + 1, 0, w - 1);
    const int v0 = std::clamp((int)v, 0, h - 1), v1 = std::clamp(v0 + 1, 0, h - 1);
    const double du = u - u0, dv = v - v0;
    auto mul = [](const Color3f& c, double f) { return Color3f{(real)(f * c.x), (real)(f * c.y), (real)(f * c.z)}; };
    auto add = [](const Color3f& a, const Color3f& b) { return Color3f{a.x + b.x, a.y + b.y, a.z + b.z}; };
    const Color3f r = add(mul(add(mul(img_->at(u0, v0), 1.0 - du), mul(img_->at(u1, v0), du)), 1.0 - dv),
                          mul(add(mul(img_->at(u0, v1), 1.0 - du), mul(img_->at(u1, v1), du)), dv));
    return Spectrum(r.x, r.y, r.z);
  }
  const Image2D<Color3f>& image() const { return *img_; }

 private:
  RC<Image2D<Color3f>> img_;
};

// ImageTexture2D (src/texture/image_texture2d.cpp:9-37): the same lookup over
// bytes, each weighted texel truncated to a byte (Point3<uint8_t>), / 255.
class ImageTexture : public Texture2D {
 public:
  explicit ImageTexture(RC<Image2D<Color3b>> img) : img_(std::move(img)) {}
  Spectrum evaluate(const Point2f& uv) const override {
    auto wrap = [](real x) { return std::clamp<real>(x - std::floor(x), 0, 1); };
    const int w = img_->width(), h = img_->height();
    const double u = std::clamp((double)wrap(uv.x), 0.0, 1.0) * (w - 1);
    const double v = std::clamp((double)wrap(uv.y), 0.0, 1.0) * (h - 1);
    const int u0 = std::clamp((int)u, 0, w - 1), u1 = std::clamp(u0 + 1, 0, w - 1);
    const int v0 = std::clamp((int)v, 0, h - 1), v1 = std::clamp(v0 + 1, 0, h - 1);
    const double du = u - u0, dv = v - v0;
    auto mul = [](const Color3b& c, double f) {
      return Color3b{(uint8_t)(f * c.x), (uint8_t)(f * c.y), (uint8_t)(f * c.z)};
    };
    auto add = [](const Color3b& a, const Color3b& b) {
      return Color3b{(uint8_t)(a.x + b.x), (uint8_t)(a.y + b.y), (uint8_t)(a.z + b.z)};
    };
    const Color3b r = add(mul(add(mul(img_->at(u0, v0), 1.0 - du), mul(img_->at(u1, v0), du)), 1.0 - dv),
                          mul(add(mul(img_->at(u0, v1), 1.0 - du), mul(img_->at(u1, v1), du)), dv));
    return Spectrum(r.x / real(255.0), r.y / real(255.0), r.z / real(255.0));
  }
  const Image2D<Color3b>& image() const { return *img_; }

 private:
  RC<Image2D<Color3b>> img_;
};

bool is_image(const Texture2D* t) {
  return dynamic_cast<const HdrTexture*>(t) || dynamic_cast<const ImageTexture*>(t);
}

// A factory argument: a constant texture gives its value; an image texture
// (HDR or 8-bit) is kept as map `slot` of the material and evaluated at each
// hit's uv (the constant field stays zero).
struct Args {
  RC<const Texture2D> maps[13];
  Spectrum col(const RC<const Texture2D>& t, const char* what, int slot) {
    if (!t) throw std::invalid_argument(std::string("null texture: ") + what);
    if (is_image(t.get())) {
      maps[slot] = t;
      return Spectrum(0);
    }
    if (!dynamic_cast<const ConstantTexture*>(t.get()))
      throw TracerError(TR_ERR_UNSUPPORTED, std::string("texture kind outside the GPU path: ") + what);
    return t->evaluate(Point2f{});
  }
  real scl(const RC<const Texture2D>& t, const char* what, int slot) { return col(t, what, slot).r; }
  RC<Material> make(const tr_material& m) {
    auto mat = std::make_shared<Material>(m);
    for (int k = 0; k < 13; ++k) mat->maps[k] = maps[k];
    return mat;
  }
};

class IblLight : public EnvironmentLight {
 public:
  IblLight(RC<const Texture2D> tex, const Transform& t) : tex(std::move(tex)), world_to_light(t) {}
  RC<const Texture2D> tex;
  Transform world_to_light;
};

class GeneralScene : public Scene {
 public:
  explicit GeneralScene(RC<BvhAggregate> a) : accel_(std::move(a)) {}
  void set_camera(RC<const Camera> c) override { camera_ = std::move(c); }
  RC<const Camera> get_camera() const noexcept override { return camera_; }

  void prepare_to_render() override {
    SceneDesc d;
    d.max_leaf_prims = accel_->max_leaf_prims;
    std::unordered_map<const MeshData*, int> mesh_base;
    std::unordered_map<const Material*, int> mat_index;
    std::unordered_map<const Light*, int> light_index;
    std::unordered_map<const Texture2D*, uint32_t> tex_index;
    for (size_t i = 0; i < accel_->prims.size(); ++i) {
      const auto* gp = dynamic_cast<const GeometricPrimitive*>(accel_->prims[i].get());
      if (!gp) throw std::invalid_argument("primitive not made by create_geometric_primitive");
      if (!gp->material) throw std::invalid_argument("primitive without material");
      auto mi = mat_index.find(gp->material.get());
      if (mi == mat_index.end()) {
        mi = mat_index.emplace(gp->material.get(), (int)d.materials.size()).first;
        tr_material rec = gp->material->rec;
        uint32_t* slots[13];
        const int nslots = rec.kind == TR_MAT_PHONG ? 4 : 13;
        uint32_t* phong[4] = {&rec.tex_ka, &rec.tex_kd, &rec.tex_ks, &rec.tex_ns};
        for (int k = 0; k < nslots; ++k) slots[k] = rec.kind == TR_MAT_PHONG ? phong[k] : &rec.tex_param[k];
        for (int k = 0; k < nslots; ++k) {
          const Texture2D* t = gp->material->maps[k].get();
          if (!t) continue;
          auto ti = tex_index.find(t);
          if (ti == tex_index.end()) {
            SceneDesc::TextureData td;
            if (const auto* ht = dynamic_cast<const HdrTexture*>(t)) {
              const Image2D<Color3f>& img = ht->image();
              td.width = (uint32_t)img.width();
              td.height = (uint32_t)img.height();
              for (int y = 0; y < img.height(); ++y)
                for (int x = 0; x < img.width(); ++x) {
                  const Color3f& c = img.at(x, y);
                  td.texels.insert(td.texels.end(), {c.x, c.y, c.z});
                }
            } else {
              const Image2D<Color3b>& img = static_cast<const ImageTexture*>(t)->image();
              td.width = (uint32_t)img.width();
              td.height = (uint32_t)img.height();
              for (int y = 0; y < img.height(); ++y)
                for (int x = 0; x < img.width(); ++x) {
                  const Color3b& c = img.at(x, y);
                  td.texels8.insert(td.texels8.end(), {c.x, c.y, c.z});
                }
            }
            ti = tex_index.emplace(t, (uint32_t)d.textures.size() + 1).first;
            d.textures.push_back(std::move(td));
          }
          *slots[k] = ti->second;
        }
        d.materials.push_back(rec);
      }
      if (const auto* ts = dynamic_cast<const TriangleShape*>(gp->shape.get())) {
        auto mb = mesh_base.find(ts->mesh.get());
        if (mb == mesh_base.end()) {
          mb = mesh_base.emplace(ts->mesh.get(), (int)(d.positions.size() / 3)).first;
          for (size_t v = 0; v < ts->mesh->p.size(); ++v) {
            const Point3f& p = ts->mesh->p[v];
            const Normal3f& n = ts->mesh->n[v];
            const Point2f& uv = ts->mesh->uv[v];
            d.positions.insert(d.positions.end(), {p.x, p.y, p.z});
            d.normals.insert(d.normals.end(), {n.x, n.y, n.z});
            d.uvs.insert(d.uvs.end(), {uv.x, uv.y});
          }
        }
        const int tri = (int)(d.indices.size() / 3);
        for (int k = 0; k < 3; ++k) d.indices.push_back(mb->second + ts->mesh->indices[3 * ts->index + k]);
        d.prim_shape.push_back(tri);
      } else if (const auto* ss = dynamic_cast<const SphereShape*>(gp->shape.get())) {
        const int s = (int)d.sphere_radius.size();
        d.sphere_radius.push_back(ss->radius);
        put_matrix(d.sphere_to_world, ss->local_to_world.matrix());
        put_matrix(d.sphere_to_local, ss->local_to_world.inverse_matrix());
        d.prim_shape.push_back(~s);
      } else {
        throw std::invalid_argument("unknown shape");
      }
      d.prim_material.push_back(mi->second);
      d.prim_emission.insert(d.prim_emission.end(), {gp->emission.r, gp->emission.g, gp->emission.b});
      light_index.emplace(&gp->light, (int)i);
    }
    for (size_t k = 0; k < lights.size(); ++k) {
      const Light* l = lights[k];
      if (dynamic_cast<const EnvironmentLight*>(l)) {
        if (l != environment_light.get() || k + 1 != lights.size())
          throw std::invalid_argument("an environment light must be the scene's environment_light and its last light");
        continue;
      }
      auto it = light_index.find(l);
      if (it == light_index.end()) throw std::invalid_argument("scene light is not a primitive of this scene");
      d.light_prims.push_back(it->second);
    }
    if (environment_light) {
      if (lights.empty() || lights.back() != environment_light.get())
        throw std::invalid_argument("the environment light must also be the last entry of scene->lights");
      const auto* ibl = dynamic_cast<const IblLight*>(environment_light.get());
      if (!ibl) throw std::invalid_argument("environment light not made by create_ibl_light");
      if (const auto* ht = dynamic_cast<const HdrTexture*>(ibl->tex.get())) {
        const Image2D<Color3f>& img = ht->image();
        d.env_width = (uint32_t)img.width();
        d.env_height = (uint32_t)img.height();
        for (int y = 0; y < img.height(); ++y)
          for (int x = 0; x < img.width(); ++x) {
            const Color3f& c = img.at(x, y);
            d.env_texels.insert(d.env_texels.end(), {c.x, c.y, c.z});
          }
      } else if (const auto* it = dynamic_cast<const ImageTexture*>(ibl->tex.get())) {
        const Image2D<Color3b>& img = it->image();
        d.env_width = (uint32_t)img.width();
        d.env_height = (uint32_t)img.height();
        for (int y = 0; y < img.height(); ++y)
          for (int x = 0; x < img.width(); ++x) {
            const Color3b& c = img.at(x, y);
            d.env_texels8.insert(d.env_texels8.end(), {c.x, c.y, c.z});
          }
      } else if (const auto* ct = dynamic_cast<const ConstantTexture*>(ibl->tex.get())) {
        const Spectrum c = ct->evaluate(Point2f{0, 0});  // a constant map is a 1 x 1 image
        d.env_width = d.env_height = 1;
        d.env_texels = {c.r, c.g, c.b};
      } else {
        throw std::invalid_argument("environment light texture must be an HDR, 8-bit image or constant texture");
      }
      put_matrix(d.env_to_light, ibl->world_to_light.matrix());
      put_matrix(d.env_to_world, ibl->world_to_light.inverse_matrix());
    }
    desc_ = std::move(d);
    ++revision_;
  }

  const SceneDesc& desc() const override { return desc_; }
  uint64_t revision() const noexcept override { return revision_; }

 private:
  RC<BvhAggregate> accel_;
  RC<const Camera> camera_;
  SceneDesc desc_;
  uint64_t revision_ = 0;
};

// ---------------------------------------------------------------- renderer

class GpuRenderer : public GpuPathTraceRenderer {
 public:
  explicit GpuRenderer(const GPUPTRendererParams& p) : params_(p) {
    tr_status s = tr_ctx_create(&ctx_, p.device);
    if (s != TR_OK) throw TracerError(s, std::string("tr_ctx_create: ") + tr_status_string(s));
  }
  ~GpuRenderer() override { tr_ctx_destroy(ctx_); }

  RenderTarget render(const Scene& scene, Film film) override {
    if (!scene.get_camera()) throw std::invalid_argument("scene has no camera");
    if (!film.get_filter()) throw std::invalid_argument("film has no filter");
    if (&scene != uploaded_scene_ || scene.revision() != uploaded_revision_) {
      const tr_scene_desc d = scene.desc().view();
      check(tr_scene_upload(ctx_, &d));
      uploaded_scene_ = &scene;
      uploaded_revision_ = scene.revision();
    }
    tr_render_params rp{};
    rp.width = film.width();
    rp.height = film.height();
    rp.spp = params_.spp;
    rp.min_depth = params_.min_depth;
    rp.max_depth = params_.max_depth;
    rp.direct_light_sample_num = params_.direct_light_sample_num;
    rp.seed_base = params_.seed_base;
    const size_t n = (size_t)rp.width * (size_t)rp.height;
    sums_.assign(4 * n, 0.0);
    if (params_.fp64_film) {
      check(tr_render(ctx_, &scene.get_camera()->rec, &film.get_filter()->rec, &rp, nullptr, sums_.data(),
                      &stats_));
    } else {
      std::vector<float> f(4 * n);
      check(tr_render(ctx_, &scene.get_camera()->rec, &film.get_filter()->rec, &rp, f.data(), nullptr, &stats_));
      for (size_t i = 0; i < 4 * n; ++i) sums_[i] = f[i];
    }
    // Film::write_render_target: color / weight where weight > 0
    RenderTarget rt;
    rt.color = Image2D<Spectrum>(rp.width, rp.height);
    for (int y = 0; y < rp.height; ++y)
      for (int x = 0; x < rp.width; ++x) {
        const double* s = &sums_[4 * ((size_t)y * rp.width + x)];
        const real w = (real)s[3];
        if (w > 0) rt.color.at(x, y) = Spectrum((real)s[0] / w, (real)s[1] / w, (real)s[2] / w);
      }
    return rt;
  }

  const std::vector<double>& film_sums() const override { return sums_; }
  tr_stats last_stats() const override { return stats_; }

 private:
  void check(tr_status s) {
    if (s != TR_OK) throw TracerError(s, tr_ctx_last_error(ctx_));
  }
  GPUPTRendererParams params_;
  tr_ctx* ctx_ = nullptr;
  const Scene* uploaded_scene_ = nullptr;
  uint64_t uploaded_revision_ = 0;
  std::vector<double> sums_;
  tr_stats stats_{};
};

}  // namespace

// ---------------------------------------------------------------- factories

RC<Texture2D> create_constant_texture2d(const Spectrum& constant) { return std::make_shared<ConstantTexture>(constant); }

RC<Texture2D> create_hdr_texture2d(const RC<Image2D<Color3f>>& image) {
  if (!image || image->width() <= 0 || image->height() <= 0) throw std::invalid_argument("empty HDR image");
  return std::make_shared<HdrTexture>(image);
}

RC<Texture2D> create_image_texture2d(const RC<Image2D<Color3b>>& image) {
  if (!image || image->width() <= 0 || image->height() <= 0) throw std::invalid_argument("empty image");
  return std::make_shared<ImageTexture>(image);
}

RC<EnvironmentLight> create_ibl_light(RC<const Texture2D> tex, const Transform& world_to_light) {
  if (!tex) throw std::invalid_argument("environment light without texture");
  return std::make_shared<IblLight>(std::move(tex), world_to_light);
}

RC<Shape> create_sphere(real radius, const Transform& local_to_world) {
  if (radius <= 0) throw std::runtime_error("invalid sphere radius");  // src/shape/sphere.cpp:88-90
  return std::make_shared<SphereShape>(radius, local_to_world);
}

std::vector<RC<Shape>> create_triangle_mesh(const mesh_t& mesh, const Transform& local_to_world) {
  if (mesh.indices.size() % 3 != 0) throw std::invalid_argument("mesh index count is not a multiple of 3");
  for (int i : mesh.indices)
    if (i < 0 || (size_t)i >= mesh.vertices.size()) throw std::invalid_argument("mesh index out of range");
  auto m = std::make_shared<MeshData>();
  m->indices = mesh.indices;
  for (const vertex_t& v : mesh.vertices) {
    m->p.push_back(local_to_world(v.pos));
    m->n.push_back(settled_normal(local_to_world(v.n)));
    m->uv.push_back(v.uv);
  }
  std::vector<RC<Shape>> out;
  for (size_t t = 0; t < mesh.indices.size() / 3; ++t) out.push_back(std::make_shared<TriangleShape>(m, (int)t));
  return out;
}

RC<Material> create_phong_material(RC<const Texture2D> map_ka, RC<const Texture2D> map_kd,
                                   RC<const Texture2D> map_ks, RC<const Texture2D> map_ns) {
  tr_material m{};
  m.kind = TR_MAT_PHONG;
  // constants are recorded as values, image maps as textures of the material
  const RC<const Texture2D> in[4] = {map_ka, map_kd, map_ks, map_ns};
  const char* names[4] = {"ka", "kd", "ks", "ns"};
  Spectrum v[4];
  RC<const Texture2D> maps[4];
  for (int k = 0; k < 4; ++k) {
    if (!in[k]) throw std::invalid_argument(std::string("null texture: ") + names[k]);
    if (dynamic_cast<const HdrTexture*>(in[k].get()) || dynamic_cast<const ImageTexture*>(in[k].get()))
      maps[k] = in[k];
    else
      v[k] = tex(in[k], names[k]);
  }
  const float a[3] = {v[0].r, v[0].g, v[0].b}, d[3] = {v[1].r, v[1].g, v[1].b}, s[3] = {v[2].r, v[2].g, v[2].b};
  std::memcpy(m.ka, a, sizeof(a));
  std::memcpy(m.kd, d, sizeof(d));
  std::memcpy(m.ks, s, sizeof(s));
  m.ns = v[3].r;
  auto mat = std::make_shared<Material>(m);
  for (int k = 0; k < 4; ++k) mat->maps[k] = maps[k];
  return mat;
}

RC<Material> create_glass(RC<const Texture2D> map_kr, RC<const Texture2D> map_kt, RC<const Texture2D> map_ior) {
  tr_material m{};
  m.kind = TR_MAT_GLASS;
  Args a;
  const Spectrum kr = a.col(map_kr, "kr", 0), kt = a.col(map_kt, "kt", 1);
  const float r[3] = {kr.r, kr.g, kr.b}, t[3] = {kt.r, kt.g, kt.b};
  std::memcpy(m.kr, r, sizeof(r));
  std::memcpy(m.kt, t, sizeof(t));
  m.ior = a.scl(map_ior, "ior", 2);
  return a.make(m);
}

RC<Material> create_disney(RC<const Texture2D> base_color, RC<const Texture2D> metallic,
                           RC<const Texture2D> roughness, RC<const Texture2D> transmission,
                           RC<const Texture2D> transmission_roughness, RC<const Texture2D> ior,
                           RC<const Texture2D> specular_scale, RC<const Texture2D> specular_tint,
                           RC<const Texture2D> anisotropic, RC<const Texture2D> sheen,
                           RC<const Texture2D> sheen_tint, RC<const Texture2D> clearcoat,
                           RC<const Texture2D> clearcoat_gloss) {
  tr_material m{};
  m.kind = TR_MAT_DISNEY15;
  Args a;
  const Spectrum bc = a.col(base_color, "base_color", 0), ss = a.col(specular_scale, "specular_scale", 6);
  const float b3[3] = {bc.r, bc.g, bc.b}, s3[3] = {ss.r, ss.g, ss.b};
  std::memcpy(m.base_color, b3, sizeof(b3));
  std::memcpy(m.specular_scale, s3, sizeof(s3));
  m.metallic = a.scl(metallic, "metallic", 1);
  m.roughness = a.scl(roughness, "roughness", 2);
  m.transmission = a.scl(transmission, "transmission", 3);
  m.transmission_roughness = a.scl(transmission_roughness, "transmission_roughness", 4);
  m.ior = a.scl(ior, "ior", 5);
  m.specular_tint = a.scl(specular_tint, "specular_tint", 7);
  m.anisotropic = a.scl(anisotropic, "anisotropic", 8);
  m.sheen = a.scl(sheen, "sheen", 9);
  m.sheen_tint = a.scl(sheen_tint, "sheen_tint", 10);
  m.clearcoat = a.scl(clearcoat, "clearcoat", 11);
  m.clearcoat_gloss = a.scl(clearcoat_gloss, "clearcoat_gloss", 12);
  return a.make(m);
}

RC<Material> create_metal(RC<const Texture2D> color, RC<const Texture2D> eta, RC<const Texture2D> k,
                          RC<const Texture2D> roughness, RC<const Texture2D> anisotropic) {
  tr_material m{};
  m.kind = TR_MAT_METAL;
  Args a;
  const Spectrum c = a.col(color, "color", 0), e = a.col(eta, "eta", 1), kk = a.col(k, "k", 2);
  const float cv[3] = {c.r, c.g, c.b}, ev[3] = {e.r, e.g, e.b}, kv[3] = {kk.r, kk.g, kk.b};
  std::memcpy(m.color, cv, sizeof(cv));
  std::memcpy(m.eta, ev, sizeof(ev));
  std::memcpy(m.k, kv, sizeof(kv));
  m.roughness = a.scl(roughness, "roughness", 3);
  m.anisotropic = a.scl(anisotropic, "anisotropic", 4);
  return a.make(m);
}

RC<Material> create_disney_brdf(RC<const Texture2D> base_color, RC<const Texture2D> subsurface,
                                RC<const Texture2D> metallic, RC<const Texture2D> specular,
                                RC<const Texture2D> specular_tint, RC<const Texture2D> roughness,
                                RC<const Texture2D> anisotropic, RC<const Texture2D> sheen,
                                RC<const Texture2D> sheen_tint, RC<const Texture2D> clearcoat,
                                RC<const Texture2D> clearcoat_gloss) {
  tr_material m{};
  m.kind = TR_MAT_DISNEY12;
  Args a;
  const Spectrum bc = a.col(base_color, "base_color", 0);
  m.base_color[0] = bc.r;
  m.base_color[1] = bc.g;
  m.base_color[2] = bc.b;
  m.subsurface = a.scl(subsurface, "subsurface", 1);
  m.metallic = a.scl(metallic, "metallic", 2);
  m.specular = a.scl(specular, "specular", 3);
  m.specular_tint = a.scl(specular_tint, "specular_tint", 4);
  m.roughness = a.scl(roughness, "roughness", 5);
  m.anisotropic = a.scl(anisotropic, "anisotropic", 6);
  m.sheen = a.scl(sheen, "sheen", 7);
  m.sheen_tint = a.scl(sheen_tint, "sheen_tint", 8);
  m.clearcoat = a.scl(clearcoat, "clearcoat", 9);
  m.clearcoat_gloss = a.scl(clearcoat_gloss, "clearcoat_gloss", 10);
  return a.make(m);
}

RC<Medium> create_vacuum() { return std::make_shared<VacuumMedium>(); }

RC<Primitive> create_geometric_primitive(const RC<Shape>& shape, const RC<Material>& material,
                                         const MediumInterface& mi, const Spectrum& emission) {
  if (!shape) throw std::invalid_argument("null shape");
  for (const RC<const Medium>& m : {mi.inside, mi.outside})
    if (m && !dynamic_cast<const VacuumMedium*>(m.get()))
      throw std::invalid_argument("only the vacuum medium is on the GPU path");
  return std::make_shared<GeometricPrimitive>(shape, material, emission);
}

RC<Aggregate> create_bvh_accel(int max_leaf_primitives) {
  if (max_leaf_primitives < 1) throw std::invalid_argument("max_leaf_primitives must be >= 1");
  return std::make_shared<BvhAggregate>(max_leaf_primitives);
}

RC<Camera> create_thin_lens_camera(real film_aspect, const Point3f& cam_pos, const Point3f& target,
                                   const Vector3f& up, real fov, real lens_radius, real focal_dist) {
  tr_camera c{};
  c.film_aspect = film_aspect;
  const float p[3] = {cam_pos.x, cam_pos.y, cam_pos.z}, t[3] = {target.x, target.y, target.z},
              u[3] = {up.x, up.y, up.z};
  std::memcpy(c.pos, p, sizeof(p));
  std::memcpy(c.target, t, sizeof(t));
  std::memcpy(c.up, u, sizeof(u));
  c.fov = fov;
  c.lens_radius = lens_radius;
  c.focal_dist = focal_dist;
  return std::make_shared<Camera>(c);
}

RC<Filter> create_gaussin_filter(real radius, real alpha) {
  if (!(radius > 0)) throw std::invalid_argument("filter radius must be positive");
  return std::make_shared<Filter>(tr_filter{radius, alpha});
}

RC<Scene> create_general_scene(const RC<Aggregate>& accel) {
  auto b = std::dynamic_pointer_cast<BvhAggregate>(accel);
  if (!b) throw std::invalid_argument("aggregate not made by create_bvh_accel");
  return std::make_shared<GeneralScene>(b);
}

RC<GpuPathTraceRenderer> create_gpu_pt_renderer(const GPUPTRendererParams& params) {
  return std::make_shared<GpuRenderer>(params);
}

tr_scene_desc SceneDesc::view() const {
  tr_scene_desc d{};
  d.num_vertices = (uint32_t)(positions.size() / 3);
  d.positions = positions.data();
  d.normals = normals.data();
  d.uvs = uvs.data();
  d.num_triangles = (uint32_t)(indices.size() / 3);
  d.indices = indices.data();
  d.num_spheres = (uint32_t)sphere_radius.size();
  d.sphere_radius = sphere_radius.data();
  d.sphere_to_world = sphere_to_world.data();
  d.sphere_to_local = sphere_to_local.data();
  d.num_materials = (uint32_t)materials.size();
  d.materials = materials.data();
  d.num_prims = (uint32_t)prim_shape.size();
  d.prim_shape = prim_shape.data();
  d.prim_material = prim_material.data();
  d.prim_emission = prim_emission.data();
  d.num_lights = (uint32_t)light_prims.size();
  d.light_prims = light_prims.data();
  d.max_leaf_prims = max_leaf_prims;
  texture_recs_.resize(textures.size());
  for (size_t k = 0; k < textures.size(); ++k) {
    texture_recs_[k].width = textures[k].width;
    texture_recs_[k].height = textures[k].height;
    texture_recs_[k].texels = textures[k].texels.empty() ? nullptr : textures[k].texels.data();
    texture_recs_[k].texels8 = textures[k].texels8.empty() ? nullptr : textures[k].texels8.data();
  }
  d.num_textures = (uint32_t)textures.size();
  d.textures = texture_recs_.empty() ? nullptr : texture_recs_.data();
  if (env_width && env_height) {
    d.env_width = env_width;
    d.env_height = env_height;
    d.env_texels = env_texels.empty() ? nullptr : env_texels.data();
    d.env_texels8 = env_texels8.empty() ? nullptr : env_texels8.data();
    d.env_to_light = env_to_light.data();
    d.env_to_world = env_to_world.data();
  }
  return d;
}

}  // namespace tracer
