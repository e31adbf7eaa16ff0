// ref_harness.cpp -- extern "C" entry points around the UNMODIFIED reference
// sources of wyzwzz/Tracer, compiled from where they lie by oracle/Makefile.
//
// Test infrastructure only. It exists to pin the CPU restatement
// (oracle/tracer_oracle.cpp) against the reference itself and to generate the
// golden fixtures under tests/golden/. Nothing in the product links it.
//
// It builds a scene through the reference's own factory API and calls:
//  * Scene::intersect_p / Scene::intersect        (src/core/scene.cpp:32-38)
//  * PathTraceRenderer::eval_pixel_li per camera sample, with one
//    SimpleUniformSampler per pixel seeded by the pixel index -- the body of
//    PixelSamplerRenderer::render (src/renderer/pixel_sampler_renderer.cpp:60-94)
//  * the stock create_pt_renderer(...)->render(...) for CPU timing.

#include "renderer/path_trace_renderer.cpp"  // PathTraceRenderer (eval_pixel_li is public)
// BVHAccel keeps its flattened nodes private; open them to read the tree out.
#define private public
#include "accelerator/bvh.cpp"
#undef private

#include <chrono>
#include <thread>
#include <unordered_map>
#include <vector>

#include "core/bssrdf.hpp"
#include "core/camera.hpp"
#include "core/light.hpp"
#include "core/render.hpp"
#include "core/sampler.hpp"
#include "core/scene.hpp"
#include "factory/accelerator.hpp"
#include "factory/camera.hpp"
#include "factory/filter.hpp"
#include "factory/light.hpp"
#include "factory/material.hpp"
#include "factory/medium.hpp"
#include "factory/primivite.hpp"
#include "factory/renderer.hpp"
#include "factory/scene.hpp"
#include "factory/shape.hpp"
#include "factory/texture.hpp"
#include "utility/image.hpp"
#include "utility/transform.hpp"

#include "tracer_gpu.h"

using namespace tracer;

namespace {

struct RefScene {
  std::vector<RC<Material>> materials;
  std::vector<RC<Primitive>> prims;
  std::unordered_map<const Primitive*, int32_t> id_of;
  RC<Aggregate> bvh;
  RC<Scene> scene;
  RC<Camera> camera;
  RC<Filter> filter;
};

Matrix4x4 to_matrix(const float* m) {
  real a[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) a[i][j] = m[4 * i + j];
  return Matrix4x4(a);
}

RC<Texture2D> ctex(float v) { return create_constant_texture2d(Spectrum(v)); }
RC<Texture2D> ctex3(const float* v) { return create_constant_texture2d(Spectrum(v[0], v[1], v[2])); }

template <class F>
void parallel_rows(int n, int threads, F&& f) {
  if (threads <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&] {
      for (;;) {
        int i = next++;
        if (i >= n) return;
        f(i);
      }
    });
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

void* ref_scene_create(const tr_scene_desc* d) {
  auto* s = new RefScene();
  auto vacuum = create_vacuum();
  MediumInterface mi;
  mi.inside = vacuum;
  mi.outside = vacuum;

  // image textures of the materials (create_hdr_texture2d / create_image_texture2d)
  std::vector<RC<Texture2D>> textures;
  for (uint32_t k = 0; k < d->num_textures; ++k) {
    const tr_texture& t = d->textures[k];
    if (t.texels) {
      auto img = newRC<Image2D<Color3f>>((int)t.width, (int)t.height);
      for (uint32_t y = 0; y < t.height; ++y)
        for (uint32_t x = 0; x < t.width; ++x) {
          const float* p = t.texels + 3 * ((size_t)x + (size_t)y * t.width);
          img->at((int)x, (int)y) = Color3f(p[0], p[1], p[2]);
        }
      textures.push_back(create_hdr_texture2d(img));
    } else {
      auto img = newRC<Image2D<Color3b>>((int)t.width, (int)t.height);
      for (uint32_t y = 0; y < t.height; ++y)
        for (uint32_t x = 0; x < t.width; ++x) {
          const uint8_t* p = t.texels8 + 3 * ((size_t)x + (size_t)y * t.width);
          img->at((int)x, (int)y) = Color3b(p[0], p[1], p[2]);
        }
      textures.push_back(create_image_texture2d(img));
    }
  }
  auto map = [&](uint32_t k, RC<Texture2D> constant) { return k ? textures[k - 1] : constant; };
  for (uint32_t i = 0; i < d->num_materials; ++i) {
    const tr_material& m = d->materials[i];
    if (m.kind == TR_MAT_PHONG) {
      s->materials.push_back(create_phong_material(map(m.tex_ka, ctex3(m.ka)), map(m.tex_kd, ctex3(m.kd)),
                                                   map(m.tex_ks, ctex3(m.ks)), map(m.tex_ns, ctex(m.ns))));
    } else if (m.kind == TR_MAT_GLASS) {
      const uint32_t* t = m.tex_param;  // the factory's arguments: image maps or constants
      s->materials.push_back(create_glass(map(t[0], ctex3(m.kr)), map(t[1], ctex3(m.kt)), map(t[2], ctex(m.ior))));
    } else if (m.kind == TR_MAT_DISNEY15) {
      const uint32_t* t = m.tex_param;
      s->materials.push_back(create_disney(
          map(t[0], ctex3(m.base_color)), map(t[1], ctex(m.metallic)), map(t[2], ctex(m.roughness)),
          map(t[3], ctex(m.transmission)), map(t[4], ctex(m.transmission_roughness)), map(t[5], ctex(m.ior)),
          map(t[6], ctex3(m.specular_scale)), map(t[7], ctex(m.specular_tint)), map(t[8], ctex(m.anisotropic)),
          map(t[9], ctex(m.sheen)), map(t[10], ctex(m.sheen_tint)), map(t[11], ctex(m.clearcoat)),
          map(t[12], ctex(m.clearcoat_gloss)), newBox<const NormalMapper>(nullptr), newRC<BSSRDFSurface>()));
    } else if (m.kind == TR_MAT_METAL) {
      const uint32_t* t = m.tex_param;
      s->materials.push_back(create_metal(map(t[0], ctex3(m.color)), map(t[1], ctex3(m.eta)), map(t[2], ctex3(m.k)),
                                          map(t[3], ctex(m.roughness)), map(t[4], ctex(m.anisotropic)),
                                          newBox<NormalMapper>()));
    } else {
      const uint32_t* t = m.tex_param;
      s->materials.push_back(create_disney_brdf(
          map(t[0], ctex3(m.base_color)), map(t[1], ctex(m.subsurface)), map(t[2], ctex(m.metallic)),
          map(t[3], ctex(m.specular)), map(t[4], ctex(m.specular_tint)), map(t[5], ctex(m.roughness)),
          map(t[6], ctex(m.anisotropic)), map(t[7], ctex(m.sheen)), map(t[8], ctex(m.sheen_tint)),
          map(t[9], ctex(m.clearcoat)), map(t[10], ctex(m.clearcoat_gloss))));
    }
  }

  std::vector<RC<Shape>> tris;
  if (d->num_triangles) {
    mesh_t mesh;
    mesh.vertices.resize(d->num_vertices);
    for (uint32_t v = 0; v < d->num_vertices; ++v) {
      mesh.vertices[v].pos = Point3f(d->positions[3 * v], d->positions[3 * v + 1], d->positions[3 * v + 2]);
      mesh.vertices[v].n = Normal3f(d->normals[3 * v], d->normals[3 * v + 1], d->normals[3 * v + 2]);
      mesh.vertices[v].uv = Point2f(d->uvs[2 * v], d->uvs[2 * v + 1]);
    }
    mesh.indices.assign(d->indices, d->indices + 3 * d->num_triangles);
    tris = create_triangle_mesh(mesh, Transform());
  }
  std::vector<RC<Shape>> spheres;
  for (uint32_t i = 0; i < d->num_spheres; ++i) {
    Transform t(to_matrix(d->sphere_to_world + 16 * i), to_matrix(d->sphere_to_local + 16 * i));
    spheres.push_back(create_sphere(d->sphere_radius[i], t));
  }
  for (uint32_t p = 0; p < d->num_prims; ++p) {
    int32_t sh = d->prim_shape[p];
    RC<Shape> shape = sh >= 0 ? tris[sh] : spheres[~sh];
    const float* e = d->prim_emission + 3 * p;
    s->prims.push_back(create_geometric_primitive(shape, s->materials[d->prim_material[p]], mi,
                                                  Spectrum(e[0], e[1], e[2])));
    s->id_of[s->prims.back().get()] = (int32_t)p;
  }
  s->bvh = create_bvh_accel(d->max_leaf_prims);
  s->bvh->build(s->prims);
  s->scene = create_general_scene(s->bvh);
  for (uint32_t l = 0; l < d->num_lights; ++l)
    s->scene->lights.push_back(s->prims[d->light_prims[l]]->as_area_light());
  if ((d->env_texels || d->env_texels8) && d->env_width > 0 && d->env_height > 0) {
    // the demo driver's environment light (src/main.cpp:59-67) over an HDR or 8-bit image
    RC<Texture2D> tex;
    if (d->env_texels) {
      auto img = newRC<Image2D<Color3f>>((int)d->env_width, (int)d->env_height);
      for (uint32_t y = 0; y < d->env_height; ++y)
        for (uint32_t x = 0; x < d->env_width; ++x) {
          const float* t = d->env_texels + 3 * ((size_t)x + (size_t)y * d->env_width);
          img->at((int)x, (int)y) = Color3f(t[0], t[1], t[2]);
        }
      tex = create_hdr_texture2d(img);
    } else {
      auto img = newRC<Image2D<Color3b>>((int)d->env_width, (int)d->env_height);
      for (uint32_t y = 0; y < d->env_height; ++y)
        for (uint32_t x = 0; x < d->env_width; ++x) {
          const uint8_t* t = d->env_texels8 + 3 * ((size_t)x + (size_t)y * d->env_width);
          img->at((int)x, (int)y) = Color3b(t[0], t[1], t[2]);
        }
      tex = create_image_texture2d(img);
    }
    auto ibl = create_ibl_light(tex, Transform(to_matrix(d->env_to_light), to_matrix(d->env_to_world)));
    s->scene->environment_light = ibl;
    s->scene->lights.push_back(ibl.get());
  }
  s->scene->prepare_to_render();
  return s;
}

void ref_scene_destroy(void* h) { delete static_cast<RefScene*>(h); }

void ref_set_camera(void* h, const tr_camera* c, const tr_filter* f) {
  auto* s = static_cast<RefScene*>(h);
  s->camera = create_thin_lens_camera(c->film_aspect, Point3f(c->pos[0], c->pos[1], c->pos[2]),
                                      Point3f(c->target[0], c->target[1], c->target[2]),
                                      Vector3f(c->up[0], c->up[1], c->up[2]), c->fov,
                                      c->lens_radius, c->focal_dist);
  s->scene->set_camera(s->camera);
  s->filter = create_gaussin_filter(f->radius, f->alpha);
}

void ref_trace_closest(void* h, const tr_ray* rays, size_t n, int32_t* prim, float* t, int threads) {
  auto* s = static_cast<RefScene*>(h);
  const size_t chunk = 4096;
  parallel_rows((int)((n + chunk - 1) / chunk), threads, [&](int c) {
    for (size_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) {
      Ray r;
      r.o = Point3f(rays[i].o[0], rays[i].o[1], rays[i].o[2]);
      r.d = Vector3f(rays[i].d[0], rays[i].d[1], rays[i].d[2]);
      r.t_min = rays[i].t_min;
      r.t_max = rays[i].t_max;
      SurfaceIntersection isect;
      bool hit = s->scene->intersect_p(r, &isect);
      prim[i] = hit ? s->id_of.at(isect.primitive) : -1;
      t[i] = r.t_max;
    }
  });
}

void ref_trace_any(void* h, const tr_ray* rays, size_t n, uint8_t* hit, int threads) {
  auto* s = static_cast<RefScene*>(h);
  const size_t chunk = 4096;
  parallel_rows((int)((n + chunk - 1) / chunk), threads, [&](int c) {
    for (size_t i = c * chunk; i < std::min(n, (c + 1) * chunk); ++i) {
      Ray r;
      r.o = Point3f(rays[i].o[0], rays[i].o[1], rays[i].o[2]);
      r.d = Vector3f(rays[i].d[0], rays[i].d[1], rays[i].d[2]);
      r.t_min = rays[i].t_min;
      r.t_max = rays[i].t_max;
      hit[i] = s->scene->intersect(r) ? 1 : 0;
    }
  });
}

// Reference Ray constructor (src/utility/geometry.hpp:791-792).
void ref_make_ray(const float* o, const float* d, float t_min, float t_max, tr_ray* out) {
  Ray r(Point3f(o[0], o[1], o[2]), Vector3f(d[0], d[1], d[2]), t_min, t_max);
  out->o[0] = r.o.x; out->o[1] = r.o.y; out->o[2] = r.o.z;
  out->d[0] = r.d.x; out->d[1] = r.d.y; out->d[2] = r.d.z;
  out->t_min = r.t_min; out->t_max = r.t_max;
}

// Per-pixel-seeded render: pixel (x, y) owns SimpleUniformSampler((int)(seed_base + y*W + x))
// and runs the body of PixelSamplerRenderer::render's sample loop
// (src/renderer/pixel_sampler_renderer.cpp:60-94) into its own Film::Tile; the
// tiles are merged in pixel order like Film::merge_film_tile
// (src/core/render.hpp:90-100). Output: rgbw[4*(y*W+x)] = color sums + weight.
void ref_render(void* h, const tr_render_params* p, float* rgbw, int threads) {
  auto* s = static_cast<RefScene*>(h);
  PTRendererParams pp;
  pp.worker_count = 1;
  pp.task_tile_size = 16;
  pp.spp = p->spp;
  pp.min_depth = p->min_depth;
  pp.max_depth = p->max_depth;
  pp.direct_light_sample_num = p->direct_light_sample_num;
  PathTraceRenderer renderer(pp);
  const int W = p->width, H = p->height;
  Film film({W, H}, s->filter);
  std::vector<std::vector<Box<Film::Tile>>> rows(H);
  parallel_rows(H, threads, [&](int y) {
    MemoryArena arena;
    rows[y].resize(W);
    for (int x = 0; x < W; ++x) {
      Bounds2i pb{{x, y}, {x + 1, y + 1}};
      auto tile = film.get_film_tile(pb);
      SimpleUniformSampler sampler((int)(p->seed_base + (uint32_t)y * (uint32_t)W + (uint32_t)x));
      for (int i = 0; i < p->spp; ++i) {
        const Sample2 film_sample = sampler.sample2();
        const Sample2 lens_sample = sampler.sample2();
        const real pixel_x = x + film_sample.u;
        const real pixel_y = y + film_sample.v;
        const real film_x = pixel_x / W;
        const real film_y = pixel_y / H;
        CameraSample cs{{film_x, film_y}, {lens_sample.u, lens_sample.v}};
        Ray ray;
        real w = s->camera->generate_ray(cs, ray);
        Spectrum L(0.0);
        if (w > 0.0) L = renderer.eval_pixel_li(*s->scene, ray, sampler, arena);
        if (std::isfinite(L.r) && std::isfinite(L.g) && std::isfinite(L.b))
          tile->add_sample({pixel_x, pixel_y}, L);
        arena.reset();
      }
      rows[y][x] = std::move(tile);
    }
  });
  std::vector<Spectrum> color(W * H);
  std::vector<real> weight(W * H, 0);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      auto& tile = rows[y][x];
      for (Point2i px : tile->get_pixel_bound()) {
        const auto& tp = tile->get_pixel(px);
        int o = px.x + px.y * W;
        color[o] += tp.contrib_sum;
        weight[o] += tp.filter_weight_sum;
      }
    }
  for (int i = 0; i < W * H; ++i) {
    rgbw[4 * i + 0] = color[i].r;
    rgbw[4 * i + 1] = color[i].g;
    rgbw[4 * i + 2] = color[i].b;
    rgbw[4 * i + 3] = weight[i];
  }
}

// The stock renderer, timed: create_pt_renderer(...)->render(scene, Film)
// (src/renderer/pixel_sampler_renderer.cpp:24-109). Returns wall seconds of
// render() and writes the final image (color / weight) into rgb if non-null.
double ref_render_stock(void* h, const tr_render_params* p, int workers, float* rgb) {
  auto* s = static_cast<RefScene*>(h);
  PTRendererParams pp;
  pp.worker_count = workers;
  pp.task_tile_size = 16;
  pp.spp = p->spp;
  pp.min_depth = p->min_depth;
  pp.max_depth = p->max_depth;
  pp.direct_light_sample_num = p->direct_light_sample_num;
  auto renderer = create_pt_renderer(pp);
  auto t0 = std::chrono::steady_clock::now();
  RenderTarget rt = renderer->render(*s->scene, Film({p->width, p->height}, s->filter));
  auto t1 = std::chrono::steady_clock::now();
  if (rgb)
    for (int y = 0; y < p->height; ++y)
      for (int x = 0; x < p->width; ++x) {
        const Spectrum& c = rt.color.at(x, y);
        float* o = rgb + 3 * (y * p->width + x);
        o[0] = c.r; o[1] = c.g; o[2] = c.b;
      }
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"

extern "C" {
// Unit entry points over the reference's own inline math
// (src/utility/geometry.hpp:570-590, 837-864; src/core/sampler.hpp:30-86).
void ref_cross(const float* a, const float* b, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    Vector3f r = cross(Vector3f(a[3 * i], a[3 * i + 1], a[3 * i + 2]), Vector3f(b[3 * i], b[3 * i + 1], b[3 * i + 2]));
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
  }
}
void ref_normalize(const float* a, float* out, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    Vector3f r = normalize(Vector3f(a[3 * i], a[3 * i + 1], a[3 * i + 2]));
    out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
  }
}
void ref_pcg_uniform(int seed, float* out, size_t n) {
  SimpleUniformSampler s(seed);
  for (size_t i = 0; i < n; ++i) out[i] = s.sample1().u;
}
}

extern "C" {
// The reference's flattened BVH (BVHAccel::linear_nodes, ::primitives;
// src/accelerator/bvh.cpp:290-312). Returns the node count; with non-null
// outputs also copies the nodes and the primitive id of every leaf slot.
static size_t ref_count_nodes(const LinearBVHNode* nodes, size_t i) {
  if (nodes[i].primitive_count > 0) return 1;
  return 1 + ref_count_nodes(nodes, i + 1) + ref_count_nodes(nodes, (size_t)nodes[i].second_child_offset);
}
size_t ref_bvh_export(void* h, tr_bvh_node32* out, uint32_t* order) {
  auto* s = static_cast<RefScene*>(h);
  auto* bvh = static_cast<BVHAccel*>(s->bvh.get());
  if (!bvh->linear_nodes) return 0;
  size_t n = ref_count_nodes(bvh->linear_nodes, 0);
  if (out) {
    for (size_t i = 0; i < n; ++i) {
      const LinearBVHNode& nd = bvh->linear_nodes[i];
      out[i].lo[0] = nd.bounds.low.x; out[i].lo[1] = nd.bounds.low.y; out[i].lo[2] = nd.bounds.low.z;
      out[i].hi[0] = nd.bounds.high.x; out[i].hi[1] = nd.bounds.high.y; out[i].hi[2] = nd.bounds.high.z;
      out[i].offset = nd.primitive_offset;
      out[i].count = nd.primitive_count;
      out[i].axis = nd.primitive_count > 0 ? 0 : nd.axis;
      out[i].pad = 0;
    }
  }
  if (order)
    for (size_t i = 0; i < bvh->primitives.size(); ++i) order[i] = (uint32_t)s->id_of.at(bvh->primitives[i].get());
  return n;
}
}

#include "core/post_processor.hpp"
#include "factory/post_processor.hpp"

extern "C" {
// The reference's post-processors on a w x h RGB float image, in place:
// kind 0 create_aces_tone_mapper(param), kind 1 create_gamma_corrector(param)
// (src/post_processor/aces.cpp, src/post_processor/gamma.cpp), applied by
// PostProcessor::process to a RenderTarget holding the image.
void ref_post_process(float* rgb, int w, int h, int kind, float param) {
  RenderTarget rt;
  rt.color = Image2D<Spectrum>(w, h);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const float* p = rgb + 3 * ((size_t)y * w + x);
      rt.color.at(x, y) = Spectrum(p[0], p[1], p[2]);
    }
  RC<PostProcessor> pp = kind == 0 ? create_aces_tone_mapper(param) : create_gamma_corrector(param);
  pp->process(rt);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float* p = rgb + 3 * ((size_t)y * w + x);
      const Spectrum& c = rt.color.at(x, y);
      p[0] = c.r;
      p[1] = c.g;
      p[2] = c.b;
    }
}
}

// ---------------------------------------------------------------- images
// The reference's 8-bit image reader (load_image_from_file, src/utility/
// image_file.cpp:26-58, over its vendored stb_image: format found from the
// file's bytes, rows flipped, 1 and 4 channels to RGB) and the vendored
// stb_image_write encoders its image_file.cpp compiles, which make the
// reader-test files (JPEG, TGA, BMP) here.
#include "utility/image_file.hpp"
#include <stb_image_write.h>

extern "C" {

// Reads `path` with the reference's reader; rgb (3 * w * h bytes) may be null
// to ask for the size. Returns 0, or -1 when the reference throws.
int ref_load_image(const char* path, int* w, int* h, uint8_t* rgb) {
  try {
    auto img = load_image_from_file(path);
    *w = img->width();
    *h = img->height();
    if (rgb)
      for (int y = 0; y < *h; ++y)
        for (int x = 0; x < *w; ++x) {
          const Color3b& c = img->at(x, y);
          uint8_t* o = rgb + 3 * ((size_t)y * *w + x);
          o[0] = c.x; o[1] = c.y; o[2] = c.z;
        }
    return 0;
  } catch (...) {
    return -1;
  }
}

// kind: 0 JPEG (quality q), 1 TGA (run-length encoded unless q == 0), 2 BMP.
int ref_write_image(const char* path, int kind, int w, int h, int comp, const uint8_t* px, int q) {
  if (kind == 0) return stbi_write_jpg(path, w, h, comp, px, q);
  if (kind == 1) {
    stbi_write_tga_with_rle = q != 0;
    return stbi_write_tga(path, w, h, comp, px);
  }
  return stbi_write_bmp(path, w, h, comp, px);
}

}  // extern "C"
