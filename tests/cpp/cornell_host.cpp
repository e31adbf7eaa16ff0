// cornell_host.cpp -- builds the Cornell box through the C++ factory API
// (include/tracer_gb300.hpp) the way a Tracer program builds a scene
// (reference src/main.cpp:226-294), then optionally renders it with
// create_gpu_pt_renderer.
//
//   cornell_host <out_prefix> <width> <height> <spp> [render]
//
// Writes <out_prefix>.desc (the uploaded scene description) and, with
// "render", <out_prefix>.sums (width*height*4 doubles: r, g, b, weight) and
// <out_prefix>.rgb (width*height*3 floats: the RenderTarget).
// Also checks that construction errors throw as the reference's do.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <string>

#include "tracer_gb300.hpp"

using namespace tracer;

namespace {

mesh_t quad_mesh(Point3f p0, Point3f p1, Point3f p2, Point3f p3, Normal3f n) {
  mesh_t m;
  m.name = "quad";
  const Point2f uv[4] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
  const Point3f p[4] = {p0, p1, p2, p3};
  for (int i = 0; i < 4; ++i) m.vertices.push_back(vertex_t{p[i], n, uv[i]});
  m.indices = {0, 1, 2, 0, 2, 3};
  return m;
}

// unit cube [-0.5, 0.5]^3, 6 faces x 2 triangles, outward normals
mesh_t cube_mesh() {
  mesh_t m;
  m.name = "cube";
  for (int axis = 0; axis < 3; ++axis)
    for (int sgn = -1; sgn <= 1; sgn += 2) {
      const int u = (axis + 1) % 3, v = (axis + 2) % 3;
      float n[3] = {0, 0, 0};
      n[axis] = (float)sgn;
      const int base = (int)m.vertices.size();
      const float su[4] = {-0.5f, 0.5f, 0.5f, -0.5f}, sv[4] = {-0.5f, -0.5f, 0.5f, 0.5f};
      for (int k = 0; k < 4; ++k) {
        float c[3];
        c[axis] = 0.5f * sgn;
        c[u] = su[k];
        c[v] = sv[k];
        m.vertices.push_back(vertex_t{{c[0], c[1], c[2]}, {n[0], n[1], n[2]}, {su[k] + 0.5f, sv[k] + 0.5f}});
      }
      // wind so that cross(B - A, C - A) points along the outward normal
      if (sgn > 0) m.indices.insert(m.indices.end(), {base, base + 1, base + 2, base, base + 2, base + 3});
      else m.indices.insert(m.indices.end(), {base, base + 2, base + 1, base, base + 3, base + 2});
    }
  return m;
}

template <class T>
void put(FILE* f, const std::vector<T>& v) {
  const uint64_t n = v.size();
  std::fwrite(&n, 8, 1, f);
  if (n) std::fwrite(v.data(), sizeof(T), n, f);
}

bool throws(void (*fn)()) {
  try {
    fn();
  } catch (const std::exception&) {
    return true;
  }
  return false;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s out_prefix width height spp [render|describe] [glass_metal]\n", argv[0]);
    return 2;
  }
  const std::string out = argv[1];
  const int W = std::atoi(argv[2]), H = std::atoi(argv[3]), spp = std::atoi(argv[4]);
  const bool render = argc > 5 && std::strcmp(argv[5], "render") == 0;
  // the short box in metal and the tall one in glass; an environment light
  const bool glass_metal = argc > 6 && std::strstr(argv[6], "glass_metal") != nullptr;
  const bool sky = argc > 6 && std::strstr(argv[6], "sky") != nullptr;
  const bool d15 = argc > 6 && std::strstr(argv[6], "disney15") != nullptr;
  const bool textured = argc > 6 && std::strstr(argv[6], "textured") != nullptr;

  // construction errors throw (src/shape/sphere.cpp:88-90)
  if (!throws([] { create_sphere(-1.0f, Transform()); }) ||
      !throws([] { create_gaussin_filter(0.0f, 1.0f); }) ||
      !throws([] { create_triangle_mesh(mesh_t{"bad", {}, {0, 1, 2}, {}}, Transform()); })) {
    std::fprintf(stderr, "construction error not reported\n");
    return 1;
  }

  auto konst = [](float r, float g, float b) { return create_constant_texture2d(Spectrum(r, g, b)); };
  auto zero = konst(0, 0, 0);
  auto white = create_phong_material(zero, konst(0.73f, 0.73f, 0.73f), zero, konst(1, 1, 1));
  auto red = create_phong_material(zero, konst(0.65f, 0.05f, 0.05f), zero, konst(1, 1, 1));
  auto green = create_phong_material(zero, konst(0.12f, 0.45f, 0.15f), zero, konst(1, 1, 1));
  auto metal = create_metal(konst(0.95f, 0.64f, 0.54f), konst(0.2f, 0.92f, 1.1f), konst(3.9f, 2.45f, 2.14f),
                            konst(0.35f, 0.35f, 0.35f), konst(0.4f, 0.4f, 0.4f));
  auto glass = create_glass(konst(1, 1, 1), konst(1, 1, 1), konst(1.5f, 1.5f, 1.5f));
  // 2015 Disney: a rough transmitter and an anisotropic, clearcoated metal
  auto d15_trans = create_disney(konst(0.9f, 0.9f, 0.9f), konst(0, 0, 0), konst(0.2f, 0.2f, 0.2f),
                                 konst(0.8f, 0.8f, 0.8f), konst(0.3f, 0.3f, 0.3f), konst(1.5f, 1.5f, 1.5f),
                                 konst(1, 1, 1), zero, zero, zero, zero, zero, zero);
  auto d15_metal = create_disney(konst(0.9f, 0.7f, 0.4f), konst(0.9f, 0.9f, 0.9f), konst(0.3f, 0.3f, 0.3f), zero,
                                 zero, konst(1.5f, 1.5f, 1.5f), zero, konst(0.2f, 0.2f, 0.2f), konst(0.5f, 0.5f, 0.5f),
                                 zero, zero, konst(0.6f, 0.6f, 0.6f), konst(0.5f, 0.5f, 0.5f));
  // an 8-bit checkerboard kd for the floor (create_image_texture2d)
  auto board = std::make_shared<Image2D<Color3b>>(8, 8);
  for (int y = 0; y < 8; ++y)
    for (int x = 0; x < 8; ++x)
      board->at(x, y) = ((x / 2 + y / 2) % 2) ? Color3b{30, 80, 200} : Color3b{220, 210, 190};
  auto floor_mat = textured ? create_phong_material(zero, create_image_texture2d(board), zero, konst(1, 1, 1)) : white;
  auto vacuum = create_vacuum();
  const MediumInterface mi(vacuum);

  std::vector<RC<Primitive>> primitives;
  Span<const Light*> area_lights;
  auto add = [&](const mesh_t& mesh, const Transform& t, const RC<Material>& mat, const Spectrum& emission) {
    for (auto& shape : create_triangle_mesh(mesh, t)) {
      primitives.push_back(create_geometric_primitive(shape, mat, mi, emission));
      if (emission) area_lights.emplace_back(primitives.back()->as_area_light());
    }
  };
  const Transform id;
  const Spectrum black;
  add(quad_mesh({-1, -1, -1}, {-1, -1, 1}, {1, -1, 1}, {1, -1, -1}, {0, 1, 0}), id, floor_mat, black);  // floor
  add(quad_mesh({-1, 1, -1}, {1, 1, -1}, {1, 1, 1}, {-1, 1, 1}, {0, -1, 0}), id, white, black);       // ceiling
  add(quad_mesh({-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {0, 0, 1}), id, white, black);    // back
  add(quad_mesh({-1, -1, -1}, {-1, 1, -1}, {-1, 1, 1}, {-1, -1, 1}, {1, 0, 0}), id, red, black);      // left
  add(quad_mesh({1, -1, -1}, {1, -1, 1}, {1, 1, 1}, {1, 1, -1}, {-1, 0, 0}), id, green, black);       // right
  const float pi = 3.14159265358979f;
  add(cube_mesh(), translate({-0.35f, -0.7f, -0.3f}) * rotate_y(15.0f * pi / 180.0f) * scale(0.6f, 0.6f, 0.6f),
      glass_metal ? metal : (d15 ? d15_metal : white), black);
  add(cube_mesh(), translate({0.35f, -0.4f, 0.3f}) * rotate_y(-18.0f * pi / 180.0f) * scale(0.6f, 1.2f, 0.6f),
      glass_metal ? glass : (d15 ? d15_trans : white), black);
  add(quad_mesh({-0.25f, 0.99f, -0.25f}, {0.25f, 0.99f, -0.25f}, {0.25f, 0.99f, 0.25f}, {-0.25f, 0.99f, 0.25f},
                {0, -1, 0}),
      id, white, Spectrum(17, 12, 4));

  auto bvh = create_bvh_accel(3);
  bvh->build(std::move(primitives));
  auto scene = create_general_scene(bvh);
  scene->lights = area_lights;
  if (sky) {
    // a 32 x 16 map: a blue-to-white sky, a dark ground, a bright sun texel
    auto img = std::make_shared<Image2D<Color3f>>(32, 16);
    for (int y = 0; y < 16; ++y)
      for (int x = 0; x < 32; ++x) {
        const float t = std::min(1.0f, (float)y / 7.5f);
        img->at(x, y) = y < 8 ? Color3f{0.25f + 0.65f * t, 0.45f + 0.45f * t, 0.9f + 0.1f * t}
                              : Color3f{0.18f, 0.14f, 0.1f};
      }
    img->at(5, 3) = Color3f{120.0f, 110.0f, 90.0f};
    scene->environment_light = create_ibl_light(create_hdr_texture2d(img), rotate_x(3.14159265358979f / 2));
    scene->lights.push_back(scene->environment_light.get());
  }
  scene->set_camera(create_thin_lens_camera((float)W / (float)H, {0, 0, 3.5f}, {0, 0, 0}, {0, 1, 0},
                                            40.0f * pi / 180.0f, 0.0f, 1.0f));
  scene->prepare_to_render();

  const SceneDesc& d = scene->desc();
  FILE* f = std::fopen((out + ".desc").c_str(), "wb");
  if (!f) return 3;
  put(f, d.positions);
  put(f, d.normals);
  put(f, d.uvs);
  put(f, d.indices);
  put(f, d.sphere_radius);
  put(f, d.sphere_to_world);
  put(f, d.sphere_to_local);
  put(f, d.materials);
  put(f, d.prim_shape);
  put(f, d.prim_material);
  put(f, d.prim_emission);
  put(f, d.light_prims);
  std::fwrite(&d.max_leaf_prims, 4, 1, f);
  std::fwrite(&scene->get_camera()->rec, sizeof(tr_camera), 1, f);
  std::fwrite(&d.env_width, 4, 1, f);
  std::fwrite(&d.env_height, 4, 1, f);
  put(f, d.env_texels);
  put(f, d.env_to_light);
  put(f, d.env_to_world);
  const uint32_t ntex = (uint32_t)d.textures.size();
  std::fwrite(&ntex, 4, 1, f);
  for (const auto& t : d.textures) {
    std::fwrite(&t.width, 4, 1, f);
    std::fwrite(&t.height, 4, 1, f);
    put(f, t.texels);
    put(f, t.texels8);
  }
  std::fclose(f);
  std::printf("scene: %zu triangles, %zu lights, %zu materials\n", d.indices.size() / 3, d.light_prims.size(),
              d.materials.size());
  if (!render) return 0;

  GPUPTRendererParams params;
  params.spp = spp;
  params.min_depth = 5;
  params.max_depth = 5;
  auto renderer = create_gpu_pt_renderer(params);
  auto filter = create_gaussin_filter(0.5f, 0.6f);
  RenderTarget rt = renderer->render(*scene, Film({W, H}, filter));
  const tr_stats st = renderer->last_stats();
  std::printf("rendered: %llu samples, %llu extend + %llu shadow rays\n", (unsigned long long)st.samples,
              (unsigned long long)st.extend_rays, (unsigned long long)st.shadow_rays);
  f = std::fopen((out + ".sums").c_str(), "wb");
  if (!f) return 3;
  std::fwrite(renderer->film_sums().data(), sizeof(double), renderer->film_sums().size(), f);
  std::fclose(f);
  f = std::fopen((out + ".rgb").c_str(), "wb");
  if (!f) return 3;
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) std::fwrite(&rt.color.at(x, y), sizeof(float), 3, f);
  std::fclose(f);
  return 0;
}
