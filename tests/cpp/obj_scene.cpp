// The reference's OBJ scene flow through the C++ host API
// (include/tracer_gb300.hpp): load_model_from_file, create_texture_from_file
// per MTL material, create_phong_material (or create_glass), one
// create_triangle_mesh per mesh, an area light from the emissive material,
// the scene, prepare_to_render. Writes the scene description, in
// tests/cpp/cornell_host.cpp's format, for tests/test_obj_scene.py.
//   obj_scene <scene.obj> <out_prefix>
#include <cstdio>
#include <string>
#include <vector>

#include "tracer_gb300.hpp"

using namespace tracer;

namespace {

template <class T>
void put(FILE* f, const std::vector<T>& v) {
  const uint64_t n = v.size();
  std::fwrite(&n, 8, 1, f);
  if (n) std::fwrite(v.data(), sizeof(T), n, f);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  try {
    const model_t model = load_model_from_file(argv[1]);
    std::vector<RC<Material>> materials;
    std::vector<Spectrum> emission;
    for (const material_t& mt : model.material) {
      const MaterialTexture t = create_texture_from_file(mt);
      materials.push_back(t.as_glass ? create_glass(t.map_ks, t.map_kt, t.ior)
                                     : create_phong_material(t.map_ka, t.map_kd, t.map_ks, t.map_ns));
      emission.push_back(t.has_emission ? t.map_ke->evaluate(Point2f{0, 0}) : Spectrum());
    }
    auto vacuum = create_vacuum();
    std::vector<RC<Primitive>> primitives;
    Span<const Light*> lights;
    for (const mesh_t& mesh : model.mesh) {
      auto shapes = create_triangle_mesh(mesh, Transform());
      for (size_t t = 0; t < shapes.size(); ++t) {
        const int mi = mesh.materials[t];
        if (mi < 0) throw TracerError(TR_ERR_ARG, "triangle without material");
        primitives.push_back(create_geometric_primitive(shapes[t], materials[mi], MediumInterface(vacuum),
                                                        emission[mi]));
        if (emission[mi]) lights.push_back(primitives.back()->as_area_light());
      }
    }
    auto bvh = create_bvh_accel(3);
    bvh->build(std::move(primitives));
    auto scene = create_general_scene(bvh);
    scene->lights = lights;
    scene->set_camera(create_thin_lens_camera(1.0f, {0, 0, 3.5f}, {0, 0, 0}, {0, 1, 0}, 0.7f, 0.0f, 1.0f));
    scene->prepare_to_render();
    const SceneDesc& d = scene->desc();
    FILE* f = std::fopen((std::string(argv[2]) + ".desc").c_str(), "wb");
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
    std::printf("scene: %zu triangles, %zu lights, %zu materials, %zu textures\n", d.indices.size() / 3,
                d.light_prims.size(), d.materials.size(), d.textures.size());
  } catch (const TracerError& e) {
    std::printf("error %d %s\n", (int)e.status, e.what());
    return 1;
  }
  return 0;
}
