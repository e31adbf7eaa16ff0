// Reads an OBJ/MTL pair with load_model_from_file and prints what it got,
// one fact per line, for tests/test_obj_load.py.
#include <cstdio>

#include "tracer_gb300.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  try {
    const tracer::model_t m = tracer::load_model_from_file(argv[1]);
    std::printf("name %s\n", m.name.c_str());
    std::printf("materials %zu\n", m.material.size());
    for (const auto& mt : m.material)
      std::printf("material %s %g %g %g %g %g %g %s\n", mt.name.c_str(), mt.diffuse[0], mt.diffuse[1], mt.diffuse[2],
                  mt.ior, mt.roughness, mt.emission[0], mt.map_kd.c_str());
    std::printf("meshes %zu\n", m.mesh.size());
    for (const auto& me : m.mesh) {
      std::printf("mesh %s %zu %zu\n", me.name.c_str(), me.vertices.size(), me.indices.size() / 3);
      for (const auto& v : me.vertices)
        std::printf("v %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g\n", v.pos.x, v.pos.y, v.pos.z, v.n.x, v.n.y, v.n.z,
                    v.uv.x, v.uv.y);
      for (size_t t = 0; t < me.indices.size() / 3; ++t)
        std::printf("t %d %d %d %d\n", me.indices[3 * t], me.indices[3 * t + 1], me.indices[3 * t + 2],
                    me.materials[t]);
    }
  } catch (const tracer::TracerError& e) {
    std::printf("error %s\n", e.what());
    return 1;
  }
  return 0;
}
