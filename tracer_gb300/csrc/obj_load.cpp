// obj_load.cpp -- load_model_from_file (src/utility/mesh_load.cpp:25-113)
// with a project-written Wavefront OBJ/MTL reader in place of the
// reference's tinyobjloader dependency: the same model_t (one mesh per
// shape, vertices deduplicated by position, normal and uv, a material id per
// triangle, the MTL materials with their map file names).
#include <cmath>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tracer_gb300.hpp"

namespace tracer {
namespace {

[[noreturn]] void fail(const std::string& path, int line, const std::string& what) {
  throw TracerError(TR_ERR_ARG, path + ":" + std::to_string(line) + ": " + what);
}

std::string dir_of(const std::string& path) {
  const size_t p = path.find_last_of("/\\");
  return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}

// extract_name_from_path (src/utility/mesh_load.cpp:7-20): from the last
// separator on (the separator included), or the whole path.
std::string name_of(const std::string& path) {
  const size_t p = path.find_last_of("/\\");
  return p == std::string::npos ? path : path.substr(p);
}

std::string rest_of(std::istringstream& in) {
  std::string r;
  std::getline(in, r);
  const size_t a = r.find_first_not_of(" \t"), b = r.find_last_not_of(" \t\r");
  return a == std::string::npos ? std::string() : r.substr(a, b - a + 1);
}

void read3(std::istringstream& in, real* v, const std::string& path, int line) {
  for (int k = 0; k < 3; ++k)
    if (!(in >> v[k])) fail(path, line, "expected three numbers");
}

void load_mtl(const std::string& path, std::vector<material_t>& out, std::unordered_map<std::string, int>& ids) {
  std::ifstream f(path);
  if (!f) throw TracerError(TR_ERR_ARG, "cannot open material library " + path);
  std::string text;
  int line = 0;
  material_t* m = nullptr;
  while (std::getline(f, text)) {
    ++line;
    std::istringstream in(text);
    std::string key;
    if (!(in >> key) || key[0] == '#') continue;
    if (key == "newmtl") {
      out.emplace_back();
      m = &out.back();
      m->name = rest_of(in);
      ids[m->name] = (int)out.size() - 1;
      continue;
    }
    if (!m) fail(path, line, "statement before newmtl");
    if (key == "Ka") read3(in, m->ambient, path, line);
    else if (key == "Kd") read3(in, m->diffuse, path, line);
    else if (key == "Ks") read3(in, m->specular, path, line);
    else if (key == "Ke") read3(in, m->emission, path, line);
    else if (key == "Tf" || key == "Kt") read3(in, m->transmittance, path, line);
    else if (key == "Ns") in >> m->shininess;
    else if (key == "Ni") in >> m->ior;
    else if (key == "d") in >> m->dissolve;
    else if (key == "Tr") {
      real tr = 0;
      in >> tr;
      m->dissolve = 1 - tr;
    } else if (key == "illum") in >> m->illum;
    else if (key == "Pr") in >> m->roughness;
    else if (key == "Pm") in >> m->metallic;
    else if (key == "Ps") in >> m->sheen;
    else if (key == "Pc") in >> m->clearcoat_thickness;
    else if (key == "Pcr") in >> m->clearcoat_roughness;
    else if (key == "map_Ka") m->map_ka = rest_of(in);
    else if (key == "map_Kd") m->map_kd = rest_of(in);
    else if (key == "map_Ks") m->map_ks = rest_of(in);
    else if (key == "map_Ns") m->map_ns = rest_of(in);
    else if (key == "map_bump" || key == "bump") m->map_bump = rest_of(in);
    else if (key == "disp") m->disp = rest_of(in);
    else if (key == "map_d") m->map_d = rest_of(in);
    else if (key == "refl") m->refl = rest_of(in);
    else if (key == "map_Pr") m->map_pr = rest_of(in);
    else if (key == "map_Pm") m->map_pm = rest_of(in);
    else if (key == "map_Ps") m->map_ps = rest_of(in);
    else if (key == "map_Ke") m->map_ke = rest_of(in);
    else if (key == "norm") m->norm = rest_of(in);
    // other statements (texture options, PBR extensions not in material_t) are skipped
  }
}

struct VertexKey {
  float p[3], n[3], uv[2];
  bool operator==(const VertexKey& o) const { return std::memcmp(this, &o, sizeof(*this)) == 0; }
};
struct VertexHash {
  size_t operator()(const VertexKey& k) const {
    size_t h = 1469598103934665603ull;
    const unsigned char* b = reinterpret_cast<const unsigned char*>(&k);
    for (size_t i = 0; i < sizeof(k); ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
  }
};

// OBJ index (1-based, negative = relative to the end) to a 0-based one.
int resolve(long v, size_t count, const std::string& path, int line) {
  const long r = v > 0 ? v - 1 : (long)count + v;
  if (v == 0 || r < 0 || (size_t)r >= count) fail(path, line, "index out of range");
  return (int)r;
}

}  // namespace

model_t load_model_from_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw TracerError(TR_ERR_ARG, "cannot open " + path);
  model_t model;
  model.name = name_of(path);
  std::vector<real> pos, nrm, tex;
  std::unordered_map<std::string, int> mat_ids;
  std::unordered_map<VertexKey, uint32_t, VertexHash> unique;
  int cur_mat = -1;
  mesh_t* mesh = nullptr;
  std::string pending_name;
  auto start_mesh = [&]() {
    model.mesh.emplace_back();
    mesh = &model.mesh.back();
    mesh->name = pending_name;
    unique.clear();
  };
  std::string text;
  int line = 0;
  while (std::getline(f, text)) {
    ++line;
    std::istringstream in(text);
    std::string key;
    if (!(in >> key) || key[0] == '#') continue;
    if (key == "v") {
      real v[3];
      read3(in, v, path, line);
      pos.insert(pos.end(), v, v + 3);
    } else if (key == "vn") {
      real v[3];
      read3(in, v, path, line);
      nrm.insert(nrm.end(), v, v + 3);
    } else if (key == "vt") {
      real u = 0, v = 0;
      if (!(in >> u >> v)) fail(path, line, "expected two texture coordinates");
      tex.push_back(u);
      tex.push_back(v);
    } else if (key == "o" || key == "g") {
      pending_name = rest_of(in);
      mesh = nullptr;  // a new shape starts at its first face
    } else if (key == "usemtl") {
      const std::string name = rest_of(in);
      auto it = mat_ids.find(name);
      cur_mat = it == mat_ids.end() ? -1 : it->second;
    } else if (key == "mtllib") {
      std::string lib;
      while (in >> lib) load_mtl(dir_of(path) + lib, model.material, mat_ids);
    } else if (key == "f") {
      if (!mesh) start_mesh();
      std::vector<uint32_t> poly;
      std::string tok;
      while (in >> tok) {
        long vi = 0, ti = 0, ni = 0;
        const size_t s1 = tok.find('/');
        try {
          vi = std::stol(tok.substr(0, s1));
          if (s1 != std::string::npos) {
            const size_t s2 = tok.find('/', s1 + 1);
            const std::string t = tok.substr(s1 + 1, s2 == std::string::npos ? std::string::npos : s2 - s1 - 1);
            if (!t.empty()) ti = std::stol(t);
            if (s2 != std::string::npos && s2 + 1 < tok.size()) ni = std::stol(tok.substr(s2 + 1));
          }
        } catch (const std::exception&) {
          fail(path, line, "malformed face vertex '" + tok + "'");
        }
        if (ni == 0) fail(path, line, "face vertex without a normal");
        const int p = resolve(vi, pos.size() / 3, path, line), n = resolve(ni, nrm.size() / 3, path, line);
        VertexKey k{};
        for (int c = 0; c < 3; ++c) k.p[c] = pos[3 * p + c];
        // Normal3::normalize (double length, float result)
        const double len = std::sqrt((double)(nrm[3 * n] * nrm[3 * n] + nrm[3 * n + 1] * nrm[3 * n + 1] +
                                              nrm[3 * n + 2] * nrm[3 * n + 2]));
        const double inv = 1.0 / len;
        for (int c = 0; c < 3; ++c) k.n[c] = (float)(nrm[3 * n + c] * inv);
        if (ti != 0) {
          const int t = resolve(ti, tex.size() / 2, path, line);
          k.uv[0] = tex[2 * t];
          k.uv[1] = tex[2 * t + 1];
        }
        auto it = unique.find(k);
        uint32_t id;
        if (it == unique.end()) {
          id = (uint32_t)mesh->vertices.size();
          unique.emplace(k, id);
          vertex_t v;
          v.pos = Point3f{k.p[0], k.p[1], k.p[2]};
          v.n = Normal3f{k.n[0], k.n[1], k.n[2]};
          v.uv = Point2f{k.uv[0], k.uv[1]};
          mesh->vertices.push_back(v);
        } else {
          id = it->second;
        }
        poly.push_back(id);
      }
      if (poly.size() < 3) fail(path, line, "face with fewer than three vertices");
      for (size_t i = 1; i + 1 < poly.size(); ++i) {  // fan
        mesh->indices.push_back((int)poly[0]);
        mesh->indices.push_back((int)poly[i]);
        mesh->indices.push_back((int)poly[i + 1]);
        mesh->materials.push_back(cur_mat);
      }
    }
    // s, l, p and other statements are skipped
  }
  return model;
}

}  // namespace tracer
