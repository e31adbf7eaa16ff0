// Drives the image-file helpers of the C++ host API for tests/test_image_file.py:
//   image_file load <file.hdr>       prints "size w h" and every pixel
//   image_file png <file>            the same for load_image_from_file (bytes; PNG, JPEG, BMP or TGA)
//   image_file write <file.hdr> w h  writes a w x h test pattern with write_image_to_hdr
//   image_file tex <file>            create_texture2d_from_file, one lookup
//   image_file mtl <file.obj>        prints create_texture_from_file for each material
#include <cstdio>
#include <cstring>
#include <string>

#include "tracer_gb300.hpp"

using namespace tracer;

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const std::string cmd = argv[1], path = argv[2];
  try {
    if (cmd == "load") {
      auto img = load_hdr_from_file(path);
      std::printf("size %d %d\n", img->width(), img->height());
      for (int y = 0; y < img->height(); ++y)
        for (int x = 0; x < img->width(); ++x) {
          const Color3f& c = img->at(x, y);
          std::printf("%.9g %.9g %.9g\n", c.x, c.y, c.z);
        }
    } else if (cmd == "png") {
      auto img = load_image_from_file(path);
      std::printf("size %d %d\n", img->width(), img->height());
      for (int y = 0; y < img->height(); ++y)
        for (int x = 0; x < img->width(); ++x) {
          const Color3b& c = img->at(x, y);
          std::printf("%d %d %d\n", c.x, c.y, c.z);
        }
    } else if (cmd == "write" && argc >= 5) {
      const int w = std::atoi(argv[3]), h = std::atoi(argv[4]);
      Image2D<Spectrum> img(w, h);
      for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) img.at(x, y) = Spectrum(0.01f * x + 0.5f * y, 3.0f + x, x == y ? 0.0f : 120.5f);
      write_image_to_hdr(img, path);
    } else if (cmd == "tex") {
      auto t = create_texture2d_from_file(path);
      const Spectrum c = t->evaluate(Point2f{0.25f, 0.5f});
      std::printf("texture %.9g %.9g %.9g\n", c.r, c.g, c.b);
    } else if (cmd == "mtl") {
      const model_t m = load_model_from_file(path);
      for (const material_t& mt : m.material) {
        const MaterialTexture t = create_texture_from_file(mt);
        const Spectrum kd = t.map_kd->evaluate(Point2f{0.5f, 0.5f}), ks = t.map_ks->evaluate(Point2f{0.5f, 0.5f});
        const Spectrum ke = t.map_ke->evaluate(Point2f{0.5f, 0.5f});
        std::printf("material %s kd %g %g %g ks %g %g %g ns %g ke %g %g %g emission %d glass %d", mt.name.c_str(),
                    kd.r, kd.g, kd.b, ks.r, ks.g, ks.b, t.map_ns->evaluate_s(Point2f{0, 0}), ke.r, ke.g, ke.b,
                    (int)t.has_emission, (int)t.as_glass);
        if (t.as_glass)
          std::printf(" kt %g ior %g", t.map_kt->evaluate_s(Point2f{0, 0}), t.ior->evaluate_s(Point2f{0, 0}));
        std::printf("\n");
      }
    } else {
      return 2;
    }
  } catch (const TracerError& e) {
    std::printf("error %d %s\n", (int)e.status, e.what());
    return 1;
  }
  return 0;
}
