// Test-oracle driver over the reference renderer's own objects (built by
// oracle/Makefile into oracle/_ref/; test infrastructure only).
//
// For a .muon scene it parses with the reference Parser (muon/parser.cc:230),
// casts the sample-0 ray through every pixel centre with Camera::CastRay
// (muon/camera.cc:37, pixel centre per muon/sampling.cc:89-91) and intersects
// it with the reference acceleration structure (muon/acceleration.cc:65).
// Output (binary, little endian):
//   header: "MUONHIT1", int32 width, int32 height
//   per pixel (row-major, y outer): int32 hit, float distance, float pos[3],
//   float normal[3], float diffuse[3], float specular[3], int32 is_light
// The integrator's Shade() is not called; the fields above are exactly the
// inputs of NormalsTracer/AlbedoTracer/DepthTracer (muon/integration.cc:47-72).
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>

#include "muon/acceleration.h"
#include "muon/options.h"
#include "muon/parser.h"

int main(int argc, char **argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_driver scene.muon out.bin [linear]\n");
    return 2;
  }
  muon::Options options;
  options.output = "";
  options.acceleration = (argc > 3 && std::string(argv[3]) == "linear")
                             ? muon::AccelerationType::kLinear
                             : muon::AccelerationType::kBVH;
  options.partition_strategy = muon::PartitionStrategy::kSAH;
  options.parallelism = 1;
  options.show_stats = false;
  muon::Parser parser(argv[1], options);
  muon::SceneConfig sc = parser.Parse();
  auto ws = sc.scene->root->CreateWorkspace();
  int w = sc.scene->width, h = sc.scene->height;
  std::ofstream out(argv[2], std::ios::binary);
  out.write("MUONHIT1", 8);
  out.write(reinterpret_cast<const char *>(&w), 4);
  out.write(reinterpret_cast<const char *>(&h), 4);
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      muon::Ray r = sc.scene->camera->CastRay(x + 0.5f, y + 0.5f);
      auto hit = sc.scene->root->Intersect(ws.get(), r);
      int32_t is_hit = hit ? 1 : 0;
      float rec[13] = {0};
      int32_t is_light = 0;
      if (hit) {
        rec[0] = hit->distance;
        for (int k = 0; k < 3; ++k) {
          rec[1 + k] = hit->pos[k];
          rec[4 + k] = hit->normal[k];
          rec[7 + k] = hit->obj->material->diffuse[k];
          rec[10 + k] = hit->obj->material->specular[k];
        }
        is_light = hit->obj->light != nullptr;
      }
      out.write(reinterpret_cast<const char *>(&is_hit), 4);
      out.write(reinterpret_cast<const char *>(rec), sizeof(rec));
      out.write(reinterpret_cast<const char *>(&is_light), 4);
    }
  }
  return 0;
}
