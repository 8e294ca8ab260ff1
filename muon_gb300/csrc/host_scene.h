// Host-side scene representation shared by the parser, the BVH builder and the
// device upload. It is the flattened form of the reference's object graph
// (muon/scene.h:22-95, muon/objects.h, muon/materials.h, muon/lighting.h):
// primitives refer to transforms, materials and lights by index instead of
// shared pointers.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/muon_gpu.h"
#include "mmath.h"

namespace muon_gpu {

struct ParsedScene {
  std::vector<MuonTransformDesc> transforms;
  std::vector<MuonMaterialDesc> materials;
  std::vector<MuonLightDesc> lights;
  std::vector<MuonTriangleDesc> triangles;
  std::vector<MuonSphereDesc> spheres;
  MuonCameraDesc camera{};
  bool has_camera = false;
  int32_t width = 150, height = 150;
  MuonRenderParams params{};
  float gamma = 1.0f;
  std::string output;
  bool has_output = false;
  int32_t warnings = 0;
};

// Parses a .muon scene from a stream of lines (see scene_parser.cc).
bool ParseScene(const std::string &text, const std::string &base_dir, ParsedScene *out,
                std::string *error);

// Thread-local error reporting used by every C entry point.
void SetLastError(const std::string &msg);

MuonTransformDesc MakeTransformDesc(const mm::m4 &m);

}  // namespace muon_gpu
