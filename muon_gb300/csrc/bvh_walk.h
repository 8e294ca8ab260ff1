// Host walk of the flattened BVH (bvh_walk.cc): traversal work per ray in the
// GPU kernels' visiting order, for measuring algorithmic bytes.
#pragma once

#include <cstdint>
#include <string>

#include "../../include/muon_gpu.h"
#include "host_scene.h"
#include "scene_build.h"

namespace muon_gpu {

struct WalkRayIn {
  float o[3], d[3];
  float tmax;
  int32_t root;  // BVH node the walk starts at (a batch keeps one root per scene)
};

// Walks one ray (closest hit, or any hit); adds its counts to *cnt and returns
// the leaf slot of the primitive hit, or -1.
int WalkRay(const SceneImage &im, const float o[3], const float d[3], float tmax, int root, bool any_hit, int mode,
            MuonWalkCounts *cnt);

// Walks n rays on all host threads; hit_slots (optional) receives each ray's
// leaf slot or -1; counts are added to *total.
void WalkMany(const SceneImage &im, const WalkRayIn *rays, int64_t n, bool any_hit, int mode, int32_t *hit_slots,
              MuonWalkCounts *total);

inline int WalkFail(int code, const std::string &msg) {
  SetLastError(msg);
  return code;
}

}  // namespace muon_gpu
