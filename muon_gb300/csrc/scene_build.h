// Host-side construction of the device scene image: world-space primitive
// records, shading records, the flattened BVH, materials and lights.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/muon_gpu.h"
#include "dev_layout.h"
#include "mmath.h"

namespace muon_gpu {

struct Aabb {
  float lo[3], hi[3];
};

struct BvhBuildStats {
  int64_t nodes = 0;
  int64_t leaves = 0;
  int32_t max_depth = 0;
  int32_t max_leaf = 0;
  double sah_cost = 0.0;
};

// Builds a binary BVH over `boxes` and flattens it into 64-byte two-child
// nodes. `order` receives, for each leaf-order slot, the index of the input
// box; `last` marks the final slot of each leaf. strategy is MUON_PARTITION_*;
// accel MUON_ACCEL_LINEAR puts every primitive into one leaf.
void BuildBvh(const std::vector<Aabb> &boxes, int accel, int strategy, int max_leaf,
              std::vector<BvhNode> *nodes, std::vector<int32_t> *order, std::vector<uint8_t> *last,
              BvhBuildStats *stats);

struct SceneImage {
  std::vector<BvhNode> nodes;
  std::vector<PrimRecord> prims;          // leaf order, world space
  std::vector<PrimRecord> prims_obj;      // leaf order, object space (exact mode)
  std::vector<ShadeRecord> shade;         // leaf order
  std::vector<F4> smooth_normals;         // 3 per leaf slot when any triangle is smooth
  std::vector<F4> smooth_normals_obj;     // the same in object space
  std::vector<DevTransform> transforms;
  std::vector<DevMaterial> materials;
  std::vector<DevLight> lights;           // quad lights only
  std::vector<DevLight> other_lights;     // point / directional lights
  std::vector<DevLight> all_lights;       // every light, in scene order
  std::vector<int32_t> leaf_of_prim_id;   // parse-order id -> leaf slot (-1 = never hit)
  int64_t num_prims = 0;                  // primitives in the scene, including never-hit ones
  bool any_smooth = false;
  std::vector<float> boxes;               // 6 per record, when the GPU builds the BVH
  std::vector<int32_t> quad_index;        // light index -> quad-light index (-1: not a quad)
  MuonCameraDesc camera{};
  int32_t width = 0, height = 0;
  BvhBuildStats bvh;
};

// Flattens a scene description. Returns false with a message on invalid input.
// With defer_bvh the BVH is left to the GPU builder: `nodes` stays empty, the
// records are in input order and `boxes` holds their world bounds. With
// device_records (which implies defer_bvh) the triangles are only validated:
// the records and boxes hold the spheres alone, to follow the hittable
// triangles' records that the device computes (scene_records.h).
bool BuildSceneImage(const MuonSceneDesc &desc, SceneImage *img, std::string *error, bool defer_bvh = false,
                     bool device_records = false);

}  // namespace muon_gpu
