// Memory layout of a scene resident in GPU memory. Shared by the host-side
// builder (which fills these arrays) and the kernels (which read them).
//
// BVH: a binary BVH stored as 64-byte nodes that hold the boxes of BOTH
// children, so one 64-byte load (four 16-byte vectors) gives a traversal step
// two box tests:
//   a = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   b = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   c = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   d = (link0, link1, -, -)
// A link >= 0 is an interior node index; a link < 0 is a leaf whose first
// primitive record is ~link. Leaves end at the record flagged kPrimLast.
// Node 0 is the root; an empty child slot has an inverted box.
//
// Primitive records (64 bytes, leaf order), world space:
//   triangle: p0 = (a.xyz, dot(a,n)), p1 = (b.xyz, eps), p2 = (c.xyz, -),
//             p3 = (n.xyz, flags)       n = (b-a) x (c-a), unnormalised
//   sphere:   p0 = (centre.xyz, radius), p1 = (-, transform, -, -),
//             p2 = -, p3 = (-, -, -, flags)
// and the same in object space for the exact mode:
//   triangle: p0 = (a.xyz, -), p1 = (b.xyz, transform), p2 = (c.xyz, |n|^2),
//             p3 = (n.xyz, flags)
//   sphere:   as above
// Shading records (32 bytes, leaf order): s0 = (unit normal.xyz, material),
// s1 = (light, prim_id, transform, flags).
#pragma once

#include <stdint.h>

namespace muon_gpu {

constexpr uint32_t kPrimSphere = 1u;   // record is a sphere (else triangle)
constexpr uint32_t kPrimLast = 2u;     // last record of its leaf
constexpr uint32_t kPrimSmooth = 4u;   // triangle interpolates vertex normals
// Shading class of a primitive (bits 8..10 of the shading record's flags,
// and of the primitive records' flags): 3 * (is sphere) + BRDF (MUON_BRDF_*).
// Hits are shaded grouped by class.
constexpr int kClassShift = 8;
constexpr int kNumClasses = 6;
constexpr int32_t kEmptyLink = INT32_MIN;

struct alignas(16) F4 {
  float x, y, z, w;
};
struct alignas(16) I4 {
  int32_t x, y, z, w;
};

struct alignas(16) BvhNode {
  F4 a, b, c;
  I4 d;
};
static_assert(sizeof(BvhNode) == 64, "BVH node must be 64 bytes");

struct alignas(16) PrimRecord {
  F4 p0, p1, p2, p3;
};
static_assert(sizeof(PrimRecord) == 64, "primitive record must be 64 bytes");

struct alignas(16) ShadeRecord {
  F4 s0;
  I4 s1;
};
static_assert(sizeof(ShadeRecord) == 32, "shading record must be 32 bytes");

// Affine transforms, rows 0..2 of each 4x4 column-major matrix stored as
// columns: m[col] = (row0, row1, row2) packed as 12 floats.
struct alignas(16) DevTransform {
  float o2w[12];
  float w2o[12];
  float n2w[12];
  float pad[4];
};

struct alignas(16) DevMaterial {
  F4 diffuse;   // xyz, w = shininess
  F4 specular;  // xyz, w = roughness
  F4 emission;  // xyz, w = brdf (as int bits)
  F4 ambient;   // xyz, w = reflectiveness (lobe-selection probability)
};

// Quad area light (muon/lighting.h:14-23, 74-83) with the quantities the
// shading code derives from it precomputed on the host.
struct alignas(16) DevLight {
  F4 corner;       // xyz, w = type (int bits)
  F4 edge0;        // xyz, w = |edge0|
  F4 edge1;        // xyz, w = |edge1|
  F4 color;        // xyz, w = area |edge0 x edge1|
  F4 rev_normal;   // normalize(edge0 x edge1)
  F4 quad_normal;  // normalize(edge1 x edge0), the Quad::Intersect normal
};

// Pointers into one scene's device arrays (all leaf order where relevant).
struct DevScene {
  const BvhNode *nodes;
  const PrimRecord *prims;      // world-space records (fast / watertight)
  const PrimRecord *prims_obj;  // object-space records (exact)
  const ShadeRecord *shade;
  const F4 *smooth_normals;      // 3 per slot, carried to world space, or null
  const F4 *smooth_normals_obj;  // 3 per slot, object space, or null
  const DevTransform *transforms;
  const DevMaterial *materials;
  const DevLight *lights;       // quad lights
  const PrimRecord *light_tris; // 2 per quad light, in light order (for MIS)
  const PrimRecord *light_tris_obj;  // the same in the object-space format
  const int32_t *light_tri_ok;  // per light triangle: 1 if it can be hit
  const DevLight *other_lights; // point/directional
  const DevLight *all_lights;   // every light in scene order (ray tracer)
  int32_t num_nodes;
  int32_t num_lights;
  int32_t num_other_lights;
  int32_t num_all_lights;
};

// Camera::CastRay state (muon/camera.h:9-32) with the host-computed frame.
struct DevCamera {
  float eye[3];
  float u[3], v[3], w[3];
  float tan_fov_x, tan_fov_y;
  int32_t width, height;  // the camera's own size (Camera::width_/height_)
};

}  // namespace muon_gpu
