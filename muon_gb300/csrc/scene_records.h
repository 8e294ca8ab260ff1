// Triangle records computed on the device (scene_records.cu), bit for bit the
// host scene builder's (tri_records.h).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/muon_gpu.h"
#include "dev_layout.h"

namespace muon_gpu {

// Scratch bytes for CountHittableTriangles over n triangles.
size_t HittableScanBytes(int64_t n);
// pos[i] = the number of hittable triangles (TriangleCanBeHit) before
// triangle i, keep[i] = whether it is hittable; *count receives the total
// (device memory). n >= 1.
cudaError_t CountHittableTriangles(const MuonTriangleDesc *tris, int64_t n, int32_t *keep, int32_t *pos,
                                   int32_t *count, void *scratch, size_t scratch_bytes, cudaStream_t st);
// Writes the records and box of every hittable triangle i at slot pos[i]
// (records in input order of the hittable triangles, as the host builder's
// deferred layout): world / object / shading records, smooth normals (3 per
// slot, when `normals` is not null) and the box as 6 floats (lo xyz, hi xyz).
void LaunchTriangleRecords(const MuonTriangleDesc *tris, int64_t n, const MuonTransformDesc *transforms,
                           const DevMaterial *materials, const int32_t *quad_index, const int32_t *keep,
                           const int32_t *pos, PrimRecord *world, PrimRecord *object, ShadeRecord *shade,
                           F4 *normals, F4 *normals_obj, float *boxes, cudaStream_t st);

// Index offsets of one scene inside a merged (batched) scene.
struct MergeOffsets {
  int32_t node_off, prim_off, xf_off, mat_off, light_off;
};
// Appends one scene's device arrays to merged ones: nodes at node_off (links
// shifted), records at prim_off with their transform, material and light
// indices shifted; smooth normals copied (zeros when the scene has none and
// the merged scene has some: sn_out set, sn_in null).
void LaunchMergeScene(const BvhNode *nodes_in, int64_t num_nodes, const PrimRecord *prims_in,
                      const PrimRecord *obj_in, const ShadeRecord *shade_in, const F4 *sn_in, const F4 *sno_in,
                      int64_t num_prims, MergeOffsets off, BvhNode *nodes_out, PrimRecord *prims_out,
                      PrimRecord *obj_out, ShadeRecord *shade_out, F4 *sn_out, F4 *sno_out, cudaStream_t st);

}  // namespace muon_gpu
