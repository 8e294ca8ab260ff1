// BVH construction on the GPU (bvh_build.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "dev_layout.h"

namespace muon_gpu {

// Scratch bytes LaunchGpuLbvh needs for n primitives.
size_t GpuLbvhScratchBytes(int n);
// Builds the BVH of n primitive boxes (n x 6 floats: lo xyz, hi xyz) into
// `nodes` (max(n - 1, 1) entries; node 0 is the root), the leaf order
// (`order`: sorted slot -> primitive) and leaf-end flags (`last`, n bytes).
void LaunchGpuLbvh(const float *boxes, int n, void *scratch, size_t scratch_bytes, BvhNode *nodes, int32_t *order,
                   uint8_t *last, cudaStream_t st);
// Binned-SAH build on the device with the host builder's split decisions
// (bvh_sah.cu): nodes (root first, at most max(n - 1, 1)), the leaf order and
// the leaf-end flags, as LaunchGpuLbvh. Synchronises `st` between the levels
// of its top phase. A non-zero result.error means an internal list or stack
// limit was reached (no tree).
struct GpuSahResult {
  int error = 0;
  int nodes = 0;
  int64_t leaves = 0;
  int max_depth = 0;  // deepest node, the root at depth 0 (leaves included)
  int max_leaf = 0;
};
size_t GpuSahScratchBytes(int n);
cudaError_t BuildGpuSah(const float *boxes, int n, int max_leaf, void *scratch, BvhNode *nodes, int32_t *order,
                        uint8_t *last, GpuSahResult *result, cudaStream_t st);
// Gathers primitive, shading and smooth-normal records into leaf order and
// sets their leaf-end flags. sn_in / sno_in may be null (no smooth triangles).
void LaunchGatherPrims(const int32_t *order, const uint8_t *last, int n, const PrimRecord *prims_in,
                       const PrimRecord *obj_in, const ShadeRecord *shade_in, const F4 *sn_in, const F4 *sno_in,
                       PrimRecord *prims_out, PrimRecord *obj_out, ShadeRecord *shade_out, F4 *sn_out, F4 *sno_out,
                       cudaStream_t st);

}  // namespace muon_gpu
