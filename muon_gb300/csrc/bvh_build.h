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
// Gathers primitive, shading and smooth-normal records into leaf order and
// sets their leaf-end flags. sn_in / sno_in may be null (no smooth triangles).
void LaunchGatherPrims(const int32_t *order, const uint8_t *last, int n, const PrimRecord *prims_in,
                       const PrimRecord *obj_in, const ShadeRecord *shade_in, const F4 *sn_in, const F4 *sno_in,
                       PrimRecord *prims_out, PrimRecord *obj_out, ShadeRecord *shade_out, F4 *sn_out, F4 *sno_out,
                       cudaStream_t st);

}  // namespace muon_gpu
