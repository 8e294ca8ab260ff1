// Scene records on the device: the host builder's per-triangle loop
// (scene_build.cc) run as one thread per triangle over the scene
// description, so a scene's records need not be built on the host and
// uploaded (both sides call TriangleRecords, tri_records.h); and the merge of
// scenes' device arrays into one batched scene.
#include <cub/device/device_scan.cuh>

#include "scene_records.h"
#include "tri_records.h"

namespace muon_gpu {

namespace {

constexpr int kThreads = 256;

inline unsigned Grid(int64_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

__global__ void KeepKernel(const MuonTriangleDesc *tris, int64_t n, int32_t *keep) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x;
  if (i < n) keep[i] = TriangleCanBeHit(tris[i]) ? 1 : 0;
}

__global__ void TotalKernel(const int32_t *keep, const int32_t *pos, int64_t n, int32_t *count) {
  *count = pos[n - 1] + keep[n - 1];
}

__global__ void RecordsKernel(const MuonTriangleDesc *tris, int64_t n, const MuonTransformDesc *transforms,
                              const DevMaterial *materials, const int32_t *quad_index, const int32_t *keep,
                              const int32_t *pos, PrimRecord *world, PrimRecord *object, ShadeRecord *shade,
                              F4 *normals, F4 *normals_obj, float *boxes) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x;
  if (i >= n || !keep[i]) return;
  const MuonTriangleDesc t = tris[i];
  TriangleOut o;
  TriangleRecords(t, transforms, materials, quad_index, &o);
  const int64_t s = pos[i];
  world[s] = o.world;
  object[s] = o.object;
  shade[s] = o.shade;
  if (normals) {
    for (int k = 0; k < 3; ++k) {
      normals[3 * s + k] = t.smooth ? o.normals[k] : F4{0.0f, 0.0f, 0.0f, 0.0f};
      normals_obj[3 * s + k] = t.smooth ? o.normals_obj[k] : F4{0.0f, 0.0f, 0.0f, 0.0f};
    }
  }
  for (int k = 0; k < 3; ++k) boxes[6 * s + k] = o.lo[k], boxes[6 * s + 3 + k] = o.hi[k];
}

__device__ __forceinline__ int32_t ShiftIndex(int32_t v, int32_t off) { return v >= 0 ? v + off : v; }
__device__ __forceinline__ float ShiftIndexBits(float bits, int32_t off) {
  return __int_as_float(ShiftIndex(__float_as_int(bits), off));
}
__device__ __forceinline__ int32_t ShiftLink(int32_t link, int32_t node_off, int32_t prim_off) {
  if (link == kEmptyLink) return link;
  if (link >= 0) return link + node_off;
  return ~(~link + prim_off);
}

__global__ void MergeNodesKernel(const BvhNode *in, int64_t n, MergeOffsets off, BvhNode *out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x;
  if (i >= n) return;
  BvhNode nd = in[i];
  nd.d.x = ShiftLink(nd.d.x, off.node_off, off.prim_off);
  nd.d.y = ShiftLink(nd.d.y, off.node_off, off.prim_off);
  out[off.node_off + i] = nd;
}

__global__ void MergePrimsKernel(const PrimRecord *prims_in, const PrimRecord *obj_in, const ShadeRecord *shade_in,
                                 const F4 *sn_in, const F4 *sno_in, int64_t n, MergeOffsets off,
                                 PrimRecord *prims_out, PrimRecord *obj_out, ShadeRecord *shade_out, F4 *sn_out,
                                 F4 *sno_out) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kThreads + threadIdx.x;
  if (i >= n) return;
  PrimRecord r = prims_in[i], ro = obj_in[i];
  if (__float_as_uint(r.p3.w) & kPrimSphere) {
    r.p1.y = ShiftIndexBits(r.p1.y, off.xf_off);
    ro.p1.y = ShiftIndexBits(ro.p1.y, off.xf_off);
  } else {
    ro.p1.w = ShiftIndexBits(ro.p1.w, off.xf_off);
  }
  ShadeRecord sh = shade_in[i];
  sh.s0.w = ShiftIndexBits(sh.s0.w, off.mat_off);
  sh.s1.x = ShiftIndex(sh.s1.x, off.light_off);
  sh.s1.z = ShiftIndex(sh.s1.z, off.xf_off);
  const int64_t o = off.prim_off + i;
  prims_out[o] = r;
  obj_out[o] = ro;
  shade_out[o] = sh;
  if (sn_out) {
    for (int k = 0; k < 3; ++k) {
      sn_out[3 * o + k] = sn_in ? sn_in[3 * i + k] : F4{0.0f, 0.0f, 0.0f, 0.0f};
      sno_out[3 * o + k] = sno_in ? sno_in[3 * i + k] : F4{0.0f, 0.0f, 0.0f, 0.0f};
    }
  }
}

}  // namespace

void LaunchMergeScene(const BvhNode *nodes_in, int64_t num_nodes, const PrimRecord *prims_in,
                      const PrimRecord *obj_in, const ShadeRecord *shade_in, const F4 *sn_in, const F4 *sno_in,
                      int64_t num_prims, MergeOffsets off, BvhNode *nodes_out, PrimRecord *prims_out,
                      PrimRecord *obj_out, ShadeRecord *shade_out, F4 *sn_out, F4 *sno_out, cudaStream_t st) {
  if (num_nodes > 0) MergeNodesKernel<<<Grid(num_nodes), kThreads, 0, st>>>(nodes_in, num_nodes, off, nodes_out);
  if (num_prims > 0)
    MergePrimsKernel<<<Grid(num_prims), kThreads, 0, st>>>(prims_in, obj_in, shade_in, sn_in, sno_in, num_prims, off,
                                                          prims_out, obj_out, shade_out, sn_out, sno_out);
}

size_t HittableScanBytes(int64_t n) {
  size_t bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, bytes, static_cast<const int32_t *>(nullptr),
                                static_cast<int32_t *>(nullptr), static_cast<int>(n));
  return bytes;
}

cudaError_t CountHittableTriangles(const MuonTriangleDesc *tris, int64_t n, int32_t *keep, int32_t *pos,
                                   int32_t *count, void *scratch, size_t scratch_bytes, cudaStream_t st) {
  KeepKernel<<<Grid(n), kThreads, 0, st>>>(tris, n, keep);
  const cudaError_t e = cub::DeviceScan::ExclusiveSum(scratch, scratch_bytes, keep, pos, static_cast<int>(n), st);
  if (e != cudaSuccess) return e;
  TotalKernel<<<1, 1, 0, st>>>(keep, pos, n, count);
  return cudaGetLastError();
}

void LaunchTriangleRecords(const MuonTriangleDesc *tris, int64_t n, const MuonTransformDesc *transforms,
                           const DevMaterial *materials, const int32_t *quad_index, const int32_t *keep,
                           const int32_t *pos, PrimRecord *world, PrimRecord *object, ShadeRecord *shade,
                           F4 *normals, F4 *normals_obj, float *boxes, cudaStream_t st) {
  if (n > 0)
    RecordsKernel<<<Grid(n), kThreads, 0, st>>>(tris, n, transforms, materials, quad_index, keep, pos, world, object,
                                                shade, normals, normals_obj, boxes);
}

}  // namespace muon_gpu
