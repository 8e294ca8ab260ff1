// Triangle records on the device: the host builder's per-triangle loop
// (scene_build.cc) run as one thread per triangle over the scene
// description, so a scene's records need not be built on the host and
// uploaded. Both sides call TriangleRecords (tri_records.h).
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

}  // namespace

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
