// muon_gpu_render_noalloc: the path-tracing render of muon_gpu_render_device
// with no device (or pinned host) allocation during the call.
//
// Who needs it: a host application that hands the GPU's memory to its own
// allocator up front (a game engine or a machine-learning framework that
// reserves nearly all device memory for its caching pool), or a real-time
// loop whose rule is that nothing is allocated after start-up, cannot let a
// renderer call cudaMalloc per frame. The scene itself is still created once
// with muon_gpu_scene_create at start-up; per-frame rendering then touches
// only the caller's film and the fixed buffer below.
//
// All working memory of a render (path queues, per-path state, shadow slots,
// queue counters, counters of work done) is carved out of `g_scratch`, a
// file-scope device array of kScratchBytes. This file is its own module, and
// CUDA loads modules lazily, so the array is placed on a device when its
// address is first looked up there: muon_gpu_scene_create does that
// (NoAllocPrepare), so the 64 MiB is taken when the first scene is created on
// a device, not during a render, and held until the process exits. Host code
// cannot use the array's name as a device address, so every call looks the
// address up with cudaGetSymbolAddress while the scene's device is current
// (cheap once the module is loaded, and never stale after a context reset).
//
// Limits and rules:
//  * Paths in flight per wavefront are capped by the buffer: at most about
//    kScratchBytes / (196 + 36 * S) paths, S = shadow slots per path. A
//    requested wave_paths above that, or a scene whose S leaves room for fewer
//    than 256 paths, is rejected with MUON_ERR_INVALID_ARG.
//  * Every call reuses the same buffer and leaves its contents behind; the
//    parts that must start at zero are cleared at the start of each call.
//    Two calls whose work overlaps on the GPU (different streams or scenes,
//    or other host threads) race on the buffer and corrupt each other.
//  * No CUDA graph and no CUDA events are used, counters are read back into
//    host stack memory and the waves are enumerated without storage, so the
//    call creates no runtime objects and allocates nothing on the host heap.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "host_cuda.h"
#include "host_scene.h"
#include "kernels.cuh"
#include "scene_access.h"

namespace muon_gpu {
namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;  // MUON_NOALLOC_SCRATCH_BYTES
static_assert(kScratchBytes == MUON_NOALLOC_SCRATCH_BYTES, "scratch size of the public header");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch on the current device.
cudaError_t ScratchAddress(unsigned char **out) {
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess) return e;
  *out = static_cast<unsigned char *>(p);
  return cudaSuccess;
}

// Carves 256-byte-aligned arrays out of the scratch buffer (with a null base
// it only measures).
struct Carver {
  unsigned char *base;
  size_t used = 0;
  template <class T>
  T *Take(size_t count) {
    used = (used + 255) & ~size_t(255);
    T *p = base ? reinterpret_cast<T *>(base + used) : nullptr;
    used += count * sizeof(T);
    return p;
  }
};

// Lays out every working array of a render of `paths` paths per wave in the
// buffer at `base` (null: only measures). Returns the bytes used.
size_t Carve(unsigned char *base, int64_t paths, int slots, int bounces, PathBuffers *b, uint32_t **counters) {
  Carver c{base};
  PathBuffers pb{};
  for (int k = 0; k < 2; ++k) pb.ray_o[k] = c.Take<float4>(paths);
  for (int k = 0; k < 2; ++k) pb.ray_d[k] = c.Take<float4>(paths);
  for (int k = 0; k < 2; ++k) pb.tp[k] = c.Take<float4>(paths);
  for (int k = 0; k < 2; ++k) pb.rad[k] = c.Take<float4>(paths);
  pb.hits = c.Take<int2>(paths);
  pb.link = c.Take<int32_t>(paths);
  pb.final_rad = c.Take<float4>(paths);
  pb.org = c.Take<float4>(paths);
  const size_t sl = static_cast<size_t>(paths) * std::max(slots, 1);
  pb.contrib = c.Take<float4>(sl);
  pb.slot_dir = c.Take<float4>(sl);
  pb.shq = c.Take<uint32_t>(sl);
  pb.order = c.Take<int32_t>(static_cast<size_t>(OrderInts(paths)));
  pb.order_cap = static_cast<int32_t>(paths);
  uint32_t *ctr = c.Take<uint32_t>(WaveCounterWords(bounces));
  pb.stats = c.Take<unsigned long long>(kNumStats);
  if (b) *b = pb;
  if (counters) *counters = ctr;
  return c.used;
}

// Largest multiple of 256 paths whose arrays fit the buffer (0 if none).
int64_t Capacity(int slots, int bounces) {
  int64_t lo = 0, hi = static_cast<int64_t>(kScratchBytes / WorkBytesPerPath(slots)) / 256 + 1;
  while (lo + 1 < hi) {  // Carve(lo * 256) fits, Carve(hi * 256) does not
    const int64_t mid = (lo + hi) / 2;
    if (Carve(nullptr, mid * 256, slots, bounces, nullptr, nullptr) <= kScratchBytes) lo = mid;
    else hi = mid;
  }
  return std::min<int64_t>(lo * 256, kMaxWavePaths);
}

}  // namespace

// Places the scratch array on the current device (loads this module) and
// checks that its address can be taken; called when a scene is created.
cudaError_t NoAllocPrepare() {
  unsigned char *base = nullptr;
  return ScratchAddress(&base);
}

}  // namespace muon_gpu

using namespace muon_gpu;

extern "C" int muon_gpu_render_noalloc(MuonScene *scene, const MuonRenderParams *params, double *d_sum,
                                       double *d_sum_sq, uint32_t *d_count) {
  SceneView v;
  if (!GetSceneView(scene, &v) || !params || !d_sum || !d_sum_sq || !d_count)
    return Fail(MUON_ERR_INVALID_ARG, "null argument");
  const MuonRenderParams &p = *params;
  int rc = ValidateParams(p);
  if (rc != MUON_OK) return rc;
  if (p.integrator != MUON_INTEGRATOR_PATHTRACER && p.integrator != MUON_INTEGRATOR_NORMALS &&
      p.integrator != MUON_INTEGRATOR_ALBEDO && p.integrator != MUON_INTEGRATOR_DEPTH)
    return Fail(MUON_ERR_INVALID_ARG, "integrator not available on the no-allocation path");
  const bool pt = p.integrator == MUON_INTEGRATOR_PATHTRACER;
  ShadeParams sp;
  const int slots = SetupShade(p, v.dev->num_lights, v.dev->num_other_lights, &sp);
  const BouncePlan bp = PlanBounces(p, sp);

  // Paths per wavefront that fit the buffer.
  const int64_t capacity = Capacity(slots, bp.bounces);
  if (capacity < 256)
    return Fail(MUON_ERR_INVALID_ARG, "scene needs too many shadow slots per path for the fixed scratch buffer");
  if (p.wave_paths > capacity)
    return Fail(MUON_ERR_INVALID_ARG, "wave_paths exceeds the fixed scratch buffer (at most " +
                                          std::to_string(capacity) + " paths for this scene)");
  const int64_t budget = p.wave_paths > 0 ? p.wave_paths : capacity;

  cudaError_t e = cudaSetDevice(v.device);
  unsigned char *base = nullptr;
  if (e == cudaSuccess) e = ScratchAddress(&base);
  if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));
  PathBuffers b{};
  uint32_t *counters = nullptr;
  Carve(base, budget, slots, bp.bounces, &b, &counters);

  cudaStream_t st = v.stream;
  const WavePlan plan = PlanWaves(v.width, v.height, p, budget);
  const int64_t npix_total = plan.npix;
  if (!(p.flags & MUON_RENDER_ACCUMULATE)) {
    e = cudaMemsetAsync(d_sum, 0, 3 * npix_total * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_sum_sq, 0, 3 * npix_total * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_count, 0, npix_total * sizeof(uint32_t), st);
    if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("film clear: ") + cudaGetErrorString(e));
  }
  // Counters of work done start at zero on every call.
  e = cudaMemsetAsync(b.stats, 0, kNumStats * sizeof(unsigned long long), st);
  if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("scratch clear: ") + cudaGetErrorString(e));
  const bool stats_on = (p.flags & MUON_RENDER_STATS) != 0;
  const size_t stride = WaveCounterWords(bp.bounces);
  const size_t nwaves = plan.Count();
  for (size_t wi = 0; wi < nwaves; ++wi) {
    const WaveInfo w = plan.At(wi);
    // Queue counters of this wavefront start at zero.
    e = cudaMemsetAsync(counters, 0, stride * sizeof(uint32_t), st);
    if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("scratch clear: ") + cudaGetErrorString(e));
    WaveCounters wc{counters};
    LaunchCamera(*v.cam, w, b, wc, st);
    for (int k = 0; k < bp.bounces; ++k) {
      LaunchExtend(*v.dev, b, wc, k, w.n, p.intersect_mode, stats_on, st);
      if (!pt) {
        LaunchShadeDebug(*v.dev, b, wc, p.integrator, w.n, p.intersect_mode, st);
        break;
      }
      LaunchShadePath(*v.dev, w, sp, b, wc, k, w.n, st);
      if (slots > 0)
        LaunchOcclude(*v.dev, b, wc, k, slots, static_cast<int>(std::min<int64_t>(int64_t(w.n) * slots, INT32_MAX)),
                      p.intersect_mode, stats_on, st);
      LaunchFold(b, wc, k, slots, w.n, st);
      if (!bp.bounded) {
        uint32_t next = 0;  // host stack memory: no pinned allocation
        e = cudaMemcpyAsync(&next, wc.count(k + 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, cudaGetErrorString(e));
        if (next == 0) break;
      }
    }
    LaunchFilm(w, b, d_sum, d_sum_sq, d_count, st);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
  return MUON_OK;
}
