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
// file-scope device array of kScratchBytes. Every GPU that loads the library
// holds it until the process exits. Host code cannot use the array's name as
// a device address, so the first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current, and caches it.
//
// Limits and rules:
//  * Paths in flight per wavefront are capped by the buffer: at most
//    kScratchBytes / (196 + 36 * S) paths, S = shadow slots per path. A
//    requested wave_paths above that, or a scene whose S leaves room for fewer
//    than 256 paths, is rejected with MUON_ERR_INVALID_ARG.
//  * Every call reuses the same buffer and leaves its contents behind; the
//    parts that must start at zero are cleared at the start of each call.
//    Two calls whose work overlaps on the GPU (different streams or scenes,
//    or other host threads) race on the buffer and corrupt each other.
//  * No CUDA graph and no CUDA events are used, and counters are read back
//    into host stack memory, so the call creates no runtime objects.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "host_scene.h"
#include "kernels.cuh"
#include "scene_access.h"

namespace muon_gpu {
namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;  // MUON_NOALLOC_SCRATCH_BYTES
constexpr int kNoAllocMaxBounces = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mutex;
void *g_scratch_addr[kMaxDevices] = {nullptr};

int Fail(int code, const std::string &msg) {
  SetLastError(msg);
  return code;
}

// Device address of g_scratch on the current device (set-up on first use).
cudaError_t ScratchAddress(int device, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[device] = p;
  }
  *out = static_cast<unsigned char *>(g_scratch_addr[device]);
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

size_t BytesFor(int64_t paths, int slots, int bounces) {
  Carver c{nullptr};
  for (int k = 0; k < 8; ++k) c.Take<float4>(paths);  // ray_o, ray_d, tp, rad (x2)
  c.Take<int2>(paths);
  c.Take<int32_t>(paths);
  c.Take<float4>(paths);  // final_rad
  c.Take<float4>(paths);  // org
  const size_t sl = static_cast<size_t>(paths) * std::max(slots, 1);
  c.Take<float4>(sl);
  c.Take<float4>(sl);
  c.Take<uint32_t>(sl);
  c.Take<int32_t>(static_cast<size_t>(paths) * kNumClasses);
  c.Take<uint32_t>(WaveCounterWords(bounces));
  c.Take<unsigned long long>(kNumStats);
  return c.used;
}

}  // namespace
}  // namespace muon_gpu

using namespace muon_gpu;

extern "C" int muon_gpu_render_noalloc(MuonScene *scene, const MuonRenderParams *params, double *d_sum,
                                       double *d_sum_sq, uint32_t *d_count) {
  SceneView v;
  if (!GetSceneView(scene, &v) || !params || !d_sum || !d_sum_sq || !d_count)
    return Fail(MUON_ERR_INVALID_ARG, "null argument");
  const MuonRenderParams &p = *params;
  if (p.integrator != MUON_INTEGRATOR_PATHTRACER && p.integrator != MUON_INTEGRATOR_NORMALS &&
      p.integrator != MUON_INTEGRATOR_ALBEDO && p.integrator != MUON_INTEGRATOR_DEPTH)
    return Fail(MUON_ERR_INVALID_ARG, "integrator not available on the GPU path");
  if (p.pixel_samples < 1 || p.max_depth < -1 || p.wave_paths < 0 || p.next_event_estimation < MUON_NEE_OFF ||
      p.next_event_estimation > MUON_NEE_MIS || p.importance_sampling < MUON_IS_HEMISPHERE ||
      p.importance_sampling > MUON_IS_BRDF || p.intersect_mode < MUON_ISECT_FAST ||
      p.intersect_mode > MUON_ISECT_EXACT)
    return Fail(MUON_ERR_INVALID_ARG, "render parameters out of range");
  const bool pt = p.integrator == MUON_INTEGRATOR_PATHTRACER;
  if (pt && p.next_event_estimation != MUON_NEE_OFF && p.light_samples < 1)
    return Fail(MUON_ERR_INVALID_ARG, "light_samples must be >= 1");

  ShadeParams sp{};
  sp.integrator = p.integrator;
  sp.nee = p.next_event_estimation;
  sp.is_mode = p.importance_sampling;
  sp.rr = p.russian_roulette;
  sp.min_depth = p.min_depth;
  sp.max_trace_depth = p.max_depth < 0 ? -1 : (p.next_event_estimation != MUON_NEE_OFF ? p.max_depth - 1 : p.max_depth);
  sp.strata = p.light_stratify ? static_cast<int>(std::sqrt(static_cast<double>(p.light_samples))) : 1;
  sp.per_section = p.light_stratify ? 1 : p.light_samples;
  sp.per_light = sp.strata * sp.strata * sp.per_section;
  sp.light_samples = std::max(1, p.light_samples);
  sp.isect = p.intersect_mode;
  sp.max_bounces = kNoAllocMaxBounces;
  int slots = 0;
  sp.mis_slot = -1;
  if (pt && p.next_event_estimation != MUON_NEE_OFF) {
    slots = v.dev->num_lights * sp.per_light + v.dev->num_other_lights;
    if (p.next_event_estimation == MUON_NEE_MIS) sp.mis_slot = slots++;
  }
  sp.slots = slots;
  const bool traces = !(p.max_depth >= 0 && sp.max_trace_depth < 0);
  const bool bounded = !pt || sp.max_trace_depth >= 0;
  const int bounces = !traces ? 0 : (!pt ? 1 : (bounded ? sp.max_trace_depth + 1 : kNoAllocMaxBounces));

  // Paths per wavefront that fit the buffer.
  int64_t capacity = static_cast<int64_t>(kScratchBytes / (196 + 36 * static_cast<size_t>(std::max(slots, 1))));
  capacity &= ~int64_t(255);
  while (capacity > 0 && BytesFor(capacity, slots, bounces) > kScratchBytes) capacity -= 256;
  if (capacity < 256)
    return Fail(MUON_ERR_INVALID_ARG, "scene needs too many shadow slots per path for the fixed scratch buffer");
  if (p.wave_paths > capacity)
    return Fail(MUON_ERR_INVALID_ARG, "wave_paths exceeds the fixed scratch buffer (at most " +
                                          std::to_string(capacity) + " paths for this scene)");
  const int64_t budget = p.wave_paths > 0 ? p.wave_paths : capacity;

  cudaError_t e = cudaSetDevice(v.device);
  unsigned char *base = nullptr;
  if (e == cudaSuccess) e = ScratchAddress(v.device, &base);
  if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));

  Carver c{base};
  PathBuffers b{};
  b.ray_o[0] = c.Take<float4>(budget), b.ray_o[1] = c.Take<float4>(budget);
  b.ray_d[0] = c.Take<float4>(budget), b.ray_d[1] = c.Take<float4>(budget);
  b.tp[0] = c.Take<float4>(budget), b.tp[1] = c.Take<float4>(budget);
  b.rad[0] = c.Take<float4>(budget), b.rad[1] = c.Take<float4>(budget);
  b.hits = c.Take<int2>(budget);
  b.link = c.Take<int32_t>(budget);
  b.final_rad = c.Take<float4>(budget);
  b.org = c.Take<float4>(budget);
  const size_t sl = static_cast<size_t>(budget) * std::max(slots, 1);
  b.contrib = c.Take<float4>(sl);
  b.slot_dir = c.Take<float4>(sl);
  b.shq = c.Take<uint32_t>(sl);
  b.order = c.Take<int32_t>(static_cast<size_t>(budget) * kNumClasses);
  b.order_cap = static_cast<int32_t>(budget);
  const size_t stride = WaveCounterWords(bounces);
  uint32_t *counters = c.Take<uint32_t>(stride);
  b.stats = c.Take<unsigned long long>(kNumStats);

  cudaStream_t st = v.stream;
  const int W = v.width, H = v.height;
  const int64_t npix_total = static_cast<int64_t>(W) * H;
  const int spp = p.pixel_samples;
  const int ns = static_cast<int>(std::min<int64_t>(spp, budget));
  const int64_t pix_per_wave = std::max<int64_t>(1, budget / ns);
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
  for (int64_t p0 = 0; p0 < npix_total; p0 += pix_per_wave) {
    for (int s0 = 0; s0 < spp; s0 += ns) {
      WaveInfo w{};
      w.width = W;
      w.p0 = static_cast<int32_t>(p0);
      w.npix = static_cast<int>(std::min<int64_t>(pix_per_wave, npix_total - p0));
      w.s0 = s0;
      w.ns = std::min(ns, spp - s0);
      w.n = w.npix * w.ns;
      w.sample_offset = static_cast<uint32_t>(p.sample_offset);
      w.seed = p.seed;
      // Queue counters of this wavefront start at zero.
      e = cudaMemsetAsync(counters, 0, stride * sizeof(uint32_t), st);
      if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("scratch clear: ") + cudaGetErrorString(e));
      WaveCounters wc{counters};
      LaunchCamera(*v.cam, w, b, wc, st);
      for (int k = 0; k < bounces; ++k) {
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
        if (!bounded) {
          uint32_t next = 0;  // host stack memory: no pinned allocation
          e = cudaMemcpyAsync(&next, wc.count(k + 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
          if (e == cudaSuccess) e = cudaStreamSynchronize(st);
          if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, cudaGetErrorString(e));
          if (next == 0) break;
        }
      }
      LaunchFilm(w, b, d_sum, d_sum_sq, d_count, st);
    }
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return Fail(MUON_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
  return MUON_OK;
}
