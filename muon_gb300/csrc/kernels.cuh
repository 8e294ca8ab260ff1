// Kernel launch interface of the wavefront renderer (implemented in
// kernels.cu; driven from render.cc).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/muon_gpu.h"
#include "dev_layout.h"

namespace muon_gpu {

// Device counters (uint32) used by the queue kernels.
enum Counter : int { kCntNext = 0, kCntShadow = 1, kNumCounters = 4 };
// Device statistics (uint64).
enum Stat : int {
  kStatPrimary = 0,
  kStatSecondary,
  kStatShadow,
  kStatBoxTests,
  kStatBoxHits,
  kStatPrimTests,
  kStatPrimHits,
  kStatOverflow,
  kStatOccBoxTests,
  kStatOccBoxHits,
  kStatOccPrimTests,
  kStatOccPrimHits,
  kNumStats
};

// One wavefront: `n` paths covering pixels [p0, p0 + npix) with samples
// [s0, s0 + ns) each; path i is pixel p0 + i / ns, sample s0 + i % ns.
struct WaveInfo {
  int32_t width;      // film width (pixel index = y * width + x)
  int32_t p0, npix;
  int32_t s0, ns;
  int32_t n;
  uint32_t sample_offset;
  int32_t pad;
  uint64_t seed;
};

struct PathBuffers {
  float4 *ray_o[2];   // path-ray queue: (origin, path id bits)
  float4 *ray_d[2];   // path-ray queue: (direction, tmax)
  int2 *hits;         // (t bits, leaf slot) per queued ray
  float4 *tp;         // throughput per path
  float4 *rad;        // radiance per path
  float4 *org;        // shadow-ray origin per path (the shifted hit point)
  float4 *contrib;    // S shadow slots per path: (radiance if unblocked, -)
  float4 *slot_dir;   // S shadow slots per path: (direction, max distance)
  uint32_t *shq;      // shadow queue: slot indices
  uint32_t *counters;
  unsigned long long *stats;
};

struct ShadeParams {
  int32_t integrator;
  int32_t nee, is_mode, rr;
  int32_t min_depth;
  int32_t max_trace_depth;  // deepest Trace() depth that casts a ray; -1 = unbounded
  int32_t strata, per_section, per_light;  // samples per quad light = strata^2 * per_section
  int32_t light_samples;
  int32_t slots;           // shadow slots per path
  int32_t mis_slot;        // slot index of the MIS ray, -1 if none
  int32_t isect;
  int32_t max_bounces;
};

void LaunchCamera(const DevCamera &cam, const WaveInfo &w, const PathBuffers &b, int slots, cudaStream_t st);
void LaunchExtend(const DevScene &s, const PathBuffers &b, int buf, int n, int isect, bool stats,
                  cudaStream_t st);
void LaunchShadeDebug(const DevScene &s, const WaveInfo &w, const PathBuffers &b, int integrator, int n, int isect,
                      cudaStream_t st);
void LaunchShadePath(const DevScene &s, const WaveInfo &w, const ShadeParams &sp, const PathBuffers &b, int buf,
                     int n, int bounce, cudaStream_t st);
void LaunchOcclude(const DevScene &s, const PathBuffers &b, int slots, int n, int isect, bool stats, cudaStream_t st);
void LaunchFilm(const WaveInfo &w, const PathBuffers &b, int slots, double *sum, double *sum_sq, uint32_t *count,
                cudaStream_t st);
// Ray-level queries for the batched Intersect/HasIntersection seams.
void LaunchIntersectRays(const DevScene &s, const float *rays, int64_t n, int isect, float *out_hit,
                         cudaStream_t st);
void LaunchOccludedRays(const DevScene &s, const float *rays, const float *maxd, int64_t n, int isect,
                        uint8_t *out, cudaStream_t st);

}  // namespace muon_gpu
