// Kernel launch interface of the wavefront renderer (implemented in
// kernels.cu; driven from render.cc).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/muon_gpu.h"
#include "dev_layout.h"

namespace muon_gpu {

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
  int32_t width;  // film width (pixel index = y * width + x)
  int32_t p0, npix;
  int32_t s0, ns;
  int32_t n;
  uint32_t sample_offset;
  int32_t pad;
  uint64_t seed;
};

// A path record's id word (ray_o.w) holds the wave-local path index in its low
// kPathBits bits and, in a batched wave, the segment index above them; a
// wave holds at most 2^kPathBits paths and kMaxSegments segments.
constexpr int kPathBits = 24;
constexpr uint32_t kPathMask = (1u << kPathBits) - 1u;
constexpr int kMaxWavePaths = 1 << kPathBits;
constexpr int kMaxSegments = 256;

// Queue counters of one wavefront, all on the device so that a wavefront is a
// fixed launch sequence: count(k) = paths queued at bounce k (count(0) = n),
// shadow(k) = shadow rays emitted at bounce k.
struct WaveCounters {
  uint32_t *c;
  __host__ __device__ uint32_t *count(int k) const { return c + 16 * k; }
  __host__ __device__ uint32_t *shadow(int k) const { return c + 16 * k + 1; }
  // rays handed out so far by the persistent traversal kernels of bounce k
  __host__ __device__ uint32_t *fetch_extend(int k) const { return c + 16 * k + 2; }
  __host__ __device__ uint32_t *fetch_occlude(int k) const { return c + 16 * k + 3; }
  // hits of bounce k per shading class (kNumClasses entries)
  __host__ __device__ uint32_t *classes(int k) const { return c + 16 * k + 4; }
};
// Words of one wavefront's counter block for `bounces` bounces.
inline size_t WaveCounterWords(int bounces) { return 16 * static_cast<size_t>(bounces + 2); }

// Path state lives in queue order: entry j of bounce k's queue holds its ray,
// hit, throughput and radiance at index j, so every per-path access in the
// bounce kernels is coalesced. `link[j]` is the entry's index in the next
// bounce's queue (-1 when the path ends there); `final_rad[path]` receives
// the radiance of a path when it ends (path = wave-local sample index).
struct PathBuffers {
  float4 *ray_o[2];   // (origin, path id bits)
  float4 *ray_d[2];   // (direction, tmax)
  float4 *tp[2];      // throughput
  float4 *rad[2];     // radiance so far
  int2 *hits;         // (t bits, leaf slot)
  int32_t *link;      // next-queue index or -1
  float4 *final_rad;  // per path
  float4 *org;        // shadow-ray origin per queue entry
  float4 *contrib;    // S slots per queue entry: radiance if unblocked
  float4 *slot_dir;   // S slots per queue entry: (direction, max distance)
  uint32_t *shq;      // shadow queue: slot indices (entry * S + slot)
  int32_t *order;     // hit entries grouped by shading class: class c at c * order_cap
  int32_t order_cap;  // entries per class (the wavefront size)
  unsigned long long *stats;
};

// The `order` array of a wavefront of `cap` paths: kNumClasses class lists
// of cap entries each, then 8 class counts per tile of kClassTile queue
// entries (the stable class partition's, MUON_STABLE_CLASSES in kernels.cu).
constexpr int kClassTile = 1024;
inline int64_t OrderInts(int64_t cap) { return cap * kNumClasses + (cap / kClassTile + 1) * 8; }

struct ShadeParams {
  int32_t integrator;
  int32_t nee, is_mode, rr;
  int32_t min_depth;
  int32_t max_trace_depth;  // deepest Trace() depth that casts a ray; -1 = unbounded
  int32_t strata, per_section, per_light;  // samples per quad light = strata^2 * per_section
  int32_t light_samples;
  int32_t slots;     // shadow slots per path
  int32_t mis_slot;  // slot index of the MIS ray, -1 if none
  int32_t isect;
  int32_t max_bounces;
};

// Batched rendering: several scenes share one wavefront. Their device arrays
// are concatenated into one DevScene (each scene's BVH under its own root
// node, its lights a contiguous range); a wave is a list of segments, each a
// block of one scene's pixels and samples.
struct BatchScene {
  DevCamera cam;
  ShadeParams sp;      // slots/mis_slot of this scene; the wave's slot stride may be larger
  int32_t light_off, num_lights;   // quad lights (and their triangles at 2x)
  int32_t other_off, num_other;    // point / directional lights
  int32_t width;
  uint32_t sample_offset;
  uint64_t seed;
  double *sum, *sum_sq;
  uint32_t *count;
};
struct BatchSeg {
  int32_t scene;
  int32_t path0;  // first wave-local path of the segment
  int32_t pix0;   // first wave-local pixel of the segment
  int32_t p0, npix, s0, ns;  // film pixels [p0, p0 + npix), samples [s0, s0 + ns)
  int32_t root;   // BVH root node of the scene
};

// Upper bound on the blocks of the device-counted launches (they loop over
// their queue with a grid stride), and the block count of the persistent
// traversal kernels; set from the SM count at scene creation.
void SetPersistentGrid(int blocks);
void SetTraversalGrid(int sms);

void LaunchCamera(const DevCamera &cam, const WaveInfo &w, const PathBuffers &b, WaveCounters wc, cudaStream_t st);
void LaunchExtend(const DevScene &s, const PathBuffers &b, WaveCounters wc, int bounce, int bound, int isect,
                  bool stats, cudaStream_t st);
void LaunchShadeDebug(const DevScene &s, const PathBuffers &b, WaveCounters wc, int integrator, int bound, int isect,
                      cudaStream_t st);
// Raytracer / AnalyticDirect for every path of a wave; rays are traced up to
// depth max_trace_depth (0 = primary rays only).
void LaunchWhitted(const DevScene &s, const PathBuffers &b, const WaveInfo &w, int integrator, int max_trace_depth,
                   int isect, bool stats, cudaStream_t st);
void LaunchShadePath(const DevScene &s, const WaveInfo &w, const ShadeParams &sp, const PathBuffers &b,
                     WaveCounters wc, int bounce, int bound, cudaStream_t st);
void LaunchOcclude(const DevScene &s, const PathBuffers &b, WaveCounters wc, int bounce, int slots, int bound,
                   int isect, bool stats, cudaStream_t st);
void LaunchFold(const PathBuffers &b, WaveCounters wc, int bounce, int slots, int bound, cudaStream_t st);
void LaunchFilm(const WaveInfo &w, const PathBuffers &b, double *sum, double *sum_sq, uint32_t *count,
                cudaStream_t st);
// Batched counterparts: `segs` (nseg entries) and `scenes` are device tables;
// `paths` and `pixels` are the wave's totals, `slot_stride` the wave's shadow
// slots per entry (the largest of its scenes').
void LaunchCameraBatch(const BatchScene *scenes, const BatchSeg *segs, int nseg, int paths, const PathBuffers &b,
                       WaveCounters wc, cudaStream_t st);
void LaunchShadePathBatch(const DevScene &s, const BatchScene *scenes, const BatchSeg *segs, int slot_stride,
                          int isect, const PathBuffers &b, WaveCounters wc, int bounce, int bound, cudaStream_t st);
void LaunchFilmBatch(const BatchScene *scenes, const BatchSeg *segs, int nseg, int pixels, const PathBuffers &b,
                     cudaStream_t st);
// Grid of the persistent traversal kernels for the launches that follow
// (0 restores the default of filling every SM once).
void SetTraversalBlocksOverride(int blocks);
// Ray-level queries for the batched Intersect/HasIntersection seams.
void LaunchIntersectRays(const DevScene &s, const float *rays, int64_t n, int isect, float *out_hit,
                         cudaStream_t st);
void LaunchOccludedRays(const DevScene &s, const float *rays, const float *maxd, int64_t n, int isect,
                        uint8_t *out, cudaStream_t st);

// Measurement: a sample of bounce `bounce`'s closest-hit (kind 0) or shadow
// (kind 1) queue, up to m rays, into out (1 + 2m float4s; see SampleQueueKernel).
void LaunchSampleQueue(const PathBuffers &b, WaveCounters wc, int bounce, int kind, int slots, int m, float4 *out,
                       cudaStream_t st);
// Read-bandwidth kernel of `blocks` blocks of 256 threads over n4 float4s,
// `passes` times; level as in muon_gpu_measure_read_bandwidth.
void LaunchReadBandwidth(const float4 *buf, int64_t n4, int passes, int level, int blocks, float *sink,
                         cudaStream_t st);

}  // namespace muon_gpu
