// Host-side CUDA helpers shared by the render entry points (render.cc,
// batch.cc): error propagation, owned device buffers, and the render setup
// that single-scene and batched renders have in common.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/muon_gpu.h"
#include "kernels.cuh"

namespace muon_gpu {

struct CudaError {
  cudaError_t code;
  const char *where;
};

#define CUDA_TRY(expr)                                                              \
  do {                                                                              \
    cudaError_t _e = (expr);                                                        \
    if (_e != cudaSuccess) throw ::muon_gpu::CudaError{_e, #expr};                  \
  } while (0)

struct DeviceBuffer {
  void *ptr = nullptr;
  size_t bytes = 0;
  DeviceBuffer() = default;
  DeviceBuffer(const DeviceBuffer &) = delete;
  DeviceBuffer &operator=(const DeviceBuffer &) = delete;
  DeviceBuffer(DeviceBuffer &&o) noexcept : ptr(o.ptr), bytes(o.bytes) {
    o.ptr = nullptr;
    o.bytes = 0;
  }
  DeviceBuffer &operator=(DeviceBuffer &&o) noexcept {
    if (this != &o) {
      if (ptr) cudaFree(ptr);
      ptr = o.ptr;
      bytes = o.bytes;
      o.ptr = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DeviceBuffer() {
    if (ptr) cudaFree(ptr);
  }
  void Ensure(size_t want) {
    if (want <= bytes && ptr) return;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    if (want == 0) return;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) throw CudaError{e, "cudaMalloc"};
    bytes = want;
  }
  template <typename T>
  T *as() const {
    return static_cast<T *>(ptr);
  }
};

// A process-wide cache of device blocks, per device, for the large per-scene
// work arrays: a destroyed scene gives its blocks back (PoolGive) and the next
// scene's EnsurePooled takes one of at least the wanted size (at most 1.5x),
// so that creating and destroying scenes does not pay cudaMalloc/cudaFree of
// gigabytes each time. Only blocks whose last use on the device has finished
// may be given. The cache holds at most 1/8 of the device's memory (oldest
// blocks are freed first) and is emptied before an allocation is allowed to
// fail; muon_gpu_release_cached() empties it on request.
void PoolGive(DeviceBuffer &buf, int device) noexcept;
void EnsurePooled(DeviceBuffer &buf, size_t want, int device);
void PoolTrim(int device) noexcept;  // device < 0: every device

template <typename T>
void Upload(DeviceBuffer &buf, const std::vector<T> &v, cudaStream_t st) {
  buf.Ensure(std::max<size_t>(v.size() * sizeof(T), 16));
  if (!v.empty()) CUDA_TRY(cudaMemcpyAsync(buf.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

// Upload into a block of the device block cache (EnsurePooled).
template <typename T>
void UploadPooled(DeviceBuffer &buf, const std::vector<T> &v, cudaStream_t st, int device) {
  EnsurePooled(buf, std::max<size_t>(v.size() * sizeof(T), 16), device);
  if (!v.empty()) CUDA_TRY(cudaMemcpyAsync(buf.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  int kind = 0;  // 0 extend, 1 occlude, 2 other
};

// Sets the thread's last error and returns `code`.
int Fail(int code, const std::string &msg);
int FailCuda(const CudaError &e);
// Camera::Camera (muon/camera.cc:15-35) evaluated on the host.
void ComputeCamera(const MuonCameraDesc &c, DevCamera *out);
// Checks a MuonRenderParams; MUON_OK or an error code (last error set).
int ValidateParams(const MuonRenderParams &p);
// Records of the two triangles of each quad light (world and object format)
// and whether each can be hit.
void BuildLightTris(const std::vector<DevLight> &lights, std::vector<PrimRecord> *lt,
                    std::vector<PrimRecord> *lt_obj, std::vector<int32_t> *lt_ok);
// ShadeParams of a render; returns the shadow slots per path vertex.
int SetupShade(const MuonRenderParams &p, int num_quad_lights, int num_other_lights, ShadeParams *out);

// How a render cuts the film's samples into wavefronts: pixels in groups of
// `pix_per_wave`, each group's samples in runs of at most `ns`; wave i is
// pixel group i / SampleGroups(), sample run i % SampleGroups(). No storage:
// callers that may not allocate enumerate the waves with At().
struct WavePlan {
  int width = 0;
  int64_t npix = 0;
  int spp = 1, ns = 1;
  int64_t pix_per_wave = 1;
  uint32_t sample_offset = 0;
  uint64_t seed = 0;
  int64_t PixelGroups() const { return (npix + pix_per_wave - 1) / pix_per_wave; }
  int64_t SampleGroups() const { return (spp + ns - 1) / ns; }
  size_t Count() const { return static_cast<size_t>(PixelGroups() * SampleGroups()); }
  WaveInfo At(size_t i) const {
    const int64_t pg = static_cast<int64_t>(i) / SampleGroups(), sg = static_cast<int64_t>(i) % SampleGroups();
    WaveInfo w{};
    w.width = width;
    w.p0 = static_cast<int32_t>(pg * pix_per_wave);
    w.npix = static_cast<int>(std::min<int64_t>(pix_per_wave, npix - pg * pix_per_wave));
    w.s0 = static_cast<int>(sg * ns);
    w.ns = std::min(ns, spp - w.s0);
    w.n = w.npix * w.ns;
    w.sample_offset = sample_offset;
    w.seed = seed;
    return w;
  }
};
// Wavefronts of at most `budget` paths for a width x height film.
WavePlan PlanWaves(int width, int height, const MuonRenderParams &p, int64_t budget);

// Bounces a wavefront runs: `traces` is false when Integrator::Trace casts no
// ray at all (max_depth 0 with lights sampled); `bounded` when the depth is
// bounded (or the integrator is not the path tracer), so that the launch
// sequence is fixed; `bounces` is the number of extend passes.
struct BouncePlan {
  bool traces = false, bounded = true;
  int bounces = 0;
};
BouncePlan PlanBounces(const MuonRenderParams &p, const ShadeParams &sp);

// Places the static scratch buffer of muon_gpu_render_noalloc on the current
// device (loading its module) and checks that its address can be taken
// (noalloc.cu). Scene creation calls it, so that the buffer is taken then and
// not during a render.
cudaError_t NoAllocPrepare();

// Bytes of per-wavefront path state per path with `slots` shadow slots (the
// arrays of PathBuffers, unpadded).
inline int64_t WorkBytesPerPath(int slots) {
  return 8 * 16 /* ray_o, ray_d, tp, rad (double-buffered) */ + 8 /* hits */ + 4 /* link */ +
         16 /* final_rad */ + 16 /* org */ + int64_t(kNumClasses) * 4 /* order */ +
         int64_t(std::max(slots, 1)) * (16 + 16 + 4) /* contrib, slot_dir, shq */;
}

}  // namespace muon_gpu
