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

}  // namespace muon_gpu
