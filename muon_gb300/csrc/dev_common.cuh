// Device-side scene view, vector helpers and the counter-based RNG.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/muon_gpu.h"
#include "dev_layout.h"
#include "mmath.h"

namespace muon_gpu {

constexpr float kEps = 0.0001f;  // kEpsilon, muon/types.h:13

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 f3(const F4 &v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 f3(const float4 &v) { return make_float3(v.x, v.y, v.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator-(float3 a) { return f3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float3 operator*(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return f3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float length3(float3 v) { return sqrtf(dot3(v, v)); }
__device__ __forceinline__ float3 normalize3(float3 v) { return v * (1.0f / sqrtf(dot3(v, v))); }
__device__ __forceinline__ float3 reflect3(float3 d, float3 n) { return d - (2.0f * dot3(d, n)) * n; }
__device__ __forceinline__ float max3c(float3 v) { return fmaxf(fmaxf(v.x, v.y), v.z); }
__device__ __forceinline__ bool nonzero3(float3 v) { return v.x != 0.0f || v.y != 0.0f || v.z != 0.0f; }

__device__ __forceinline__ float3 xform_point3(const float *m, float3 p) {
  // rows 0..2 of M * (p, 1), columns packed as m[3c..3c+2]
  return f3((m[0] * p.x + m[3] * p.y) + (m[6] * p.z + m[9]), (m[1] * p.x + m[4] * p.y) + (m[7] * p.z + m[10]),
            (m[2] * p.x + m[5] * p.y) + (m[8] * p.z + m[11]));
}
__device__ __forceinline__ float3 xform_vec3(const float *m, float3 d) {
  return f3((m[0] * d.x + m[3] * d.y) + m[6] * d.z, (m[1] * d.x + m[4] * d.y) + m[7] * d.z,
            (m[2] * d.x + m[5] * d.y) + m[8] * d.z);
}

// ---------------------------------------------------------------------------
// Counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC 2011). A 128-bit counter and a
// 64-bit key give four independent 32-bit outputs per evaluation, so every
// (sample, bounce, draw) has its own stream without stored state.
// ---------------------------------------------------------------------------
struct Philox {
  static constexpr uint32_t kMul0 = 0xD2511F53u;
  static constexpr uint32_t kMul1 = 0xCD9E8D57u;
  static constexpr uint32_t kWeyl0 = 0x9E3779B9u;
  static constexpr uint32_t kWeyl1 = 0xBB67AE85u;

  __device__ __forceinline__ static uint4 Eval(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
      uint32_t hi0 = __umulhi(kMul0, c.x), lo0 = kMul0 * c.x;
      uint32_t hi1 = __umulhi(kMul1, c.z), lo1 = kMul1 * c.z;
      c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
      k.x += kWeyl0;
      k.y += kWeyl1;
    }
    return c;
  }
};

// Uniform floats in [0, 1) for one (sample, bounce) pair; draws are consumed
// four at a time from successive counters.
struct Rng {
  uint4 ctr;
  uint2 key;
  uint4 buf;
  int left;

  __device__ __forceinline__ Rng(uint64_t seed, uint64_t sample, uint32_t bounce) {
    key = make_uint2(static_cast<uint32_t>(seed), static_cast<uint32_t>(seed >> 32));
    ctr = make_uint4(static_cast<uint32_t>(sample), static_cast<uint32_t>(sample >> 32), bounce, 0u);
    left = 0;
  }
  __device__ __forceinline__ float Next() {
    if (left == 0) {
      buf = Philox::Eval(ctr, key);
      ctr.w += 1u;
      left = 4;
    }
    uint32_t x;
    switch (left) {
      case 4: x = buf.x; break;
      case 3: x = buf.y; break;
      case 2: x = buf.z; break;
      default: x = buf.w; break;
    }
    --left;
    return static_cast<float>(x >> 8) * (1.0f / 16777216.0f);
  }
};

}  // namespace muon_gpu
