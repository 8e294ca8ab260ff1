// Learned path guiding, device side: network layout, tensor-core inference
// for one warp, and the von Mises-Fisher mixture it predicts.
//
// Model (restated for the CPU in oracle/guiding.py): 8 features in [0, 1]
// (position in the scene box, shading normal and outgoing direction as
// (theta / pi, phi / 2pi + 1/2), roughness), one-blob encoded into 32 bins
// each (Mueller et al., "Neural Importance Sampling", 2019), an MLP
// 256 -> 64 -> 64 -> 64 -> 64 -> 40 with ReLU, and 8 vMF lobes of 5 outputs
// each (weight logit, unnormalised mean direction, log concentration).
//
// Inference runs on the tensor cores: mma.sync m16n8k16 with BF16 operands
// and FP32 accumulation, one warp per 32 samples (two 16-row tiles). The
// accumulator fragment of two adjacent 8-column tiles has the layout of the
// next layer's 16-column operand fragment, so activations stay in registers
// from layer to layer; weights are read from shared memory, stored
// transposed (output-major) with rows padded by 8 elements, which makes every
// operand fetch one conflict-free 32-bit load.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace muon_gpu {
namespace guide {

constexpr int kBins = 32;
constexpr int kFeatures = 8;
constexpr int kIn = kFeatures * kBins;  // 256
constexpr int kWidth = 64;
constexpr int kLobes = 8;
constexpr int kOut = 5 * kLobes;        // 40
constexpr int kLayers = 5;
constexpr float kBMin = -3.0f, kBMax = 8.0f;

// Layer l maps In(l) -> Out(l).
__host__ __device__ constexpr int In(int l) { return l == 0 ? kIn : kWidth; }
__host__ __device__ constexpr int Out(int l) { return l == kLayers - 1 ? kOut : kWidth; }
// Transposed BF16 weights: Out(l) rows of In(l) + 8 elements.
__host__ __device__ constexpr int Stride(int l) { return In(l) + 8; }
__host__ __device__ constexpr int WtOffset(int l) {
  int off = 0;
  for (int k = 0; k < l; ++k) off += Out(k) * Stride(k);
  return off;
}
constexpr int kWtElems = WtOffset(kLayers);                  // BF16 elements of all layers
constexpr int kBiasFloats = 4 * kWidth + kOut;               // FP32 biases of all layers
__host__ __device__ constexpr int BiasOffset(int l) { return l * kWidth; }
// FP32 master weights [in][out] then biases, per layer, concatenated.
__host__ __device__ constexpr int MasterOffset(int l) {
  int off = 0;
  for (int k = 0; k < l; ++k) off += In(k) * Out(k) + Out(k);
  return off;
}
constexpr int kParams = MasterOffset(kLayers);
constexpr int kSmemBytes = kWtElems * 2 + kBiasFloats * 4;

#ifdef __CUDACC__

__device__ __forceinline__ void MmaBf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t PackBf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

// One-blob value of feature s at bin k.
__device__ __forceinline__ float Blob(float s, int k) {
  const float d = s - (static_cast<float>(k) + 0.5f) * (1.0f / kBins);
  return __expf(-d * d * (0.5f * kBins * kBins));
}

// Copies the network (transposed BF16 weights and FP32 biases) into shared
// memory; all threads of the block take part.
__device__ __forceinline__ void LoadNetwork(const __nv_bfloat16 *wt, const float *bias, unsigned char *smem) {
  const int4 *src = reinterpret_cast<const int4 *>(wt);
  int4 *dst = reinterpret_cast<int4 *>(smem);
  for (int i = threadIdx.x; i < kWtElems * 2 / 16; i += blockDim.x) dst[i] = src[i];
  float *sb = reinterpret_cast<float *>(smem + kWtElems * 2);
  for (int i = threadIdx.x; i < kBiasFloats; i += blockDim.x) sb[i] = bias[i];
}

// Forward pass of one warp over 32 samples: sample r of the warp has
// features feat(r, d). Writes the 40 raw outputs of sample r to out[r * 40 + c]
// (shared memory of the warp). `smem` holds the network (LoadNetwork).
template <class Feat>
__device__ __forceinline__ void ForwardWarp(const unsigned char *smem, Feat feat, float *out) {
  const __nv_bfloat16 *sw = reinterpret_cast<const __nv_bfloat16 *>(smem);
  const float *sb = reinterpret_cast<const float *>(smem + kWtElems * 2);
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;

  uint32_t act[2][4][4];  // BF16 operand fragments of a 64-wide activation
  float acc[2][8][4];
  // ---- layer 0: one-blob input, 16 k-blocks
#pragma unroll
  for (int m = 0; m < 2; ++m)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.0f;
  {
    const __nv_bfloat16 *w = sw + WtOffset(0);
#pragma unroll 2
    for (int kb = 0; kb < kIn / 16; ++kb) {
      // columns 16 kb + 2t (+1) and +8: feature kb / 2, bins 16 (kb & 1) + 2t ...
      const int d = kb >> 1;
      const int k0 = 16 * (kb & 1) + 2 * t;
      uint32_t a[2][4];
#pragma unroll
      for (int m = 0; m < 2; ++m) {
        // this thread's rows of tile m: g and g + 8
        const float s0 = feat(16 * m + g, d), s1 = feat(16 * m + g + 8, d);
        a[m][0] = PackBf16(Blob(s0, k0), Blob(s0, k0 + 1));
        a[m][1] = PackBf16(Blob(s1, k0), Blob(s1, k0 + 1));
        a[m][2] = PackBf16(Blob(s0, k0 + 8), Blob(s0, k0 + 9));
        a[m][3] = PackBf16(Blob(s1, k0 + 8), Blob(s1, k0 + 9));
      }
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const __nv_bfloat16 *row = w + (8 * j + g) * Stride(0) + 16 * kb + 2 * t;
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row);
        const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + 8);
        MmaBf16(acc[0][j], a[0], b0, b1);
        MmaBf16(acc[1][j], a[1], b0, b1);
      }
    }
  }
  // bias + ReLU, repacked as the next layer's operand
  auto to_act = [&](int layer) {
    const float *b = sb + BiasOffset(layer);
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int kb = 0; kb < 4; ++kb) {
        const int c0 = 16 * kb + 2 * t, c1 = c0 + 8;
        const float *lo = acc[m][2 * kb], *hi = acc[m][2 * kb + 1];
        act[m][kb][0] = PackBf16(fmaxf(lo[0] + b[c0], 0.0f), fmaxf(lo[1] + b[c0 + 1], 0.0f));
        act[m][kb][1] = PackBf16(fmaxf(lo[2] + b[c0], 0.0f), fmaxf(lo[3] + b[c0 + 1], 0.0f));
        act[m][kb][2] = PackBf16(fmaxf(hi[0] + b[c1], 0.0f), fmaxf(hi[1] + b[c1 + 1], 0.0f));
        act[m][kb][3] = PackBf16(fmaxf(hi[2] + b[c1], 0.0f), fmaxf(hi[3] + b[c1 + 1], 0.0f));
      }
  };
  to_act(0);
  // ---- hidden layers 1..3
#pragma unroll 1
  for (int layer = 1; layer < kLayers - 1; ++layer) {
    const __nv_bfloat16 *w = sw + WtOffset(layer);
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[m][j][0] = acc[m][j][1] = acc[m][j][2] = acc[m][j][3] = 0.0f;
#pragma unroll
    for (int kb = 0; kb < 4; ++kb)
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const __nv_bfloat16 *row = w + (8 * j + g) * Stride(1) + 16 * kb + 2 * t;
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row);
        const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + 8);
        MmaBf16(acc[0][j], act[0][kb], b0, b1);
        MmaBf16(acc[1][j], act[1][kb], b0, b1);
      }
    to_act(layer);
  }
  // ---- output layer: 5 tiles of 8 columns
  {
    const __nv_bfloat16 *w = sw + WtOffset(kLayers - 1);
    const float *b = sb + BiasOffset(kLayers - 1);
    float o[2][5][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int j = 0; j < 5; ++j) o[m][j][0] = o[m][j][1] = o[m][j][2] = o[m][j][3] = 0.0f;
#pragma unroll
    for (int kb = 0; kb < 4; ++kb)
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const __nv_bfloat16 *row = w + (8 * j + g) * Stride(kLayers - 1) + 16 * kb + 2 * t;
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(row);
        const uint32_t b1 = *reinterpret_cast<const uint32_t *>(row + 8);
        MmaBf16(o[0][j], act[0][kb], b0, b1);
        MmaBf16(o[1][j], act[1][kb], b0, b1);
      }
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const int c = 8 * j + 2 * t;
        const int r0 = 16 * m + g, r1 = r0 + 8;
        out[r0 * kOut + c] = o[m][j][0] + b[c];
        out[r0 * kOut + c + 1] = o[m][j][1] + b[c + 1];
        out[r1 * kOut + c] = o[m][j][2] + b[c];
        out[r1 * kOut + c + 1] = o[m][j][3] + b[c + 1];
      }
  }
}

// ---- the mixture -----------------------------------------------------------
// Processed form, 40 floats: pi[8] (weights), kappa[8] (concentrations) and
// mu[8][3] (unit mean directions), read in place from memory.
constexpr int kMixFloats = 40;

// Raw network outputs -> weights (softmax), concentrations, unit means.
__device__ __forceinline__ void MakeMixture(const float *raw, float *mx) {
  float amax = -INFINITY;
  for (int i = 0; i < kLobes; ++i) amax = fmaxf(amax, raw[5 * i]);
  float sum = 0.0f;
  float e[kLobes];
  for (int i = 0; i < kLobes; ++i) {
    e[i] = __expf(raw[5 * i] - amax);
    sum += e[i];
  }
  const float inv = 1.0f / sum;
  for (int i = 0; i < kLobes; ++i) {
    mx[i] = e[i] * inv;
    mx[kLobes + i] = __expf(fminf(fmaxf(raw[5 * i + 4], kBMin), kBMax));
    float x = raw[5 * i + 1], y = raw[5 * i + 2], z = raw[5 * i + 3];
    const float n2 = x * x + y * y + z * z;
    if (n2 > 1e-24f) {
      const float r = rsqrtf(n2);
      x *= r, y *= r, z *= r;
    } else {
      x = 0.0f, y = 0.0f, z = 1.0f;
    }
    mx[2 * kLobes + 3 * i] = x, mx[2 * kLobes + 3 * i + 1] = y, mx[2 * kLobes + 3 * i + 2] = z;
  }
}

// vMF density kappa / (2 pi (1 - exp(-2 kappa))) exp(kappa (mu . w - 1)).
__device__ __forceinline__ float VmfPdf(float mx, float my, float mz, float kappa, float wx, float wy, float wz) {
  const float c = mx * wx + my * wy + mz * wz;
  return kappa / (2.0f * 3.14159265358979f * -expm1f(-2.0f * kappa)) * __expf(kappa * (c - 1.0f));
}

__device__ __forceinline__ float MixturePdf(const float *mx, float wx, float wy, float wz) {
  float p = 0.0f;
#pragma unroll 1
  for (int i = 0; i < kLobes; ++i) {
    const float *m = mx + 2 * kLobes + 3 * i;
    p += __ldg(mx + i) * VmfPdf(__ldg(m), __ldg(m + 1), __ldg(m + 2), __ldg(mx + kLobes + i), wx, wy, wz);
  }
  return p;
}

// Draws a direction: lobe by weight, then the vMF sampling of W. Jakob,
// "Numerically stable sampling of the von Mises-Fisher distribution on S^2"
// (2012): cos = 1 + log(u1 + (1 - u1) exp(-2 kappa)) / kappa, azimuth 2 pi
// u2, in an orthonormal frame around mu (Duff et al., "Building an
// Orthonormal Basis, Revisited", 2017).
__device__ __forceinline__ void SampleMixture(const float *mx, float u0, float u1, float u2, float *wx, float *wy,
                                              float *wz) {
  int lobe = kLobes - 1;
  float acc = 0.0f;
#pragma unroll 1
  for (int i = 0; i < kLobes; ++i) {
    acc += __ldg(mx + i);
    if (u0 < acc) {
      lobe = i;
      break;
    }
  }
  const float k = __ldg(mx + kLobes + lobe);
  const float m0 = __ldg(mx + 2 * kLobes + 3 * lobe), m1 = __ldg(mx + 2 * kLobes + 3 * lobe + 1),
              m2 = __ldg(mx + 2 * kLobes + 3 * lobe + 2);
  float c = 1.0f + __logf(u1 + (1.0f - u1) * __expf(-2.0f * k)) / k;
  c = fminf(fmaxf(c, -1.0f), 1.0f);
  const float s = sqrtf(fmaxf(0.0f, 1.0f - c * c));
  float sn, cs;
  __sincosf(2.0f * 3.14159265358979f * u2, &sn, &cs);
  const float sign = copysignf(1.0f, m2);
  const float a = -1.0f / (sign + m2);
  const float b = m0 * m1 * a;
  const float t1x = 1.0f + sign * m0 * m0 * a, t1y = sign * b, t1z = -sign * m0;
  const float t2x = b, t2y = sign + m1 * m1 * a, t2z = -m1;
  *wx = s * (cs * t1x + sn * t2x) + c * m0;
  *wy = s * (cs * t1y + sn * t2y) + c * m1;
  *wz = s * (cs * t1z + sn * t2z) + c * m2;
}

#endif  // __CUDACC__

}  // namespace guide
}  // namespace muon_gpu
