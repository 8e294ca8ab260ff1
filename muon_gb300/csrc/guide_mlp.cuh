// Learned path guiding, device side: network layout, the tensor-core operand
// image of the weights, and the von Mises-Fisher mixture the network predicts.
//
// Model (restated for the CPU in oracle/guiding.py): 8 features in [0, 1]
// (position in the scene box, shading normal and outgoing direction as
// (theta / pi, phi / 2pi + 1/2), roughness), one-blob encoded into 32 bins
// each (Mueller et al., "Neural Importance Sampling", 2019), an MLP
// 256 -> 64 -> 64 -> 64 -> 64 -> 40 with ReLU, and 8 vMF lobes of 5 outputs
// each (weight logit, unnormalised mean direction, log concentration).
//
// Inference runs on the tensor cores through tcgen05 (guide_tc.cuh); training
// is FP32 (guide.cu).
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
constexpr int kBiasFloats = 4 * kWidth + kOut;               // FP32 biases of all layers
__host__ __device__ constexpr int BiasOffset(int l) { return l * kWidth; }
// FP32 master weights [in][out] then biases, per layer, concatenated.
__host__ __device__ constexpr int MasterOffset(int l) {
  int off = 0;
  for (int k = 0; k < l; ++k) off += In(k) * Out(k) + Out(k);
  return off;
}
constexpr int kParams = MasterOffset(kLayers);

// ---- the inference image ----------------------------------------------------
// The network as the tensor cores read it: per layer the BF16 weights as an
// N x K operand (N = outputs, padded to a multiple of 16 with zero rows; K =
// inputs), K-major in 8 x 8 core matrices of 128 contiguous bytes (8 rows of
// 16 bytes): element (r, k) of an R x K operand sits at byte
// (r / 8) * (K / 8) * 128 + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2, so
// core matrices adjacent in K are 128 bytes apart and those adjacent in R are
// K / 8 * 128 bytes apart. The FP32 biases follow the last layer.
__host__ __device__ constexpr int NPad(int l) { return l == kLayers - 1 ? 48 : kWidth; }
__host__ __device__ constexpr int OperandByte(int r, int k, int K) {
  return (r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}
__host__ __device__ constexpr int ImgOffset(int l) {
  int off = 0;
  for (int k = 0; k < l; ++k) off += NPad(k) * In(k) * 2;
  return off;
}
constexpr int kImgBiasOffset = ImgOffset(kLayers);
constexpr int kImgBytes = kImgBiasOffset + kBiasFloats * 4;
static_assert(kImgBytes % 16 == 0, "bulk copies move multiples of 16 bytes");

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t PackBf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

// One-blob value of feature s at bin k.
__device__ __forceinline__ float Blob(float s, int k) {
  const float d = s - (static_cast<float>(k) + 0.5f) * (1.0f / kBins);
  return __expf(-d * d * (0.5f * kBins * kBins));
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
