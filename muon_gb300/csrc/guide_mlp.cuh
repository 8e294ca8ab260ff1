// Learned path guiding, device side: network layout, the tensor-core operand
// image of the weights, and the mixture of anisotropic lobes the network
// predicts.
//
// Model (restated for the CPU in oracle/guiding.py): 8 features in [0, 1]
// (position in the scene box, shading normal and outgoing direction as
// (theta / pi, phi / 2pi + 1/2), roughness), one-blob encoded into 32 bins
// each (Mueller et al., "Neural Importance Sampling", 2019), an MLP
// 256 -> 64 -> 64 -> 64 -> 64 -> 64 with ReLU, and 8 lobes of 8 outputs each
// (weight logit, unnormalised mean direction, log isotropic precision,
// anisotropy vector). A lobe is a 2D Gaussian in the plane tangent to the
// sphere at its mean, mapped to the sphere by gnomonic projection, so that it
// can stretch along one direction (light seen through a slit is a thin
// sliver of directions); a uniform component of weight 0.02 keeps the
// density positive everywhere.
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
constexpr int kLobeOut = 8;             // a, m (3), b, u (3)
constexpr int kOut = kLobeOut * kLobes; // 64
constexpr int kLayers = 5;
constexpr float kBMin = -3.0f, kBMax = 8.0f;
constexpr float kEpsUniform = 0.02f;    // probability of the uniform component
constexpr float kCMin = 1e-4f;          // a lobe is zero where mu . w <= kCMin
constexpr float kPi = 3.14159265358979f;

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
__host__ __device__ constexpr int NPad(int l) { return (Out(l) + 15) / 16 * 16; }
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

// The processed mixture, 72 floats per queue entry: pi[8] (weights), s[8]
// (isotropic precisions), norm[8] = sqrt(s (s + |pu|^2)) / (2 pi), mu[8][3]
// (unit means) and pu[8][3] (anisotropy, tangent to mu).
constexpr int kMixFloats = 9 * kLobes;
constexpr int kMixVec = kMixFloats / 4;  // float4 per queue entry

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

// Raw network outputs -> processed mixture.
__device__ __forceinline__ void MakeMixture(const float *raw, float *mx) {
  float amax = -INFINITY;
  for (int i = 0; i < kLobes; ++i) amax = fmaxf(amax, raw[kLobeOut * i]);
  float sum = 0.0f;
  float e[kLobes];
  for (int i = 0; i < kLobes; ++i) {
    e[i] = __expf(raw[kLobeOut * i] - amax);
    sum += e[i];
  }
  const float inv = 1.0f / sum;
  for (int i = 0; i < kLobes; ++i) {
    const float *r = raw + kLobeOut * i;
    float x = r[1], y = r[2], z = r[3];
    const float n2 = x * x + y * y + z * z;
    if (n2 > 1e-24f) {
      const float k = rsqrtf(n2);
      x *= k, y *= k, z *= k;
    } else {
      x = 0.0f, y = 0.0f, z = 1.0f;
    }
    const float s = __expf(fminf(fmaxf(r[4], kBMin), kBMax));
    const float um = r[5] * x + r[6] * y + r[7] * z;
    const float px = r[5] - um * x, py = r[6] - um * y, pz = r[7] - um * z;
    const float p2 = px * px + py * py + pz * pz;
    mx[i] = e[i] * inv;
    mx[kLobes + i] = s;
    mx[2 * kLobes + i] = sqrtf(s * (s + p2)) * (0.5f / kPi);
    float *m = mx + 3 * kLobes + 3 * i;
    m[0] = x, m[1] = y, m[2] = z;
    float *pu = mx + 6 * kLobes + 3 * i;
    pu[0] = px, pu[1] = py, pu[2] = pz;
  }
}

// Mixture density at the unit direction w: (1 - eps) sum_i pi_i p_i(w) +
// eps / (4 pi), p_i(w) = norm_i exp(-(s_i |v|^2 + (pu_i . v)^2) / 2) / c^3 with
// c = mu_i . w > kCMin and v = w / c - mu_i.
__device__ __forceinline__ float MixturePdf(const float *mx, float wx, float wy, float wz) {
  float p = 0.0f;
#pragma unroll 1
  for (int i = 0; i < kLobes; ++i) {
    const float *m = mx + 3 * kLobes + 3 * i;
    const float mu0 = __ldg(m), mu1 = __ldg(m + 1), mu2 = __ldg(m + 2);
    const float c = mu0 * wx + mu1 * wy + mu2 * wz;
    if (!(c > kCMin)) continue;
    const float ic = 1.0f / c;
    const float v0 = wx * ic - mu0, v1 = wy * ic - mu1, v2 = wz * ic - mu2;
    const float *pu = mx + 6 * kLobes + 3 * i;
    const float d = __ldg(pu) * v0 + __ldg(pu + 1) * v1 + __ldg(pu + 2) * v2;
    const float q = __ldg(mx + kLobes + i) * (v0 * v0 + v1 * v1 + v2 * v2) + d * d;
    p += __ldg(mx + i) * __ldg(mx + 2 * kLobes + i) * __expf(-0.5f * q) * (ic * ic * ic);
  }
  return (1.0f - kEpsUniform) * p + kEpsUniform * (0.25f / kPi);
}

// Draws a direction: the uniform component with probability eps (u1, u2 ->
// a point of the sphere), else a lobe by weight (u0 rescaled), then the
// tangent-plane Gaussian by Box-Muller (u1, u2) along e1 = mu x e2 and
// e2 = pu / |pu| (any tangent frame when pu = 0; Duff et al., "Building an
// Orthonormal Basis, Revisited", 2017), projected: w = normalize(mu + x).
__device__ __forceinline__ void SampleMixture(const float *mx, float u0, float u1, float u2, float *wx, float *wy,
                                              float *wz) {
  if (u0 < kEpsUniform) {
    const float z = 1.0f - 2.0f * u1;
    const float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float sn, cs;
    __sincosf(2.0f * kPi * u2, &sn, &cs);
    *wx = r * cs, *wy = r * sn, *wz = z;
    return;
  }
  const float x = (u0 - kEpsUniform) * (1.0f / (1.0f - kEpsUniform));
  int lobe = kLobes - 1;
  float acc = 0.0f;
#pragma unroll 1
  for (int i = 0; i < kLobes; ++i) {
    acc += __ldg(mx + i);
    if (x < acc) {
      lobe = i;
      break;
    }
  }
  const float *m = mx + 3 * kLobes + 3 * lobe;
  const float m0 = __ldg(m), m1 = __ldg(m + 1), m2 = __ldg(m + 2);
  const float *pu = mx + 6 * kLobes + 3 * lobe;
  float e2x = __ldg(pu), e2y = __ldg(pu + 1), e2z = __ldg(pu + 2);
  const float s = __ldg(mx + kLobes + lobe);
  const float p2 = e2x * e2x + e2y * e2y + e2z * e2z;
  if (p2 > 1e-20f) {
    const float k = rsqrtf(p2);
    e2x *= k, e2y *= k, e2z *= k;
  } else {
    const float sign = copysignf(1.0f, m2);
    const float a = -1.0f / (sign + m2);
    e2x = 1.0f + sign * m0 * m0 * a, e2y = sign * m0 * m1 * a, e2z = -sign * m0;
  }
  const float e1x = m1 * e2z - m2 * e2y, e1y = m2 * e2x - m0 * e2z, e1z = m0 * e2y - m1 * e2x;
  const float r = sqrtf(-2.0f * __logf(fmaxf(u1, 1e-30f)));
  float sn, cs;
  __sincosf(2.0f * kPi * u2, &sn, &cs);
  const float g1 = r * cs * rsqrtf(s), g2 = r * sn * rsqrtf(s + p2);
  float dx = m0 + g1 * e1x + g2 * e2x, dy = m1 + g1 * e1y + g2 * e2y, dz = m2 + g1 * e1z + g2 * e2z;
  const float k = rsqrtf(dx * dx + dy * dy + dz * dz);
  *wx = dx * k, *wy = dy * k, *wz = dz * k;
}

#endif  // __CUDACC__

}  // namespace guide
}  // namespace muon_gpu
