// Learned path guiding: network initialisation and packing, tensor-core
// forward pass for given features, and the training step.
//
// Training is a hand-written FP32 pipeline over a batch of samples: the
// forward pass layer by layer (inputs of every layer kept), the mixture loss
// gradient per sample, the backward pass layer by layer, and weight gradients
// as per-chunk partial sums reduced in a fixed order, so a step's gradients do
// not depend on scheduling. Adam then updates the FP32 master weights, which
// are repacked as the BF16 tensor-core operand image for inference.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "dev_common.cuh"
#include "guide.h"
#include "guide_mlp.cuh"
#include "guide_tc.cuh"

namespace muon_gpu {

namespace {

using namespace guide;

constexpr int kThreads = 256;
constexpr int kChunk = 512;  // samples per weight-gradient partial

// ---- packing and initialisation ------------------------------------------------
// The inference image (guide_mlp.cuh): one thread per 16-byte chunk of a
// layer's operand (8 BF16 weights of one output along K) or per bias.
constexpr int kImgChunks = kImgBiasOffset / 16;

__global__ void PackKernel(const float *params, unsigned char *img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kImgChunks) {
    const int byte = 16 * i;
    int l = 0;
    while (l + 1 < kLayers && byte >= ImgOffset(l + 1)) ++l;
    const int K = In(l);
    const int local = byte - ImgOffset(l);
    const int rb = local / ((K / 8) * 128), rem = local % ((K / 8) * 128);
    const int kb = rem / 128, r = rb * 8 + (rem % 128) / 16;
    uint32_t w[4];
    for (int e = 0; e < 4; ++e) {
      const int k = 8 * kb + 2 * e;
      float lo = 0.0f, hi = 0.0f;
      if (r < Out(l)) {
        lo = params[MasterOffset(l) + k * Out(l) + r];
        hi = params[MasterOffset(l) + (k + 1) * Out(l) + r];
      }
      w[e] = PackBf16(lo, hi);
    }
    *reinterpret_cast<uint4 *>(img + byte) = make_uint4(w[0], w[1], w[2], w[3]);
  }
  if (i < kBiasFloats) {
    const int l = i < 4 * kWidth ? i / kWidth : kLayers - 1;
    const int o = i - BiasOffset(l);
    reinterpret_cast<float *>(img + kImgBiasOffset)[i] = params[MasterOffset(l) + In(l) * Out(l) + o];
  }
}

// He-uniform weights U(-sqrt(6 / fan_in), sqrt(6 / fan_in)), zero biases.
__global__ void InitKernel(float *params, uint64_t seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  int l = 0;
  while (l + 1 < kLayers && i >= MasterOffset(l + 1)) ++l;
  const int local = i - MasterOffset(l);
  if (local >= In(l) * Out(l)) {
    params[i] = 0.0f;
    return;
  }
  Rng r(seed, 0, 0);
  r.ctr = make_uint4(static_cast<uint32_t>(i), 0x6d6c70u, 0u, 0u);
  const float lim = sqrtf(6.0f / static_cast<float>(In(l)));
  params[i] = (2.0f * r.Next() - 1.0f) * lim;
}

// ---- tensor-core forward for given features ------------------------------------
// The inference kernel's network pass (guide_tc.cuh) over features read from
// memory: one CTA per SM, 128 rows per group.
__global__ void __launch_bounds__(kTcThreads, 1) ForwardKernel(const void *img, const float *features, int n,
                                                               float *out, int32_t *status) {
  extern __shared__ __align__(1024) unsigned char smem[];
  if (static_cast<int>(blockIdx.x) * kTcThreads >= n) return;  // the whole CTA
  TcGroup grp;
  bool ok = TcBegin(smem, img, &grp);
  const int group = threadIdx.x / kTcRows;
  for (int base = (blockIdx.x * 2 + group) * kTcRows; ok && base < n; base += gridDim.x * kTcThreads) {
    const int r = base + grp.row;
    float f[kFeatures];
#pragma unroll
    for (int d = 0; d < kFeatures; ++d) f[d] = r < n ? features[static_cast<int64_t>(r) * kFeatures + d] : 0.0f;
    float o[kOut];
    ok = TcForward(grp, f, o);
    if (ok && r < n)
#pragma unroll
      for (int c = 0; c < kOut; ++c) out[static_cast<int64_t>(r) * kOut + c] = o[c];
  }
  TcEnd(smem, grp, status);
}

// T consecutive floats of shared memory into registers, as 16- or 8-byte
// loads where T allows (p is aligned to T floats).
template <int T>
__device__ __forceinline__ void LoadRow(const float *p, float (&v)[T]) {
  if constexpr (T % 4 == 0) {
#pragma unroll
    for (int q = 0; q < T / 4; ++q) {
      const float4 f = reinterpret_cast<const float4 *>(p)[q];
      v[4 * q] = f.x, v[4 * q + 1] = f.y, v[4 * q + 2] = f.z, v[4 * q + 3] = f.w;
    }
  } else if constexpr (T % 2 == 0) {
#pragma unroll
    for (int q = 0; q < T / 2; ++q) {
      const float2 f = reinterpret_cast<const float2 *>(p)[q];
      v[2 * q] = f.x, v[2 * q + 1] = f.y;
    }
  } else {
#pragma unroll
    for (int q = 0; q < T; ++q) v[q] = p[q];
  }
}

// ---- sampling the mixture for given network outputs ------------------------------
__global__ void MixKernel(const float *raw, int n, float *mix) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) MakeMixture(raw + static_cast<int64_t>(i) * kOut, mix + static_cast<int64_t>(i) * kMixFloats);
}

__global__ void SampleKernel(const float *mix, int n, const float *u, float *dirs, float *pdf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *mx = mix + static_cast<int64_t>(i) * kMixFloats;
  float wx, wy, wz;
  SampleMixture(mx, u[3 * i], u[3 * i + 1], u[3 * i + 2], &wx, &wy, &wz);
  dirs[3 * i] = wx, dirs[3 * i + 1] = wy, dirs[3 * i + 2] = wz;
  pdf[i] = MixturePdf(mx, wx, wy, wz);
}

// ---- training: forward ----------------------------------------------------------
// y[b][n] = act(sum_k x[b][k] w[k][n] + bias[n]) for a tile of 64 samples;
// with kBlob, x is the one-blob encoding of features (batch x 8).
template <bool kBlob, bool kRelu>
__global__ void __launch_bounds__(kThreads) FwdLayerKernel(const float *x, const float *w, const float *bias, int K,
                                                           int N, float *y, int batch) {
  __shared__ float xs[64][33];
  __shared__ __align__(16) float ws[32][64];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int b0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 32) {
    for (int i = tid; i < 64 * 32; i += kThreads) {
      const int r = i >> 5, c = i & 31, b = b0 + r, k = k0 + c;
      float v = 0.0f;
      if (b < batch) {
        if (kBlob) v = Blob(x[static_cast<int64_t>(b) * kFeatures + k / kBins], k % kBins);
        else v = x[static_cast<int64_t>(b) * K + k];
      }
      xs[r][c] = v;
    }
    for (int i = tid; i < 32 * 64; i += kThreads) {
      const int r = i >> 6, c = i & 63;
      ws[r][c] = c < N ? w[(k0 + r) * N + c] : 0.0f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      float a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = xs[ty * 4 + i][kk];
      LoadRow<4>(&ws[kk][tx * 4], bb);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * bb[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = b0 + ty * 4 + i;
    if (b >= batch) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tx * 4 + j;
      if (c >= N) continue;
      float v = acc[i][j] + bias[c];
      y[static_cast<int64_t>(b) * N + c] = kRelu ? fmaxf(v, 0.0f) : v;
    }
  }
}

// ---- training: loss ---------------------------------------------------------------
// Replaces z (raw outputs) by d(mean loss)/dz and writes per-block loss sums.
// Per sample: loss -weight log q(w) and its gradient with respect to the 64
// raw outputs (written over them), mean over the batch. q = (1 - eps)
// sum_i pi_i p_i + eps / (4 pi) with the lobes of guide_mlp.cuh; the
// gradient of log p_i follows oracle/guiding.py (loss_grad), through
// s = exp(b) (inside the clip range), the tangent projection pu = u - (u.mu) mu
// and mu = m / |m|.
__global__ void __launch_bounds__(kThreads) LossKernel(float *z, const float *dirs, const float *weights, int batch,
                                                       double *loss_out) {
  __shared__ double red[kThreads];
  const int b = blockIdx.x * kThreads + threadIdx.x;
  double loss = 0.0;
  if (b < batch) {
    float *r = z + static_cast<int64_t>(b) * kOut;
    const float w[3] = {dirs[3 * b], dirs[3 * b + 1], dirs[3 * b + 2]};
    const float wt = weights[b];
    float amax = -INFINITY;
    for (int i = 0; i < kLobes; ++i) amax = fmaxf(amax, r[kLobeOut * i]);
    float se = 0.0f;
    for (int i = 0; i < kLobes; ++i) se += expf(r[kLobeOut * i] - amax);
    const float lse = amax + logf(se);
    // pass 1: log of each lobe's share of q (-inf where the lobe is zero)
    float t[kLobes];
    const float log_keep = logf(1.0f - kEpsUniform), t_uniform = logf(kEpsUniform * 0.25f / kPi);
    float tmax = t_uniform;
    for (int i = 0; i < kLobes; ++i) {
      const float *ri = r + kLobeOut * i;
      t[i] = -INFINITY;
      const float n2 = ri[1] * ri[1] + ri[2] * ri[2] + ri[3] * ri[3];
      float mu[3] = {0.0f, 0.0f, 1.0f};
      if (n2 > 1e-24f) {
        const float k = 1.0f / sqrtf(n2);
        mu[0] = ri[1] * k, mu[1] = ri[2] * k, mu[2] = ri[3] * k;
      }
      const float c = mu[0] * w[0] + mu[1] * w[1] + mu[2] * w[2];
      if (!(c > kCMin)) continue;
      const float s = expf(fminf(fmaxf(ri[4], kBMin), kBMax));
      const float um = ri[5] * mu[0] + ri[6] * mu[1] + ri[7] * mu[2];
      float pu[3], v[3], p2 = 0.0f, v2 = 0.0f, d = 0.0f;
      for (int k = 0; k < 3; ++k) {
        pu[k] = ri[5 + k] - um * mu[k];
        v[k] = w[k] / c - mu[k];
        p2 += pu[k] * pu[k], v2 += v[k] * v[k], d += pu[k] * v[k];
      }
      const float logp = 0.5f * logf(s) + 0.5f * logf(s + p2) - logf(2.0f * kPi) - 0.5f * (s * v2 + d * d) -
                         3.0f * logf(c);
      t[i] = log_keep + (ri[0] - lse) + logp;
      tmax = fmaxf(tmax, t[i]);
    }
    float qs = expf(t_uniform - tmax);
    for (int i = 0; i < kLobes; ++i) qs += expf(t[i] - tmax);
    const float logq = tmax + logf(qs);
    loss = -static_cast<double>(wt) * logq;
    const float coef = -wt / static_cast<float>(batch);
    float resp[kLobes], rsum = 0.0f;
    for (int i = 0; i < kLobes; ++i) {
      resp[i] = expf(t[i] - logq);
      rsum += resp[i];
    }
    // pass 2: gradients, written over the raw outputs
    for (int i = 0; i < kLobes; ++i) {
      float *ri = r + kLobeOut * i;
      const float pi = expf(ri[0] - lse);
      float g[kLobeOut] = {coef * (resp[i] - pi * rsum), 0, 0, 0, 0, 0, 0, 0};
      const float n2 = ri[1] * ri[1] + ri[2] * ri[2] + ri[3] * ri[3];
      float mu[3] = {0.0f, 0.0f, 1.0f};
      const float nrm = sqrtf(n2);
      if (n2 > 1e-24f) mu[0] = ri[1] / nrm, mu[1] = ri[2] / nrm, mu[2] = ri[3] / nrm;
      const float c = mu[0] * w[0] + mu[1] * w[1] + mu[2] * w[2];
      if (resp[i] > 0.0f && c > kCMin) {
        const float cr = coef * resp[i];
        const float braw = ri[4];
        const float s = expf(fminf(fmaxf(braw, kBMin), kBMax));
        const float um = ri[5] * mu[0] + ri[6] * mu[1] + ri[7] * mu[2];
        float pu[3], v[3], p2 = 0.0f, v2 = 0.0f, d = 0.0f, vw = 0.0f, pw = 0.0f;
        for (int k = 0; k < 3; ++k) {
          pu[k] = ri[5 + k] - um * mu[k];
          v[k] = w[k] / c - mu[k];
          p2 += pu[k] * pu[k], v2 += v[k] * v[k], d += pu[k] * v[k];
          vw += v[k] * w[k], pw += pu[k] * w[k];
        }
        const float sp2 = s + p2;
        if (braw > kBMin && braw < kBMax) g[4] = cr * (0.5f + 0.5f * s / sp2 - 0.5f * s * v2);
        for (int k = 0; k < 3; ++k) g[5 + k] = cr * (pu[k] / sp2 - d * v[k]);
        if (n2 > 1e-24f) {
          const float ic2 = 1.0f / (c * c);
          float gm[3], dot = 0.0f;
          for (int k = 0; k < 3; ++k) {
            gm[k] = -um * pu[k] / sp2 + s * (vw * w[k] * ic2 + v[k]) + d * (um * v[k] + pw * w[k] * ic2 + pu[k]) -
                    3.0f * w[k] / c;
            dot += gm[k] * mu[k];
          }
          for (int k = 0; k < 3; ++k) g[1 + k] = cr * (gm[k] - dot * mu[k]) / nrm;
        }
      }
      for (int k = 0; k < kLobeOut; ++k) ri[k] = g[k];
    }
  }
  red[threadIdx.x] = loss;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) loss_out[blockIdx.x] = red[0];
}

// ---- training: backward -------------------------------------------------------------
// dx[b][k] = (sum_n dz[b][n] w[k][n]) * (h[b][k] > 0), K = 64, N <= 64.
__global__ void __launch_bounds__(kThreads) BwdDataKernel(const float *dz, const float *w, const float *h, int N,
                                                          float *dx, int batch) {
  __shared__ float ds[64][65];
  __shared__ __align__(16) float wt[64][68];  // wt[n][k] = w[k][n], rows 16-byte aligned
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int b0 = blockIdx.x * 64;
  for (int i = tid; i < 64 * 64; i += kThreads) {
    const int r = i >> 6, c = i & 63, b = b0 + r;
    ds[r][c] = (b < batch && c < N) ? dz[static_cast<int64_t>(b) * N + c] : 0.0f;
    wt[c][r] = c < N ? w[r * N + c] : 0.0f;  // w row k = r, column n = c
  }
  __syncthreads();
  float acc[4][4] = {};
  for (int n = 0; n < N; ++n) {
    float a[4], bb[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) a[i] = ds[ty * 4 + i][n];
    LoadRow<4>(&wt[n][tx * 4], bb);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * bb[j];
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int b = b0 + ty * 4 + i;
    if (b >= batch) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int k = tx * 4 + j;
      const int64_t o = static_cast<int64_t>(b) * kWidth + k;
      dx[o] = h[o] > 0.0f ? acc[i][j] : 0.0f;
    }
  }
}

// Per chunk of samples: partial[k * N + n] = sum_b x[b][k] dz[b][n] and the
// bias part partial[K * N + n] = sum_b dz[b][n]. Each thread owns a TK x TN
// block of outputs.
// Weight and bias gradients of one layer over one chunk of kChunk samples:
// partial[chunk][k][n] = sum over the chunk's samples of x[b][k] dz[b][n].
// Each thread owns a TK x TN tile of the K x N gradient; 32 samples at a time
// are staged in shared memory (rows of K and N floats, read back as vectors).
template <bool kBlob, int K, int N, int TK, int TN>
__global__ void __launch_bounds__(kThreads) WgradKernel(const float *x, const float *dz, int batch, float *partial,
                                                        int stride, int layer_off) {
  static_assert((K / TK) * (N / TN) == kThreads, "thread tiling");
  static_assert(K % 4 == 0 && N % 4 == 0, "rows of whole 16-byte vectors");
  __shared__ __align__(16) float xs[32][K];
  __shared__ __align__(16) float ds[32][N];
  __shared__ float fs[32][kFeatures];  // one-blob input: the slab's features
  const int tid = threadIdx.x;
  const int kg = tid / (N / TN), ng = tid % (N / TN);
  const int b0 = blockIdx.x * kChunk;
  float acc[TK][TN] = {};
  float bacc = 0.0f;
  for (int s0 = b0; s0 < b0 + kChunk && s0 < batch; s0 += 32) {
    if (kBlob) {
      for (int i = tid; i < 32 * kFeatures; i += kThreads) {
        const int r = i / kFeatures, b = s0 + r;
        fs[r][i % kFeatures] = b < batch ? x[static_cast<int64_t>(b) * kFeatures + i % kFeatures] : 0.0f;
      }
      __syncthreads();
    }
    for (int i = tid; i < 32 * K; i += kThreads) {
      const int r = i / K, k = i % K, b = s0 + r;
      float v = 0.0f;
      if (b < batch) {
        if (kBlob) v = Blob(fs[r][k / kBins], k % kBins);
        else v = x[static_cast<int64_t>(b) * K + k];
      }
      xs[r][k] = v;
    }
    for (int i = tid; i < 32 * N; i += kThreads) {
      const int r = i / N, n = i % N, b = s0 + r;
      ds[r][n] = b < batch ? dz[static_cast<int64_t>(b) * N + n] : 0.0f;
    }
    __syncthreads();
#pragma unroll 4
    for (int r = 0; r < 32; ++r) {
      float a[TK], d[TN];
      LoadRow<TK>(&xs[r][kg * TK], a);
      LoadRow<TN>(&ds[r][ng * TN], d);
#pragma unroll
      for (int i = 0; i < TK; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] += a[i] * d[j];
    }
    if (tid < N)
      for (int r = 0; r < 32; ++r) bacc += ds[r][tid];
    __syncthreads();
  }
  float *p = partial + static_cast<int64_t>(blockIdx.x) * stride + layer_off;
#pragma unroll
  for (int i = 0; i < TK; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) p[(kg * TK + i) * N + ng * TN + j] = acc[i][j];
  if (tid < N) p[K * N + tid] = bacc;
}

__global__ void ReduceKernel(const float *partial, int chunks, float *grad) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  float s = 0.0f;
  for (int c = 0; c < chunks; ++c) s += partial[static_cast<int64_t>(c) * kParams + i];
  grad[i] = s;
}

// Adam (Kingma and Ba, 2015) with bias correction.
__global__ void AdamKernel(float *params, float *m, float *v, const float *grad, float lr, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kParams) return;
  const float g = grad[i];
  const float mi = 0.9f * m[i] + 0.1f * g;
  const float vi = 0.999f * v[i] + 0.001f * g * g;
  m[i] = mi;
  v[i] = vi;
  params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

// ---- sample gathering -----------------------------------------------------------------
__global__ void GatherKernel(const GuideSample *pool, uint64_t available, uint32_t cap, int batch, uint64_t seed,
                             float *features, float *dirs, float *weights) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch) return;
  const uint64_t valid = available < cap ? available : cap;
  Rng r(seed, 0, 0);
  r.ctr = make_uint4(static_cast<uint32_t>(i), 0x67617468u, static_cast<uint32_t>(seed >> 32), 0u);
  const uint64_t j = static_cast<uint64_t>(r.Next() * static_cast<float>(valid)) % (valid ? valid : 1);
  const GuideSample s = pool[j];
  float *f = features + static_cast<int64_t>(i) * kFeatures;
  f[0] = s.f0.x, f[1] = s.f0.y, f[2] = s.f0.z, f[3] = s.f0.w;
  f[4] = s.f1.x, f[5] = s.f1.y, f[6] = s.f1.z, f[7] = s.f1.w;
  dirs[3 * i] = s.dir_w.x, dirs[3 * i + 1] = s.dir_w.y, dirs[3 * i + 2] = s.dir_w.z;
  weights[i] = s.dir_w.w;
}

// Divides the weights by their mean (one block; fixed summation order).
// Training weights divided by their batch mean, in two deterministic passes:
// per-block sums in a fixed order, then every block forms the total from them.
constexpr int kSumBlocks = 256;

__global__ void __launch_bounds__(256) WeightSumKernel(const float *weights, int batch, double *part) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = blockIdx.x * 256 + threadIdx.x; i < batch; i += kSumBlocks * 256) s += weights[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(256) WeightScaleKernel(float *weights, int batch, const double *part) {
  __shared__ float inv;
  if (threadIdx.x == 0) {
    double total = 0.0;
    for (int b = 0; b < kSumBlocks; ++b) total += part[b];
    const double mean = total / static_cast<double>(batch);
    inv = mean > 0.0 ? static_cast<float>(1.0 / mean) : 0.0f;
  }
  __syncthreads();
  for (int i = blockIdx.x * 256 + threadIdx.x; i < batch; i += gridDim.x * 256) weights[i] *= inv;
}

inline unsigned Grid(int64_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

}  // namespace

void LaunchGuidePack(const float *params, void *img, cudaStream_t st) {
  PackKernel<<<Grid(std::max(kImgChunks, kBiasFloats), 256), 256, 0, st>>>(params, static_cast<unsigned char *>(img));
}

void LaunchGuideInit(float *params, uint64_t seed, cudaStream_t st) {
  InitKernel<<<Grid(kParams, 256), 256, 0, st>>>(params, seed);
}

void LaunchGuideForward(const void *img, const float *features, int n, float *out, int32_t *status,
                        cudaStream_t st) {
  if (n <= 0) return;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const unsigned grid = static_cast<unsigned>(std::max<int64_t>(
      1, std::min<int64_t>((static_cast<int64_t>(n) + kTcThreads - 1) / kTcThreads, std::max(sms, 1))));
  cudaFuncSetAttribute(ForwardKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmemBytes);
  ForwardKernel<<<grid, kTcThreads, kTcSmemBytes, st>>>(img, features, n, out, status);
}

void LaunchGuideSample(const float *raw, int n, const float *u, float *mix, float *dirs, float *pdf,
                       cudaStream_t st) {
  if (n <= 0) return;
  MixKernel<<<Grid(n, 256), 256, 0, st>>>(raw, n, mix);
  SampleKernel<<<Grid(n, 256), 256, 0, st>>>(mix, n, u, dirs, pdf);
}

size_t GuideTrainBytes(int batch) {
  const size_t chunks = (batch + kChunk - 1) / kChunk;
  return sizeof(float) * (4ull * batch * kWidth + static_cast<size_t>(batch) * kOut + 2ull * batch * kWidth +
                          chunks * kParams + kParams) +
         sizeof(double) * (batch / kThreads + 2 + kSumBlocks) + 256 * 9;
}

void GuideTrainCarve(void *base, int batch, GuideTrainBuffers *out) {
  char *p = static_cast<char *>(base);
  auto take = [&](size_t bytes) {
    char *r = p;
    p += (bytes + 255) / 256 * 256;
    return r;
  };
  out->h[0] = nullptr;
  for (int l = 1; l < 5; ++l) out->h[l] = reinterpret_cast<float *>(take(sizeof(float) * batch * kWidth));
  out->z = reinterpret_cast<float *>(take(sizeof(float) * batch * kOut));
  out->dz[0] = reinterpret_cast<float *>(take(sizeof(float) * batch * kWidth));
  out->dz[1] = reinterpret_cast<float *>(take(sizeof(float) * batch * kWidth));
  out->chunks = (batch + kChunk - 1) / kChunk;
  out->partial = reinterpret_cast<float *>(take(sizeof(float) * out->chunks * kParams));
  out->grad = reinterpret_cast<float *>(take(sizeof(float) * kParams));
  out->loss = reinterpret_cast<double *>(take(sizeof(double) * (batch / kThreads + 2)));
  out->wsum = reinterpret_cast<double *>(take(sizeof(double) * kSumBlocks));
}

void LaunchGuideGradients(const float *params, const float *features, const float *dirs, const float *weights,
                          int batch, const GuideTrainBuffers &tb, cudaStream_t st) {
  const unsigned tiles = Grid(batch, 64);
  auto W = [&](int l) { return params + MasterOffset(l); };
  auto B = [&](int l) { return params + MasterOffset(l) + In(l) * Out(l); };
  FwdLayerKernel<true, true><<<tiles, kThreads, 0, st>>>(features, W(0), B(0), kIn, kWidth, tb.h[1], batch);
  for (int l = 1; l < 4; ++l)
    FwdLayerKernel<false, true><<<tiles, kThreads, 0, st>>>(tb.h[l], W(l), B(l), kWidth, kWidth, tb.h[l + 1], batch);
  FwdLayerKernel<false, false><<<tiles, kThreads, 0, st>>>(tb.h[4], W(4), B(4), kWidth, kOut, tb.z, batch);
  LossKernel<<<Grid(batch, kThreads), kThreads, 0, st>>>(tb.z, dirs, weights, batch, tb.loss);
  const unsigned chunks = static_cast<unsigned>(tb.chunks);
  // layer 4: 64 x 64
  WgradKernel<false, kWidth, kOut, 4, 4><<<chunks, kThreads, 0, st>>>(tb.h[4], tb.z, batch, tb.partial, kParams,
                                                                       MasterOffset(4));
  BwdDataKernel<<<tiles, kThreads, 0, st>>>(tb.z, W(4), tb.h[4], kOut, tb.dz[0], batch);
  // layers 3..1: 64 x 64
  int cur = 0;
  for (int l = 3; l >= 1; --l) {
    WgradKernel<false, kWidth, kWidth, 4, 4><<<chunks, kThreads, 0, st>>>(tb.h[l], tb.dz[cur], batch, tb.partial,
                                                                         kParams, MasterOffset(l));
    BwdDataKernel<<<tiles, kThreads, 0, st>>>(tb.dz[cur], W(l), tb.h[l], kWidth, tb.dz[cur ^ 1], batch);
    cur ^= 1;
  }
  // layer 0: one-blob input, 256 x 64
  WgradKernel<true, kIn, kWidth, 8, 8><<<chunks, kThreads, 0, st>>>(features, tb.dz[cur], batch, tb.partial,
                                                                    kParams, MasterOffset(0));
  ReduceKernel<<<Grid(kParams, 256), 256, 0, st>>>(tb.partial, tb.chunks, tb.grad);
}

void LaunchGuideGather(const GuideSample *pool, uint64_t available, uint32_t cap, int batch, uint64_t seed,
                       float *features, float *dirs, float *weights, double *sums, cudaStream_t st) {
  GatherKernel<<<Grid(batch, 256), 256, 0, st>>>(pool, available, cap, batch, seed, features, dirs, weights);
  WeightSumKernel<<<kSumBlocks, 256, 0, st>>>(weights, batch, sums);
  WeightScaleKernel<<<std::max(1u, std::min(Grid(batch, 256), 1024u)), 256, 0, st>>>(weights, batch, sums);
}

void LaunchGuideAdam(float *params, float *m, float *v, const float *grad, float lr, int step, cudaStream_t st) {
  const float c1 = 1.0f - powf(0.9f, static_cast<float>(step));
  const float c2 = 1.0f - powf(0.999f, static_cast<float>(step));
  AdamKernel<<<Grid(kParams, 256), 256, 0, st>>>(params, m, v, grad, lr, c1, c2);
}

}  // namespace muon_gpu
