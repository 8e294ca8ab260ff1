// Learned path guiding: structures shared by the host code and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels.cuh"

namespace muon_gpu {

// What a guided render leaves behind for one path vertex whose path
// continued: its features, the sampled direction, the throughput before the
// vertex and the radiance the path had collected once the vertex's direct
// light was added. Together with the path's final radiance this gives the
// training target of the direction (see GuideCollect).
struct GuideRec {
  float4 f0, f1;   // features 0-3, 4-7
  float4 dir;      // xyz, w = path id word
  float4 tp;       // throughput before the vertex; w = 1 when recorded
  float4 after;    // radiance after the vertex's direct light
};

// One training sample: features, direction and weight (target / density).
struct GuideSample {
  float4 f0, f1;
  float4 dir_w;
};

// Device view of a guide for the render kernels.
struct GuideDev {
  const void *wt;        // the inference image (guide_mlp.cuh): BF16 operands, then FP32 biases
  int32_t *status;       // set to 1 by an inference kernel whose tensor-core wait gave up
  float4 *mix;           // guide::kMixVec per queue entry: the processed mixture
  float4 *feat;          // 2 per queue entry: the features
  GuideRec *rec;         // rec_bounces x rec_cap
  int32_t rec_cap;       // entries per bounce (the wave's capacity)
  int32_t rec_bounces;   // bounces recorded for training
  float alpha;           // probability of sampling the mixture instead of the BRDF
  float lo[3], inv_ext[3];  // scene box: feature = (p - lo) * inv_ext
  GuideSample *pool;     // training samples (ring buffer)
  unsigned long long *pool_count;  // samples ever appended
  uint32_t pool_cap;
  // shadow slots that become training samples when unblocked: the area-light
  // samples [0, area_slots) and the MIS ray (mis_slot, -1 if none); set per
  // render
  int32_t area_slots;
  int32_t mis_slot;
  int32_t direct_only;   // MUON_GUIDE_DIRECT: only the light-hit (MIS) ray is guided and
                         // only light samples train; continuations sample the BRDF
  // ordered appends of light-sample training samples (per queue entry: its
  // count and the exclusive scan of the counts; scan scratch)
  uint32_t *sample_count;
  uint32_t *sample_off;
  void *scan_tmp;
  size_t scan_bytes;
};

// A path-traced render with guiding (render.cc): the single-scene wavefront
// loop with the guide's inference before shading, guided sampling, and
// training records collected after each wave. Throws CudaError.
void RenderGuided(MuonScene *sc, const MuonRenderParams &p, double *d_sum, double *d_sq, uint32_t *d_cnt,
                  const GuideDev &g);

// Kernels of the guided render (kernels.cu).
void LaunchGuideInfer(const DevScene &s, const PathBuffers &b, WaveCounters wc, int bounce, int bound, int isect,
                      const GuideDev &g, cudaStream_t st);
void LaunchShadePathGuided(const DevScene &s, const WaveInfo &w, const ShadeParams &sp, const PathBuffers &b,
                           WaveCounters wc, int bounce, int bound, const GuideDev &g, cudaStream_t st);
// The guided fold; on bounces that collect training samples it also appends
// them to the pool in entry order (a scan of per-entry counts). Throws
// CudaError.
void LaunchFoldGuided(const PathBuffers &b, WaveCounters wc, int bounce, int slots, int bound, const GuideDev &g,
                      cudaStream_t st);
// Scratch bytes of the scan over `capacity` entries.
size_t GuideScanBytes(int capacity);
void LaunchGuideCollect(const PathBuffers &b, WaveCounters wc, int bounces, int bound, const GuideDev &g,
                        cudaStream_t st);

// Training and network kernels (guide.cu). `params` is the FP32 master copy
// (guide::MasterOffset layout).
// Writes the inference image (guide_mlp.cuh) of the master copy.
void LaunchGuidePack(const float *params, void *img, cudaStream_t st);
void LaunchGuideInit(float *params, uint64_t seed, cudaStream_t st);
// Network outputs (n x 64) for features (n x 8) on the tensor-core path;
// `status` as in GuideDev.
void LaunchGuideForward(const void *img, const float *features, int n, float *out, int32_t *status,
                        cudaStream_t st);

// Directions drawn from the mixtures of network outputs raw (n x 64) with
// uniforms u (n x 3), and the mixture density of each (guide_mlp.cuh,
// SampleMixture / MixturePdf); mix is scratch of n x kMixFloats.
void LaunchGuideSample(const float *raw, int n, const float *u, float *mix, float *dirs, float *pdf,
                       cudaStream_t st);

// Working memory of one training step over `batch` samples.
struct GuideTrainBuffers {
  float *h[5];      // inputs of layers 1..4 (h[0] unused: the one-blob input is recomputed), batch x 64
  float *z;         // batch x 64 outputs, then their gradients
  float *dz[2];     // batch x 64 gradients (ping-pong)
  float *partial;   // per chunk: all weight and bias gradients
  float *grad;      // guide::kParams
  double *loss;     // loss sum of every 256 consecutive samples
  double *wsum;     // partial sums of the training weights (LaunchGuideGather)
  int32_t chunks;
};
size_t GuideTrainBytes(int batch);
void GuideTrainCarve(void *base, int batch, GuideTrainBuffers *out);
// Gradients of the mean loss over the batch into tb.grad and the loss sums
// into tb.loss.
void LaunchGuideGradients(const float *params, const float *features, const float *dirs, const float *weights,
                          int batch, const GuideTrainBuffers &tb, cudaStream_t st);
// Gathers `batch` samples from the pool at random positions (seeded) into
// features / dirs / weights (weights normalised by their batch mean; `sums`
// is scratch of GuideTrainBuffers::wsum).
void LaunchGuideGather(const GuideSample *pool, uint64_t available, uint32_t cap, int batch, uint64_t seed,
                       float *features, float *dirs, float *weights, double *sums, cudaStream_t st);
void LaunchGuideAdam(float *params, float *m, float *v, const float *grad, float lr, int step, cudaStream_t st);

}  // namespace muon_gpu
