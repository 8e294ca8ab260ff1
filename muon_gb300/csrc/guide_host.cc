// Learned path guiding: the MuonGuide handle and its C ABI (include/muon_gpu.h,
// "learned path guiding").
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <memory>
#include <new>
#include <vector>

#include "guide.h"
#include "guide_mlp.cuh"
#include "host_cuda.h"
#include "scene_access.h"

using namespace muon_gpu;

static_assert(guide::kParams == MUON_GUIDE_PARAMS, "parameter count of the public header");

struct MuonGuide {
  MuonScene *scene = nullptr;
  SceneView view{};
  MuonGuideConfig cfg{};
  DeviceBuffer params, adam_m, adam_v, wt, status, mix, feat, rec, pool, pool_count, train, batch_feat, batch_dir,
      batch_w, io_in, io_dir, io_w, io_out, io_mix, io_u, io_pdf, sample_count, sample_off, scan_tmp;
  GuideDev dev{};
  int step = 0;
  uint64_t batches = 0;
};

namespace {

void Defaults(MuonGuideConfig *c) {
  if (c->batch <= 0) c->batch = 1 << 18;
  if (c->wave_paths <= 0) c->wave_paths = kMaxWavePaths;
  c->wave_paths = std::min(c->wave_paths, kMaxWavePaths);
  if (c->record_bounces <= 0) c->record_bounces = 4;
  if (c->pool_capacity <= 0) c->pool_capacity = 1 << 22;
  if (!(c->learning_rate > 0.0f)) c->learning_rate = 1e-3f;
  if (!(c->mixture_fraction > 0.0f) || c->mixture_fraction > 1.0f)
    c->mixture_fraction = c->targets == MUON_GUIDE_DIRECT ? 0.95f : 0.5f;
}

// Scene box from the BVH root's two child boxes.
void SceneBox(const SceneImage &im, float lo[3], float hi[3]) {
  for (int k = 0; k < 3; ++k) lo[k] = 0.0f, hi[k] = 1.0f;
  if (im.nodes.empty()) return;
  const BvhNode &r = im.nodes[0];
  const float c0[6] = {r.a.x, r.a.y, r.a.z, r.a.w, r.c.x, r.c.y};  // lo.x hi.x lo.y hi.y lo.z hi.z
  const float c1[6] = {r.b.x, r.b.y, r.b.z, r.b.w, r.c.z, r.c.w};
  for (int k = 0; k < 3; ++k) {
    float l = std::min(c0[2 * k], c1[2 * k]), h = std::max(c0[2 * k + 1], c1[2 * k + 1]);
    if (!(l <= h)) l = 0.0f, h = 1.0f;
    lo[k] = l, hi[k] = h;
  }
}

// The status word of the tensor-core inference kernels (see GuideDev::status).
int CheckInferenceStatus(const MuonGuide *g) {
  int32_t v = 0;
  CUDA_TRY(cudaMemcpyAsync(&v, g->status.ptr, sizeof(v), cudaMemcpyDeviceToHost, g->view.stream));
  CUDA_TRY(cudaStreamSynchronize(g->view.stream));
  if (v != 0) return Fail(MUON_ERR_TIMEOUT, "guide inference: a tensor-core wait timed out");
  return MUON_OK;
}

}  // namespace

extern "C" {

int muon_gpu_guide_create(MuonScene *scene, const MuonGuideConfig *config, MuonGuide **out) {
  if (!scene || !out) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  std::unique_ptr<MuonGuide> g;
  try {
    g.reset(new MuonGuide());
    g->scene = scene;
    if (!GetSceneView(scene, &g->view)) return Fail(MUON_ERR_INVALID_ARG, "null scene");
    if (config) g->cfg = *config;
    if (g->cfg.targets != MUON_GUIDE_DIRECT && g->cfg.targets != MUON_GUIDE_ALL)
      return Fail(MUON_ERR_INVALID_ARG, "unknown guide targets");
    Defaults(&g->cfg);
    const MuonGuideConfig &c = g->cfg;
    CUDA_TRY(cudaSetDevice(g->view.device));
    cudaStream_t st = g->view.stream;
    g->params.Ensure(sizeof(float) * guide::kParams);
    g->adam_m.Ensure(sizeof(float) * guide::kParams);
    g->adam_v.Ensure(sizeof(float) * guide::kParams);
    g->wt.Ensure(guide::kImgBytes);
    g->status.Ensure(sizeof(int32_t));
    const size_t cap = static_cast<size_t>(c.wave_paths);
    g->mix.Ensure(cap * guide::kMixVec * sizeof(float4));
    g->feat.Ensure(cap * 2 * sizeof(float4));
    const bool records = c.targets == MUON_GUIDE_ALL;  // continuation records (guided continuations only)
    if (records) g->rec.Ensure(cap * c.record_bounces * sizeof(GuideRec));
    g->pool.Ensure(static_cast<size_t>(c.pool_capacity) * sizeof(GuideSample));
    g->pool_count.Ensure(sizeof(unsigned long long));
    g->sample_count.Ensure(cap * sizeof(uint32_t));
    g->sample_off.Ensure(cap * sizeof(uint32_t));
    const size_t scan_bytes = GuideScanBytes(c.wave_paths);
    g->scan_tmp.Ensure(std::max<size_t>(scan_bytes, 16));
    g->train.Ensure(GuideTrainBytes(c.batch));
    g->batch_feat.Ensure(sizeof(float) * c.batch * guide::kFeatures);
    g->batch_dir.Ensure(sizeof(float) * c.batch * 3);
    g->batch_w.Ensure(sizeof(float) * c.batch);
    CUDA_TRY(cudaMemsetAsync(g->adam_m.ptr, 0, sizeof(float) * guide::kParams, st));
    CUDA_TRY(cudaMemsetAsync(g->adam_v.ptr, 0, sizeof(float) * guide::kParams, st));
    CUDA_TRY(cudaMemsetAsync(g->pool_count.ptr, 0, sizeof(unsigned long long), st));
    CUDA_TRY(cudaMemsetAsync(g->status.ptr, 0, sizeof(int32_t), st));
    if (records) CUDA_TRY(cudaMemsetAsync(g->rec.ptr, 0, cap * c.record_bounces * sizeof(GuideRec), st));
    LaunchGuideInit(g->params.as<float>(), c.seed, st);
    LaunchGuidePack(g->params.as<float>(), g->wt.ptr, st);
    CUDA_TRY(cudaGetLastError());
    GuideDev &d = g->dev;
    d.wt = g->wt.ptr;
    d.status = g->status.as<int32_t>();
    d.mix = g->mix.as<float4>();
    d.feat = g->feat.as<float4>();
    d.rec = records ? g->rec.as<GuideRec>() : nullptr;
    d.rec_cap = c.wave_paths;
    d.rec_bounces = c.record_bounces;
    d.alpha = c.mixture_fraction;
    d.direct_only = c.targets == MUON_GUIDE_DIRECT ? 1 : 0;
    float lo[3], hi[3];
    SceneBox(*g->view.img, lo, hi);
    for (int k = 0; k < 3; ++k) {
      d.lo[k] = lo[k];
      d.inv_ext[k] = hi[k] > lo[k] ? 1.0f / (hi[k] - lo[k]) : 1.0f;
    }
    d.pool = g->pool.as<GuideSample>();
    d.pool_count = g->pool_count.as<unsigned long long>();
    d.pool_cap = static_cast<uint32_t>(c.pool_capacity);
    d.sample_count = g->sample_count.as<uint32_t>();
    d.sample_off = g->sample_off.as<uint32_t>();
    d.scan_tmp = g->scan_tmp.ptr;
    d.scan_bytes = scan_bytes;
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  *out = g.release();
  return MUON_OK;
}

void muon_gpu_guide_destroy(MuonGuide *guide) { delete guide; }

int muon_gpu_guide_render_device(MuonGuide *guide, const MuonRenderParams *params, double *d_sum, double *d_sum_sq,
                                 uint32_t *d_count) {
  if (!guide || !params || !d_sum || !d_sum_sq || !d_count) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  if (params->integrator != MUON_INTEGRATOR_PATHTRACER)
    return Fail(MUON_ERR_INVALID_ARG, "guiding needs the path tracer");
  int rc = ValidateParams(*params);
  if (rc != MUON_OK) return rc;
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    MuonRenderParams p = *params;
    p.wave_paths = guide->cfg.wave_paths;
    if (!(p.flags & MUON_RENDER_ACCUMULATE)) {
      const size_t np = static_cast<size_t>(guide->view.width) * guide->view.height;
      cudaStream_t st = guide->view.stream;
      CUDA_TRY(cudaMemsetAsync(d_sum, 0, 3 * np * sizeof(double), st));
      CUDA_TRY(cudaMemsetAsync(d_sum_sq, 0, 3 * np * sizeof(double), st));
      CUDA_TRY(cudaMemsetAsync(d_count, 0, np * sizeof(uint32_t), st));
    }
    RenderGuided(guide->scene, p, d_sum, d_sum_sq, d_count, guide->dev);
    return CheckInferenceStatus(guide);
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}

int muon_gpu_guide_train(MuonGuide *guide, int32_t steps, double *loss) {
  if (!guide || steps < 0) return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    cudaStream_t st = guide->view.stream;
    unsigned long long avail = 0;
    CUDA_TRY(cudaMemcpyAsync(&avail, guide->pool_count.ptr, sizeof(avail), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (avail == 0) return Fail(MUON_ERR_INVALID_ARG, "no training samples collected yet");
    const int batch = guide->cfg.batch;
    GuideTrainBuffers tb;
    GuideTrainCarve(guide->train.ptr, batch, &tb);
    for (int s = 0; s < steps; ++s) {
      LaunchGuideGather(guide->pool.as<GuideSample>(), avail, guide->dev.pool_cap, batch,
                        guide->cfg.seed * 0x9E3779B97F4A7C15ull + (++guide->batches), guide->batch_feat.as<float>(),
                        guide->batch_dir.as<float>(), guide->batch_w.as<float>(), tb.wsum, st);
      LaunchGuideGradients(guide->params.as<float>(), guide->batch_feat.as<float>(), guide->batch_dir.as<float>(),
                           guide->batch_w.as<float>(), batch, tb, st);
      LaunchGuideAdam(guide->params.as<float>(), guide->adam_m.as<float>(), guide->adam_v.as<float>(), tb.grad,
                      guide->cfg.learning_rate, ++guide->step, st);
    }
    LaunchGuidePack(guide->params.as<float>(), guide->wt.ptr, st);
    CUDA_TRY(cudaGetLastError());
    if (loss) {
      std::vector<double> parts(batch / 256 + 1, 0.0);
      const size_t nparts = (batch + 255) / 256;
      CUDA_TRY(cudaMemcpyAsync(parts.data(), tb.loss, nparts * sizeof(double), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
      double sum = 0.0;
      for (size_t i = 0; i < nparts; ++i) sum += parts[i];
      *loss = steps > 0 ? sum / batch : 0.0;
    }
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_guide_forward(MuonGuide *guide, const float *features, int64_t n, float *out) {
  if (!guide || n < 0 || (n > 0 && (!features || !out)) || n > (int64_t(1) << 30))
    return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return MUON_OK;
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    cudaStream_t st = guide->view.stream;
    guide->io_in.Ensure(sizeof(float) * n * guide::kFeatures);
    guide->io_out.Ensure(sizeof(float) * n * guide::kOut);
    CUDA_TRY(cudaMemcpyAsync(guide->io_in.ptr, features, sizeof(float) * n * guide::kFeatures,
                             cudaMemcpyHostToDevice, st));
    LaunchGuideForward(guide->wt.ptr, guide->io_in.as<float>(), static_cast<int>(n), guide->io_out.as<float>(),
                       guide->status.as<int32_t>(), st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(out, guide->io_out.ptr, sizeof(float) * n * guide::kOut, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return CheckInferenceStatus(guide);
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_guide_sample(MuonGuide *guide, const float *features, const float *u, int64_t n, float *dirs,
                          float *pdf) {
  if (!guide || n < 0 || (n > 0 && (!features || !u || !dirs || !pdf)) || n > (int64_t(1) << 26))
    return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  if (n == 0) return MUON_OK;
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    cudaStream_t st = guide->view.stream;
    guide->io_in.Ensure(sizeof(float) * n * guide::kFeatures);
    guide->io_out.Ensure(sizeof(float) * n * guide::kOut);
    guide->io_mix.Ensure(sizeof(float) * n * guide::kMixFloats);
    guide->io_u.Ensure(sizeof(float) * n * 3);
    guide->io_dir.Ensure(sizeof(float) * n * 3);
    guide->io_pdf.Ensure(sizeof(float) * n);
    CUDA_TRY(cudaMemcpyAsync(guide->io_in.ptr, features, sizeof(float) * n * guide::kFeatures,
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(guide->io_u.ptr, u, sizeof(float) * n * 3, cudaMemcpyHostToDevice, st));
    LaunchGuideForward(guide->wt.ptr, guide->io_in.as<float>(), static_cast<int>(n), guide->io_out.as<float>(),
                       guide->status.as<int32_t>(), st);
    LaunchGuideSample(guide->io_out.as<float>(), static_cast<int>(n), guide->io_u.as<float>(),
                      guide->io_mix.as<float>(), guide->io_dir.as<float>(), guide->io_pdf.as<float>(), st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(dirs, guide->io_dir.ptr, sizeof(float) * n * 3, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(pdf, guide->io_pdf.ptr, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return CheckInferenceStatus(guide);
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
}

int muon_gpu_guide_gradients(MuonGuide *guide, const float *features, const float *dirs, const float *weights,
                             int32_t n, float *grad, double *loss) {
  if (!guide || n <= 0 || !features || !dirs || !weights || !grad) return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    cudaStream_t st = guide->view.stream;
    DeviceBuffer work;
    work.Ensure(GuideTrainBytes(n));
    GuideTrainBuffers tb;
    GuideTrainCarve(work.ptr, n, &tb);
    guide->io_in.Ensure(sizeof(float) * n * guide::kFeatures);
    guide->io_dir.Ensure(sizeof(float) * n * 3);
    guide->io_w.Ensure(sizeof(float) * n);
    CUDA_TRY(cudaMemcpyAsync(guide->io_in.ptr, features, sizeof(float) * n * guide::kFeatures,
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(guide->io_dir.ptr, dirs, sizeof(float) * n * 3, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(guide->io_w.ptr, weights, sizeof(float) * n, cudaMemcpyHostToDevice, st));
    LaunchGuideGradients(guide->params.as<float>(), guide->io_in.as<float>(), guide->io_dir.as<float>(),
                         guide->io_w.as<float>(), n, tb, st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(grad, tb.grad, sizeof(float) * guide::kParams, cudaMemcpyDeviceToHost, st));
    const size_t nparts = (n + 255) / 256;
    std::vector<double> parts(nparts);
    CUDA_TRY(cudaMemcpyAsync(parts.data(), tb.loss, nparts * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (loss) {
      double sum = 0.0;
      for (double v : parts) sum += v;
      *loss = sum / n;
    }
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_guide_get_params(const MuonGuide *guide, float *params) {
  if (!guide || !params) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    CUDA_TRY(cudaMemcpyAsync(params, guide->params.ptr, sizeof(float) * guide::kParams, cudaMemcpyDeviceToHost,
                             guide->view.stream));
    CUDA_TRY(cudaStreamSynchronize(guide->view.stream));
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_guide_set_params(MuonGuide *guide, const float *params) {
  if (!guide || !params) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    cudaStream_t st = guide->view.stream;
    CUDA_TRY(cudaMemcpyAsync(guide->params.ptr, params, sizeof(float) * guide::kParams, cudaMemcpyHostToDevice, st));
    LaunchGuidePack(guide->params.as<float>(), guide->wt.ptr, st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_guide_set_status(MuonGuide *guide, int32_t status) {
  if (!guide) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  try {
    CUDA_TRY(cudaSetDevice(guide->view.device));
    CUDA_TRY(cudaMemcpyAsync(guide->status.ptr, &status, sizeof(status), cudaMemcpyHostToDevice, guide->view.stream));
    CUDA_TRY(cudaStreamSynchronize(guide->view.stream));
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_guide_samples(const MuonGuide *guide, uint64_t *count) {
  if (!guide || !count) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  try {
    unsigned long long v = 0;
    CUDA_TRY(cudaMemcpyAsync(&v, guide->pool_count.ptr, sizeof(v), cudaMemcpyDeviceToHost, guide->view.stream));
    CUDA_TRY(cudaStreamSynchronize(guide->view.stream));
    *count = v;
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

}  // extern "C"
