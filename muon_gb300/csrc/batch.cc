// Batched rendering: many scenes in one wavefront (include/muon_gpu.h,
// "batched rendering").
//
// The scenes' device arrays are copied into one merged image: BVH node links,
// leaf starts and transform / material / light indices are shifted by each
// scene's offsets, so every scene keeps its own BVH under its own root node.
// A path record carries its BVH root (ray_d.w, and the shadow origin's w) and
// its batch segment (high bits of its id word); the traversal kernels are the
// single-scene ones unchanged, and only the camera, shading and film kernels
// look up per-scene settings. The wavefront loop is the single-scene one
// (render.cc) over waves that hold segments of several scenes, replayed as one
// CUDA graph. An autotuner picks the wavefront size and the traversal grid.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "host_cuda.h"
#include "host_scene.h"
#include "kernels.cuh"
#include "scene_access.h"
#include "scene_records.h"
#include "scene_build.h"

using namespace muon_gpu;

namespace {

constexpr int kBatchDefaultWavePaths = 1 << 22;

struct WavePlan {
  int seg_begin = 0, nseg = 0;  // into the batch's segment table
  int paths = 0, pixels = 0;
  int bounces = 0;
};

}  // namespace

struct MuonBatch {
  int device = 0;
  int sms = 0;
  cudaStream_t stream = nullptr;
  int n = 0;
  std::vector<int> schedule;  // scene indices, shortest first
  // merged scene
  DeviceBuffer nodes, prims, prims_obj, shade, smooth, smooth_obj, transforms, materials, lights, light_tris,
      light_tris_obj, light_tri_ok, other_lights;
  DevScene dev{};
  std::vector<DevCamera> cams;
  std::vector<int32_t> root, light_off, num_lights, other_off, num_other, width, height;
  std::vector<uint64_t> scene_prims;
  uint64_t total_nodes = 0, total_prims = 0;
  // work
  DeviceBuffer ray_o[2], ray_d[2], tp[2], rad[2], hits, link, final_rad, org, contrib, slot_dir, shq, order, counters,
      stats, scene_table, seg_table;
  std::vector<DeviceBuffer> film_sum, film_sq, film_cnt;
  int64_t wave_cap = 0;
  int slots_cap = -1;
  // graph of the last render
  cudaGraphExec_t graph = nullptr;
  std::string graph_key;
  uint64_t graph_launches = 0;
  std::vector<cudaEvent_t> wave_done;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  // launch configuration
  int wave_paths = 0;       // 0: default
  int blocks_per_sm = 0;    // 0: default traversal grid
  // last render
  MuonStats last{};
  std::vector<MuonBatchSceneStats> per_scene;

  ~MuonBatch() {
    if (graph) cudaGraphExecDestroy(graph);
    for (cudaEvent_t e : wave_done) cudaEventDestroy(e);
    if (t0) cudaEventDestroy(t0);
    if (t1) cudaEventDestroy(t1);
    if (stream) cudaStreamDestroy(stream);
  }

  void DropGraph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_key.clear();
  }

  PathBuffers Buffers() const {
    PathBuffers b;
    for (int k = 0; k < 2; ++k) {
      b.ray_o[k] = ray_o[k].as<float4>();
      b.ray_d[k] = ray_d[k].as<float4>();
      b.tp[k] = tp[k].as<float4>();
      b.rad[k] = rad[k].as<float4>();
    }
    b.hits = hits.as<int2>();
    b.link = link.as<int32_t>();
    b.final_rad = final_rad.as<float4>();
    b.org = org.as<float4>();
    b.contrib = contrib.as<float4>();
    b.slot_dir = slot_dir.as<float4>();
    b.shq = shq.as<uint32_t>();
    b.order = order.as<int32_t>();
    b.order_cap = static_cast<int32_t>(wave_cap);
    b.stats = stats.as<unsigned long long>();
    return b;
  }

  bool EnsureWork(int64_t paths, int slots) {
    if (paths <= wave_cap && slots <= slots_cap) return false;
    int64_t p = std::max(paths, wave_cap);
    int s = std::max(slots, slots_cap);
    for (int k = 0; k < 2; ++k) {
      ray_o[k].Ensure(p * sizeof(float4));
      ray_d[k].Ensure(p * sizeof(float4));
      tp[k].Ensure(p * sizeof(float4));
      rad[k].Ensure(p * sizeof(float4));
    }
    hits.Ensure(p * sizeof(int2));
    link.Ensure(p * sizeof(int32_t));
    final_rad.Ensure(p * sizeof(float4));
    org.Ensure(p * sizeof(float4));
    size_t sl = static_cast<size_t>(p) * std::max(s, 1);
    contrib.Ensure(sl * sizeof(float4));
    slot_dir.Ensure(sl * sizeof(float4));
    shq.Ensure(sl * sizeof(uint32_t));
    order.Ensure(static_cast<size_t>(OrderInts(p)) * sizeof(int32_t));
    wave_cap = p;
    slots_cap = s;
    return true;
  }
};

namespace {

// Builds the merged scene of `views` (creation order) into `b`: the scenes'
// device arrays are appended on the device (nodes with shifted links,
// records with shifted transform / material / light indices); the small
// tables (transforms, materials, lights) are merged on the host.
void MergeScenes(MuonBatch *b, const std::vector<SceneView> &views) {
  std::vector<DevTransform> transforms;
  std::vector<DevMaterial> materials;
  std::vector<DevLight> lights, other;
  bool any_smooth = false;
  int64_t total_nodes = 0, total_prims = 0;
  for (const SceneView &v : views) {
    any_smooth |= v.img->any_smooth;
    total_nodes += std::max<int64_t>(v.dev->num_nodes, 1);
    total_prims += v.num_slots;
    CUDA_TRY(cudaStreamSynchronize(v.stream));  // the scene's arrays are complete
  }
  if (total_nodes > INT32_MAX || total_prims > INT32_MAX) throw CudaError{cudaErrorInvalidValue, "batch too large"};
  cudaStream_t st = b->stream;
  b->nodes.Ensure(sizeof(BvhNode) * total_nodes);
  b->prims.Ensure(sizeof(PrimRecord) * std::max<int64_t>(total_prims, 1));
  b->prims_obj.Ensure(sizeof(PrimRecord) * std::max<int64_t>(total_prims, 1));
  b->shade.Ensure(sizeof(ShadeRecord) * std::max<int64_t>(total_prims, 1));
  b->smooth.Ensure(any_smooth ? sizeof(F4) * 3 * total_prims : 16);
  b->smooth_obj.Ensure(any_smooth ? sizeof(F4) * 3 * total_prims : 16);
  // No primitives: a root whose first child link is empty ends every
  // traversal at once.
  BvhNode empty{};
  empty.d.x = empty.d.y = kEmptyLink;
  int32_t node_off = 0, prim_off = 0;
  for (const SceneView &v : views) {
    const SceneImage &im = *v.img;
    const int32_t xf_off = static_cast<int32_t>(transforms.size());
    const int32_t mat_off = static_cast<int32_t>(materials.size());
    const int32_t light_off = static_cast<int32_t>(lights.size());
    b->root.push_back(node_off);
    b->light_off.push_back(light_off);
    b->num_lights.push_back(static_cast<int32_t>(im.lights.size()));
    b->other_off.push_back(static_cast<int32_t>(other.size()));
    b->num_other.push_back(static_cast<int32_t>(im.other_lights.size()));
    b->width.push_back(im.width);
    b->height.push_back(im.height);
    b->scene_prims.push_back(static_cast<uint64_t>(im.num_prims));
    b->cams.push_back(*v.cam);
    const int64_t nn = v.dev->num_nodes;
    if (nn == 0)
      CUDA_TRY(cudaMemcpyAsync(b->nodes.as<BvhNode>() + node_off, &empty, sizeof(BvhNode), cudaMemcpyHostToDevice, st));
    const MergeOffsets off{node_off, prim_off, xf_off, mat_off, light_off};
    LaunchMergeScene(v.dev->nodes, nn, v.dev->prims, v.dev->prims_obj, v.dev->shade, v.dev->smooth_normals,
                     v.dev->smooth_normals_obj, v.num_slots, off, b->nodes.as<BvhNode>(), b->prims.as<PrimRecord>(),
                     b->prims_obj.as<PrimRecord>(), b->shade.as<ShadeRecord>(),
                     any_smooth ? b->smooth.as<F4>() : nullptr, any_smooth ? b->smooth_obj.as<F4>() : nullptr, st);
    CUDA_TRY(cudaGetLastError());
    node_off += static_cast<int32_t>(std::max<int64_t>(nn, 1));
    prim_off += static_cast<int32_t>(v.num_slots);
    transforms.insert(transforms.end(), im.transforms.begin(), im.transforms.end());
    materials.insert(materials.end(), im.materials.begin(), im.materials.end());
    lights.insert(lights.end(), im.lights.begin(), im.lights.end());
    other.insert(other.end(), im.other_lights.begin(), im.other_lights.end());
  }
  std::vector<PrimRecord> lt, lt_obj;
  std::vector<int32_t> lt_ok;
  BuildLightTris(lights, &lt, &lt_obj, &lt_ok);
  Upload(b->transforms, transforms, st);
  Upload(b->materials, materials, st);
  Upload(b->lights, lights, st);
  Upload(b->light_tris, lt, st);
  Upload(b->light_tris_obj, lt_obj, st);
  Upload(b->light_tri_ok, lt_ok, st);
  Upload(b->other_lights, other, st);
  DevScene &d = b->dev;
  d = DevScene{};
  d.nodes = b->nodes.as<BvhNode>();
  d.prims = b->prims.as<PrimRecord>();
  d.prims_obj = b->prims_obj.as<PrimRecord>();
  d.shade = b->shade.as<ShadeRecord>();
  d.smooth_normals = any_smooth ? b->smooth.as<F4>() : nullptr;
  d.smooth_normals_obj = any_smooth ? b->smooth_obj.as<F4>() : nullptr;
  d.transforms = b->transforms.as<DevTransform>();
  d.materials = b->materials.as<DevMaterial>();
  d.lights = b->lights.as<DevLight>();
  d.light_tris = b->light_tris.as<PrimRecord>();
  d.light_tris_obj = b->light_tris_obj.as<PrimRecord>();
  d.light_tri_ok = b->light_tri_ok.as<int32_t>();
  d.other_lights = b->other_lights.as<DevLight>();
  d.all_lights = nullptr;
  d.num_nodes = static_cast<int32_t>(total_nodes);
  d.num_lights = static_cast<int32_t>(lights.size());
  d.num_other_lights = static_cast<int32_t>(other.size());
  d.num_all_lights = 0;
  b->total_nodes = static_cast<size_t>(total_nodes);
  b->total_prims = static_cast<size_t>(total_prims);
  CUDA_TRY(cudaStreamSynchronize(st));
}

int ValidateBatchParams(const MuonBatch *b, const MuonRenderParams *params) {
  for (int i = 0; i < b->n; ++i) {
    const MuonRenderParams &p = params[i];
    int rc = ValidateParams(p);
    if (rc != MUON_OK) return rc;
    if (p.integrator != MUON_INTEGRATOR_PATHTRACER)
      return Fail(MUON_ERR_INVALID_ARG, "batched rendering supports the path tracer only");
    if (p.max_depth < 0) return Fail(MUON_ERR_INVALID_ARG, "batched rendering needs max_depth >= 0");
    if (p.max_depth == 0 && p.next_event_estimation != MUON_NEE_OFF)
      return Fail(MUON_ERR_INVALID_ARG, "max_depth 0 with light sampling traces no ray; render it alone");
    if (p.intersect_mode != params[0].intersect_mode)
      return Fail(MUON_ERR_INVALID_ARG, "all scenes of a batch must use one intersect_mode");
  }
  return MUON_OK;
}

// Renders the batch into device films. Throws CudaError.
void RenderBatch(MuonBatch *b, const MuonRenderParams *params, double *const *d_sum, double *const *d_sq,
                 uint32_t *const *d_cnt) {
  cudaStream_t st = b->stream;
  const int n = b->n;
  std::vector<ShadeParams> sps(n);
  std::vector<int> bounces(n);
  int S = 0;
  for (int i = 0; i < n; ++i) {
    const int slots = SetupShade(params[i], b->num_lights[i], b->num_other[i], &sps[i]);
    S = std::max(S, slots);
    bounces[i] = sps[i].max_trace_depth + 1;
  }
  const bool stats_on = (params[0].flags & MUON_RENDER_STATS) != 0;
  const int isect = params[0].intersect_mode;

  // Wave plan: scenes in schedule order, cut into segments that fill waves.
  int64_t budget = b->wave_paths > 0 ? b->wave_paths : kBatchDefaultWavePaths;
  const int64_t per_path = 200 + 36 * static_cast<int64_t>(std::max(S, 1));
  budget = std::max<int64_t>(1, std::min<int64_t>({budget, (int64_t(8) << 30) / per_path, int64_t(kMaxWavePaths)}));
  std::vector<BatchSeg> segs;
  std::vector<WavePlan> waves;
  std::vector<int> last_wave(n, -1);
  WavePlan cur;
  auto close_wave = [&]() {
    if (cur.nseg > 0) waves.push_back(cur);
    cur = WavePlan{};
    cur.seg_begin = static_cast<int>(segs.size());
  };
  for (int k : b->schedule) {
    const int64_t npix = static_cast<int64_t>(b->width[k]) * b->height[k];
    const int spp = params[k].pixel_samples;
    const int ns_max = static_cast<int>(std::min<int64_t>(spp, budget));
    for (int s0 = 0; s0 < spp; s0 += ns_max) {
      const int ns = std::min(ns_max, spp - s0);
      int64_t p = 0;
      while (p < npix) {
        int64_t room = (budget - cur.paths) / ns;
        if (room <= 0 || cur.nseg >= kMaxSegments) {
          close_wave();
          continue;
        }
        const int64_t take = std::min(npix - p, room);
        BatchSeg sg{};
        sg.scene = k;
        sg.path0 = cur.paths;
        sg.pix0 = cur.pixels;
        sg.p0 = static_cast<int32_t>(p);
        sg.npix = static_cast<int32_t>(take);
        sg.s0 = s0;
        sg.ns = ns;
        sg.root = b->root[k];
        segs.push_back(sg);
        cur.nseg++;
        cur.paths += static_cast<int>(take * ns);
        cur.pixels += static_cast<int>(take);
        cur.bounces = std::max(cur.bounces, bounces[k]);
        p += take;
        last_wave[k] = static_cast<int>(waves.size());
      }
    }
  }
  close_wave();
  const size_t stride = WaveCounterWords(*std::max_element(bounces.begin(), bounces.end()));

  // Device tables.
  std::vector<BatchScene> scenes(n);
  for (int i = 0; i < n; ++i) {
    BatchScene &s = scenes[i];
    s.cam = b->cams[i];
    s.sp = sps[i];
    s.light_off = b->light_off[i];
    s.num_lights = b->num_lights[i];
    s.other_off = b->other_off[i];
    s.num_other = b->num_other[i];
    s.width = b->width[i];
    s.sample_offset = static_cast<uint32_t>(params[i].sample_offset);
    s.seed = params[i].seed;
    s.sum = d_sum[i];
    s.sum_sq = d_sq[i];
    s.count = d_cnt[i];
  }
  bool moved = b->EnsureWork(budget, S);
  const size_t table_bytes = scenes.size() * sizeof(BatchScene), seg_bytes = segs.size() * sizeof(BatchSeg);
  if (b->scene_table.bytes < table_bytes || b->seg_table.bytes < seg_bytes ||
      b->counters.bytes < stride * waves.size() * sizeof(uint32_t))
    moved = true;
  b->scene_table.Ensure(table_bytes);
  b->seg_table.Ensure(seg_bytes);
  b->counters.Ensure(stride * waves.size() * sizeof(uint32_t));
  b->stats.Ensure(sizeof(unsigned long long) * kNumStats);
  CUDA_TRY(cudaMemcpyAsync(b->scene_table.ptr, scenes.data(), table_bytes, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemcpyAsync(b->seg_table.ptr, segs.data(), seg_bytes, cudaMemcpyHostToDevice, st));
  while (b->wave_done.size() < waves.size()) {
    cudaEvent_t e;
    CUDA_TRY(cudaEventCreate(&e));
    b->wave_done.push_back(e);
  }
  if (!b->t0) CUDA_TRY(cudaEventCreate(&b->t0));
  if (!b->t1) CUDA_TRY(cudaEventCreate(&b->t1));

  PathBuffers pb = b->Buffers();
  const BatchScene *d_scenes = b->scene_table.as<BatchScene>();
  const BatchSeg *d_segs = b->seg_table.as<BatchSeg>();
  uint64_t launches = 0;
  auto enqueue = [&]() {
    CUDA_TRY(cudaMemsetAsync(b->counters.ptr, 0, stride * waves.size() * sizeof(uint32_t), st));
    CUDA_TRY(cudaMemsetAsync(b->stats.ptr, 0, sizeof(unsigned long long) * kNumStats, st));
    for (size_t wi = 0; wi < waves.size(); ++wi) {
      const WavePlan &w = waves[wi];
      WaveCounters wc{b->counters.as<uint32_t>() + wi * stride};
      const BatchSeg *wsegs = d_segs + w.seg_begin;
      LaunchCameraBatch(d_scenes, wsegs, w.nseg, w.paths, pb, wc, st);
      ++launches;
      for (int k = 0; k < w.bounces; ++k) {
        LaunchExtend(b->dev, pb, wc, k, w.paths, isect, stats_on, st);
        LaunchShadePathBatch(b->dev, d_scenes, wsegs, S, isect, pb, wc, k, w.paths, st);
        launches += 2;
        if (S > 0) {
          LaunchOcclude(b->dev, pb, wc, k, S, static_cast<int>(std::min<int64_t>(int64_t(w.paths) * S, INT32_MAX)),
                        isect, stats_on, st);
          ++launches;
        }
        LaunchFold(pb, wc, k, S, w.paths, st);
        ++launches;
      }
      LaunchFilmBatch(d_scenes, wsegs, w.nseg, w.pixels, pb, st);
      ++launches;
      CUDA_TRY(cudaEventRecordWithFlags(b->wave_done[wi], st, cudaEventRecordExternal));
    }
  };

  // Id words carry the segment index within the wave's slice of the table,
  // which the camera, shading and film kernels of that wave all receive.
  std::string key;
  {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "w%lld b%d S%d i%d st%d n%zu|", static_cast<long long>(budget), b->blocks_per_sm,
                  S, isect, stats_on ? 1 : 0, waves.size());
    key = buf;
    for (int i = 0; i < n; ++i) {
      std::snprintf(buf, sizeof(buf), "%d %d %d %d %d %d %d %d %d %d %llu %p %p %p|", params[i].pixel_samples,
                    params[i].light_samples, params[i].light_stratify, params[i].next_event_estimation,
                    params[i].russian_roulette, params[i].importance_sampling, params[i].min_depth,
                    params[i].max_depth, params[i].sample_offset, params[i].flags,
                    static_cast<unsigned long long>(params[i].seed), static_cast<void *>(d_sum[i]),
                    static_cast<void *>(d_sq[i]), static_cast<void *>(d_cnt[i]));
      key += buf;
    }
  }
  if (moved) b->DropGraph();
  if (b->graph_key != key || !b->graph) {
    b->DropGraph();
    SetTraversalBlocksOverride(b->blocks_per_sm > 0 ? b->blocks_per_sm * b->sms : 0);
    cudaGraph_t g = nullptr;
    launches = 0;
    CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue();
    } catch (...) {
      cudaGraph_t dummy = nullptr;
      cudaStreamEndCapture(st, &dummy);
      if (dummy) cudaGraphDestroy(dummy);
      SetTraversalBlocksOverride(0);
      throw;
    }
    SetTraversalBlocksOverride(0);
    CUDA_TRY(cudaStreamEndCapture(st, &g));
    cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) throw CudaError{e, "cudaGraphInstantiate"};
    b->graph_key = key;
    b->graph_launches = launches;
  }
  CUDA_TRY(cudaEventRecord(b->t0, st));
  CUDA_TRY(cudaGraphLaunch(b->graph, st));
  CUDA_TRY(cudaEventRecord(b->t1, st));
  CUDA_TRY(cudaGetLastError());
  unsigned long long hstats[kNumStats];
  std::vector<uint32_t> hc(stride * waves.size());
  CUDA_TRY(cudaMemcpyAsync(hstats, b->stats.ptr, sizeof(hstats), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(hc.data(), b->counters.ptr, hc.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));

  MuonStats &o = b->last;
  o = MuonStats{};
  uint64_t shadow = 0, ext_rays = 0, ext_launches = 0, occ_launches = 0;
  for (size_t wi = 0; wi < waves.size(); ++wi) {
    WaveCounters hw{hc.data() + wi * stride};
    for (int k = 0; k < waves[wi].bounces; ++k) {
      ext_rays += *hw.count(k);
      shadow += *hw.shadow(k);
      if (*hw.count(k) > 0) {
        ++ext_launches;
        if (S > 0) ++occ_launches;
      }
    }
  }
  b->per_scene.assign(n, MuonBatchSceneStats{});
  uint64_t primary = 0;
  for (int i = 0; i < n; ++i) {
    const uint64_t paths = static_cast<uint64_t>(b->width[i]) * b->height[i] * params[i].pixel_samples;
    b->per_scene[i].primary_rays = paths;
    primary += paths;
    float ms = 0.0f;
    if (last_wave[i] >= 0) CUDA_TRY(cudaEventElapsedTime(&ms, b->t0, b->wave_done[last_wave[i]]));
    b->per_scene[i].done_ms = ms;
    o.paths += paths;
  }
  o.primary_rays = primary;
  o.secondary_rays = hstats[kStatSecondary];
  o.shadow_rays = shadow;
  o.bounds_tests = hstats[kStatBoxTests] + hstats[kStatOccBoxTests];
  o.bounds_hits = hstats[kStatBoxHits] + hstats[kStatOccBoxHits];
  o.object_tests = hstats[kStatPrimTests] + hstats[kStatOccPrimTests];
  o.object_hits = hstats[kStatPrimHits] + hstats[kStatOccPrimHits];
  o.kernel_launches = b->graph_launches;
  o.bvh_nodes = b->total_nodes;
  o.primitives = b->total_prims;
  o.extend_rays = ext_rays;
  o.extend_launches = ext_launches;
  o.extend_box_tests = hstats[kStatBoxTests];
  o.extend_prim_tests = hstats[kStatPrimTests];
  o.occlude_rays = shadow;
  o.occlude_launches = occ_launches;
  o.occlude_box_tests = hstats[kStatOccBoxTests];
  o.occlude_prim_tests = hstats[kStatOccPrimTests];
  float ms = 0.0f;
  CUDA_TRY(cudaEventElapsedTime(&ms, b->t0, b->t1));
  o.render_ms = ms;
  if (hstats[kStatOverflow]) SetLastError("BVH traversal stack overflowed; results may miss hits");
}

void ClearFilms(MuonBatch *b, const MuonRenderParams *params, double *const *d_sum, double *const *d_sq,
                uint32_t *const *d_cnt) {
  for (int i = 0; i < b->n; ++i) {
    if (params[i].flags & MUON_RENDER_ACCUMULATE) continue;
    const size_t np = static_cast<size_t>(b->width[i]) * b->height[i];
    CUDA_TRY(cudaMemsetAsync(d_sum[i], 0, 3 * np * sizeof(double), b->stream));
    CUDA_TRY(cudaMemsetAsync(d_sq[i], 0, 3 * np * sizeof(double), b->stream));
    CUDA_TRY(cudaMemsetAsync(d_cnt[i], 0, np * sizeof(uint32_t), b->stream));
  }
}

}  // namespace

extern "C" {

int muon_gpu_batch_create(MuonScene *const *scenes, int32_t n, MuonBatch **out) {
  if (!scenes || !out || n <= 0) return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  *out = nullptr;
  std::vector<SceneView> views(n);
  for (int i = 0; i < n; ++i) {
    if (!GetSceneView(scenes[i], &views[i])) return Fail(MUON_ERR_INVALID_ARG, "null scene");
    if (views[i].device != views[0].device) return Fail(MUON_ERR_INVALID_ARG, "scenes live on different devices");
  }
  std::unique_ptr<MuonBatch> b;
  try {
    b.reset(new MuonBatch());
    b->n = n;
    b->device = views[0].device;
    CUDA_TRY(cudaSetDevice(b->device));
    CUDA_TRY(cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device));
    CUDA_TRY(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    MergeScenes(b.get(), views);
    b->schedule.resize(n);
    std::iota(b->schedule.begin(), b->schedule.end(), 0);
    // Shortest first (by film pixels), which lowers the median time to a
    // finished film; ties keep the given order.
    std::stable_sort(b->schedule.begin(), b->schedule.end(), [&](int x, int y) {
      return static_cast<int64_t>(b->width[x]) * b->height[x] < static_cast<int64_t>(b->width[y]) * b->height[y];
    });
    b->film_sum.resize(n);
    b->film_sq.resize(n);
    b->film_cnt.resize(n);
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  *out = b.release();
  return MUON_OK;
}

void muon_gpu_batch_destroy(MuonBatch *batch) { delete batch; }

int muon_gpu_batch_render_device(MuonBatch *batch, const MuonRenderParams *params, double *const *d_sum,
                                 double *const *d_sum_sq, uint32_t *const *d_count) {
  if (!batch || !params || !d_sum || !d_sum_sq || !d_count) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  for (int i = 0; i < batch->n; ++i)
    if (!d_sum[i] || !d_sum_sq[i] || !d_count[i]) return Fail(MUON_ERR_INVALID_ARG, "null film");
  int rc = ValidateBatchParams(batch, params);
  if (rc != MUON_OK) return rc;
  try {
    CUDA_TRY(cudaSetDevice(batch->device));
    ClearFilms(batch, params, d_sum, d_sum_sq, d_count);
    RenderBatch(batch, params, d_sum, d_sum_sq, d_count);
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}

int muon_gpu_batch_render(MuonBatch *batch, const MuonRenderParams *params, MuonFilm *films) {
  if (!batch || !params || !films) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  for (int i = 0; i < batch->n; ++i) {
    const MuonFilm &f = films[i];
    if (!f.sum || !f.sum_sq || !f.count) return Fail(MUON_ERR_INVALID_ARG, "null film");
    if (f.width != batch->width[i] || f.height != batch->height[i])
      return Fail(MUON_ERR_INVALID_ARG, "film size does not match its scene");
  }
  int rc = ValidateBatchParams(batch, params);
  if (rc != MUON_OK) return rc;
  try {
    CUDA_TRY(cudaSetDevice(batch->device));
    cudaStream_t st = batch->stream;
    std::vector<double *> s(batch->n), q(batch->n);
    std::vector<uint32_t *> c(batch->n);
    for (int i = 0; i < batch->n; ++i) {
      const size_t np = static_cast<size_t>(films[i].width) * films[i].height;
      batch->film_sum[i].Ensure(3 * np * sizeof(double));
      batch->film_sq[i].Ensure(3 * np * sizeof(double));
      batch->film_cnt[i].Ensure(np * sizeof(uint32_t));
      s[i] = batch->film_sum[i].as<double>();
      q[i] = batch->film_sq[i].as<double>();
      c[i] = batch->film_cnt[i].as<uint32_t>();
      if (params[i].flags & MUON_RENDER_ACCUMULATE) {
        CUDA_TRY(cudaMemcpyAsync(s[i], films[i].sum, 3 * np * sizeof(double), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(q[i], films[i].sum_sq, 3 * np * sizeof(double), cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(c[i], films[i].count, np * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
      }
    }
    ClearFilms(batch, params, s.data(), q.data(), c.data());
    RenderBatch(batch, params, s.data(), q.data(), c.data());
    for (int i = 0; i < batch->n; ++i) {
      const size_t np = static_cast<size_t>(films[i].width) * films[i].height;
      CUDA_TRY(cudaMemcpyAsync(films[i].sum, s[i], 3 * np * sizeof(double), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(films[i].sum_sq, q[i], 3 * np * sizeof(double), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaMemcpyAsync(films[i].count, c[i], np * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}

int muon_gpu_batch_autotune(MuonBatch *batch, const MuonRenderParams *params, MuonBatchTuning *out) {
  if (!batch || !params) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  int rc = ValidateBatchParams(batch, params);
  if (rc != MUON_OK) return rc;
  try {
    CUDA_TRY(cudaSetDevice(batch->device));
    // Trial: every scene at up to 4 samples per pixel into scratch films.
    std::vector<MuonRenderParams> trial(params, params + batch->n);
    int64_t paths = 0;
    for (int i = 0; i < batch->n; ++i) {
      trial[i].pixel_samples = std::min(trial[i].pixel_samples, 4);
      trial[i].flags &= ~(MUON_RENDER_STATS | MUON_RENDER_ACCUMULATE);
      paths += static_cast<int64_t>(batch->width[i]) * batch->height[i] * trial[i].pixel_samples;
    }
    std::vector<DeviceBuffer> fs(batch->n), fq(batch->n), fc(batch->n);
    std::vector<double *> s(batch->n), q(batch->n);
    std::vector<uint32_t *> c(batch->n);
    for (int i = 0; i < batch->n; ++i) {
      const size_t np = static_cast<size_t>(batch->width[i]) * batch->height[i];
      fs[i].Ensure(3 * np * sizeof(double));
      fq[i].Ensure(3 * np * sizeof(double));
      fc[i].Ensure(np * sizeof(uint32_t));
      s[i] = fs[i].as<double>();
      q[i] = fq[i].as<double>();
      c[i] = fc[i].as<uint32_t>();
    }
    // Traversal grids of 2..4 blocks per SM (4 is the most that fit at the
    // traversal kernels' register use: 64 registers x 256 threads).
    constexpr int kMaxBlocksPerSm = 4;
    int best_w = 0, best_b = 0, tried = 0;
    double best_ms = 1e300;
    for (int lw = 20; lw <= 24; ++lw) {
      const int w = 1 << lw;
      // Larger waves than the trial's paths time the same launches again.
      if (w > 2 * paths && lw > 20) break;
      for (int bps = 2; bps <= kMaxBlocksPerSm; ++bps) {
        batch->wave_paths = w;
        batch->blocks_per_sm = bps;
        ClearFilms(batch, trial.data(), s.data(), q.data(), c.data());
        RenderBatch(batch, trial.data(), s.data(), q.data(), c.data());  // capture + warm
        ClearFilms(batch, trial.data(), s.data(), q.data(), c.data());
        RenderBatch(batch, trial.data(), s.data(), q.data(), c.data());
        ++tried;
        if (batch->last.render_ms < best_ms) {
          best_ms = batch->last.render_ms;
          best_w = w;
          best_b = bps;
        }
      }
    }
    batch->wave_paths = best_w;
    batch->blocks_per_sm = best_b;
    batch->DropGraph();
    if (out) {
      out->wave_paths = best_w;
      out->traversal_blocks_per_sm = best_b;
      out->candidates = tried;
      out->pad = 0;
      out->best_ms = best_ms;
    }
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}

int muon_gpu_batch_stats(const MuonBatch *batch, MuonStats *total, MuonBatchSceneStats *per_scene) {
  if (!batch) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  if (total) *total = batch->last;
  if (per_scene) {
    for (int i = 0; i < batch->n; ++i)
      per_scene[i] = i < static_cast<int>(batch->per_scene.size()) ? batch->per_scene[i] : MuonBatchSceneStats{};
  }
  return MUON_OK;
}

int muon_gpu_render_batch(MuonScene *const *scenes, const MuonRenderParams *params, int32_t n, MuonFilm *films) {
  MuonBatch *b = nullptr;
  int rc = muon_gpu_batch_create(scenes, n, &b);
  if (rc != MUON_OK) return rc;
  rc = muon_gpu_batch_render(b, params, films);
  muon_gpu_batch_destroy(b);
  return rc;
}

}  // extern "C"
