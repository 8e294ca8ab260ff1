// Device scene management, the wavefront render loop and the GPU entry points
// of the C ABI (include/muon_gpu.h).
//
// The loop replaces Renderer::Render's thread pool (muon/renderer.cc:31-77):
// instead of threads pulling row tiles and tracing one sample at a time, the
// film's samples are cut into wavefronts of up to `wave_paths` paths and each
// wavefront is advanced one bounce at a time by whole-GPU kernels.
#include <cuda_runtime.h>

#include <mutex>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "bvh_walk.h"
#include "guide.h"
#include "host_cuda.h"
#include "host_scene.h"
#include "kernels.cuh"
#include "scene_access.h"
#include "scene_build.h"
#include "scene_records.h"

using namespace muon_gpu;

namespace {

constexpr int kDefaultWavePaths = 1 << 24;
constexpr int kMaxBounces = 256;  // hard cap for unbounded depth without Russian roulette
constexpr int kMaxEventPairs = 16384;

}  // namespace

// The path arrays of one wavefront in flight (PathBuffers).
struct WorkSet {
  DeviceBuffer ray_o[2], ray_d[2], tp[2], rad[2], hits, link, final_rad, org, contrib, slot_dir, shq, order;
  int64_t cap = 0;
  int slots = -1;

  // Grows the arrays (the scene's streams are idle); true if any moved.
  bool Ensure(int64_t paths, int slots_wanted, int device) {
    if (paths <= cap && slots_wanted <= slots) return false;
    const int64_t p = std::max(paths, cap);
    const int sl_count = std::max(slots_wanted, slots);
    for (int k = 0; k < 2; ++k) {
      EnsurePooled(ray_o[k], p * sizeof(float4), device);
      EnsurePooled(ray_d[k], p * sizeof(float4), device);
      EnsurePooled(tp[k], p * sizeof(float4), device);
      EnsurePooled(rad[k], p * sizeof(float4), device);
    }
    EnsurePooled(hits, p * sizeof(int2), device);
    EnsurePooled(link, p * sizeof(int32_t), device);
    EnsurePooled(final_rad, p * sizeof(float4), device);
    EnsurePooled(org, p * sizeof(float4), device);
    const size_t sl = static_cast<size_t>(p) * std::max(sl_count, 1);
    EnsurePooled(contrib, sl * sizeof(float4), device);
    EnsurePooled(slot_dir, sl * sizeof(float4), device);
    EnsurePooled(shq, sl * sizeof(uint32_t), device);
    EnsurePooled(order, static_cast<size_t>(OrderInts(p)) * sizeof(int32_t), device);
    cap = p;
    slots = sl_count;
    return true;
  }

  PathBuffers Buffers(const DeviceBuffer &stats) const {
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
    b.order_cap = static_cast<int32_t>(cap);
    b.stats = stats.as<unsigned long long>();
    return b;
  }

  // To the process-wide cache (the streams are idle).
  void Give(int device) {
    for (int k = 0; k < 2; ++k) {
      PoolGive(ray_o[k], device);
      PoolGive(ray_d[k], device);
      PoolGive(tp[k], device);
      PoolGive(rad[k], device);
    }
    for (DeviceBuffer *b : {&hits, &link, &final_rad, &org, &contrib, &slot_dir, &shq, &order}) PoolGive(*b, device);
  }
};

struct MuonScene {
  int device = 0;
  cudaStream_t stream = nullptr;
  // A second stream and its events, for wavefronts in flight two at a time.
  cudaStream_t stream2 = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr, film_ev[2] = {nullptr, nullptr};
  SceneImage img;
  // The leaf-order records of a scene whose BVH was built on the device live
  // on the device only (img holds them in input order) until a host reader
  // calls SyncSceneImage.
  mutable bool host_records_stale = false;
  int64_t num_slots = 0;  // primitive records on the device
  DevScene dev{};
  DevCamera cam{};
  // scene arrays
  DeviceBuffer nodes, prims, prims_obj, shade, smooth, smooth_obj, transforms, materials, lights, light_tris,
      light_tris_obj, light_tri_ok, other_lights, all_lights;
  // work arrays: the path arrays of up to two wavefronts in flight, their
  // counters and the statistics
  WorkSet work[2];
  DeviceBuffer counters, stats;
  DeviceBuffer film_sum, film_sq, film_cnt, ray_in, ray_out, ray_aux;
  uint32_t *h_counters = nullptr;  // pinned, one WaveCounters block per wave
  size_t h_counters_len = 0;
  std::vector<EventPair> events;
  int events_used = 0;
  MuonStats last{};
  // Instantiated CUDA graph of the last bounded-depth render and the launch
  // configuration it was captured for.
  cudaGraphExec_t graph = nullptr;
  std::string graph_key;
  int graph_events = 0;
  uint64_t graph_launches = 0;
  // Launch configuration of the last render launched kernel by kernel: a
  // graph is captured when the same configuration renders again (a one-off
  // render would pay more to instantiate a graph than the graph saves).
  std::string seen_key;

  ~MuonScene() {
    // The work arrays go to the process-wide cache once the stream is idle.
    if (stream && cudaStreamSynchronize(stream) == cudaSuccess &&
        (!stream2 || cudaStreamSynchronize(stream2) == cudaSuccess)) {
      for (WorkSet &ws : work) ws.Give(device);
      for (DeviceBuffer *b : {&film_sum, &film_sq, &film_cnt, &nodes, &prims, &prims_obj, &shade, &smooth, &smooth_obj})
        PoolGive(*b, device);
    }
    for (cudaEvent_t e : {fork_ev, join_ev, film_ev[0], film_ev[1]})
      if (e) cudaEventDestroy(e);
    if (stream2) cudaStreamDestroy(stream2);
    if (graph) cudaGraphExecDestroy(graph);
    for (EventPair &e : events) {
      if (e.a) cudaEventDestroy(e.a);
      if (e.b) cudaEventDestroy(e.b);
    }
    if (h_counters) cudaFreeHost(h_counters);
    if (stream) cudaStreamDestroy(stream);
  }

  EventPair *NextEvent(int kind) {
    if (events_used >= kMaxEventPairs) return nullptr;
    if (events_used == static_cast<int>(events.size())) {
      EventPair e;
      CUDA_TRY(cudaEventCreate(&e.a));
      CUDA_TRY(cudaEventCreate(&e.b));
      events.push_back(e);
    }
    EventPair *e = &events[events_used++];
    e->kind = kind;
    return e;
  }

  PathBuffers Buffers(int set = 0) const { return work[set].Buffers(stats); }

  // Grows the path arrays of `sets` wavefronts in flight; true if any moved.
  bool EnsureWork(int64_t paths, int slots, int sets = 1) {
    bool moved = false;
    for (int k = 0; k < sets; ++k) moved |= work[k].Ensure(paths, slots, device);
    return moved;
  }

  // The second stream and the events that order two wavefronts in flight.
  void EnsureStream2() {
    if (stream2) return;
    CUDA_TRY(cudaStreamCreateWithFlags(&stream2, cudaStreamNonBlocking));
    for (cudaEvent_t *e : {&fork_ev, &join_ev, &film_ev[0], &film_ev[1]})
      CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
  }

  // Grows the device and pinned host counter arrays; returns true if the
  // device pointer changed.
  bool EnsureCounters(size_t words) {
    if (words <= h_counters_len) return false;
    counters.Ensure(words * sizeof(uint32_t));
    if (h_counters) cudaFreeHost(h_counters);
    h_counters = nullptr;
    CUDA_TRY(cudaMallocHost(reinterpret_cast<void **>(&h_counters), words * sizeof(uint32_t)));
    h_counters_len = words;
    return true;
  }

  void DropGraph() {
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_key.clear();
  }
};

namespace muon_gpu {
namespace {
thread_local std::string g_last_error;
}
void SetLastError(const std::string &msg) { g_last_error = msg; }
const char *LastError() { return g_last_error.c_str(); }
}  // namespace muon_gpu

namespace muon_gpu {

int Fail(int code, const std::string &msg) {
  SetLastError(msg);
  return code;
}
int FailCuda(const CudaError &e) {
  return Fail(MUON_ERR_CUDA, std::string(e.where) + ": " + cudaGetErrorString(e.code));
}

void ComputeCamera(const MuonCameraDesc &c, DevCamera *out) {
  // Camera::Camera (muon/camera.cc:15-35) in the reference's float order.
  mm::v3 eye = mm::make3(c.eye[0], c.eye[1], c.eye[2]);
  mm::v3 look = mm::make3(c.look_at[0], c.look_at[1], c.look_at[2]);
  mm::v3 up = mm::make3(c.up[0], c.up[1], c.up[2]);
  float tan_y = tanf(mm::radians(c.fov_y_degrees) / 2.0f);
  float tan_x = tan_y * (static_cast<float>(c.width) / static_cast<float>(c.height));
  mm::v3 w = mm::normalize(eye - look);
  mm::v3 u = mm::normalize(mm::cross(up, w));
  mm::v3 v = mm::cross(w, u);
  const mm::v3 *src[4] = {&eye, &u, &v, &w};
  float *dst[4] = {out->eye, out->u, out->v, out->w};
  for (int k = 0; k < 4; ++k) {
    dst[k][0] = src[k]->x;
    dst[k][1] = src[k]->y;
    dst[k][2] = src[k]->z;
  }
  out->tan_fov_x = tan_x;
  out->tan_fov_y = tan_y;
  out->width = c.width;
  out->height = c.height;
}

// Builds the BVH of a scene on the device (binned SAH or linear BVH) from
// input-order records: those BuildSceneImage left on the host (defer_bvh),
// or, with `device_desc`, the hittable triangles' records computed on the
// device from the scene description followed by the spheres' records from
// the host (device_records). The records are gathered into leaf order in the
// scene's buffers; the nodes are copied back into the host image, and so are
// the records for the linear BVH (the binned-SAH path leaves them on the
// device until SyncSceneImage). Returns MUON_OK or an error code (last error
// set).
int BuildBvhOnGpu(MuonScene *sc, int builder, int max_leaf, cudaStream_t st, const MuonSceneDesc *device_desc) {
  SceneImage &im = sc->img;
  // temporaries come from (and go back to) the device block cache
  DeviceBuffer boxes, in_prims, in_obj, in_shade, in_sn, in_sno, scratch, order, last, tris, xfs, mats, qidx, keep,
      pos, count, scan;
  DeviceBuffer *const temps[] = {&boxes, &in_prims, &in_obj, &in_shade, &in_sn, &in_sno, &scratch, &order, &last,
                                 &tris, &xfs, &mats, &qidx, &keep, &pos, &count, &scan};
  struct GiveBack {
    DeviceBuffer *const *bufs;
    int count;
    cudaStream_t st;
    int device;
    ~GiveBack() {
      if (cudaStreamSynchronize(st) == cudaSuccess)
        for (int i = 0; i < count; ++i) PoolGive(*bufs[i], device);
    }
  } give_back{temps, static_cast<int>(sizeof(temps) / sizeof(temps[0])), st, sc->device};
  int n = static_cast<int>(im.prims.size());
  if (device_desc) {
    const int64_t ntri = device_desc->num_triangles;
    const int nsph = n;  // the host image holds the spheres alone
    int32_t nkept = 0;
    if (ntri > 0) {
      EnsurePooled(tris, sizeof(MuonTriangleDesc) * ntri, sc->device);
      CUDA_TRY(cudaMemcpyAsync(tris.ptr, device_desc->triangles, sizeof(MuonTriangleDesc) * ntri,
                               cudaMemcpyHostToDevice, st));
      EnsurePooled(xfs, sizeof(MuonTransformDesc) * std::max(device_desc->num_transforms, 1), sc->device);
      if (device_desc->num_transforms > 0)
        CUDA_TRY(cudaMemcpyAsync(xfs.ptr, device_desc->transforms,
                                 sizeof(MuonTransformDesc) * device_desc->num_transforms, cudaMemcpyHostToDevice, st));
      UploadPooled(mats, im.materials, st, sc->device);
      UploadPooled(qidx, im.quad_index, st, sc->device);
      EnsurePooled(keep, sizeof(int32_t) * ntri, sc->device);
      EnsurePooled(pos, sizeof(int32_t) * ntri, sc->device);
      EnsurePooled(count, 16, sc->device);
      const size_t scan_bytes = HittableScanBytes(ntri);
      EnsurePooled(scan, std::max<size_t>(scan_bytes, 16), sc->device);
      CUDA_TRY(CountHittableTriangles(tris.as<MuonTriangleDesc>(), ntri, keep.as<int32_t>(), pos.as<int32_t>(),
                                      count.as<int32_t>(), scan.ptr, scan_bytes, st));
      CUDA_TRY(cudaMemcpyAsync(&nkept, count.ptr, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
      CUDA_TRY(cudaStreamSynchronize(st));
    }
    n = nkept + nsph;
    sc->num_slots = n;
    if (n == 0) {
      for (DeviceBuffer *b : {&sc->nodes, &sc->prims, &sc->prims_obj, &sc->shade, &sc->smooth, &sc->smooth_obj})
        EnsurePooled(*b, 16, sc->device);
      im.nodes.clear();
      im.boxes.clear();
      im.bvh = BvhBuildStats();
      return MUON_OK;
    }
    EnsurePooled(boxes, sizeof(float) * 6 * n, sc->device);
    EnsurePooled(in_prims, sizeof(PrimRecord) * n, sc->device);
    EnsurePooled(in_obj, sizeof(PrimRecord) * n, sc->device);
    EnsurePooled(in_shade, sizeof(ShadeRecord) * n, sc->device);
    if (im.any_smooth) {
      EnsurePooled(in_sn, sizeof(F4) * 3 * n, sc->device);
      EnsurePooled(in_sno, sizeof(F4) * 3 * n, sc->device);
    }
    LaunchTriangleRecords(tris.as<MuonTriangleDesc>(), ntri, xfs.as<MuonTransformDesc>(), mats.as<DevMaterial>(),
                          qidx.as<int32_t>(), keep.as<int32_t>(), pos.as<int32_t>(), in_prims.as<PrimRecord>(),
                          in_obj.as<PrimRecord>(), in_shade.as<ShadeRecord>(),
                          im.any_smooth ? in_sn.as<F4>() : nullptr, im.any_smooth ? in_sno.as<F4>() : nullptr,
                          boxes.as<float>(), st);
    CUDA_TRY(cudaGetLastError());
    if (nsph > 0) {
      CUDA_TRY(cudaMemcpyAsync(in_prims.as<PrimRecord>() + nkept, im.prims.data(), sizeof(PrimRecord) * nsph,
                               cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(in_obj.as<PrimRecord>() + nkept, im.prims_obj.data(), sizeof(PrimRecord) * nsph,
                               cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(in_shade.as<ShadeRecord>() + nkept, im.shade.data(), sizeof(ShadeRecord) * nsph,
                               cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(boxes.as<float>() + 6 * static_cast<size_t>(nkept), im.boxes.data(),
                               sizeof(float) * 6 * nsph, cudaMemcpyHostToDevice, st));
      if (im.any_smooth) {
        CUDA_TRY(cudaMemsetAsync(in_sn.as<F4>() + 3 * static_cast<size_t>(nkept), 0, sizeof(F4) * 3 * nsph, st));
        CUDA_TRY(cudaMemsetAsync(in_sno.as<F4>() + 3 * static_cast<size_t>(nkept), 0, sizeof(F4) * 3 * nsph, st));
      }
    }
  } else {
    sc->num_slots = n;
    UploadPooled(boxes, im.boxes, st, sc->device);
    UploadPooled(in_prims, im.prims, st, sc->device);
    UploadPooled(in_obj, im.prims_obj, st, sc->device);
    UploadPooled(in_shade, im.shade, st, sc->device);
    if (im.any_smooth) {
      UploadPooled(in_sn, im.smooth_normals, st, sc->device);
      UploadPooled(in_sno, im.smooth_normals_obj, st, sc->device);
    }
  }
  int nn = std::max(n - 1, 1);
  const bool sah = builder == MUON_BUILDER_GPU_SAH;
  const size_t sbytes = sah ? GpuSahScratchBytes(n) : GpuLbvhScratchBytes(n);
  EnsurePooled(scratch, sbytes, sc->device);
  EnsurePooled(order, sizeof(int32_t) * n, sc->device);
  EnsurePooled(last, static_cast<size_t>(n), sc->device);
  EnsurePooled(sc->nodes, sizeof(BvhNode) * nn, sc->device);
  EnsurePooled(sc->prims, sizeof(PrimRecord) * n, sc->device);
  EnsurePooled(sc->prims_obj, sizeof(PrimRecord) * n, sc->device);
  EnsurePooled(sc->shade, sizeof(ShadeRecord) * n, sc->device);
  EnsurePooled(sc->smooth, im.any_smooth ? sizeof(F4) * 3 * n : 16, sc->device);
  EnsurePooled(sc->smooth_obj, im.any_smooth ? sizeof(F4) * 3 * n : 16, sc->device);
  GpuSahResult sr;
  if (sah) {
    CUDA_TRY(BuildGpuSah(boxes.as<float>(), n, max_leaf, scratch.ptr, sc->nodes.as<BvhNode>(), order.as<int32_t>(),
                         last.as<uint8_t>(), &sr, st));
    if (sr.error) return Fail(MUON_ERR_CUDA, "device BVH build: internal list or stack limit reached");
    nn = sr.nodes;
  } else {
    LaunchGpuLbvh(boxes.as<float>(), n, scratch.ptr, sbytes, sc->nodes.as<BvhNode>(), order.as<int32_t>(),
                  last.as<uint8_t>(), st);
  }
  LaunchGatherPrims(order.as<int32_t>(), last.as<uint8_t>(), n, in_prims.as<PrimRecord>(), in_obj.as<PrimRecord>(),
                    in_shade.as<ShadeRecord>(), im.any_smooth ? in_sn.as<F4>() : nullptr,
                    im.any_smooth ? in_sno.as<F4>() : nullptr, sc->prims.as<PrimRecord>(),
                    sc->prims_obj.as<PrimRecord>(), sc->shade.as<ShadeRecord>(),
                    im.any_smooth ? sc->smooth.as<F4>() : nullptr, im.any_smooth ? sc->smooth_obj.as<F4>() : nullptr,
                    st);
  CUDA_TRY(cudaGetLastError());
  im.nodes.resize(nn);
  CUDA_TRY(cudaMemcpyAsync(im.nodes.data(), sc->nodes.ptr, sizeof(BvhNode) * nn, cudaMemcpyDeviceToHost, st));
  if (sah) {
    // the records stay on the device until a host reader asks for them
    // (SyncSceneImage); the scene box and the node count come from the nodes
    CUDA_TRY(cudaStreamSynchronize(st));
    im.boxes.clear();
    im.boxes.shrink_to_fit();
    sc->host_records_stale = true;
    BvhBuildStats &bs = im.bvh;
    bs = BvhBuildStats();
    bs.nodes = nn;
    // the builder's own counts, with the host builder's depth convention
    bs.leaves = sr.leaves;
    bs.max_depth = sr.max_depth;
    bs.max_leaf = sr.max_leaf;
    return MUON_OK;
  }
  CUDA_TRY(cudaMemcpyAsync(im.prims.data(), sc->prims.ptr, sizeof(PrimRecord) * n, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(im.prims_obj.data(), sc->prims_obj.ptr, sizeof(PrimRecord) * n, cudaMemcpyDeviceToHost,
                           st));
  CUDA_TRY(cudaMemcpyAsync(im.shade.data(), sc->shade.ptr, sizeof(ShadeRecord) * n, cudaMemcpyDeviceToHost, st));
  if (im.any_smooth) {
    CUDA_TRY(cudaMemcpyAsync(im.smooth_normals.data(), sc->smooth.ptr, sizeof(F4) * 3 * n, cudaMemcpyDeviceToHost,
                             st));
    CUDA_TRY(cudaMemcpyAsync(im.smooth_normals_obj.data(), sc->smooth_obj.ptr, sizeof(F4) * 3 * n,
                             cudaMemcpyDeviceToHost, st));
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  im.boxes.clear();
  im.boxes.shrink_to_fit();
  for (int slot = 0; slot < n; ++slot) im.leaf_of_prim_id[im.shade[slot].s1.y] = slot;
  BvhBuildStats &bs = im.bvh;
  bs = BvhBuildStats();
  bs.nodes = nn;
  // statistics: depth (iterative walk from the root) and leaves
  std::vector<std::pair<int32_t, int32_t>> stack{{0, 1}};
  while (!stack.empty()) {
    auto [node, depth] = stack.back();
    stack.pop_back();
    bs.max_depth = std::max(bs.max_depth, depth);
    const int32_t links[2] = {im.nodes[node].d.x, im.nodes[node].d.y};
    for (int32_t l : links) {
      if (l >= 0) {
        if (l < nn && depth < 1000) stack.push_back({l, depth + 1});
      } else if (l != kEmptyLink) {
        ++bs.leaves;
        int count = 0;
        for (int i = ~l; i < n; ++i) {
          ++count;
          uint32_t flags;
          std::memcpy(&flags, &im.prims[i].p3.w, 4);
          if (flags & kPrimLast) break;
        }
        bs.max_leaf = std::max(bs.max_leaf, count);
      }
    }
  }
  return MUON_OK;
}

// ShadeParams of a render (PathTracer settings and the shadow-slot layout of
// a path vertex); returns the number of shadow slots.
int SetupShade(const MuonRenderParams &p, int num_quad_lights, int num_other_lights, ShadeParams *out) {
  const bool pt = p.integrator == MUON_INTEGRATOR_PATHTRACER;
  ShadeParams sp{};
  sp.integrator = p.integrator;
  sp.nee = p.next_event_estimation;
  sp.is_mode = p.importance_sampling;
  sp.rr = p.russian_roulette;
  sp.min_depth = p.min_depth;
  // Integrator::Trace casts a ray at depth d only if d <= max_depth (or
  // max_depth - 1 when lights are sampled) (muon/integration.cc:29-33).
  sp.max_trace_depth = p.max_depth < 0 ? -1 : (p.next_event_estimation != MUON_NEE_OFF ? p.max_depth - 1 : p.max_depth);
  sp.strata = p.light_stratify ? static_cast<int>(std::sqrt(static_cast<double>(p.light_samples))) : 1;
  sp.per_section = p.light_stratify ? 1 : p.light_samples;
  sp.per_light = sp.strata * sp.strata * sp.per_section;
  sp.light_samples = std::max(1, p.light_samples);
  sp.isect = p.intersect_mode;
  sp.max_bounces = kMaxBounces;
  int slots = 0;
  sp.mis_slot = -1;
  if (pt && p.next_event_estimation != MUON_NEE_OFF) {
    slots = num_quad_lights * sp.per_light + num_other_lights;
    if (p.next_event_estimation == MUON_NEE_MIS) sp.mis_slot = slots++;
  }
  sp.slots = slots;
  *out = sp;
  return slots;
}

// The two triangles of each quad light (muon/parser.cc:735-747), in the same
// record format as the BVH's, for the MIS light-hit test.
void BuildLightTris(const std::vector<DevLight> &lights, std::vector<PrimRecord> *lt_out,
                    std::vector<PrimRecord> *lt_obj_out, std::vector<int32_t> *lt_ok_out) {
  std::vector<PrimRecord> &lt = *lt_out, &lt_obj = *lt_obj_out;
  std::vector<int32_t> &lt_ok = *lt_ok_out;
  lt.assign(2 * lights.size(), PrimRecord{});
  lt_obj.assign(2 * lights.size(), PrimRecord{});
  lt_ok.assign(2 * lights.size(), 0);
  for (size_t i = 0; i < lights.size(); ++i) {
    const DevLight &l = lights[i];
    mm::v3 c = mm::make3(l.corner.x, l.corner.y, l.corner.z);
    mm::v3 e0 = mm::make3(l.edge0.x, l.edge0.y, l.edge0.z), e1 = mm::make3(l.edge1.x, l.edge1.y, l.edge1.z);
    mm::v3 va = c, vb = c + e0, vc = c + e1, vd = c + e0 + e1;
    const mm::v3 tri[2][3] = {{va, vc, vb}, {vb, vc, vd}};
    for (int t = 0; t < 2; ++t) {
      mm::v3 n = mm::cross(tri[t][1] - tri[t][0], tri[t][2] - tri[t][0]);
      PrimRecord &r = lt[2 * i + t];
      r.p0 = F4{tri[t][0].x, tri[t][0].y, tri[t][0].z, mm::dot(tri[t][0], n)};
      r.p1 = F4{tri[t][1].x, tri[t][1].y, tri[t][1].z, 1e-4f};
      r.p2 = F4{tri[t][2].x, tri[t][2].y, tri[t][2].z, 0.0f};
      r.p3 = F4{n.x, n.y, n.z, 0.0f};
      lt_ok[2 * i + t] = mm::length(n) >= 1e-4f ? 1 : 0;
      PrimRecord &ro = lt_obj[2 * i + t];
      int32_t identity = -1;
      float xf_bits;
      std::memcpy(&xf_bits, &identity, 4);
      ro.p0 = F4{tri[t][0].x, tri[t][0].y, tri[t][0].z, 0.0f};
      ro.p1 = F4{tri[t][1].x, tri[t][1].y, tri[t][1].z, xf_bits};
      ro.p2 = F4{tri[t][2].x, tri[t][2].y, tri[t][2].z, mm::dot(n, n)};
      ro.p3 = F4{n.x, n.y, n.z, 0.0f};
    }
  }
}

WavePlan PlanWaves(int width, int height, const MuonRenderParams &p, int64_t budget) {
  WavePlan wp;
  wp.width = width;
  wp.npix = static_cast<int64_t>(width) * height;
  wp.spp = p.pixel_samples;
  wp.ns = static_cast<int>(std::min<int64_t>(wp.spp, std::max<int64_t>(budget, 1)));
  wp.pix_per_wave = std::max<int64_t>(1, budget / wp.ns);
  wp.sample_offset = static_cast<uint32_t>(p.sample_offset);
  wp.seed = p.seed;
  return wp;
}

BouncePlan PlanBounces(const MuonRenderParams &p, const ShadeParams &sp) {
  const bool pt = p.integrator == MUON_INTEGRATOR_PATHTRACER;
  BouncePlan b;
  // A path traces at depths 0..max_trace_depth; with max_depth 0 and lights
  // sampled, Trace() casts no ray at all.
  b.traces = !(p.max_depth >= 0 && sp.max_trace_depth < 0);
  b.bounded = !pt || sp.max_trace_depth >= 0;  // (the ray tracer runs in one launch)
  b.bounces = !b.traces ? 0 : (!pt ? 1 : (b.bounded ? sp.max_trace_depth + 1 : sp.max_bounces));
  return b;
}

int ValidateParams(const MuonRenderParams &p) {
  if (p.integrator < MUON_INTEGRATOR_NORMALS || p.integrator > MUON_INTEGRATOR_PATHTRACER)
    return Fail(MUON_ERR_INVALID_ARG, "unknown integrator");
  if (p.pixel_samples < 1) return Fail(MUON_ERR_INVALID_ARG, "pixel_samples must be >= 1");
  if (p.next_event_estimation < MUON_NEE_OFF || p.next_event_estimation > MUON_NEE_MIS)
    return Fail(MUON_ERR_INVALID_ARG, "unknown next_event_estimation mode");
  if (p.importance_sampling < MUON_IS_HEMISPHERE || p.importance_sampling > MUON_IS_BRDF)
    return Fail(MUON_ERR_INVALID_ARG, "unknown importance_sampling mode");
  if (p.intersect_mode < MUON_ISECT_FAST || p.intersect_mode > MUON_ISECT_EXACT)
    return Fail(MUON_ERR_INVALID_ARG, "unknown intersect_mode");
  if (p.integrator == MUON_INTEGRATOR_PATHTRACER && p.next_event_estimation != MUON_NEE_OFF && p.light_samples < 1)
    return Fail(MUON_ERR_INVALID_ARG, "light_samples must be >= 1");
  if (p.max_depth < -1) return Fail(MUON_ERR_INVALID_ARG, "max_depth must be >= -1");
  if (p.wave_paths < 0) return Fail(MUON_ERR_INVALID_ARG, "wave_paths must be >= 0");
  return MUON_OK;
}

}  // namespace muon_gpu

namespace {

// Queue samples of a probed render (muon_gpu_probe_traversal): per wave,
// bounce and kind (0 closest hit, 1 shadow) a block of 1 + 2m float4s as
// SampleQueueKernel writes them.
struct QueueProbe {
  int m = 0;
  DeviceBuffer buf;
  size_t waves = 0;
  int bounces = 0;
  size_t BlockFloat4s() const { return 1 + 2 * static_cast<size_t>(m); }
  size_t Offset(size_t wave, int bounce, int kind) const {
    return ((wave * bounces + bounce) * 2 + kind) * BlockFloat4s();
  }
};

// Renders into a device film. Throws CudaError.
//
// Bounded depth: every wavefront is a fixed launch sequence (camera; per
// bounce extend, shade, occlude, fold; film) whose kernels read their queue
// lengths from device counters, so the whole frame is captured once into a
// CUDA graph and replayed; the host synchronises once per frame. Unbounded
// depth (max_depth -1): the host reads the queue length after every bounce and
// stops when no path continues.
// Wavefronts in flight at a time in a render (1 or 2).
#ifndef MUON_WAVES_IN_FLIGHT
#define MUON_WAVES_IN_FLIGHT 2
#endif

void RenderDevice(MuonScene *sc, const MuonRenderParams &p, double *d_sum, double *d_sq, uint32_t *d_cnt,
                  const GuideDev *guide = nullptr, QueueProbe *probe = nullptr) {
  cudaStream_t st = sc->stream;
  const bool pt = p.integrator == MUON_INTEGRATOR_PATHTRACER;
  // Raytracer / AnalyticDirect: one kernel follows each path to its end.
  const bool whitted = p.integrator == MUON_INTEGRATOR_RAYTRACER || p.integrator == MUON_INTEGRATOR_ANALYTIC_DIRECT;
  const bool stats_on = (p.flags & MUON_RENDER_STATS) != 0;
  const bool timing = (p.flags & MUON_RENDER_TIMING) != 0;
  ShadeParams sp;
  const int slots = SetupShade(p, sc->dev.num_lights, sc->dev.num_other_lights, &sp);
  GuideDev guide_local{};
  if (guide) {
    guide_local = *guide;
    guide_local.area_slots = sc->dev.num_lights * sp.per_light;
    guide_local.mis_slot = sp.mis_slot;
  }

  const int W = sc->img.width, H = sc->img.height;
  const int64_t npix_total = static_cast<int64_t>(W) * H;
  const int spp = p.pixel_samples;
  int64_t budget = p.wave_paths > 0 ? p.wave_paths : kDefaultWavePaths;
  // Keep per-wave path state within ~8 GiB.
  budget = std::max<int64_t>(1, std::min<int64_t>(budget, (int64_t(8) << 30) / WorkBytesPerPath(slots)));
  budget = std::min<int64_t>(budget, kMaxWavePaths);
  const WavePlan plan = PlanWaves(W, H, p, budget);
  std::vector<WaveInfo> waves(plan.Count());
  for (size_t i = 0; i < waves.size(); ++i) waves[i] = plan.At(i);
  const BouncePlan bp = PlanBounces(p, sp);
  const bool traces = bp.traces, bounded = bp.bounded;
  const int bounces = bp.bounces;
  const size_t stride = WaveCounterWords(bounces);
  // Two wavefronts in flight, on two streams with their own path arrays:
  // while one wavefront's kernels drain (the last rays of a persistent
  // traversal launch, the last blocks of a pass), the other's fill the SMs.
  // Films are still added in wave order. Per-kernel timing, probes, guiding
  // and host-driven unbounded loops run the wavefronts one after another.
  const bool concurrent = MUON_WAVES_IN_FLIGHT > 1 && bounded && !timing && !probe && !guide && waves.size() > 1;
  bool moved = sc->EnsureWork(std::min<int64_t>(plan.pix_per_wave, npix_total) * plan.ns, slots, concurrent ? 2 : 1);
  moved |= sc->EnsureCounters(stride * waves.size());
  sc->stats.Ensure(sizeof(unsigned long long) * kNumStats);
  if (concurrent) sc->EnsureStream2();
  const PathBuffers bsets[2] = {sc->Buffers(0), sc->Buffers(concurrent ? 1 : 0)};
  const PathBuffers &b = bsets[0];
  if (probe) {
    probe->waves = waves.size();
    probe->bounces = bounces;
    const size_t bytes = std::max<size_t>(16, waves.size() * bounces * 2 * probe->BlockFloat4s() * sizeof(float4));
    probe->buf.Ensure(bytes);
    CUDA_TRY(cudaMemsetAsync(probe->buf.ptr, 0, bytes, st));
  }
  auto sample_queue = [&](size_t wi, WaveCounters wc, int k, int kind) {
    if (probe)
      LaunchSampleQueue(b, wc, k, kind, slots, probe->m, probe->buf.as<float4>() + probe->Offset(wi, k, kind), st);
  };

  uint64_t launches = 0;
  int timed_pairs = 1;
  // Records the launch sequence of the whole frame on `st`.
  bool capturing = false;  // event records inside a graph capture become external event nodes
  auto enqueue = [&](bool host_loop) {
    sc->events_used = 1;  // pair 0 brackets the frame
    CUDA_TRY(cudaMemsetAsync(sc->counters.ptr, 0, stride * waves.size() * sizeof(uint32_t), st));
    CUDA_TRY(cudaMemsetAsync(sc->stats.ptr, 0, sizeof(unsigned long long) * kNumStats, st));
    const cudaStream_t main_st = st;
    if (concurrent) {  // the second stream joins after the clears
      CUDA_TRY(cudaEventRecord(sc->fork_ev, main_st));
      CUDA_TRY(cudaStreamWaitEvent(sc->stream2, sc->fork_ev, 0));
    }
    for (size_t wi = 0; wi < waves.size(); ++wi) {
      const WaveInfo &w = waves[wi];
      WaveCounters wc{sc->counters.as<uint32_t>() + wi * stride};
      // this wavefront's path arrays and stream
      const int set = concurrent ? static_cast<int>(wi & 1) : 0;
      const PathBuffers &b = bsets[set];
      const cudaStream_t st = set ? sc->stream2 : main_st;
      LaunchCamera(sc->cam, w, b, wc, st);
      ++launches;
      auto timed = [&](int kind, auto &&launch) {
        // External event nodes when captured, so they time the kernels
        // inside the replayed graph.
        EventPair *ev = timing ? sc->NextEvent(kind) : nullptr;
        if (ev) CUDA_TRY(capturing ? cudaEventRecordWithFlags(ev->a, st, cudaEventRecordExternal)
                                   : cudaEventRecord(ev->a, st));
        launch();
        if (ev) CUDA_TRY(capturing ? cudaEventRecordWithFlags(ev->b, st, cudaEventRecordExternal)
                                   : cudaEventRecord(ev->b, st));
        ++launches;
      };
      if (whitted && bounces > 0) {
        // Integrator::Trace's depth cut-off; unbounded depth stops at the
        // bounce cap (a ray between two mirrors would never end).
        const int max_d = p.integrator == MUON_INTEGRATOR_ANALYTIC_DIRECT ? 0
                          : sp.max_trace_depth >= 0 ? sp.max_trace_depth : kMaxBounces - 1;
        timed(2, [&] { LaunchWhitted(sc->dev, b, w, p.integrator, max_d, p.intersect_mode, stats_on, st); });
      }
      for (int k = 0; k < (whitted ? 0 : bounces); ++k) {
        sample_queue(wi, wc, k, 0);
        timed(0, [&] { LaunchExtend(sc->dev, b, wc, k, w.n, p.intersect_mode, stats_on, st); });
        // Guiding covers the first rec_bounces vertices of a path (where the
        // network is trained); deeper vertices sample the BRDF alone.
        const bool guided = guide && k < guide->rec_bounces;
        if (guided) {
          // two kernels: the features, then the tensor-core network pass
          timed(2, [&] { LaunchGuideInfer(sc->dev, b, wc, k, w.n, p.intersect_mode, guide_local, st); });
          ++launches;
        }
        if (!pt) {
          timed(2, [&] { LaunchShadeDebug(sc->dev, b, wc, p.integrator, w.n, p.intersect_mode, st); });
          break;
        }
        timed(2, [&] {
          if (guided) LaunchShadePathGuided(sc->dev, w, sp, b, wc, k, w.n, guide_local, st);
          else LaunchShadePath(sc->dev, w, sp, b, wc, k, w.n, st);
        });
        if (slots > 0) {
          sample_queue(wi, wc, k, 1);
          timed(1, [&] {
            LaunchOcclude(sc->dev, b, wc, k, slots, static_cast<int>(std::min<int64_t>(int64_t(w.n) * slots, INT32_MAX)),
                          p.intersect_mode, stats_on, st);
          });
        }
        timed(3, [&] {
          if (guided) LaunchFoldGuided(b, wc, k, slots, w.n, guide_local, st);
          else LaunchFold(b, wc, k, slots, w.n, st);
        });
        if (guided) launches += 2;  // the ordered append of training samples
        if (host_loop) {
          CUDA_TRY(cudaMemcpyAsync(sc->h_counters, wc.count(k + 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
          CUDA_TRY(cudaStreamSynchronize(st));
          if (sc->h_counters[0] == 0) break;
        }
      }
      // films in wave order (wavefronts may share pixels)
      if (concurrent && wi > 0) CUDA_TRY(cudaStreamWaitEvent(st, sc->film_ev[(wi - 1) & 1], 0));
      LaunchFilm(w, b, d_sum, d_sq, d_cnt, st);
      if (concurrent) CUDA_TRY(cudaEventRecord(sc->film_ev[wi & 1], st));
      ++launches;
      if (guide && !guide->direct_only) {
        LaunchGuideCollect(b, wc, std::min(bounces, guide->rec_bounces), w.n, guide_local, st);
        ++launches;
      }
    }
    if (concurrent) {  // the second stream's work ends before the frame does
      CUDA_TRY(cudaEventRecord(sc->join_ev, sc->stream2));
      CUDA_TRY(cudaStreamWaitEvent(main_st, sc->join_ev, 0));
    }
    timed_pairs = sc->events_used;
  };

  cudaEvent_t t0 = sc->NextEvent(2)->a;
  cudaEvent_t t1 = sc->events[0].b;
  char keybuf[640];
  int klen = std::snprintf(keybuf, sizeof(keybuf), "%d %d %d %d %d %d %d %d %d %d %llu %d %d %u %p %p %p %zu %d",
                           p.integrator, p.pixel_samples, p.light_samples, p.light_stratify, p.next_event_estimation,
                           p.russian_roulette, p.importance_sampling, p.min_depth, p.max_depth, p.sample_offset,
                           (unsigned long long)p.seed, p.intersect_mode, p.wave_paths, p.flags, (void *)d_sum,
                           (void *)d_sq, (void *)d_cnt, waves.size(), bounces);
  if (guide && klen > 0 && klen < static_cast<int>(sizeof(keybuf)))
    std::snprintf(keybuf + klen, sizeof(keybuf) - klen, " guide %p %p %p %p %d %d %.9g %.9g %.9g %.9g", guide->wt,
                  (void *)guide->mix, (void *)guide->rec, (void *)guide->pool, guide->rec_cap, guide->rec_bounces,
                  guide->alpha, guide->lo[0], guide->lo[1], guide->inv_ext[0]);
  const bool use_graph = bounded && !(p.flags & MUON_RENDER_NO_GRAPH) && !probe;
  if (moved) sc->DropGraph();
  CUDA_TRY(cudaEventRecord(t0, st));
  const bool graph_ready = use_graph && sc->graph && sc->graph_key == keybuf;
  if (graph_ready || (use_graph && sc->seen_key == keybuf)) {
    if (!graph_ready) {
      sc->DropGraph();
      cudaGraph_t g = nullptr;
      launches = 0;
      CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      try {
        capturing = true;
        enqueue(false);
        capturing = false;
      } catch (...) {
        cudaGraph_t dummy = nullptr;
        cudaStreamEndCapture(st, &dummy);
        if (dummy) cudaGraphDestroy(dummy);
        throw;
      }
      CUDA_TRY(cudaStreamEndCapture(st, &g));
      cudaError_t e = cudaGraphInstantiate(&sc->graph, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) throw CudaError{e, "cudaGraphInstantiate"};
      sc->graph_key = keybuf;
      sc->graph_events = timed_pairs;
      sc->graph_launches = launches;
    }
    CUDA_TRY(cudaGraphLaunch(sc->graph, st));
    launches = sc->graph_launches;
    timed_pairs = sc->graph_events;
  } else {
    enqueue(!bounded);
    if (use_graph) sc->seen_key = keybuf;
  }
  CUDA_TRY(cudaEventRecord(t1, st));
  CUDA_TRY(cudaGetLastError());
  unsigned long long hstats[kNumStats];
  CUDA_TRY(cudaMemcpyAsync(hstats, sc->stats.ptr, sizeof(hstats), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(sc->h_counters, sc->counters.ptr, stride * waves.size() * sizeof(uint32_t),
                           cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  uint64_t primary = 0, ext_rays = 0, shadow = 0, ext_launches = 0, occ_launches = 0;
  for (size_t wi = 0; wi < waves.size(); ++wi) {
    const uint32_t *c = sc->h_counters + wi * stride;
    if (traces) primary += static_cast<uint64_t>(waves[wi].n);
    WaveCounters hc{const_cast<uint32_t *>(c)};
    for (int k = 0; k < bounces; ++k) {
      ext_rays += *hc.count(k);
      shadow += *hc.shadow(k);
      if (*hc.count(k) > 0) {
        ++ext_launches;
        if (slots > 0) ++occ_launches;
      }
    }
  }
  MuonStats &o = sc->last;
  o = MuonStats{};
  o.primary_rays = primary;
  o.secondary_rays = hstats[kStatSecondary];
  o.shadow_rays = shadow;
  o.bounds_tests = hstats[kStatBoxTests] + hstats[kStatOccBoxTests];
  o.bounds_hits = hstats[kStatBoxHits] + hstats[kStatOccBoxHits];
  o.object_tests = hstats[kStatPrimTests] + hstats[kStatOccPrimTests];
  o.object_hits = hstats[kStatPrimHits] + hstats[kStatOccPrimHits];
  o.paths = static_cast<uint64_t>(npix_total) * spp;
  o.kernel_launches = launches;
  o.bvh_nodes = static_cast<uint64_t>(sc->img.nodes.size());
  o.primitives = static_cast<uint64_t>(sc->img.num_prims);
  o.extend_rays = ext_rays;
  o.extend_launches = ext_launches;
  o.extend_box_tests = hstats[kStatBoxTests];
  o.extend_prim_tests = hstats[kStatPrimTests];
  o.occlude_rays = shadow;
  o.occlude_launches = occ_launches;
  o.occlude_box_tests = hstats[kStatOccBoxTests];
  o.occlude_prim_tests = hstats[kStatOccPrimTests];
  float ms = 0.0f;
  CUDA_TRY(cudaEventElapsedTime(&ms, t0, t1));
  o.render_ms = ms;
  for (int i = 1; i < timed_pairs; ++i) {
    float e = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&e, sc->events[i].a, sc->events[i].b));
    if (sc->events[i].kind == 0) o.extend_ms += e;
    else if (sc->events[i].kind == 1) o.occlude_ms += e;
    else if (sc->events[i].kind == 2) o.shade_ms += e;
    else o.fold_ms += e;
  }
  if (hstats[kStatOverflow]) SetLastError("BVH traversal stack overflowed; results may miss hits");
}

}  // namespace

namespace muon_gpu {

// ---- device block cache (host_cuda.h) ----------------------------------------------
namespace {

struct PoolBlock {
  int device;
  void *ptr;
  size_t bytes;
};

std::mutex g_pool_mu;
std::vector<PoolBlock> g_pool;  // oldest first

size_t PoolCap(int device) {
  size_t free_b = 0, total_b = 0;
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != device) cudaSetDevice(device);
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) total_b = 0;
  if (cur != device) cudaSetDevice(cur);
  return total_b / 8;
}

}  // namespace

void PoolGive(DeviceBuffer &buf, int device) noexcept {
  if (!buf.ptr) return;
  std::vector<void *> evict;
  try {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    g_pool.push_back({device, buf.ptr, buf.bytes});
    size_t held = 0;
    for (const PoolBlock &b : g_pool)
      if (b.device == device) held += b.bytes;
    const size_t cap = PoolCap(device);
    for (size_t i = 0; i < g_pool.size() && held > cap;) {
      if (g_pool[i].device == device) {
        held -= g_pool[i].bytes;
        evict.push_back(g_pool[i].ptr);
        g_pool.erase(g_pool.begin() + static_cast<std::ptrdiff_t>(i));
      } else {
        ++i;
      }
    }
  } catch (...) {  // no room to remember the block: free it
    cudaFree(buf.ptr);
  }
  buf.ptr = nullptr;
  buf.bytes = 0;
  for (void *p : evict) cudaFree(p);
}

void PoolTrim(int device) noexcept {
  std::vector<void *> drop;
  {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    for (size_t i = 0; i < g_pool.size();) {
      if (device < 0 || g_pool[i].device == device) {
        drop.push_back(g_pool[i].ptr);
        g_pool.erase(g_pool.begin() + static_cast<std::ptrdiff_t>(i));
      } else {
        ++i;
      }
    }
  }
  for (void *p : drop) cudaFree(p);
}

void EnsurePooled(DeviceBuffer &buf, size_t want, int device) {
  if (want <= buf.bytes && buf.ptr) return;
  PoolGive(buf, device);
  if (want == 0) return;
  {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    size_t best = g_pool.size();
    for (size_t i = 0; i < g_pool.size(); ++i) {
      const PoolBlock &b = g_pool[i];
      if (b.device == device && b.bytes >= want && b.bytes <= want + want / 2 &&
          (best == g_pool.size() || b.bytes < g_pool[best].bytes))
        best = i;
    }
    if (best < g_pool.size()) {
      buf.ptr = g_pool[best].ptr;
      buf.bytes = g_pool[best].bytes;
      g_pool.erase(g_pool.begin() + static_cast<std::ptrdiff_t>(best));
      return;
    }
  }
  cudaError_t e = cudaMalloc(&buf.ptr, want);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    PoolTrim(-1);
    e = cudaMalloc(&buf.ptr, want);
  }
  if (e != cudaSuccess) {
    buf.ptr = nullptr;
    throw CudaError{e, "cudaMalloc"};
  }
  buf.bytes = want;
}

void RenderGuided(MuonScene *sc, const MuonRenderParams &p, double *d_sum, double *d_sq, uint32_t *d_cnt,
                  const GuideDev &g) {
  RenderDevice(sc, p, d_sum, d_sq, d_cnt, &g);
}

}  // namespace muon_gpu


extern "C" {

const char *muon_gpu_last_error(void) { return muon_gpu::LastError(); }

int muon_gpu_scene_create(const MuonSceneDesc *desc, MuonScene **out) {
  if (!desc || !out) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  *out = nullptr;
  std::unique_ptr<MuonScene> sc;
  try {
    sc.reset(new MuonScene());
    std::string err;
    if (desc->builder != MUON_BUILDER_HOST_SAH && desc->builder != MUON_BUILDER_GPU_LBVH &&
        desc->builder != MUON_BUILDER_GPU_SAH)
      return Fail(MUON_ERR_INVALID_ARG, "unknown BVH builder");
    if (desc->builder == MUON_BUILDER_GPU_SAH && desc->acceleration == MUON_ACCEL_BVH &&
        desc->partition_strategy != MUON_PARTITION_SAH)
      return Fail(MUON_ERR_INVALID_ARG, "the GPU SAH builder takes the SAH partition strategy only");
    const bool gpu_bvh = desc->builder != MUON_BUILDER_HOST_SAH && desc->acceleration == MUON_ACCEL_BVH;
    // with the device SAH build the triangles' records are computed on the device too
    const bool device_records = gpu_bvh && desc->builder == MUON_BUILDER_GPU_SAH;
    if (!BuildSceneImage(*desc, &sc->img, &err, gpu_bvh, device_records)) return Fail(MUON_ERR_INVALID_ARG, err);
    if (sc->img.bvh.max_depth >= 60) return Fail(MUON_ERR_INVALID_ARG, "BVH too deep for the traversal stack");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return Fail(MUON_ERR_CUDA, "no CUDA device available");
    CUDA_TRY(cudaGetDevice(&sc->device));
    {
      // muon_gpu_render_noalloc's buffer is taken now, not during its renders
      const cudaError_t e = NoAllocPrepare();
      if (e != cudaSuccess) {
        cudaGetLastError();
        return Fail(MUON_ERR_CUDA, std::string("no-allocation scratch set-up: ") + cudaGetErrorString(e));
      }
    }
    int sms = 0;
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sc->device));
    SetPersistentGrid(sms * 8);
    SetTraversalGrid(sms);
    CUDA_TRY(cudaStreamCreateWithFlags(&sc->stream, cudaStreamNonBlocking));
    cudaStream_t st = sc->stream;
    const SceneImage &im = sc->img;
    if (device_records || (gpu_bvh && !im.prims.empty())) {
      const int rc = BuildBvhOnGpu(sc.get(), desc->builder, desc->max_leaf_size > 0 ? desc->max_leaf_size : 4, st,
                                   device_records ? desc : nullptr);
      if (rc != MUON_OK) return rc;
      if (sc->img.bvh.max_depth >= 60) return Fail(MUON_ERR_INVALID_ARG, "BVH too deep for the traversal stack");
    } else {
      sc->num_slots = static_cast<int64_t>(im.prims.size());
      UploadPooled(sc->nodes, im.nodes, st, sc->device);
      UploadPooled(sc->prims, im.prims, st, sc->device);
      UploadPooled(sc->prims_obj, im.prims_obj, st, sc->device);
      UploadPooled(sc->shade, im.shade, st, sc->device);
      UploadPooled(sc->smooth, im.smooth_normals, st, sc->device);
      UploadPooled(sc->smooth_obj, im.smooth_normals_obj, st, sc->device);
    }
    Upload(sc->transforms, im.transforms, st);
    Upload(sc->materials, im.materials, st);
    Upload(sc->lights, im.lights, st);
    Upload(sc->other_lights, im.other_lights, st);
    Upload(sc->all_lights, im.all_lights, st);
    std::vector<PrimRecord> lt, lt_obj;
    std::vector<int32_t> lt_ok;
    BuildLightTris(im.lights, &lt, &lt_obj, &lt_ok);
    Upload(sc->light_tris, lt, st);
    Upload(sc->light_tris_obj, lt_obj, st);
    Upload(sc->light_tri_ok, lt_ok, st);
    DevScene &d = sc->dev;
    d.nodes = sc->nodes.as<BvhNode>();
    d.prims = sc->prims.as<PrimRecord>();
    d.prims_obj = sc->prims_obj.as<PrimRecord>();
    d.shade = sc->shade.as<ShadeRecord>();
    d.smooth_normals = im.any_smooth ? sc->smooth.as<F4>() : nullptr;
    d.smooth_normals_obj = im.any_smooth ? sc->smooth_obj.as<F4>() : nullptr;
    d.transforms = sc->transforms.as<DevTransform>();
    d.materials = sc->materials.as<DevMaterial>();
    d.lights = sc->lights.as<DevLight>();
    d.light_tris = sc->light_tris.as<PrimRecord>();
    d.light_tris_obj = sc->light_tris_obj.as<PrimRecord>();
    d.light_tri_ok = sc->light_tri_ok.as<int32_t>();
    d.other_lights = sc->other_lights.as<DevLight>();
    d.all_lights = sc->all_lights.as<DevLight>();
    d.num_nodes = static_cast<int32_t>(im.nodes.size());
    d.num_lights = static_cast<int32_t>(im.lights.size());
    d.num_other_lights = static_cast<int32_t>(im.other_lights.size());
    d.num_all_lights = static_cast<int32_t>(im.all_lights.size());
    ComputeCamera(im.camera, &sc->cam);
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  *out = sc.release();
  return MUON_OK;
}

void muon_gpu_scene_destroy(MuonScene *scene) { delete scene; }

void muon_gpu_release_cached(void) { PoolTrim(-1); }

int muon_gpu_render_device(MuonScene *scene, const MuonRenderParams *params, double *d_sum, double *d_sum_sq,
                           uint32_t *d_count) {
  if (!scene || !params || !d_sum || !d_sum_sq || !d_count) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  int rc = ValidateParams(*params);
  if (rc != MUON_OK) return rc;
  try {
    CUDA_TRY(cudaSetDevice(scene->device));
    if (!(params->flags & MUON_RENDER_ACCUMULATE)) {
      size_t np = static_cast<size_t>(scene->img.width) * scene->img.height;
      CUDA_TRY(cudaMemsetAsync(d_sum, 0, 3 * np * sizeof(double), scene->stream));
      CUDA_TRY(cudaMemsetAsync(d_sum_sq, 0, 3 * np * sizeof(double), scene->stream));
      CUDA_TRY(cudaMemsetAsync(d_count, 0, np * sizeof(uint32_t), scene->stream));
    }
    RenderDevice(scene, *params, d_sum, d_sum_sq, d_count);
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}

int muon_gpu_render(MuonScene *scene, const MuonRenderParams *params, MuonFilm *film) {
  if (!scene || !params || !film || !film->sum || !film->sum_sq || !film->count)
    return Fail(MUON_ERR_INVALID_ARG, "null argument");
  if (film->width != scene->img.width || film->height != scene->img.height)
    return Fail(MUON_ERR_INVALID_ARG, "film size does not match the scene");
  int rc = ValidateParams(*params);
  if (rc != MUON_OK) return rc;
  try {
    CUDA_TRY(cudaSetDevice(scene->device));
    const size_t np = static_cast<size_t>(film->width) * film->height;
    EnsurePooled(scene->film_sum, 3 * np * sizeof(double), scene->device);
    EnsurePooled(scene->film_sq, 3 * np * sizeof(double), scene->device);
    EnsurePooled(scene->film_cnt, np * sizeof(uint32_t), scene->device);
    cudaStream_t st = scene->stream;
    if (params->flags & MUON_RENDER_ACCUMULATE) {
      CUDA_TRY(cudaMemcpyAsync(scene->film_sum.ptr, film->sum, 3 * np * sizeof(double), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(scene->film_sq.ptr, film->sum_sq, 3 * np * sizeof(double), cudaMemcpyHostToDevice, st));
      CUDA_TRY(cudaMemcpyAsync(scene->film_cnt.ptr, film->count, np * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    } else {
      CUDA_TRY(cudaMemsetAsync(scene->film_sum.ptr, 0, 3 * np * sizeof(double), st));
      CUDA_TRY(cudaMemsetAsync(scene->film_sq.ptr, 0, 3 * np * sizeof(double), st));
      CUDA_TRY(cudaMemsetAsync(scene->film_cnt.ptr, 0, np * sizeof(uint32_t), st));
    }
    RenderDevice(scene, *params, scene->film_sum.as<double>(), scene->film_sq.as<double>(),
                 scene->film_cnt.as<uint32_t>());
    CUDA_TRY(cudaMemcpyAsync(film->sum, scene->film_sum.ptr, 3 * np * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(film->sum_sq, scene->film_sq.ptr, 3 * np * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(film->count, scene->film_cnt.ptr, np * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}

int muon_gpu_intersect(MuonScene *scene, const MuonRay *rays, int64_t n, int32_t intersect_mode, MuonHit *hits) {
  if (!scene || (n > 0 && (!rays || !hits)) || n < 0) return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  if (intersect_mode < MUON_ISECT_FAST || intersect_mode > MUON_ISECT_EXACT)
    return Fail(MUON_ERR_INVALID_ARG, "unknown intersect_mode");
  if (n == 0) return MUON_OK;
  static_assert(sizeof(MuonRay) == 24 && sizeof(MuonHit) == 32, "ray/hit layout");
  try {
    CUDA_TRY(cudaSetDevice(scene->device));
    cudaStream_t st = scene->stream;
    scene->ray_in.Ensure(n * sizeof(MuonRay));
    scene->ray_out.Ensure(n * sizeof(MuonHit));
    CUDA_TRY(cudaMemcpyAsync(scene->ray_in.ptr, rays, n * sizeof(MuonRay), cudaMemcpyHostToDevice, st));
    LaunchIntersectRays(scene->dev, scene->ray_in.as<float>(), n, intersect_mode, scene->ray_out.as<float>(), st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(hits, scene->ray_out.ptr, n * sizeof(MuonHit), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_occluded(MuonScene *scene, const MuonRay *rays, const float *max_distance, int64_t n,
                      int32_t intersect_mode, uint8_t *occluded) {
  if (!scene || (n > 0 && (!rays || !max_distance || !occluded)) || n < 0)
    return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  if (intersect_mode < MUON_ISECT_FAST || intersect_mode > MUON_ISECT_EXACT)
    return Fail(MUON_ERR_INVALID_ARG, "unknown intersect_mode");
  if (n == 0) return MUON_OK;
  try {
    CUDA_TRY(cudaSetDevice(scene->device));
    cudaStream_t st = scene->stream;
    scene->ray_in.Ensure(n * sizeof(MuonRay));
    scene->ray_aux.Ensure(n * sizeof(float));
    scene->ray_out.Ensure(n);
    CUDA_TRY(cudaMemcpyAsync(scene->ray_in.ptr, rays, n * sizeof(MuonRay), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(scene->ray_aux.ptr, max_distance, n * sizeof(float), cudaMemcpyHostToDevice, st));
    LaunchOccludedRays(scene->dev, scene->ray_in.as<float>(), scene->ray_aux.as<float>(), n, intersect_mode,
                       scene->ray_out.as<uint8_t>(), st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(occluded, scene->ray_out.ptr, n, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  return MUON_OK;
}

int muon_gpu_probe_traversal(MuonScene *scene, const MuonRenderParams *params, int32_t rays_per_queue,
                             MuonTraversalProbe *out) {
  if (!scene || !params || !out || rays_per_queue < 1) return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  int rc = ValidateParams(*params);
  if (rc != MUON_OK) return rc;
  if (params->integrator != MUON_INTEGRATOR_PATHTRACER || params->max_depth < 0)
    return Fail(MUON_ERR_INVALID_ARG, "traversal probes need the path tracer with a bounded depth");
  if (params->intersect_mode != MUON_ISECT_EXACT && params->intersect_mode != MUON_ISECT_FAST)
    return Fail(MUON_ERR_INVALID_ARG, "the host walk supports the exact and fast intersection modes");
  *out = MuonTraversalProbe{};
  try {
    CUDA_TRY(cudaSetDevice(scene->device));
    SyncSceneImage(scene);  // the host walk reads the scene's own leaf-order records
    const size_t np = static_cast<size_t>(scene->img.width) * scene->img.height;
    EnsurePooled(scene->film_sum, 3 * np * sizeof(double), scene->device);
    EnsurePooled(scene->film_sq, 3 * np * sizeof(double), scene->device);
    EnsurePooled(scene->film_cnt, np * sizeof(uint32_t), scene->device);
    cudaStream_t st = scene->stream;
    CUDA_TRY(cudaMemsetAsync(scene->film_sum.ptr, 0, 3 * np * sizeof(double), st));
    CUDA_TRY(cudaMemsetAsync(scene->film_sq.ptr, 0, 3 * np * sizeof(double), st));
    CUDA_TRY(cudaMemsetAsync(scene->film_cnt.ptr, 0, np * sizeof(uint32_t), st));
    MuonRenderParams p = *params;
    p.flags = (p.flags | MUON_RENDER_STATS | MUON_RENDER_NO_GRAPH) & ~MUON_RENDER_ACCUMULATE;
    QueueProbe probe;
    probe.m = rays_per_queue;
    RenderDevice(scene, p, scene->film_sum.as<double>(), scene->film_sq.as<double>(), scene->film_cnt.as<uint32_t>(),
                 nullptr, &probe);
    const size_t blocks = probe.waves * probe.bounces * 2;
    std::vector<float4> h(blocks * probe.BlockFloat4s());
    if (!h.empty())
      CUDA_TRY(cudaMemcpy(h.data(), probe.buf.ptr, h.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    std::vector<WalkRayIn> rays;
    for (size_t wi = 0; wi < probe.waves; ++wi) {
      for (int k = 0; k < probe.bounces; ++k) {
        for (int kind = 0; kind < 2; ++kind) {
          const float4 *blk = h.data() + probe.Offset(wi, k, kind);
          int32_t taken, n;
          std::memcpy(&taken, &blk[0].x, 4);
          std::memcpy(&n, &blk[0].y, 4);
          if (taken <= 0 || n <= 0) continue;
          rays.resize(static_cast<size_t>(taken));
          for (int i = 0; i < taken; ++i) {
            const float4 o = blk[1 + 2 * i], d = blk[2 + 2 * i];
            WalkRayIn &r = rays[i];
            r.o[0] = o.x, r.o[1] = o.y, r.o[2] = o.z;
            r.d[0] = d.x, r.d[1] = d.y, r.d[2] = d.z;
            r.tmax = d.w;
            std::memcpy(&r.root, &o.w, 4);
          }
          MuonWalkCounts c{0, 0, 0, 0};
          WalkMany(scene->img, rays.data(), taken, kind == 1, p.intersect_mode, nullptr, &c);
          const double scale = static_cast<double>(n) / taken;
          MuonWalkCounts &tot = kind == 0 ? out->extend_walked : out->occlude_walked;
          tot.rays += c.rays, tot.box_tests += c.box_tests, tot.prim_tests += c.prim_tests, tot.hits += c.hits;
          if (kind == 0) {
            out->extend_rays += static_cast<uint64_t>(n);
            out->extend_box_tests += scale * static_cast<double>(c.box_tests);
            out->extend_prim_tests += scale * static_cast<double>(c.prim_tests);
          } else {
            out->occlude_rays += static_cast<uint64_t>(n);
            out->occlude_box_tests += scale * static_cast<double>(c.box_tests);
            out->occlude_prim_tests += scale * static_cast<double>(c.prim_tests);
          }
        }
      }
    }
  } catch (const CudaError &e) {
    return FailCuda(e);
  } catch (const std::bad_alloc &) {
    return Fail(MUON_ERR_OOM, "host allocation failed");
  }
  return MUON_OK;
}

int muon_gpu_measure_read_bandwidth(int32_t level, int64_t bytes, int32_t passes, double *gb_per_s) {
  if (!gb_per_s || level < 0 || level > 2 || bytes < 4096 || passes < 1)
    return Fail(MUON_ERR_INVALID_ARG, "bad argument");
  if (level == 0 && bytes > (int64_t(64) << 10)) return Fail(MUON_ERR_INVALID_ARG, "level 0 reads at most 64 KiB");
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = MUON_OK;
  try {
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t n4 = bytes / 16;
    DeviceBuffer buf, sink;
    buf.Ensure(static_cast<size_t>(n4) * 16);
    sink.Ensure(16);
    CUDA_TRY(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreate(&e0));
    CUDA_TRY(cudaEventCreate(&e1));
    CUDA_TRY(cudaMemsetAsync(buf.ptr, 0, static_cast<size_t>(n4) * 16, st));
    // level 0: two blocks per SM, each reading the whole buffer; else eight
    // blocks per SM (full occupancy) reading it once between them
    const int blocks = level == 0 ? 2 * sms : 8 * sms;
    LaunchReadBandwidth(buf.as<float4>(), n4, 1, level, blocks, sink.as<float>(), st);  // warm
    CUDA_TRY(cudaEventRecord(e0, st));
    LaunchReadBandwidth(buf.as<float4>(), n4, passes, level, blocks, sink.as<float>(), st);
    CUDA_TRY(cudaEventRecord(e1, st));
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.0f;
    CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    const double delivered = static_cast<double>(n4) * 16.0 * passes * (level == 0 ? blocks : 1);
    *gb_per_s = delivered / (static_cast<double>(ms) * 1e6);
  } catch (const CudaError &e) {
    rc = FailCuda(e);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return rc;
}

int muon_gpu_stats(const MuonScene *scene, MuonStats *stats) {
  if (!scene || !stats) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  *stats = scene->last;
  return MUON_OK;
}

int muon_gpu_scene_stream(const MuonScene *scene, void **stream) {
  if (!scene || !stream) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  *stream = static_cast<void *>(scene->stream);
  return MUON_OK;
}

int muon_gpu_scene_bvh(const MuonScene *scene, MuonBvhInfo *info, void *nodes, int32_t *slot_prim,
                       uint8_t *slot_last) {
  if (!scene || !info) return Fail(MUON_ERR_INVALID_ARG, "null argument");
  try {
    SyncSceneImage(scene);
  } catch (const CudaError &e) {
    return FailCuda(e);
  }
  const SceneImage &im = scene->img;
  info->nodes = static_cast<int64_t>(im.nodes.size());
  info->slots = static_cast<int64_t>(im.shade.size());
  info->leaves = im.bvh.leaves;
  info->max_depth = im.bvh.max_depth;
  info->max_leaf = im.bvh.max_leaf;
  if (nodes && !im.nodes.empty()) std::memcpy(nodes, im.nodes.data(), sizeof(BvhNode) * im.nodes.size());
  for (size_t slot = 0; slot < im.shade.size(); ++slot) {
    if (slot_prim) slot_prim[slot] = im.shade[slot].s1.y;
    if (slot_last) {
      uint32_t flags;
      std::memcpy(&flags, &im.prims[slot].p3.w, 4);
      slot_last[slot] = (flags & kPrimLast) ? 1 : 0;
    }
  }
  return MUON_OK;
}

}  // extern "C"

namespace muon_gpu {

void SyncSceneImage(const MuonScene *scene) {
  if (!scene || !scene->host_records_stale) return;
  MuonScene *sc = const_cast<MuonScene *>(scene);  // img is a host cache of the device arrays
  SceneImage &im = sc->img;
  const size_t n = static_cast<size_t>(sc->num_slots);
  im.prims.resize(n);
  im.prims_obj.resize(n);
  im.shade.resize(n);
  if (im.any_smooth) im.smooth_normals.resize(3 * n), im.smooth_normals_obj.resize(3 * n);
  cudaStream_t st = sc->stream;
  CUDA_TRY(cudaSetDevice(sc->device));
  CUDA_TRY(cudaMemcpyAsync(im.prims.data(), sc->prims.ptr, sizeof(PrimRecord) * n, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(im.prims_obj.data(), sc->prims_obj.ptr, sizeof(PrimRecord) * n, cudaMemcpyDeviceToHost,
                           st));
  CUDA_TRY(cudaMemcpyAsync(im.shade.data(), sc->shade.ptr, sizeof(ShadeRecord) * n, cudaMemcpyDeviceToHost, st));
  if (im.any_smooth) {
    CUDA_TRY(cudaMemcpyAsync(im.smooth_normals.data(), sc->smooth.ptr, sizeof(F4) * 3 * n, cudaMemcpyDeviceToHost,
                             st));
    CUDA_TRY(cudaMemcpyAsync(im.smooth_normals_obj.data(), sc->smooth_obj.ptr, sizeof(F4) * 3 * n,
                             cudaMemcpyDeviceToHost, st));
  }
  CUDA_TRY(cudaStreamSynchronize(st));
  for (size_t slot = 0; slot < n; ++slot) im.leaf_of_prim_id[im.shade[slot].s1.y] = static_cast<int32_t>(slot);
  sc->host_records_stale = false;
}

bool GetSceneView(const MuonScene *scene, SceneView *out) {
  if (!scene || !out) return false;
  out->dev = &scene->dev;
  out->cam = &scene->cam;
  out->stream = scene->stream;
  out->device = scene->device;
  out->width = scene->img.width;
  out->height = scene->img.height;
  out->img = &scene->img;
  out->num_slots = scene->num_slots;
  return true;
}

}  // namespace muon_gpu
