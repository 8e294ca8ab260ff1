// Wavefront path-tracing kernels for sm_103a.
//
// One wavefront holds a batch of camera samples. Per bounce:
//   extend  closest-hit BVH traversal of the queued path rays
//   shade   emission, next-event estimation, MIS and continuation sampling
//           (PathTracer::Shade, muon/integration.cc:205-328); writes one
//           contribution per shadow slot and appends shadow rays and
//           continuation rays to compacted queues
//   occlude any-hit traversal of the shadow queue; zeroes blocked slots
// and at the end of the wave
//   film    folds each sample's radiance and surviving slots into the FP64
//           film (sum, sum of squares, count), pixel by pixel in sample order
//
// Queue compaction: each warp forms its offsets with a ballot/shuffle scan,
// the block scans the warp totals in shared memory and one thread per block
// reserves the block's range with a single atomicAdd.
#include <cuda_runtime.h>

#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <numeric>
#include <type_traits>

#include "dev_shade.cuh"
#include "dev_trace.cuh"
#include "kernels.cuh"
#include "guide.h"
#include "guide_mlp.cuh"
#include "guide_tc.cuh"
#include "host_cuda.h"

namespace muon_gpu {

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;

__device__ __forceinline__ void AddStat(unsigned long long *stats, int idx, unsigned long long v) {
  // one atomic per warp
  unsigned long long s = v;
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(stats + idx, s);
}

// Continuation rays of a shading block are queued grouped by direction
// octant (1: BlockReserveGrouped) or in thread order (0: BlockReserve).
#ifndef MUON_CONT_OCTANTS
#define MUON_CONT_OCTANTS 1
#endif

#if !MUON_CONT_OCTANTS
// Exclusive block-wide scan of a (count_a, count_b) pair; returns this
// thread's offsets into two global queues whose tails are reserved with one
// atomicAdd each per block. All threads of the block must call it.
__device__ __forceinline__ void BlockReserve(uint32_t a, uint32_t b, uint32_t *ctr_a, uint32_t *ctr_b, uint32_t *off_a,
                                             uint32_t *off_b) {
  __shared__ unsigned long long warp_tot[kWarps];
  __shared__ unsigned long long base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long v = (static_cast<unsigned long long>(a) << 32) | b;
  unsigned long long incl = v;
  for (int off = 1; off < 32; off <<= 1) {
    unsigned long long y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned long long t = lane < kWarps ? warp_tot[lane] : 0ull;
    unsigned long long ti = t;
    for (int off = 1; off < kWarps; off <<= 1) {
      unsigned long long y = __shfl_up_sync(0xffffffffu, ti, off);
      if (lane >= off) ti += y;
    }
    if (lane < kWarps) warp_tot[lane] = ti - t;  // exclusive
    if (lane == kWarps - 1) {
      uint32_t ta = static_cast<uint32_t>(ti >> 32), tb = static_cast<uint32_t>(ti & 0xffffffffu);
      uint32_t ba = ta ? atomicAdd(ctr_a, ta) : 0u;
      uint32_t bb = tb ? atomicAdd(ctr_b, tb) : 0u;
      base = (static_cast<unsigned long long>(ba) << 32) | bb;
    }
  }
  __syncthreads();
  unsigned long long excl = warp_tot[warp] + incl - v;
  *off_a = static_cast<uint32_t>(base >> 32) + static_cast<uint32_t>(excl >> 32);
  *off_b = static_cast<uint32_t>(base & 0xffffffffu) + static_cast<uint32_t>(excl & 0xffffffffu);
}

#else
// Like BlockReserve, with the block's `a` items laid out by group (0..7,
// each group in thread order; -1: no item) instead of in thread order.
constexpr int kReserveGroups = 8;
__device__ __forceinline__ void BlockReserveGrouped(int group, uint32_t nb, uint32_t *ctr_a, uint32_t *ctr_b,
                                                    uint32_t *off_a, uint32_t *off_b) {
  __shared__ uint32_t cnt[kWarps][kReserveGroups + 1];  // per warp: a per group, then b
  __shared__ uint32_t group_base[kReserveGroups];
  __shared__ uint32_t base_a, base_b;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  unsigned mine = 0;
  for (int g = 0; g < kReserveGroups; ++g) {
    const unsigned m = __ballot_sync(0xffffffffu, group == g);
    if (lane == 0) cnt[warp][g] = static_cast<uint32_t>(__popc(m));
    if (group == g) mine = m;
  }
  uint32_t incl = nb;
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  if (lane == 31) cnt[warp][kReserveGroups] = incl;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t ta = 0, tb = 0;
    for (int g = 0; g < kReserveGroups; ++g) {
      group_base[g] = ta;
      for (int w = 0; w < kWarps; ++w) ta += cnt[w][g];
    }
    for (int w = 0; w < kWarps; ++w) tb += cnt[w][kReserveGroups];
    base_a = ta ? atomicAdd(ctr_a, ta) : 0u;
    base_b = tb ? atomicAdd(ctr_b, tb) : 0u;
  }
  __syncthreads();
  uint32_t pa = 0, pb = base_b + incl - nb;
  if (group >= 0) {
    pa = base_a + group_base[group] + static_cast<uint32_t>(__popc(mine & below));
    for (int w = 0; w < warp; ++w) pa += cnt[w][group];
  }
  for (int w = 0; w < warp; ++w) pb += cnt[w][kReserveGroups];
  *off_a = pa;
  *off_b = pb;
  __syncthreads();  // cnt and the bases are written again by the next call
}
#endif

// Surface point, shading normal and material of a hit (Primitive::Intersect,
// muon/objects.cc:29-46, and the normals of Tri/Sphere::IntersectObjectSpace).
__device__ __forceinline__ void HitSurface(const DevScene &s, int slot, float3 o, float3 d, float t, float3 *p_out,
                                           float3 *n_out, int *mat_out, int *light_out, int *prim_id_out) {
  const float4 *q = reinterpret_cast<const float4 *>(s.shade + slot);
  float4 s0 = __ldg(q);
  int4 s1 = __ldg(reinterpret_cast<const int4 *>(q + 1));
  float3 p = o + d * t;
  float3 n;
  if (s1.w & kPrimSphere) {
    PrimRecord pr = LoadPrim(s.prims, slot);
    float3 c = f3(pr.p0);
    if (s1.z < 0) {
      n = normalize3(p - c);
    } else {
      const DevTransform &T = s.transforms[s1.z];
      float3 po = xform_point3(T.w2o, p);
      n = normalize3(xform_vec3(T.n2w, normalize3(po - c)));
    }
  } else if (s1.w & kPrimSmooth) {
    PrimRecord pr = LoadPrim(s.prims, slot);
    float3 a = f3(pr.p0), b = f3(pr.p1), c = f3(pr.p2), nn = f3(pr.p3);
    float inv = 1.0f / dot3(nn, nn);
    float v = dot3(nn, cross3(b - a, p - a)) * inv;
    float w = dot3(nn, cross3(c - b, p - b)) * inv;
    float u = dot3(nn, cross3(a - c, p - c)) * inv;
    const float4 *vn = reinterpret_cast<const float4 *>(s.smooth_normals) + 3 * slot;
    n = normalize3(w * f3(__ldg(vn)) + u * f3(__ldg(vn + 1)) + v * f3(__ldg(vn + 2)));
  } else {
    n = f3(s0.x, s0.y, s0.z);
  }
  *p_out = p;
  *n_out = n;
  *mat_out = __float_as_int(s0.w);
  *light_out = s1.x;
  *prim_id_out = s1.y;
}

// Exact counterpart of HitSurface: the hit rebuilt in the primitive's object
// space from the object-space ray parameter and carried back with the
// reference's transforms (muon/objects.cc:29-46, 160-174, 261-262).
__device__ __forceinline__ void HitSurfaceExact(const DevScene &s, int slot, float3 o, float3 d, float t_obj,
                                                float3 *p_out, float3 *n_out, float *dist_out, int *mat_out,
                                                int *light_out, int *prim_id_out) {
  using namespace mm;
  const float4 *q4 = reinterpret_cast<const float4 *>(s.shade + slot);
  float4 s0 = __ldg(q4);
  int4 s1 = __ldg(reinterpret_cast<const int4 *>(q4 + 1));
  PrimRecord pr = LoadPrim(s.prims_obj, slot);
  const uint32_t flags = __float_as_uint(pr.p3.w);
  const int xf = __float_as_int((flags & kPrimSphere) ? pr.p1.y : pr.p1.w);
  v3 oo, dd;
  if (xf < 0) {
    oo = V(o);
    dd = normalize(V(d));
  } else {
    oo = XPointExact(s.transforms[xf].w2o, V(o));
    dd = XDirExact(s.transforms[xf].w2o, V(d));
  }
  v3 q = oo + dd * t_obj;
  v3 n;
  if (flags & kPrimSphere) {
    n = normalize(q - V(pr.p0));
  } else if (flags & kPrimSmooth) {
    v3 a = V(pr.p0), b = V(pr.p1), c = V(pr.p2), fn = V(pr.p3);
    float len2 = pr.p2.w;
    float v = div(dot(fn, cross(b - a, q - a)), len2);
    float w = div(dot(fn, cross(c - b, q - b)), len2);
    float u = div(dot(fn, cross(a - c, q - c)), len2);
    const F4 *vn = s.smooth_normals_obj + 3 * slot;
    n = w * V(vn[0]) + u * V(vn[1]) + v * V(vn[2]);
  } else {
    n = normalize(V(pr.p3));
  }
  v3 pw = xf < 0 ? q : XPointExact(s.transforms[xf].o2w, q);
  v3 nw = xf < 0 ? normalize(n) : XDirExact(s.transforms[xf].n2w, n);
  *p_out = f3(pw.x, pw.y, pw.z);
  *n_out = f3(nw.x, nw.y, nw.z);
  *dist_out = length(pw - V(o));
  *mat_out = __float_as_int(s0.w);
  *light_out = s1.x;
  *prim_id_out = s1.y;
}

// Surface at a path vertex in the given intersection mode; `tv` is the value
// the extend kernel stored (world distance, or the object-space t in exact
// mode).
template <int kMode>
__device__ __forceinline__ void Surface(const DevScene &s, int slot, float3 o, float3 d, float tv, float3 *p,
                                        float3 *n, float *dist, int *mat, int *light, int *pid) {
  if (kMode == MUON_ISECT_EXACT) {
    HitSurfaceExact(s, slot, o, d, tv, p, n, dist, mat, light, pid);
  } else {
    HitSurface(s, slot, o, d, tv, p, n, mat, light, pid);
    *dist = tv;
  }
}

__device__ __forceinline__ Rng MakeRng(const WaveInfo &w, int path, uint32_t bounce) {
  int pixel = w.p0 + path / w.ns;
  uint32_t sample = w.sample_offset + static_cast<uint32_t>(w.s0 + path % w.ns);
  Rng r(w.seed, 0, bounce);
  r.ctr = make_uint4(sample, static_cast<uint32_t>(pixel), bounce, 0u);
  return r;
}


// Device-counted loops: `bound` (a host-known upper bound of the queue) sizes
// the grid, the true length is read on the device, and blocks stride over it.
#define QUEUE_LOOP(j, n)                                                                     \
  for (int j##_base = blockIdx.x * kBlock; j##_base < (n); j##_base += gridDim.x * kBlock)

// Double-buffered arrays are chosen with selects, not by indexing the
// parameter arrays with a runtime value (which would copy them to local
// memory).
template <class T>
__device__ __forceinline__ T *Pick(T *const (&a)[2], int i) {
  return i ? a[1] : a[0];
}

__device__ __forceinline__ int PathOf(float id) { return static_cast<int>(__float_as_uint(id) & kPathMask); }
__device__ __forceinline__ int SegOf(float id) { return static_cast<int>(__float_as_uint(id) >> kPathBits); }

// Index of the last segment whose `field` start is <= i (segments are in
// ascending order of both path0 and pix0).
template <int32_t BatchSeg::*kField>
__device__ __forceinline__ int FindSeg(const BatchSeg *segs, int nseg, int i) {
  int lo = 0, hi = nseg - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (__ldg(&(segs[mid].*kField)) <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ---- camera ------------------------------------------------------------
// Sampler::NextSample (muon/sampling.cc:80-121): sample 0 at the pixel centre,
// later samples jittered uniformly inside the pixel. Fills bounce 0's queue in
// path order and clears each path's final radiance.
__device__ __forceinline__ void CameraSample(const DevCamera &cam, int width, uint64_t seed, int pixel,
                                             uint32_t sample, float3 *o, float3 *d) {
  int px = pixel % width, py = pixel / width;
  float x, y;
  if (sample == 0) {
    x = mm::add(static_cast<float>(px), 0.5f);
    y = mm::add(static_cast<float>(py), 0.5f);
  } else {
    Rng rng(seed, 0, 0xffffffffu);
    rng.ctr = make_uint4(sample, static_cast<uint32_t>(pixel), 0xffffffffu, 0u);
    float u = rng.Next(), v = rng.Next();
    float fx = static_cast<float>(px), fy = static_cast<float>(py);
    x = mm::add(fx, u);
    y = mm::add(fy, v);
    if (x == mm::add(fx, 1.0f)) x = nextafterf(x, -INFINITY);
    if (y == mm::add(fy, 1.0f)) y = nextafterf(y, -INFINITY);
  }
  CastRay(cam, x, y, o, d);
}

// Writes bounce 0's queue entry i: the ray, its id word and its BVH root.
__device__ __forceinline__ void StartPath(const PathBuffers &b, int i, uint32_t id, int root, float3 o, float3 d) {
  b.ray_o[0][i] = make_float4(o.x, o.y, o.z, __uint_as_float(id));
  b.ray_d[0][i] = make_float4(d.x, d.y, d.z, __int_as_float(root));
  b.tp[0][i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
  b.rad[0][i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  b.final_rad[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(kBlock) CameraKernel(DevCamera cam, WaveInfo w, PathBuffers b, WaveCounters wc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *wc.count(0) = static_cast<uint32_t>(w.n);
  if (i >= w.n) return;
  int pixel = w.p0 + i / w.ns;
  uint32_t sample = w.sample_offset + static_cast<uint32_t>(w.s0 + i % w.ns);
  float3 o, d;
  CameraSample(cam, w.width, w.seed, pixel, sample, &o, &d);
  StartPath(b, i, static_cast<uint32_t>(i), 0, o, d);
}

__global__ void __launch_bounds__(kBlock) CameraBatchKernel(const BatchScene *scenes, const BatchSeg *segs, int nseg,
                                                            int paths, PathBuffers b, WaveCounters wc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) *wc.count(0) = static_cast<uint32_t>(paths);
  if (i >= paths) return;
  const int k = FindSeg<&BatchSeg::path0>(segs, nseg, i);
  const BatchSeg sg = segs[k];
  const BatchScene &sc = scenes[sg.scene];
  const int local = i - sg.path0;
  int pixel = sg.p0 + local / sg.ns;
  uint32_t sample = sc.sample_offset + static_cast<uint32_t>(sg.s0 + local % sg.ns);
  float3 o, d;
  CameraSample(sc.cam, sc.width, sc.seed, pixel, sample, &o, &d);
  StartPath(b, i, static_cast<uint32_t>(i) | (static_cast<uint32_t>(k) << kPathBits), sg.root, o, d);
}

// ---- extend / occlude ------------------------------------------------------
// Persistent traversal: each warp takes rays from a per-launch counter, 32 at
// a time, and a lane whose ray is done takes the next one as soon as fewer
// than kRefillThreshold lanes of its warp are still traversing, so warps stay
// full while the work per ray varies (dynamic fetch, after Aila and Laine,
// "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009).
#ifndef MUON_REFILL_THRESHOLD
#define MUON_REFILL_THRESHOLD 24
#endif
constexpr int kRefillThreshold = MUON_REFILL_THRESHOLD;
// Minimum resident blocks per SM the traversal kernels are compiled for.
#ifndef MUON_TRAVERSAL_MIN_BLOCKS
#define MUON_TRAVERSAL_MIN_BLOCKS 4
#endif

template <bool kAnyHit, bool kStats, int kMode, class Load, class Finish>
__device__ __forceinline__ void PersistentTraverse(const DevScene &s, int n, uint32_t *fetch, Load load,
                                                   Finish finish, TraceCounters &c, bool &overflow) {
  const int lane = threadIdx.x & 31;
  int ray = -1;
  bool exhausted = false;
  RayPre r;
  TravState t;
#if MUON_SHORT_STACK
  __shared__ int short_stack[kShortStack * kBlock];
  t.sh = short_stack + threadIdx.x;
  t.stride = kBlock;
#else
  t.sh = nullptr;
  t.stride = 0;
#endif
  while (true) {
    const unsigned need = __ballot_sync(0xffffffffu, ray < 0 && !exhausted);
    if (need) {
      const int leader = __ffs(need) - 1;
      uint32_t base = 0;
      if (lane == leader) base = atomicAdd(fetch, static_cast<uint32_t>(__popc(need)));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (ray < 0 && !exhausted) {
        const uint32_t mine = base + static_cast<uint32_t>(__popc(need & ((1u << lane) - 1u)));
        if (mine < static_cast<uint32_t>(n)) {
          ray = static_cast<int>(mine);
          float3 o, d;
          float tmax;
          int root;
          load(ray, &o, &d, &tmax, &root);
          r = Prepare<kMode>(o, d);
          TravBegin(t, tmax, root);
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, ray >= 0)) break;
    if (ray >= 0 && (MUON_SPECULATIVE ? TravRunSpeculative<kAnyHit, kStats, kMode>(s, r, t, &c, &overflow,
                                                                                    kRefillThreshold)
                                      : TravRun<kAnyHit, kStats, kMode>(s, r, t, &c, &overflow, kRefillThreshold))) {
      finish(ray, t);
      ray = -1;
    }
  }
}

// The extend kernel reads a hit's shading class from its primitive record (1)
// or its shading record (0).
#ifndef MUON_CLASS_FROM_PRIM
#define MUON_CLASS_FROM_PRIM 1
#endif
// Class lists of the shading kernel in queue order (1): the extend kernel
// leaves each hit's class in link[] and a stable partition (per-tile counts,
// a scan per class, a scatter) builds the lists, so that queue order, and the
// pixel locality the camera gave it, carries over from bounce to bounce; or
// in the order rays finish (0): the extend kernel appends each hit as its
// lane finishes.
#ifndef MUON_STABLE_CLASSES
#define MUON_STABLE_CLASSES 1
#endif

template <bool kStats, int kTri>
__global__ void __launch_bounds__(kBlock, MUON_TRAVERSAL_MIN_BLOCKS) ExtendKernel(DevScene s, PathBuffers b, WaveCounters wc, int bounce) {
  const int n = static_cast<int>(*wc.count(bounce));
  const float4 *__restrict__ ray_o = Pick(b.ray_o, bounce & 1);
  const float4 *__restrict__ ray_d = Pick(b.ray_d, bounce & 1);
  TraceCounters c;
  bool overflow = false;
  PersistentTraverse<false, kStats, kTri>(
      s, n, wc.fetch_extend(bounce),
      [&](int j, float3 *o, float3 *d, float *tmax, int *root) {
        float4 o4 = ray_o[j], d4 = ray_d[j];
        *o = f3(o4.x, o4.y, o4.z);
        *d = f3(d4.x, d4.y, d4.z);
        *tmax = INFINITY;
        *root = __float_as_int(d4.w);
      },
      [&](int j, const TravState &t) {
        b.hits[j] = make_int2(__float_as_int(kTri == MUON_ISECT_EXACT ? t.t_obj : t.tmax), t.hit);
        // Group hits by shading class for the shading kernel (one atomic per
        // class per group of lanes finishing together); a miss ends its path.
        int cls = kNumClasses;
#if MUON_CLASS_FROM_PRIM
        // the hit's record was just tested, so its flags are likely in L1
        if (t.hit >= 0)
          cls = (__float_as_uint(__ldg(&(kTri == MUON_ISECT_EXACT ? s.prims_obj : s.prims)[t.hit].p3.w)) >>
                 kClassShift) & 7;
#else
        if (t.hit >= 0) cls = (__ldg(&s.shade[t.hit].s1.w) >> kClassShift) & 7;
#endif
#if MUON_STABLE_CLASSES
        b.link[j] = cls < kNumClasses ? cls : -1;
#else
        const unsigned active = __activemask();
        const unsigned peers = __match_any_sync(active, cls);
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(peers) - 1;
        if (cls < kNumClasses) {
          uint32_t pos = 0;
          if (lane == leader) pos = atomicAdd(wc.classes(bounce) + cls, static_cast<uint32_t>(__popc(peers)));
          pos = __shfl_sync(peers, pos, leader) + static_cast<uint32_t>(__popc(peers & ((1u << lane) - 1u)));
          b.order[static_cast<int64_t>(cls) * b.order_cap + pos] = j;
        } else {
          b.link[j] = -1;
        }
#endif
      },
      c, overflow);
  if (kStats) {
    AddStat(b.stats, kStatBoxTests, c.box_tests);
    AddStat(b.stats, kStatBoxHits, c.box_hits);
    AddStat(b.stats, kStatPrimTests, c.prim_tests);
    AddStat(b.stats, kStatPrimHits, c.prim_hits);
  }
  if (overflow) atomicAdd(b.stats + kStatOverflow, 1ull);
}

// ---- stable class partition (MUON_STABLE_CLASSES) ---------------------------------
// Tile t holds queue entries [t * kClassTile, (t + 1) * kClassTile); its
// class counts, then their exclusive prefix over tiles, live in the ints
// after the class lists of b.order.
constexpr int kClassThreads = 256;
static_assert(kClassTile % kClassThreads == 0, "a tile is a whole number of block passes");

__device__ __forceinline__ int32_t *ClassTiles(const PathBuffers &b) {
  return b.order + static_cast<int64_t>(b.order_cap) * kNumClasses;
}

__global__ void __launch_bounds__(kClassThreads) ClassCountKernel(PathBuffers b, WaveCounters wc, int bounce) {
  const int n = static_cast<int>(*wc.count(bounce));
  const int base = blockIdx.x * kClassTile;
  if (base >= n) return;
  __shared__ int cnt[kNumClasses];
  if (threadIdx.x < kNumClasses) cnt[threadIdx.x] = 0;
  __syncthreads();
  for (int k = 0; k < kClassTile / kClassThreads; ++k) {
    const int j = base + k * kClassThreads + threadIdx.x;
    const int c = j < n ? b.link[j] : -1;
    if (c >= 0 && c < kNumClasses) atomicAdd(&cnt[c], 1);
  }
  __syncthreads();
  if (threadIdx.x < kNumClasses) ClassTiles(b)[blockIdx.x * 8 + threadIdx.x] = cnt[threadIdx.x];
}

// One block per class: the exclusive prefix of the class's tile counts, and
// the class total for the shading kernel.
__global__ void __launch_bounds__(1024) ClassScanKernel(PathBuffers b, WaveCounters wc, int bounce) {
  const int n = static_cast<int>(*wc.count(bounce));
  const int tiles = (n + kClassTile - 1) / kClassTile;
  const int c = blockIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t *t8 = ClassTiles(b);
  const int per = (tiles + 1023) / 1024;
  const int t0 = threadIdx.x * per, t1 = min(t0 + per, tiles);
  int sum = 0;
  for (int t = t0; t < t1; ++t) sum += t8[t * 8 + c];
  __shared__ int warp_sums[32];
  int x = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  if (w == 0) {
    const int v = warp_sums[lane];
    int y = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int z = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += z;
    }
    warp_sums[lane] = y - v;  // exclusive over warps
  }
  __syncthreads();
  int acc = warp_sums[w] + x - sum;
  for (int t = t0; t < t1; ++t) {
    const int v = t8[t * 8 + c];
    t8[t * 8 + c] = acc;
    acc += v;
  }
  if (threadIdx.x == 1023) wc.classes(bounce)[c] = static_cast<uint32_t>(acc);
}

// Each hit entry to its class list, in queue order.
__global__ void __launch_bounds__(kClassThreads) ClassScatterKernel(PathBuffers b, WaveCounters wc, int bounce) {
  const int n = static_cast<int>(*wc.count(bounce));
  const int base = blockIdx.x * kClassTile;
  if (base >= n) return;
  constexpr int kW = kClassThreads / 32;
  __shared__ int running[kNumClasses];
  __shared__ int warp_cnt[kW][kNumClasses];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (threadIdx.x < kNumClasses) running[threadIdx.x] = ClassTiles(b)[blockIdx.x * 8 + threadIdx.x];
  for (int k = 0; k < kClassTile / kClassThreads; ++k) {
    const int j = base + k * kClassThreads + threadIdx.x;
    int c = j < n ? b.link[j] : -1;
    if (c >= kNumClasses) c = -1;
    unsigned mine = 0;
    for (int q = 0; q < kNumClasses; ++q) {
      const unsigned m = __ballot_sync(0xffffffffu, c == q);
      if (lane == 0) warp_cnt[w][q] = __popc(m);
      if (c == q) mine = m;
    }
    __syncthreads();
    if (c >= 0) {
      int pos = running[c] + __popc(mine & ((1u << lane) - 1u));
      for (int v = 0; v < w; ++v) pos += warp_cnt[v][c];
      if (pos < b.order_cap) b.order[static_cast<int64_t>(c) * b.order_cap + pos] = j;
    }
    __syncthreads();
    if (threadIdx.x < kNumClasses) {
      int tot = 0;
      for (int v = 0; v < kW; ++v) tot += warp_cnt[v][threadIdx.x];
      running[threadIdx.x] += tot;
    }
    __syncthreads();
  }
}

// Shadow queue entries are slot indices (entry * S + slot). A blocked slot's
// contribution is zeroed.
template <bool kStats, int kTri>
__global__ void __launch_bounds__(kBlock, MUON_TRAVERSAL_MIN_BLOCKS) OccludeKernel(DevScene s, PathBuffers b, WaveCounters wc, int bounce,
                                                        int slots) {
  const int n = static_cast<int>(*wc.shadow(bounce));
  TraceCounters c;
  bool overflow = false;
  PersistentTraverse<true, kStats, kTri>(
      s, n, wc.fetch_occlude(bounce),
      [&](int j, float3 *o, float3 *d, float *tmax, int *root) {
        uint32_t slot = b.shq[j];
        float4 o4 = b.org[slot / slots], d4 = b.slot_dir[slot];
        *o = f3(o4.x, o4.y, o4.z);
        *d = f3(d4.x, d4.y, d4.z);
        *tmax = d4.w;
        *root = __float_as_int(o4.w);
      },
      [&](int j, const TravState &t) {
        if (t.hit >= 0) b.contrib[b.shq[j]] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      },
      c, overflow);
  if (kStats) {
    AddStat(b.stats, kStatOccBoxTests, c.box_tests);
    AddStat(b.stats, kStatOccBoxHits, c.box_hits);
    AddStat(b.stats, kStatOccPrimTests, c.prim_tests);
    AddStat(b.stats, kStatOccPrimHits, c.prim_hits);
  }
  if (overflow) atomicAdd(b.stats + kStatOverflow, 1ull);
}

// ---- deterministic integrators --------------------------------------------
// NormalsTracer / AlbedoTracer / DepthTracer (muon/integration.cc:47-72).
template <int kMode>
__global__ void __launch_bounds__(kBlock) ShadeDebugKernel(DevScene s, PathBuffers b, WaveCounters wc,
                                                           int integrator) {
  const int n = static_cast<int>(*wc.count(0));
  for (int j = blockIdx.x * kBlock + threadIdx.x; j < n; j += gridDim.x * kBlock) {
    float4 o4 = b.ray_o[0][j], d4 = b.ray_d[0][j];
    int path = PathOf(o4.w);
    int2 h = b.hits[j];
    float4 out = make_float4(0, 0, 0, 0);
    if (h.y >= 0) {
      float3 p, nrm;
      float dist;
      int mat, light, pid;
      Surface<kMode>(s, h.y, f3(o4.x, o4.y, o4.z), f3(d4.x, d4.y, d4.z), __int_as_float(h.x), &p, &nrm, &dist, &mat,
                     &light, &pid);
      using mm::add;
      using mm::mul;
      if (integrator == MUON_INTEGRATOR_NORMALS) {
        out = make_float4(add(mul(nrm.x, 0.5f), 0.5f), add(mul(nrm.y, 0.5f), 0.5f), add(mul(nrm.z, 0.5f), 0.5f),
                          0.0f);
      } else if (integrator == MUON_INTEGRATOR_ALBEDO) {
        Mat m = LoadMat(s.materials, mat);
        out = make_float4(add(m.kd.x, m.ks.x), add(m.kd.y, m.ks.y), add(m.kd.z, m.ks.z), 0.0f);
      } else {
        float v = mm::div(1.0f, add(1.0f, dist));
        out = make_float4(v, v, v, 0.0f);
      }
    }
    b.final_rad[path] = out;
  }
}

// ---- ray tracer and analytic direct lighting ---------------------------------
// Raytracer::Shade (muon/integration.cc:74-124) and AnalyticDirect::Shade
// (muon/integration.cc:126-199), one thread per path. The ray tracer's
// recursion color_k = local_k + ks_k * color_(k+1) is evaluated from the
// deepest level back, in the reference's order, for the first kExactLevels
// levels; deeper levels (max_depth above 7) are summed forward into the
// value that stands for level kExactLevels.
constexpr int kExactLevels = 8;

// glm::max / std::max: (a < b) ? b : a (keeps a NaN in a).
__device__ __forceinline__ float GlmMax(float a, float b) { return a < b ? b : a; }

struct LightInfo {
  mm::v3 color, dir;
  float dist;
  bool area;
};

// Light::ShadingInfoAt (muon/lighting.cc:38-72): a quad light reports no
// direction and distance 0.
__device__ __forceinline__ LightInfo ShadingInfoAt(const DevLight &l, mm::v3 p) {
  using namespace mm;
  LightInfo r;
  const int type = __float_as_int(l.corner.w);
  r.color = V(l.color);
  r.area = false;
  if (type == MUON_LIGHT_DIRECTIONAL) {
    r.dir = V(l.corner);
    r.dist = INFINITY;
  } else if (type == MUON_LIGHT_POINT) {
    v3 ptl = V(l.corner) - p;
    r.dir = normalize(ptl);
    float d = length(ptl);
    float att = add(add(l.edge0.x, mul(l.edge0.y, d)), mul(mul(l.edge0.z, d), d));
    r.color = r.color / att;
    r.dist = d;
  } else {
    r.dir = make3(0.0f, 0.0f, 0.0f);
    r.dist = 0.0f;
    r.area = true;
  }
  return r;
}

template <bool kStats, int kMode>
__global__ void __launch_bounds__(kBlock) WhittedKernel(DevScene s, PathBuffers b, WaveInfo w, int integrator,
                                                        int max_trace_depth) {
  using namespace mm;
  const int i = blockIdx.x * kBlock + threadIdx.x;
  TraceCounters ce, co;
  bool overflow = false;
  uint32_t secondary = 0;
  if (i < w.n) {
    float4 o4 = b.ray_o[0][i], d4 = b.ray_d[0][i];
    float3 o = f3(o4.x, o4.y, o4.z), d = f3(d4.x, d4.y, d4.z);
    v3 local[kExactLevels], ks[kExactLevels];
    v3 tail = splat3(0.0f), tail_tp = splat3(1.0f);
    int levels = 0;
    for (int depth = 0; depth <= max_trace_depth; ++depth) {
      if (depth > 0) ++secondary;
      float t, t_obj = 0.0f;
      const int h = Trace<false, kStats, kMode>(s, o, d, INFINITY, &t, &ce, &overflow, &t_obj);
      if (h < 0) break;
      float3 p3, n3;
      float dist;
      int mat, light, pid;
      Surface<kMode>(s, h, o, d, kMode == MUON_ISECT_EXACT ? t_obj : t, &p3, &n3, &dist, &mat, &light, &pid);
      const v3 p = V(p3), n = V(n3), rd = V(d);
      const float4 *mq = reinterpret_cast<const float4 *>(s.materials + mat);
      const float4 kd4 = __ldg(mq), ks4 = __ldg(mq + 1), ke4 = __ldg(mq + 2), ka4 = __ldg(mq + 3);
      const v3 kd = make3(kd4.x, kd4.y, kd4.z), kspec = make3(ks4.x, ks4.y, ks4.z);
      const v3 ke = make3(ke4.x, ke4.y, ke4.z), ka = make3(ka4.x, ka4.y, ka4.z);
      v3 color;
      bool cont = false;
      if (integrator == MUON_INTEGRATOR_ANALYTIC_DIRECT) {
        color = ke;
        for (int li = 0; li < s.num_all_lights; ++li) {
          const DevLight l = s.all_lights[li];
          LightInfo info = ShadingInfoAt(l, p);
          if (!info.area) continue;
          v3 vtx[4];
          vtx[0] = V(l.corner);
          vtx[1] = V(l.corner) + V(l.edge0);
          vtx[2] = vtx[1] + V(l.edge1);
          vtx[3] = V(l.corner) + V(l.edge1);
          const v3 brdf = kd * 0.318309886183790671537767526745028724f;
          v3 irr = splat3(0.0f);
          for (int k = 0; k < 4; ++k) {
            v3 ui = normalize(vtx[k] - p), un = normalize(vtx[(k + 1) & 3] - p);
            float theta = acosf(dot(ui, un));
            irr = irr + theta * normalize(cross(ui, un));
          }
          irr = irr * 0.5f;
          color = color + (brdf * info.color) * dot(irr, n);
        }
      } else {
        color = ka + ke;
        const v3 shift = p + kEps * n;
        for (int li = 0; li < s.num_all_lights; ++li) {
          const DevLight l = s.all_lights[li];
          LightInfo info = ShadingInfoAt(l, p);
          // A quad light's zero-length shadow ray can hit nothing.
          if (!info.area) {
            float ts;
            const float3 dir = f3(info.dir.x, info.dir.y, info.dir.z);
            if (Trace<true, kStats, kMode>(s, f3(shift.x, shift.y, shift.z), dir, info.dist, &ts, &co, &overflow) >= 0)
              continue;
          }
          v3 dc = kd * GlmMax(dot(n, info.dir), 0.0f);
          v3 half = normalize(info.dir - rd);
          // pow in double rounded to float: the correctly rounded value,
          // which the host libm's powf also returns on all but rare inputs.
          v3 sc = kspec * static_cast<float>(pow(static_cast<double>(GlmMax(dot(n, half), 0.0f)),
                                                 static_cast<double>(kd4.w)));
          color = color + info.color * (dc + sc);
        }
        if (kspec.x > 0.0f || kspec.y > 0.0f || kspec.z > 0.0f) {
          cont = true;
          const v3 r = reflect(rd, n);
          o = f3(shift.x, shift.y, shift.z);
          d = f3(r.x, r.y, r.z);
        }
      }
      if (levels < kExactLevels) {
        local[levels] = color;
        ks[levels] = kspec;
        ++levels;
      } else {
        tail = tail + tail_tp * color;
        tail_tp = tail_tp * kspec;
      }
      if (!cont) break;
    }
    v3 c = tail;
    for (int k = levels - 1; k >= 0; --k) c = local[k] + ks[k] * c;
    b.final_rad[i] = make_float4(c.x, c.y, c.z, 0.0f);
  }
  AddStat(b.stats, kStatSecondary, secondary);
  if (kStats) {
    AddStat(b.stats, kStatBoxTests, ce.box_tests);
    AddStat(b.stats, kStatBoxHits, ce.box_hits);
    AddStat(b.stats, kStatPrimTests, ce.prim_tests);
    AddStat(b.stats, kStatPrimHits, ce.prim_hits);
    AddStat(b.stats, kStatOccBoxTests, co.box_tests);
    AddStat(b.stats, kStatOccBoxHits, co.box_hits);
    AddStat(b.stats, kStatOccPrimTests, co.prim_tests);
    AddStat(b.stats, kStatOccPrimHits, co.prim_hits);
  }
  if (overflow) atomicAdd(b.stats + kStatOverflow, 1ull);
}

// ---- path tracer shading ----------------------------------------------------
// PathTracer::Shade for every queued path vertex at depth `bounce`
// (muon/integration.cc:205-328). Each shadow slot receives the radiance it
// adds if its shadow ray turns out unblocked; the shadow rays go to the
// compacted shadow queue as slot indices, continuing paths to the next
// bounce's queue (with their throughput and a link from this entry).
constexpr int kMaskSlots = 64;
// Minimum resident blocks per SM the shading kernel is compiled for (sets its
// register budget: 2 -> up to 128 registers, 3 -> 80).
#ifndef MUON_SHADE_MIN_BLOCKS
#define MUON_SHADE_MIN_BLOCKS 2
#endif
// Shade hits grouped by shading class (1, through the extend kernel's class
// lists) or in queue order (0; measured 1.8x slower shading on the sphere
// field: warps mix materials).
#ifndef MUON_SHADE_SORTED
#define MUON_SHADE_SORTED 1
#endif


// ---- guided sampling ----------------------------------------------------------------
// Direction sampling of a guided render: with probability alpha from the
// learned mixture of the vertex, else from the render's own sampler
// (hemisphere, cosine or BRDF); the sample is weighted by the density of the
// combination (one-sample MIS, balance heuristic), so the estimator stays
// unbiased whatever the network predicts. Light-sample MIS weights use the
// same combined density.
__device__ __forceinline__ float GuidedPdf(const GuideDev *g, const float *mx, float base_pdf, float3 w) {
  return g->alpha * guide::MixturePdf(mx, w.x, w.y, w.z) + (1.0f - g->alpha) * base_pdf;
}

__device__ __forceinline__ bool SampleGuided(const GuideDev *g, const float *mx, int mode, const Mat &m, float3 n,
                                             float3 ray_dir, float3 tp, Rng &rng, float3 *dir, float *pdf,
                                             float3 *next_tp) {
  float3 w;
  if (rng.Next() < g->alpha) {
    const float u0 = rng.Next(), u1 = rng.Next(), u2 = rng.Next();
    guide::SampleMixture(mx, u0, u1, u2, &w.x, &w.y, &w.z);
  } else if (mode == MUON_IS_HEMISPHERE) {
    w = SampleHemisphere(n, rng);
  } else if (mode == MUON_IS_COSINE) {
    w = SampleCosine(n, rng);
  } else {
    w = BrdfSample(m, ray_dir, n, rng);
  }
  const float cosn = dot3(w, n);
  if (cosn <= 0.0f) return false;
  const float p = GuidedPdf(g, mx, IsPdf(mode, m, w, ray_dir, n), w);
  if (!(p > 0.0f)) return false;
  *next_tp = tp * BrdfEval(m, w, ray_dir, n) * (cosn / p);
  *dir = w;
  *pdf = p;
  return true;
}

// Shading of one queued hit (PathTracer::Shade); `local` is the path's index
// in its wave (or batch segment), which seeds its random numbers.
struct ShadeOut {
  uint32_t want_cont = 0, nshadow = 0;
  unsigned long long mask = 0;  // nonzero slots (first 64)
  float3 cont_o, cont_d, cont_tp;
};

template <int kMode>
__device__ __forceinline__ void ShadeEntry(const DevScene &s, const WaveInfo &w, const ShadeParams &sp,
                                           const PathBuffers &b, int cur, int bounce, int S, int jj, float4 o4,
                                           float4 d4, int local, unsigned long long &counted, ShadeOut &out,
                                           const GuideDev *gd) {
    // the vertex's learned mixture when guided
    const float *mx = gd ? reinterpret_cast<const float *>(gd->mix + guide::kMixVec * static_cast<int64_t>(jj)) : nullptr;
    const float3 o = f3(o4.x, o4.y, o4.z), d = f3(d4.x, d4.y, d4.z);
    const int2 h = b.hits[jj];
    float4 *contrib = b.contrib + static_cast<int64_t>(jj) * S;
    float4 *sdir = b.slot_dir + static_cast<int64_t>(jj) * S;
    for (int k = 0; k < S; ++k) contrib[k] = make_float4(0, 0, 0, 0);
    float3 L = f3(Pick(b.rad, cur)[jj]);
    const float3 tp = f3(Pick(b.tp, cur)[jj]);

    if (h.y >= 0) {
      float3 p, nrm;
      float hit_dist;
      int mat_id, light_id, pid;
      Surface<kMode>(s, h.y, o, d, __int_as_float(h.x), &p, &nrm, &hit_dist, &mat_id, &light_id, &pid);
      const Mat m = LoadMat(s.materials, mat_id);
      const float3 shift = p + kEps * nrm;
      Rng rng = MakeRng(w, local, static_cast<uint32_t>(bounce));
      const bool direct = bounce >= sp.min_depth;
      const bool mis = direct && sp.nee == MUON_NEE_MIS;

      if (direct) {
        // Emission: only at the first vertex when lights are sampled, and
        // only from the front face (muon/integration.cc:257-264).
        if ((sp.nee == MUON_NEE_OFF || bounce == 0) && !(dot3(nrm, -d) < 0.0f)) L = L + tp * m.ke;
        if (sp.nee != MUON_NEE_OFF) {
          int slot = 0;
          // Area lights: ShadeDirectNEE (muon/integration.cc:371-462).
#pragma unroll 1
          for (int li = 0; li < s.num_lights; ++li) {
            const DevLight &l = s.lights[li];
            const float3 corner = f3(l.corner), e0 = f3(l.edge0), e1 = f3(l.edge1), rev = f3(l.rev_normal);
            const float3 lcol = f3(l.color) * (l.color.w / static_cast<float>(sp.light_samples));
            const float inv_strata = 1.0f / static_cast<float>(sp.strata);
#pragma unroll 1
            for (int q = 0; q < sp.per_light; ++q, ++slot) {
              const int si = (q / sp.per_section) / sp.strata, sj = (q / sp.per_section) % sp.strata;
              float u = rng.Next(), v = rng.Next();
              float fu = (static_cast<float>(si) + u) * inv_strata;
              float fv = (static_cast<float>(sj) + v) * inv_strata;
              float3 ptl = corner + fu * e0 + fv * e1 - kEps * rev - shift;
              float dist = sqrtf(dot3(ptl, ptl));
              float3 ldir = ptl * (1.0f / dist);
              float ci = fmaxf(dot3(nrm, ldir), 0.0f);
              float cl = fmaxf(dot3(rev, ldir), 0.0f);
              if (ci == 0.0f || cl == 0.0f) continue;
              float3 c = BrdfEval(m, ldir, d, nrm) * (ci * cl / (dist * dist));
              if (mis) {
                float bp = IsPdf(sp.is_mode, m, ldir, d, nrm);
                if (gd) bp = GuidedPdf(gd, mx, bp, ldir);
                c = c * PowerHeuristic(NeePdf(s, shift, ldir), bp);
              }
              c = tp * lcol * c;
              if (!nonzero3(c)) continue;
              contrib[slot] = make_float4(c.x, c.y, c.z, 0.0f);
              sdir[slot] = make_float4(ldir.x, ldir.y, ldir.z, dist);
              ++out.nshadow;
              if (slot < kMaskSlots) out.mask |= 1ull << slot;
            }
          }
          // Point and directional lights (muon/integration.cc:350-369,
          // muon/lighting.cc:38-64).
#pragma unroll 1
          for (int li = 0; li < s.num_other_lights; ++li, ++slot) {
            const DevLight &l = s.other_lights[li];
            float3 lcol = f3(l.color);
            float3 ldir;
            float dist;
            if (__float_as_int(l.corner.w) == MUON_LIGHT_POINT) {
              float3 ptl = f3(l.corner) - p;
              ldir = normalize3(ptl);
              dist = length3(ptl);
              float att = l.edge0.x + l.edge0.y * dist + l.edge0.z * dist * dist;
              lcol = lcol / att;
              lcol = lcol / (dist * dist);
            } else {
              ldir = f3(l.corner);
              dist = INFINITY;
            }
            float ci = fmaxf(dot3(nrm, ldir), 0.0f);
            float3 c = tp * lcol * BrdfEval(m, ldir, d, nrm) * ci;
            if (!nonzero3(c)) continue;
            contrib[slot] = make_float4(c.x, c.y, c.z, 0.0f);
            sdir[slot] = make_float4(ldir.x, ldir.y, ldir.z, dist);
            ++out.nshadow;
            if (slot < kMaskSlots) out.mask |= 1ull << slot;
          }
        }
      }
      // Two BRDF samples share one code path: first the MIS light-hit ray
      // (ShadeDirectImportanceSampling, muon/integration.cc:468-501), then
      // the continuation (ShadeIndirect, muon/integration.cc:294-328).
#pragma unroll 1
      for (int pass = mis ? 0 : 1; pass < 2; ++pass) {
        float3 dir, ntp;
        float pdf;
        const bool guided = gd && (pass == 0 || !gd->direct_only);
        if (!(guided ? SampleGuided(gd, mx, sp.is_mode, m, nrm, d, tp, rng, &dir, &pdf, &ntp)
                     : SampleReflection(sp.is_mode, m, nrm, d, tp, rng, &dir, &pdf, &ntp)))
          continue;
        if (pass == 0) {
          ++counted;
          // The sampled ray's closest hit is a light triangle exactly when
          // some light triangle is hit at t_L and nothing is hit before
          // t_L: an any-hit query up to t_L, none if no light is met. Same
          // triangle test and ray preparation as the traversal, so t_L is
          // bit-identical to what the query compares against.
          float best = INFINITY;
          int best_light = -1;
          RayPre rp = Prepare<kMode>(shift, dir);
          const PrimRecord *lts = kMode == MUON_ISECT_EXACT ? s.light_tris_obj : s.light_tris;
#pragma unroll 1
          for (int lt = 0; lt < 2 * s.num_lights; ++lt) {
            if (!s.light_tri_ok[lt]) continue;
            PrimRecord lp = LoadPrim(lts, lt);
            float t_obj;
            float t = PrimTest<kMode>(s, rp, lp, __float_as_uint(lp.p3.w), &t_obj);
            if (t > 0.0f && t < best) best = t, best_light = lt >> 1;
          }
          if (best_light < 0) continue;
          float3 c = ntp * f3(s.lights[best_light].color) * PowerHeuristic(pdf, NeePdf(s, shift, dir));
          if (!nonzero3(c)) continue;
          const int slot = sp.mis_slot;
          contrib[slot] = make_float4(c.x, c.y, c.z, 0.0f);
          sdir[slot] = make_float4(dir.x, dir.y, dir.z, best);
          ++out.nshadow;
          if (slot < kMaskSlots) out.mask |= 1ull << slot;
        } else {
          bool survive = true;
          if (sp.rr) {
            float q = fminf(max3c(ntp), 1.0f);
            if (q < rng.Next()) survive = false;
            else ntp = ntp / q;
          }
          const int next_depth = bounce + 1;
          const bool depth_ok = sp.max_trace_depth < 0 || next_depth <= sp.max_trace_depth;
          if (survive && depth_ok && next_depth < sp.max_bounces) {
            out.want_cont = 1;
            ++counted;
            out.cont_o = shift;
            out.cont_d = dir;
            out.cont_tp = ntp;
            if (gd && !gd->direct_only && bounce < gd->rec_bounces) {
              // training record; the fold adds the radiance after this vertex
              GuideRec &r = gd->rec[static_cast<int64_t>(bounce) * gd->rec_cap + jj];
              r.f0 = gd->feat[2 * static_cast<int64_t>(jj)];
              r.f1 = gd->feat[2 * static_cast<int64_t>(jj) + 1];
              r.dir = make_float4(dir.x, dir.y, dir.z, o4.w);
              r.tp = make_float4(tp.x, tp.y, tp.z, 1.0f);
            }
          }
        }
      }
      if (out.nshadow) b.org[jj] = make_float4(shift.x, shift.y, shift.z, d4.w);  // w: BVH root
    }
    Pick(b.rad, cur)[jj] = make_float4(L.x, L.y, L.z, 0.0f);
}

template <int kMode, bool kBatch, bool kGuide>
__global__ void __launch_bounds__(kBlock, MUON_SHADE_MIN_BLOCKS)
    ShadePathKernel(DevScene s, WaveInfo w, ShadeParams sp, PathBuffers b, WaveCounters wc, int bounce,
                    const BatchScene *bscenes, const BatchSeg *segs, int slot_stride, GuideDev gdev) {
  // Hits of this bounce, grouped by shading class: position i of the
  // concatenated class lists is entry order[c * cap + (i - start[c])].
  __shared__ uint32_t class_start[kNumClasses + 1];
  if (threadIdx.x == 0) {
    uint32_t acc = 0;
    for (int c = 0; c < kNumClasses; ++c) {
      class_start[c] = acc;
      acc += wc.classes(bounce)[c];
    }
    class_start[kNumClasses] = acc;
  }
  __syncthreads();
  const int cur = bounce & 1, nxt = cur ^ 1;
  const int S = slot_stride;
  unsigned long long counted = 0;  // secondary rays in the reference's sense
#if MUON_SHADE_SORTED
  const int n = static_cast<int>(class_start[kNumClasses]);
#else
  const int n = static_cast<int>(*wc.count(bounce));
#endif
  QUEUE_LOOP(j, n) {
    const int ii = j_base + threadIdx.x;
#if MUON_SHADE_SORTED
    const bool active = ii < n;
    int jj = 0;
    if (active) {
      int c = 0;
      while (c + 1 < kNumClasses && static_cast<uint32_t>(ii) >= class_start[c + 1]) ++c;
      jj = b.order[static_cast<int64_t>(c) * b.order_cap + (ii - static_cast<int>(class_start[c]))];
    }
#else
    // queue order: coalesced per-entry reads, materials mixed in a warp
    const int jj = ii;
    const bool active = ii < n && b.hits[ii].y >= 0;
#endif
    ShadeOut so;
    float id = 0.0f, root = 0.0f;
    if (active) {
      const float4 o4 = Pick(b.ray_o, cur)[jj], d4 = Pick(b.ray_d, cur)[jj];
      id = o4.w;
      root = d4.w;
      if (kBatch) {
        // This path's scene: its lights, settings and sample numbering.
        const BatchSeg &sg = segs[SegOf(o4.w)];
        const BatchScene &bs = bscenes[sg.scene];
        DevScene sv = s;
        sv.lights = s.lights + bs.light_off;
        sv.light_tris = s.light_tris + 2 * bs.light_off;
        sv.light_tris_obj = s.light_tris_obj + 2 * bs.light_off;
        sv.light_tri_ok = s.light_tri_ok + 2 * bs.light_off;
        sv.num_lights = bs.num_lights;
        sv.other_lights = s.other_lights + bs.other_off;
        sv.num_other_lights = bs.num_other;
        WaveInfo wv = w;
        wv.p0 = sg.p0;
        wv.s0 = sg.s0;
        wv.ns = sg.ns;
        wv.seed = bs.seed;
        wv.sample_offset = bs.sample_offset;
        ShadeEntry<kMode>(sv, wv, bs.sp, b, cur, bounce, S, jj, o4, d4, PathOf(o4.w) - sg.path0, counted, so,
                          nullptr);
      } else {
        ShadeEntry<kMode>(s, w, sp, b, cur, bounce, S, jj, o4, d4, PathOf(o4.w), counted, so,
                          kGuide ? &gdev : nullptr);
      }
    }

    uint32_t off_c, off_s;
#if MUON_CONT_OCTANTS
    // a block's continuation rays grouped by direction octant
    const int octant = so.want_cont ? (so.cont_d.x < 0.0f ? 1 : 0) | (so.cont_d.y < 0.0f ? 2 : 0) |
                                          (so.cont_d.z < 0.0f ? 4 : 0)
                                    : -1;
    BlockReserveGrouped(octant, so.nshadow, wc.count(bounce + 1), wc.shadow(bounce), &off_c, &off_s);
#else
    BlockReserve(so.want_cont, so.nshadow, wc.count(bounce + 1), wc.shadow(bounce), &off_c, &off_s);
#endif
    if (active) b.link[jj] = so.want_cont ? static_cast<int32_t>(off_c) : -1;
    if (so.want_cont) {
      Pick(b.ray_o, nxt)[off_c] = make_float4(so.cont_o.x, so.cont_o.y, so.cont_o.z, id);
      Pick(b.ray_d, nxt)[off_c] = make_float4(so.cont_d.x, so.cont_d.y, so.cont_d.z, root);
      Pick(b.tp, nxt)[off_c] = make_float4(so.cont_tp.x, so.cont_tp.y, so.cont_tp.z, 0.0f);
    }
    if (so.nshadow) {
      const uint32_t base = static_cast<uint32_t>(jj) * static_cast<uint32_t>(S);
      uint32_t k = off_s;
      if (S <= kMaskSlots) {
        while (so.mask) {
          int slot = __ffsll(static_cast<long long>(so.mask)) - 1;
          so.mask &= so.mask - 1;
          b.shq[k++] = base + slot;
        }
      } else {
        const float4 *contrib = b.contrib + static_cast<int64_t>(jj) * S;
        for (int slot = 0; slot < S; ++slot) {
          float4 c = contrib[slot];
          if (c.x != 0.0f || c.y != 0.0f || c.z != 0.0f) b.shq[k++] = base + slot;
        }
      }
    }
  }
  AddStat(b.stats, kStatSecondary, counted);
}

// ---- fold -----------------------------------------------------------------------
// After the occlusion pass of a bounce: each entry's radiance plus its
// unblocked shadow slots moves to its next-bounce entry, or to the path's
// final radiance when the path ends here.
// Training samples from a guided vertex's direct light: every unblocked
// area-light sample and MIS ray becomes (features, direction, weight) with
// weight = luminance of its contribution / throughput, i.e. f cos L_e times
// the MIS weight over the density it was drawn from. Together with the
// continuation records (indirect light) these estimate the full incident
// radiance the mixture learns. They enter the pool at positions fixed by the
// bounce, the path and the slot (the fold stores each path's count at
// Mix(path), an exclusive scan over the wave's paths gives the offsets, then
// GuideAppendKernel writes), so the pool, and training, are reproducible
// whatever order the queues hold the paths in. Mix is a fixed permutation of
// the wave's path indices (p -> a p mod n, a coprime to n, near 0.618 n): the
// pool keeps the latest samples, and in path (pixel) order those would all
// come from the bottom of the image.
__device__ __forceinline__ uint32_t Mix(uint32_t path, uint32_t a, uint32_t n) {
  return static_cast<uint32_t>((static_cast<uint64_t>(path) * a) % n);
}
__device__ __forceinline__ bool GuideSlotKept(const GuideDev &g, const float4 *c, int k) {
  if (k >= g.area_slots && k != g.mis_slot) return false;
  const float4 v = c[k];
  return v.x != 0.0f || v.y != 0.0f || v.z != 0.0f;
}

__device__ __forceinline__ uint32_t GuideSampleCount(const PathBuffers &b, const GuideDev &g, int slots, int j) {
  if (b.hits[j].y < 0) return 0;
  const float4 *c = b.contrib + static_cast<int64_t>(j) * slots;
  uint32_t count = 0;
  for (int k = 0; k < slots; ++k) count += GuideSlotKept(g, c, k) ? 1u : 0u;
  return count;
}

// Writes entry j's training samples from pool position base + off[path of j].
__global__ void __launch_bounds__(kBlock) GuideAppendKernel(PathBuffers b, WaveCounters wc, int bounce, int slots,
                                                            GuideDev g, uint32_t mix_a, uint32_t paths) {
  const int n = static_cast<int>(*wc.count(bounce));
  const unsigned long long base = *g.pool_count;
  for (int j = blockIdx.x * kBlock + threadIdx.x; j < n; j += gridDim.x * kBlock) {
    const uint32_t key = Mix(PathOf(Pick(b.ray_o, bounce & 1)[j].w), mix_a, paths);
    if (g.sample_count[key] == 0) continue;
    unsigned long long idx = base + g.sample_off[key];
    const float4 *c = b.contrib + static_cast<int64_t>(j) * slots;
    const float4 tp = Pick(b.tp, bounce & 1)[j];
    const float4 f0 = g.feat[2 * static_cast<int64_t>(j)], f1 = g.feat[2 * static_cast<int64_t>(j) + 1];
    const float tpc[3] = {tp.x, tp.y, tp.z};
    const float lum[3] = {0.2126f, 0.7152f, 0.0722f};
    for (int k = 0; k < slots; ++k) {
      if (!GuideSlotKept(g, c, k)) continue;
      const float4 v = c[k];
      const float vc[3] = {v.x, v.y, v.z};
      float wgt = 0.0f;
      for (int q = 0; q < 3; ++q)
        if (tpc[q] > 0.0f) wgt += lum[q] * fmaxf(vc[q], 0.0f) / tpc[q];
      const float4 dir = b.slot_dir[static_cast<int64_t>(j) * slots + k];
      GuideSample smp;
      smp.f0 = f0;
      smp.f1 = f1;
      // a non-finite weight becomes 0, which training ignores
      smp.dir_w = make_float4(dir.x, dir.y, dir.z, isfinite(wgt) ? wgt : 0.0f);
      g.pool[idx % g.pool_cap] = smp;
      ++idx;
    }
  }
}

// Samples ever appended += this bounce's total over the wave's `paths` paths
// (one thread, after the append).
__global__ void GuideAdvanceKernel(int paths, GuideDev g) {
  *g.pool_count += static_cast<unsigned long long>(g.sample_off[paths - 1]) + g.sample_count[paths - 1];
}

template <bool kGuide>
__global__ void __launch_bounds__(kBlock) FoldKernel(PathBuffers b, WaveCounters wc, int bounce, int slots,
                                                     GuideDev g, uint32_t mix_a = 1, uint32_t paths = 1) {
  const int n = static_cast<int>(*wc.count(bounce));
  const int cur = bounce & 1, nxt = cur ^ 1;
  for (int base = blockIdx.x * kBlock; base < n; base += gridDim.x * kBlock) {
    const int j = base + threadIdx.x;
    if (j < n) {
      float4 r = Pick(b.rad, cur)[j];
      // Only shaded entries (hits) wrote shadow slots this bounce.
      if (b.hits[j].y >= 0) {
        const float4 *c = b.contrib + static_cast<int64_t>(j) * slots;
        for (int k = 0; k < slots; ++k) {
          float4 v = c[k];
          r.x += v.x, r.y += v.y, r.z += v.z;
        }
      }
      int next = b.link[j];
      if (kGuide && !g.direct_only && bounce < g.rec_bounces) {
        GuideRec &rc = g.rec[static_cast<int64_t>(bounce) * g.rec_cap + j];
        if (next >= 0) rc.after = r;
        else rc.tp.w = 0.0f;  // no continuation: nothing to learn from this vertex
      }
      if (next >= 0) Pick(b.rad, nxt)[next] = r;
      else b.final_rad[PathOf(Pick(b.ray_o, cur)[j].w)] = r;
    }
    if (kGuide && bounce < g.rec_bounces && j < n)
      g.sample_count[Mix(PathOf(Pick(b.ray_o, cur)[j].w), mix_a, paths)] = GuideSampleCount(b, g, slots, j);
  }
}

// ---- film ----------------------------------------------------------------------
// Film::SetPixel accumulation (muon/film.cc:10-19) in FP64: one thread per
// pixel adds its samples in sample order, so the film is reproducible.
__global__ void __launch_bounds__(kBlock) FilmKernel(WaveInfo w, PathBuffers b, double *sum, double *sum_sq,
                                                     uint32_t *count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= w.npix) return;
  const int pixel = w.p0 + i;
  double s0 = 0, s1 = 0, s2 = 0, q0 = 0, q1 = 0, q2 = 0;
  for (int k = 0; k < w.ns; ++k) {
    float4 r = b.final_rad[i * w.ns + k];
    s0 += r.x, s1 += r.y, s2 += r.z;
    q0 += static_cast<double>(r.x) * r.x, q1 += static_cast<double>(r.y) * r.y, q2 += static_cast<double>(r.z) * r.z;
  }
  sum[3 * pixel + 0] += s0;
  sum[3 * pixel + 1] += s1;
  sum[3 * pixel + 2] += s2;
  sum_sq[3 * pixel + 0] += q0;
  sum_sq[3 * pixel + 1] += q1;
  sum_sq[3 * pixel + 2] += q2;
  count[pixel] += static_cast<uint32_t>(w.ns);
}

// ---- learned guiding: features, inference, training records -----------------------
// Spherical coordinates of a unit vector scaled to [0, 1]^2.
__device__ __forceinline__ void Spherical01(float3 v, float *a, float *b) {
  *a = acosf(fminf(fmaxf(v.z, -1.0f), 1.0f)) * kInvPi;
  *b = atan2f(v.y, v.x) * (0.5f * kInvPi) + 0.5f;
}

// The 8 guiding features of a shading point.
__device__ __forceinline__ void GuideFeatures(const GuideDev &g, float3 p, float3 n, float3 d, const Mat &m,
                                              float *f) {
  f[0] = fminf(fmaxf((p.x - g.lo[0]) * g.inv_ext[0], 0.0f), 1.0f);
  f[1] = fminf(fmaxf((p.y - g.lo[1]) * g.inv_ext[1], 0.0f), 1.0f);
  f[2] = fminf(fmaxf((p.z - g.lo[2]) * g.inv_ext[2], 0.0f), 1.0f);
  Spherical01(n, &f[3], &f[4]);
  Spherical01(-d, &f[5], &f[6]);
  // GGX alpha; for Phong the Beckmann-equivalent sqrt(2 / (s + 2)); Lambertian 1
  float r = 1.0f;
  if (m.brdf == MUON_BRDF_GGX) r = m.roughness;
  else if (m.brdf == MUON_BRDF_PHONG) r = sqrtf(2.0f / (m.shininess + 2.0f));
  f[7] = fminf(fmaxf(r, 0.0f), 1.0f);
}

// For every hit of the bounce's queue: its guiding features (one thread per
// entry at full occupancy, which hides the dependent loads of the surface).
template <int kMode>
__global__ void __launch_bounds__(kBlock) GuideFeatureKernel(DevScene s, PathBuffers b, WaveCounters wc, int bounce,
                                                            GuideDev g) {
  const int n = static_cast<int>(*wc.count(bounce));
  const int cur = bounce & 1;
  for (int j = blockIdx.x * kBlock + threadIdx.x; j < n; j += gridDim.x * kBlock) {
    const int2 h = b.hits[j];
    if (h.y < 0) continue;
    const float4 o4 = Pick(b.ray_o, cur)[j], d4 = Pick(b.ray_d, cur)[j];
    float3 p, nrm;
    float dist;
    int mat, light, pid;
    const float3 d = f3(d4.x, d4.y, d4.z);
    Surface<kMode>(s, h.y, f3(o4.x, o4.y, o4.z), d, __int_as_float(h.x), &p, &nrm, &dist, &mat, &light, &pid);
    float f[guide::kFeatures];
    GuideFeatures(g, p, nrm, d, LoadMat(s.materials, mat), f);
    g.feat[2 * static_cast<int64_t>(j)] = make_float4(f[0], f[1], f[2], f[3]);
    g.feat[2 * static_cast<int64_t>(j) + 1] = make_float4(f[4], f[5], f[6], f[7]);
  }
}

// For every hit of the bounce's queue: the network's mixture for its features.
// Tensor-core inference (guide_tc.cuh): one CTA per SM, two groups of 128
// queue entries in flight, one thread per entry; the next tile's hits and
// features are loaded while the current tile runs.
__global__ void __launch_bounds__(guide::kTcThreads, 1) GuideInferKernel(PathBuffers b, WaveCounters wc, int bounce,
                                                                         GuideDev g) {
  extern __shared__ __align__(1024) unsigned char smem[];
  const int n = static_cast<int>(*wc.count(bounce));
  if (static_cast<int>(blockIdx.x) * guide::kTcThreads >= n) return;  // the whole CTA
  guide::TcGroup grp;
  bool ok = guide::TcBegin(smem, g.wt, &grp);
  const int group = threadIdx.x / guide::kTcRows;
  const int stride = gridDim.x * guide::kTcThreads;
  auto fetch = [&](int j, bool *hit, float4 *f0, float4 *f1) {
    *hit = j < n && b.hits[j].y >= 0;
    *f0 = *f1 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (*hit) {
      *f0 = g.feat[2 * static_cast<int64_t>(j)];
      *f1 = g.feat[2 * static_cast<int64_t>(j) + 1];
    }
  };
  int base = (blockIdx.x * 2 + group) * guide::kTcRows;
  bool hit;
  float4 f0, f1;
  fetch(base + grp.row, &hit, &f0, &f1);
  for (; ok && base < n; base += stride) {
    const int j = base + grp.row;
    const float f[guide::kFeatures] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
    const bool cur_hit = hit;
    fetch(j + stride, &hit, &f0, &f1);
    float raw[guide::kOut];
    ok = guide::TcForward(grp, f, raw);
    if (!ok) break;
    if (cur_hit) guide::MakeMixture(raw, guide::TcMixRow(grp));  // rows of misses stay unused
    guide::TcStoreMix(grp, base, n, g.mix);
  }
  guide::TcEnd(smem, grp, g.status);
}

// After a guided wave: every recorded vertex becomes a training sample whose
// weight is the luminance of (final radiance - radiance after the vertex) /
// throughput before it, i.e. f cos L_i / density of the sampled direction.
__global__ void __launch_bounds__(kBlock) GuideCollectKernel(PathBuffers b, WaveCounters wc, int bounces, GuideDev g) {
  for (int k = 0; k < bounces; ++k) {
    const int n = static_cast<int>(*wc.count(k));
    for (int base = blockIdx.x * kBlock; base < n; base += gridDim.x * kBlock) {
      const int j = base + threadIdx.x;
      bool keep = false;
      GuideSample smp;
      if (j < n) {
        const GuideRec rc = g.rec[static_cast<int64_t>(k) * g.rec_cap + j];
        if (rc.tp.w == 1.0f) {
          const float4 L = b.final_rad[PathOf(rc.dir.w)];
          const float dl[3] = {L.x - rc.after.x, L.y - rc.after.y, L.z - rc.after.z};
          const float tp[3] = {rc.tp.x, rc.tp.y, rc.tp.z};
          const float lum[3] = {0.2126f, 0.7152f, 0.0722f};
          float wgt = 0.0f;
          for (int c = 0; c < 3; ++c)
            if (tp[c] > 0.0f) wgt += lum[c] * fmaxf(dl[c], 0.0f) / tp[c];
          if (wgt > 0.0f && isfinite(wgt)) {
            keep = true;
            smp.f0 = rc.f0;
            smp.f1 = rc.f1;
            smp.dir_w = make_float4(rc.dir.x, rc.dir.y, rc.dir.z, wgt);
          }
        }
      }
      const unsigned mask = __ballot_sync(0xffffffffu, keep);
      if (mask) {
        const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
        unsigned long long base_idx = 0;
        if (lane == leader) base_idx = atomicAdd(g.pool_count, static_cast<unsigned long long>(__popc(mask)));
        base_idx = __shfl_sync(0xffffffffu, base_idx, leader);
        if (keep) {
          const unsigned long long idx = base_idx + __popc(mask & ((1u << lane) - 1u));
          g.pool[idx % g.pool_cap] = smp;
        }
      }
    }
  }
}

// Batched film: one thread per pixel of the wave's segments.
__global__ void __launch_bounds__(kBlock) FilmBatchKernel(const BatchScene *scenes, const BatchSeg *segs, int nseg,
                                                          int pixels, PathBuffers b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= pixels) return;
  const BatchSeg sg = segs[FindSeg<&BatchSeg::pix0>(segs, nseg, i)];
  const BatchScene &sc = scenes[sg.scene];
  const int local = i - sg.pix0;
  const int pixel = sg.p0 + local;
  double s0 = 0, s1 = 0, s2 = 0, q0 = 0, q1 = 0, q2 = 0;
  const float4 *fr = b.final_rad + sg.path0 + static_cast<int64_t>(local) * sg.ns;
  for (int k = 0; k < sg.ns; ++k) {
    float4 r = fr[k];
    s0 += r.x, s1 += r.y, s2 += r.z;
    q0 += static_cast<double>(r.x) * r.x, q1 += static_cast<double>(r.y) * r.y, q2 += static_cast<double>(r.z) * r.z;
  }
  double *sum = sc.sum, *sum_sq = sc.sum_sq;
  sum[3 * pixel + 0] += s0;
  sum[3 * pixel + 1] += s1;
  sum[3 * pixel + 2] += s2;
  sum_sq[3 * pixel + 0] += q0;
  sum_sq[3 * pixel + 1] += q1;
  sum_sq[3 * pixel + 2] += q2;
  sc.count[pixel] += static_cast<uint32_t>(sg.ns);
}

// ---- ray-level queries -----------------------------------------------------------
// rays: n x 6 floats (origin, direction); out: n x 8 floats
// (distance, prim id bits, position xyz, normal xyz).
template <int kTri>
__global__ void __launch_bounds__(kBlock) IntersectRaysKernel(DevScene s, const float *rays, int64_t n, float *out) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *r = rays + 6 * i;
  float3 o = f3(r[0], r[1], r[2]), d = f3(r[3], r[4], r[5]);
  TraceCounters c;
  bool of = false;
  float t, t_obj = 0.0f;
  int h = Trace<false, false, kTri>(s, o, d, INFINITY, &t, &c, &of, &t_obj);
  float *q = out + 8 * i;
  if (h < 0) {
    q[0] = INFINITY;
    q[1] = __int_as_float(-1);
    for (int k = 2; k < 8; ++k) q[k] = 0.0f;
    return;
  }
  float3 p, nrm;
  float dist;
  int mat, light, pid;
  Surface<kTri>(s, h, o, d, kTri == MUON_ISECT_EXACT ? t_obj : t, &p, &nrm, &dist, &mat, &light, &pid);
  q[0] = dist;
  q[1] = __int_as_float(pid);
  q[2] = p.x, q[3] = p.y, q[4] = p.z;
  q[5] = nrm.x, q[6] = nrm.y, q[7] = nrm.z;
}

template <int kTri>
__global__ void __launch_bounds__(kBlock) OccludedRaysKernel(DevScene s, const float *rays, const float *maxd,
                                                             int64_t n, uint8_t *out) {
  int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *r = rays + 6 * i;
  TraceCounters c;
  bool of = false;
  float t;
  int h = Trace<true, false, kTri>(s, f3(r[0], r[1], r[2]), f3(r[3], r[4], r[5]), maxd[i], &t, &c, &of);
  out[i] = h >= 0 ? 1 : 0;
}

inline unsigned Blocks(int64_t n) { return static_cast<unsigned>((n + kBlock - 1) / kBlock); }

int g_persistent_blocks = 152 * 8;
int g_traversal_blocks = 152 * 4;
int g_sms = 152;

// Grid for a device-counted launch whose queue holds at most `bound` entries.
inline unsigned CountedBlocks(int64_t bound) {
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(Blocks(bound), g_persistent_blocks)));
}

int g_traversal_override = 0;

inline unsigned TraversalBlocks(int64_t bound) {
  const int grid = g_traversal_override > 0 ? g_traversal_override : g_traversal_blocks;
  return static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>(Blocks(bound), grid)));
}

// Calls f(std::integral_constant<int, mode>) for a runtime intersection mode.
template <class F>
void WithMode(int mode, F &&f) {
  if (mode == MUON_ISECT_WATERTIGHT) f(std::integral_constant<int, MUON_ISECT_WATERTIGHT>());
  else if (mode == MUON_ISECT_EXACT) f(std::integral_constant<int, MUON_ISECT_EXACT>());
  else f(std::integral_constant<int, MUON_ISECT_FAST>());
}

// ---- measurement ---------------------------------------------------------------
// A sample of one bounce's traversal queue, copied for the host walk that
// counts traversal work: kind 0 the closest-hit queue, kind 1 the shadow
// queue. out[0] = (sampled, queue length) as int bits; ray i of the sample
// (queue entry i * length / sampled) follows as (origin, root), (direction,
// tmax), i.e. exactly what the traversal kernels load for it.
__global__ void __launch_bounds__(kBlock) SampleQueueKernel(PathBuffers b, WaveCounters wc, int bounce, int kind,
                                                            int slots, int m, float4 *out) {
  const int n = static_cast<int>(kind == 0 ? *wc.count(bounce) : *wc.shadow(bounce));
  const int taken = min(m, n);
  if (blockIdx.x == 0 && threadIdx.x == 0) out[0] = make_float4(__int_as_float(taken), __int_as_float(n), 0.0f, 0.0f);
  for (int i = blockIdx.x * kBlock + threadIdx.x; i < taken; i += gridDim.x * kBlock) {
    const int j = static_cast<int>((static_cast<int64_t>(i) * n) / taken);
    float4 o, d;
    if (kind == 0) {
      o = Pick(b.ray_o, bounce & 1)[j];
      d = Pick(b.ray_d, bounce & 1)[j];
      o.w = d.w;  // root
      d.w = INFINITY;
    } else {
      const uint32_t slot = b.shq[j];
      o = b.org[slot / slots];  // w: root
      d = b.slot_dir[slot];     // w: distance to the light sample
    }
    out[1 + 2 * static_cast<int64_t>(i)] = o;
    out[2 + 2 * static_cast<int64_t>(i)] = d;
  }
}

// Read-bandwidth ceiling: each pass reads the buffer (n4 float4s) once per
// block through L1 (level 0), or once across the grid bypassing L1 (levels 1
// and 2). Four independent accumulators keep loads in flight; the sum is
// stored only if it equals an impossible value, so the loads stay.
__global__ void __launch_bounds__(kBlock) ReadBandwidthKernel(const float4 *buf, int64_t n4, int passes, int level,
                                                              float *sink) {
  float4 a0 = make_float4(0, 0, 0, 0), a1 = a0, a2 = a0, a3 = a0;
  const int64_t start = level == 0 ? threadIdx.x : static_cast<int64_t>(blockIdx.x) * kBlock + threadIdx.x;
  const int64_t step = level == 0 ? kBlock : static_cast<int64_t>(gridDim.x) * kBlock;
  for (int p = 0; p < passes; ++p) {
    int64_t i = start;
    for (; i + 3 * step < n4; i += 4 * step) {
      const float4 v0 = level == 0 ? __ldg(buf + i) : __ldcg(buf + i);
      const float4 v1 = level == 0 ? __ldg(buf + i + step) : __ldcg(buf + i + step);
      const float4 v2 = level == 0 ? __ldg(buf + i + 2 * step) : __ldcg(buf + i + 2 * step);
      const float4 v3 = level == 0 ? __ldg(buf + i + 3 * step) : __ldcg(buf + i + 3 * step);
      a0.x += v0.x, a0.y += v0.y, a0.z += v0.z, a0.w += v0.w;
      a1.x += v1.x, a1.y += v1.y, a1.z += v1.z, a1.w += v1.w;
      a2.x += v2.x, a2.y += v2.y, a2.z += v2.z, a2.w += v2.w;
      a3.x += v3.x, a3.y += v3.y, a3.z += v3.z, a3.w += v3.w;
    }
    for (; i < n4; i += step) {
      const float4 v = level == 0 ? __ldg(buf + i) : __ldcg(buf + i);
      a0.x += v.x, a0.y += v.y, a0.z += v.z, a0.w += v.w;
    }
  }
  const float t = (a0.x + a0.y + a0.z + a0.w) + (a1.x + a1.y + a1.z + a1.w) + (a2.x + a2.y + a2.z + a2.w) +
                  (a3.x + a3.y + a3.z + a3.w);
  if (t == 1.2345e-37f) sink[0] = t;
}

}  // namespace

void SetPersistentGrid(int blocks) { g_persistent_blocks = std::max(1, blocks); }

void SetTraversalBlocksOverride(int blocks) { g_traversal_override = std::max(0, blocks); }

void SetTraversalGrid(int sms) {
  // Enough resident blocks to fill every SM once; the persistent traversal
  // kernels hand out rays themselves.
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ExtendKernel<false, MUON_ISECT_EXACT>, kBlock, 0) !=
          cudaSuccess ||
      per_sm < 1)
    per_sm = 4;
  g_traversal_blocks = std::max(1, sms * per_sm);
  g_sms = std::max(1, sms);
}

void LaunchSampleQueue(const PathBuffers &b, WaveCounters wc, int bounce, int kind, int slots, int m, float4 *out,
                       cudaStream_t st) {
  SampleQueueKernel<<<Blocks(std::max(m, 1)), kBlock, 0, st>>>(b, wc, bounce, kind, std::max(slots, 1), m, out);
}

void LaunchReadBandwidth(const float4 *buf, int64_t n4, int passes, int level, int blocks, float *sink,
                         cudaStream_t st) {
  ReadBandwidthKernel<<<static_cast<unsigned>(std::max(blocks, 1)), kBlock, 0, st>>>(buf, n4, passes, level, sink);
}

void LaunchCamera(const DevCamera &cam, const WaveInfo &w, const PathBuffers &b, WaveCounters wc, cudaStream_t st) {
  CameraKernel<<<Blocks(std::max(w.n, 1)), kBlock, 0, st>>>(cam, w, b, wc);
}

void LaunchExtend(const DevScene &s, const PathBuffers &b, WaveCounters wc, int bounce, int bound, int isect,
                  bool stats, cudaStream_t st) {
  if (bound <= 0) return;
  WithMode(isect, [&](auto m) {
    constexpr int M = decltype(m)::value;
    const unsigned g = TraversalBlocks(bound);
    if (stats) ExtendKernel<true, M><<<g, kBlock, 0, st>>>(s, b, wc, bounce);
    else ExtendKernel<false, M><<<g, kBlock, 0, st>>>(s, b, wc, bounce);
  });
  if (MUON_STABLE_CLASSES) {
    const unsigned tiles = static_cast<unsigned>((bound + kClassTile - 1) / kClassTile);
    ClassCountKernel<<<tiles, kClassThreads, 0, st>>>(b, wc, bounce);
    ClassScanKernel<<<kNumClasses, 1024, 0, st>>>(b, wc, bounce);
    ClassScatterKernel<<<tiles, kClassThreads, 0, st>>>(b, wc, bounce);
  }
}

void LaunchShadeDebug(const DevScene &s, const PathBuffers &b, WaveCounters wc, int integrator, int bound, int isect,
                      cudaStream_t st) {
  if (bound <= 0) return;
  WithMode(isect, [&](auto m) {
    ShadeDebugKernel<decltype(m)::value><<<CountedBlocks(bound), kBlock, 0, st>>>(s, b, wc, integrator);
  });
}

void LaunchWhitted(const DevScene &s, const PathBuffers &b, const WaveInfo &w, int integrator, int max_trace_depth,
                   int isect, bool stats, cudaStream_t st) {
  if (w.n <= 0) return;
  WithMode(isect, [&](auto m) {
    constexpr int M = decltype(m)::value;
    if (stats) WhittedKernel<true, M><<<Blocks(w.n), kBlock, 0, st>>>(s, b, w, integrator, max_trace_depth);
    else WhittedKernel<false, M><<<Blocks(w.n), kBlock, 0, st>>>(s, b, w, integrator, max_trace_depth);
  });
}

void LaunchShadePath(const DevScene &s, const WaveInfo &w, const ShadeParams &sp, const PathBuffers &b,
                     WaveCounters wc, int bounce, int bound, cudaStream_t st) {
  if (bound <= 0) return;
  WithMode(sp.isect, [&](auto m) {
    ShadePathKernel<decltype(m)::value, false, false>
        <<<CountedBlocks(bound), kBlock, 0, st>>>(s, w, sp, b, wc, bounce, nullptr, nullptr, sp.slots, GuideDev{});
  });
}

void LaunchOcclude(const DevScene &s, const PathBuffers &b, WaveCounters wc, int bounce, int slots, int bound,
                   int isect, bool stats, cudaStream_t st) {
  if (bound <= 0 || slots <= 0) return;
  WithMode(isect, [&](auto m) {
    constexpr int M = decltype(m)::value;
    const unsigned g = TraversalBlocks(bound);
    if (stats) OccludeKernel<true, M><<<g, kBlock, 0, st>>>(s, b, wc, bounce, slots);
    else OccludeKernel<false, M><<<g, kBlock, 0, st>>>(s, b, wc, bounce, slots);
  });
}

void LaunchFold(const PathBuffers &b, WaveCounters wc, int bounce, int slots, int bound, cudaStream_t st) {
  if (bound <= 0) return;
  FoldKernel<false><<<CountedBlocks(bound), kBlock, 0, st>>>(b, wc, bounce, slots, GuideDev{});
}

void LaunchFilm(const WaveInfo &w, const PathBuffers &b, double *sum, double *sum_sq, uint32_t *count,
                cudaStream_t st) {
  if (w.npix > 0) FilmKernel<<<Blocks(w.npix), kBlock, 0, st>>>(w, b, sum, sum_sq, count);
}

void LaunchCameraBatch(const BatchScene *scenes, const BatchSeg *segs, int nseg, int paths, const PathBuffers &b,
                       WaveCounters wc, cudaStream_t st) {
  CameraBatchKernel<<<Blocks(std::max(paths, 1)), kBlock, 0, st>>>(scenes, segs, nseg, paths, b, wc);
}

void LaunchShadePathBatch(const DevScene &s, const BatchScene *scenes, const BatchSeg *segs, int slot_stride,
                          int isect, const PathBuffers &b, WaveCounters wc, int bounce, int bound, cudaStream_t st) {
  if (bound <= 0) return;
  WaveInfo w{};
  ShadeParams sp{};
  WithMode(isect, [&](auto m) {
    ShadePathKernel<decltype(m)::value, true, false>
        <<<CountedBlocks(bound), kBlock, 0, st>>>(s, w, sp, b, wc, bounce, scenes, segs, slot_stride, GuideDev{});
  });
}

void LaunchFilmBatch(const BatchScene *scenes, const BatchSeg *segs, int nseg, int pixels, const PathBuffers &b,
                     cudaStream_t st) {
  if (pixels > 0) FilmBatchKernel<<<Blocks(pixels), kBlock, 0, st>>>(scenes, segs, nseg, pixels, b);
}

void LaunchGuideInfer(const DevScene &s, const PathBuffers &b, WaveCounters wc, int bounce, int bound, int isect,
                      const GuideDev &g, cudaStream_t st) {
  if (bound <= 0) return;
  WithMode(isect, [&](auto m) {
    GuideFeatureKernel<decltype(m)::value><<<CountedBlocks(bound), kBlock, 0, st>>>(s, b, wc, bounce, g);
  });
  // one CTA per SM (the shared memory of the two groups fills an SM)
  const unsigned grid = static_cast<unsigned>(
      std::max<int64_t>(1, std::min<int64_t>((bound + guide::kTcThreads - 1) / guide::kTcThreads, g_sms)));
  cudaFuncSetAttribute(GuideInferKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, guide::kTcSmemBytes);
  GuideInferKernel<<<grid, guide::kTcThreads, guide::kTcSmemBytes, st>>>(b, wc, bounce, g);
}

void LaunchShadePathGuided(const DevScene &s, const WaveInfo &w, const ShadeParams &sp, const PathBuffers &b,
                           WaveCounters wc, int bounce, int bound, const GuideDev &g, cudaStream_t st) {
  if (bound <= 0) return;
  WithMode(sp.isect, [&](auto m) {
    ShadePathKernel<decltype(m)::value, false, true>
        <<<CountedBlocks(bound), kBlock, 0, st>>>(s, w, sp, b, wc, bounce, nullptr, nullptr, sp.slots, g);
  });
}

void LaunchFoldGuided(const PathBuffers &b, WaveCounters wc, int bounce, int slots, int bound, const GuideDev &g,
                      cudaStream_t st) {
  if (bound <= 0) return;
  // `bound` is the wave's path count: sample counts are kept per path index
  // (paths without a vertex at this bounce count none)
  const bool sampling = bounce < g.rec_bounces;
  const uint32_t paths = static_cast<uint32_t>(bound);
  uint32_t mix_a = std::max<uint32_t>(1u, static_cast<uint32_t>(0.6180339887 * paths));
  while (std::gcd(mix_a, paths) != 1u) ++mix_a;
  if (sampling) CUDA_TRY(cudaMemsetAsync(g.sample_count, 0, sizeof(uint32_t) * bound, st));
  FoldKernel<true><<<CountedBlocks(bound), kBlock, 0, st>>>(b, wc, bounce, slots, g, mix_a, paths);
  if (!sampling) return;
  size_t tmp = g.scan_bytes;
  CUDA_TRY(cub::DeviceScan::ExclusiveSum(g.scan_tmp, tmp, g.sample_count, g.sample_off, bound, st));
  GuideAppendKernel<<<CountedBlocks(bound), kBlock, 0, st>>>(b, wc, bounce, slots, g, mix_a, paths);
  GuideAdvanceKernel<<<1, 1, 0, st>>>(bound, g);
}

size_t GuideScanBytes(int capacity) {
  size_t bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, bytes, static_cast<const uint32_t *>(nullptr), static_cast<uint32_t *>(nullptr),
                                capacity);
  return bytes;
}

void LaunchGuideCollect(const PathBuffers &b, WaveCounters wc, int bounces, int bound, const GuideDev &g,
                        cudaStream_t st) {
  if (bound <= 0 || bounces <= 0) return;
  GuideCollectKernel<<<CountedBlocks(bound), kBlock, 0, st>>>(b, wc, bounces, g);
}

void LaunchIntersectRays(const DevScene &s, const float *rays, int64_t n, int isect, float *out_hit, cudaStream_t st) {
  if (n <= 0) return;
  WithMode(isect, [&](auto m) {
    IntersectRaysKernel<decltype(m)::value><<<Blocks(n), kBlock, 0, st>>>(s, rays, n, out_hit);
  });
}

void LaunchOccludedRays(const DevScene &s, const float *rays, const float *maxd, int64_t n, int isect, uint8_t *out,
                        cudaStream_t st) {
  if (n <= 0) return;
  WithMode(isect, [&](auto m) {
    OccludedRaysKernel<decltype(m)::value><<<Blocks(n), kBlock, 0, st>>>(s, rays, maxd, n, out);
  });
}

}  // namespace muon_gpu
