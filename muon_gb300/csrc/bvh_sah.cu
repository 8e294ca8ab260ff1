// BVH construction on the GPU with the host builder's binned SAH: the same
// split decisions as the top-down builder of scene_build.cc (32 centroid
// bins per axis, SAH with unit traversal and intersection costs, a leaf when
// a node of at most max_leaf references is no dearer as a leaf, the
// reference's BVH build replaced there as muon/acceleration.cc:204-458), so
// the tree has the host tree's nodes and boxes. Only the order of references
// inside a leaf and the node numbering differ: partitions here are stable,
// and interior nodes are numbered root first, then sibling pairs in the order
// of their parents' split positions.
//
// Every decision is taken with the same float operations as on the host,
// written with round-to-nearest intrinsics so that nothing is contracted into
// a fused multiply-add: centroid 0.5 (lo + hi), bin floor((c - lo) * 32 /
// extent), box areas, and the sweep's costs in the host's order. Bin
// contents (counts, min / max of boxes and centroids) are exact whatever the
// order in which references arrive.
//
// Two phases:
//  * nodes of at least kSmallRefs references, level by level: a pass bins
//    the level's references into per-node bins (blocks of kChunk references
//    accumulate in shared memory, then merge into global bins); one warp per
//    node sweeps the bins and decides; a stable partition (per-chunk counts,
//    per-node prefix, scatter) moves the references;
//  * smaller nodes, also level by level: one warp per node bins it in shared
//    memory, sweeps the bins with one lane per bin, and partitions it with
//    warp ballots.
//
// A node's box and its children's centroid bounds come from its bins. A node
// writes its own box and link into its parent's child slot, and an interior
// node keeps its entry at index (split position - 1) of a sparse array; a
// scan of the entries' interior-child counts gives the dense numbering at
// the end, siblings side by side.
#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "bvh_build.h"

namespace muon_gpu {

namespace {

constexpr int kSahBins = 32;
// Words of one bin: reference count, box lo / hi, centroid lo / hi (floats
// as order-preserving keys).
constexpr int kBinWords = 13;
constexpr int kNodeBinWords = 3 * kSahBins * kBinWords;
constexpr int kSmallRefs = 2048;
constexpr int kChunk = 2048;
constexpr int kLevelThreads = 256;
constexpr int kSmallWarps = 4;
constexpr int kMaxLevels = 64;
// levels of the small-node phase between checks of its queue, and at most
constexpr int kSmallLevelsPerCheck = 4;
constexpr int kMaxSmallLevels = 4096;

inline unsigned Blocks(int64_t n, int threads) { return static_cast<unsigned>((n + threads - 1) / threads); }

__device__ __forceinline__ unsigned FloatKey(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float KeyFloat(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// A node waiting to be split: its references idx[start, end), the child slot
// of its parent it fills (sparse index * 2 + slot) and its centroid bounds.
struct PendingNode {
  int32_t start, end, parent, depth;
  float clo[3], chi[3];
};

// How a level node was split: axis >= 0 binned SAH at `bin`; -1 leaf; -2 the
// first half by position (every centroid coincides).
struct Decision {
  int32_t axis, bin, mid, pad;
  float lo, scale;
};

struct SahStats {
  unsigned long long leaves;
  int max_depth, max_leaf, root, error;
  int next_count, small_count, small_next;
};

__device__ __forceinline__ float Centroid(float lo, float hi) { return __fmul_rn(0.5f, __fadd_rn(lo, hi)); }

// scale_axis as the host builder forms it: kBins / extent, 0 for no extent.
__device__ __forceinline__ float BinScale(float lo, float hi) {
  const float extent = __fsub_rn(hi, lo);
  return extent > 0.0f ? __fdiv_rn(static_cast<float>(kSahBins), extent) : 0.0f;
}
__device__ __forceinline__ int BinOf(float c, float lo, float scale) {
  const int k = __float2int_rz(__fmul_rn(__fsub_rn(c, lo), scale));
  return max(0, min(kSahBins - 1, k));
}

// Area of a box as the host builder computes it (0 for an empty box).
__device__ __forceinline__ float BoxArea(const float *lo, const float *hi) {
  const float dx = __fsub_rn(hi[0], lo[0]), dy = __fsub_rn(hi[1], lo[1]), dz = __fsub_rn(hi[2], lo[2]);
  if (!(dx >= 0.0f) || !(dy >= 0.0f) || !(dz >= 0.0f)) return 0.0f;
  return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dx, dz)), __fmul_rn(dy, dz)));
}

__device__ __forceinline__ void LoadRef(const float4 *box8, int ref, float *lo, float *hi) {
  const float4 a = __ldg(box8 + 2 * ref), b = __ldg(box8 + 2 * ref + 1);
  lo[0] = a.x, lo[1] = a.y, lo[2] = a.z;
  hi[0] = b.x, hi[1] = b.y, hi[2] = b.z;
}

__device__ __forceinline__ void InitBins(uint32_t *bins, int i0, int step) {
  for (int w = i0; w < kNodeBinWords; w += step) {
    const int f = w % kBinWords;
    // count 0; lower bounds start at the largest key, upper bounds at 0
    bins[w] = f == 0 ? 0u : ((f >= 1 && f <= 3) || (f >= 7 && f <= 9) ? 0xffffffffu : 0u);
  }
}

// Adds one reference to a node's bins (shared or global memory).
__device__ __forceinline__ void BinRef(uint32_t *bins, const float *lo, const float *hi, const float *clo,
                                       const float *scale) {
  float c[3];
  for (int k = 0; k < 3; ++k) c[k] = Centroid(lo[k], hi[k]);
  for (int axis = 0; axis < 3; ++axis) {
    uint32_t *b = bins + (axis * kSahBins + BinOf(c[axis], clo[axis], scale[axis])) * kBinWords;
    atomicAdd(b, 1u);
    for (int k = 0; k < 3; ++k) {
      atomicMin(b + 1 + k, FloatKey(lo[k]));
      atomicMax(b + 4 + k, FloatKey(hi[k]));
      atomicMin(b + 7 + k, FloatKey(c[k]));
      atomicMax(b + 10 + k, FloatKey(c[k]));
    }
  }
}

// Merges shared bins into global ones (bins that received nothing are
// skipped).
__device__ __forceinline__ void FlushBins(const uint32_t *s, uint32_t *g, int i0, int step) {
  for (int w = i0; w < kNodeBinWords; w += step) {
    const int f = w % kBinWords;
    if (s[w - f] == 0) continue;
    if (f == 0) atomicAdd(g + w, s[w]);
    else if ((f >= 1 && f <= 3) || (f >= 7 && f <= 9)) atomicMin(g + w, s[w]);
    else atomicMax(g + w, s[w]);
  }
}

// A node's box and split, from its bins; the same in every lane of the warp.
struct NodeSplit {
  float lo[3], hi[3];  // the node's box
  int axis, bin;       // Decision::axis / bin
  int left_n;          // references that go left
  float lclo[3], lchi[3], rclo[3], rchi[3];  // the children's centroid bounds
};

__device__ __forceinline__ float WarpMin(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float WarpMax(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int WarpSum(int v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// SplitSah's two sweeps over one axis (scene_build.cc), lane b holding bin
// b: the right sweep's box of bins b..31 and the left sweep's box of bins
// 0..b are unions (exact in any order), so suffix and prefix scans across
// the lanes give the host's boxes, areas and costs; the cheapest split of the
// axis, the first bin at the minimum, in every lane; bin -1 when none leaves
// both sides non-empty.
__device__ void SweepAxis(const uint32_t *ab, int lane, float *best_cost, int *best_bin) {
  const uint32_t *x = ab + lane * kBinWords;
  const int c = static_cast<int>(x[0]);
  float blo[3], bhi[3];
  for (int k = 0; k < 3; ++k) {
    blo[k] = c ? KeyFloat(x[1 + k]) : INFINITY;
    bhi[k] = c ? KeyFloat(x[4 + k]) : -INFINITY;
  }
  float llo[3], lhi[3], rlo[3], rhi[3];
  int ln = c, rn = c;
  for (int k = 0; k < 3; ++k) llo[k] = rlo[k] = blo[k], lhi[k] = rhi[k] = bhi[k];
  for (int o = 1; o < kSahBins; o <<= 1) {
    const int up_n = __shfl_up_sync(0xffffffffu, ln, o), down_n = __shfl_down_sync(0xffffffffu, rn, o);
    if (lane >= o) ln += up_n;
    if (lane + o < kSahBins) rn += down_n;
    for (int k = 0; k < 3; ++k) {
      const float ul = __shfl_up_sync(0xffffffffu, llo[k], o), uh = __shfl_up_sync(0xffffffffu, lhi[k], o);
      const float dl = __shfl_down_sync(0xffffffffu, rlo[k], o), dh = __shfl_down_sync(0xffffffffu, rhi[k], o);
      if (lane >= o) llo[k] = fminf(llo[k], ul), lhi[k] = fmaxf(lhi[k], uh);
      if (lane + o < kSahBins) rlo[k] = fminf(rlo[k], dl), rhi[k] = fmaxf(rhi[k], dh);
    }
  }
  // the right side of split b is bins b+1..31
  const float right_area = __shfl_down_sync(0xffffffffu, BoxArea(rlo, rhi), 1);
  const int right_n = __shfl_down_sync(0xffffffffu, rn, 1);
  float cost = INFINITY;
  if (lane < kSahBins - 1 && ln != 0 && right_n != 0)
    cost = __fadd_rn(__fmul_rn(BoxArea(llo, lhi), __int2float_rn(ln)),
                     __fmul_rn(right_area, __int2float_rn(right_n)));
  int bin = cost < INFINITY ? lane : kSahBins;
  for (int o = 16; o > 0; o >>= 1) {
    const float oc = __shfl_xor_sync(0xffffffffu, cost, o);
    const int ob = __shfl_xor_sync(0xffffffffu, bin, o);
    if (oc < cost || (oc == cost && ob < bin)) cost = oc, bin = ob;
  }
  *best_cost = cost;
  *best_bin = bin < kSahBins ? bin : -1;
}

// Evaluates a node of n >= 2 references from its bins (all 32 lanes call;
// lane b reads bin b). Decision as in Builder::Build / SplitSah.
__device__ NodeSplit EvaluateNode(const uint32_t *bins, const PendingNode &nd, int max_leaf, int lane) {
  NodeSplit s;
  const int n = nd.end - nd.start;
  {
    // the node box: the union of every bin of axis 0
    const uint32_t *x = bins + lane * kBinWords;
    const bool full = x[0] != 0u;
    for (int k = 0; k < 3; ++k) {
      s.lo[k] = WarpMin(full ? KeyFloat(x[1 + k]) : INFINITY);
      s.hi[k] = WarpMax(full ? KeyFloat(x[4 + k]) : -INFINITY);
    }
  }
  float best_cost = INFINITY;
  int best_axis = -1, best_bin = -1;
  for (int a = 0; a < 3; ++a) {
    if (!(__fsub_rn(nd.chi[a], nd.clo[a]) > 0.0f)) continue;
    float c;
    int b;
    SweepAxis(bins + a * kSahBins * kBinWords, lane, &c, &b);
    if (b >= 0 && c < best_cost) best_cost = c, best_axis = a, best_bin = b;
  }
  s.bin = best_bin;
  if (best_axis < 0) {
    s.axis = n <= max_leaf ? -1 : -2;
  } else {
    const float parent_area = BoxArea(s.lo, s.hi);
    const float split_cost = __fadd_rn(1.0f, __fdiv_rn(__fmul_rn(1.0f, best_cost), fmaxf(parent_area, 1e-30f)));
    const float leaf_cost = __fmul_rn(1.0f, __int2float_rn(n));
    s.axis = (n <= max_leaf && leaf_cost <= split_cost) ? -1 : best_axis;
  }
  if (s.axis >= 0) {
    const uint32_t *x = bins + (s.axis * kSahBins + lane) * kBinWords;
    const bool full = x[0] != 0u, left = lane <= s.bin;
    s.left_n = WarpSum(left ? static_cast<int>(x[0]) : 0);
    for (int k = 0; k < 3; ++k) {
      const float cl = full ? KeyFloat(x[7 + k]) : INFINITY, ch = full ? KeyFloat(x[10 + k]) : -INFINITY;
      s.lclo[k] = WarpMin(left ? cl : INFINITY);
      s.lchi[k] = WarpMax(left ? ch : -INFINITY);
      s.rclo[k] = WarpMin(left ? INFINITY : cl);
      s.rchi[k] = WarpMax(left ? -INFINITY : ch);
    }
  } else {
    // a leaf, or halves by position when every centroid coincides (the
    // halves keep the node's centroid bounds)
    s.left_n = n / 2;
    for (int k = 0; k < 3; ++k) s.lclo[k] = s.rclo[k] = nd.clo[k], s.lchi[k] = s.rchi[k] = nd.chi[k];
  }
  return s;
}

// Writes a child's padded box and link into slot (parent & 1) of sparse
// entry parent >> 1 (the padding of the host builder's Pad).
__device__ void WriteSlot(BvhNode *sparse, int parent, const float *lo, const float *hi, int link) {
  float plo[3], phi[3];
  for (int k = 0; k < 3; ++k) {
    if (!(lo[k] <= hi[k])) {
      plo[k] = lo[k], phi[k] = hi[k];
      continue;
    }
    const float m = __fadd_rn(fmaxf(fabsf(lo[k]), fabsf(hi[k])), __fsub_rn(hi[k], lo[k]));
    const float e = __fadd_rn(__fmul_rn(m, 4e-7f), 1e-30f);
    plo[k] = __fsub_rn(lo[k], e);
    phi[k] = __fadd_rn(hi[k], e);
  }
  BvhNode &nd = sparse[parent >> 1];
  if ((parent & 1) == 0) {
    nd.a = F4{plo[0], phi[0], plo[1], phi[1]};
    nd.c.x = plo[2], nd.c.y = phi[2];
    nd.d.x = link;
  } else {
    nd.b = F4{plo[0], phi[0], plo[1], phi[1]};
    nd.c.z = plo[2], nd.c.w = phi[2];
    nd.d.y = link;
  }
}

// Lane 0: records a decided node (leaf or interior) and returns the
// children to build (false for a leaf).
__device__ bool EmitNode(const PendingNode &nd, const NodeSplit &s, BvhNode *sparse, int *used, uint8_t *last,
                         SahStats *st, PendingNode *left, PendingNode *right) {
  atomicMax(&st->max_depth, nd.depth);
  if (s.axis == -1) {
    WriteSlot(sparse, nd.parent, s.lo, s.hi, ~nd.start);
    last[nd.end - 1] = 1;
    atomicAdd(&st->leaves, 1ull);
    atomicMax(&st->max_leaf, nd.end - nd.start);
    return false;
  }
  const int mid = nd.start + s.left_n;
  const int p = mid - 1;
  used[p] = 1;
  WriteSlot(sparse, nd.parent, s.lo, s.hi, p);
  *left = PendingNode{nd.start, mid, 2 * p, nd.depth + 1, {s.lclo[0], s.lclo[1], s.lclo[2]},
                      {s.lchi[0], s.lchi[1], s.lchi[2]}};
  *right = PendingNode{mid, nd.end, 2 * p + 1, nd.depth + 1, {s.rclo[0], s.rclo[1], s.rclo[2]},
                       {s.rchi[0], s.rchi[1], s.rchi[2]}};
  return true;
}

__device__ __forceinline__ Decision MakeDecision(const PendingNode &nd, const NodeSplit &s) {
  Decision d{};
  d.axis = s.axis;
  d.bin = s.bin;
  d.mid = nd.start + s.left_n;
  if (s.axis >= 0) {
    d.lo = nd.clo[s.axis];
    d.scale = BinScale(nd.clo[s.axis], nd.chi[s.axis]);
  }
  return d;
}

// Whether reference `ref` goes to the left child (false for a value that is
// not a reference; the binning pass flags those).
__device__ __forceinline__ bool GoesLeft(const Decision &d, const float4 *box8, int n, int ref) {
  if (static_cast<unsigned>(ref) >= static_cast<unsigned>(n)) return false;
  const float4 a = __ldg(box8 + 2 * ref), b = __ldg(box8 + 2 * ref + 1);
  const float lo = d.axis == 0 ? a.x : (d.axis == 1 ? a.y : a.z);
  const float hi = d.axis == 0 ? b.x : (d.axis == 1 ? b.y : b.z);
  return BinOf(Centroid(lo, hi), d.lo, d.scale) <= d.bin;
}

// Boxes into two float4s per reference, the identity reference order, and
// the root's centroid bounds (order-preserving keys, min then max).
__global__ void PackKernel(const float *boxes, int n, float4 *box8, int32_t *idx, unsigned *cbounds) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  if (i < n) {
    const float *b = boxes + 6 * static_cast<int64_t>(i);
    box8[2 * i] = make_float4(b[0], b[1], b[2], 0.0f);
    box8[2 * i + 1] = make_float4(b[3], b[4], b[5], 0.0f);
    idx[i] = i;
    for (int k = 0; k < 3; ++k) lo[k] = hi[k] = FloatKey(Centroid(b[k], b[3 + k]));
  }
  for (int k = 0; k < 3; ++k) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0 && i - static_cast<int>(threadIdx.x & 31) < n) {
    for (int k = 0; k < 3; ++k) atomicMin(cbounds + k, lo[k]), atomicMax(cbounds + 3 + k, hi[k]);
  }
}

// The root as a pending node: all references, the virtual parent slot
// (sparse entry n - 1), its centroid bounds; into the level list or, when it
// is small, the small list.
__global__ void RootKernel(int n, const unsigned *cbounds, PendingNode *level, PendingNode *small, SahStats *st) {
  PendingNode r{};
  r.start = 0;
  r.end = n;
  r.parent = 2 * (n - 1);
  r.depth = 0;
  for (int k = 0; k < 3; ++k) r.clo[k] = KeyFloat(cbounds[k]), r.chi[k] = KeyFloat(cbounds[3 + k]);
  if (n >= kSmallRefs) {
    level[0] = r;
    st->next_count = 1;
  } else {
    small[0] = r;
    st->small_count = 1;
  }
}

__global__ void InitBinsKernel(uint32_t *bins, int nodes) {
  const int64_t w = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (w >= static_cast<int64_t>(nodes) * kNodeBinWords) return;
  const int f = static_cast<int>(w % kBinWords);
  bins[w] = f == 0 ? 0u : ((f >= 1 && f <= 3) || (f >= 7 && f <= 9) ? 0xffffffffu : 0u);
}

// One block per work item (level node, chunk of up to kChunk references).
__global__ void __launch_bounds__(kLevelThreads) LevelBinKernel(const float4 *box8, const int32_t *idx, int n,
                                                                 const PendingNode *level, const int2 *work,
                                                                 uint32_t *bins, SahStats *st) {
  __shared__ uint32_t sb[kNodeBinWords];
  const int2 w = work[blockIdx.x];
  const PendingNode nd = level[w.x];
  InitBins(sb, threadIdx.x, kLevelThreads);
  float scale[3];
  for (int k = 0; k < 3; ++k) scale[k] = BinScale(nd.clo[k], nd.chi[k]);
  __syncthreads();
  const int end = min(w.y + kChunk, nd.end);
  for (int i = w.y + threadIdx.x; i < end; i += kLevelThreads) {
    const int ref = idx[i];
    if (static_cast<unsigned>(ref) >= static_cast<unsigned>(n)) {
      atomicExch(&st->error, 5);  // not a reference: the partition went wrong
      continue;
    }
    float lo[3], hi[3];
    LoadRef(box8, ref, lo, hi);
    BinRef(sb, lo, hi, nd.clo, scale);
  }
  __syncthreads();
  FlushBins(sb, bins + static_cast<int64_t>(w.x) * kNodeBinWords, threadIdx.x, kLevelThreads);
}

// One warp per level node: decide, record, queue the children.
__global__ void LevelSplitKernel(const PendingNode *level, int m, const uint32_t *bins, int max_leaf, Decision *dec,
                                 BvhNode *sparse, int *used, uint8_t *last, PendingNode *next, int next_cap,
                                 PendingNode *small, int small_cap, SahStats *st) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= m) return;
  const PendingNode nd = level[warp];
  const NodeSplit s = EvaluateNode(bins + static_cast<int64_t>(warp) * kNodeBinWords, nd, max_leaf, lane);
  if (lane != 0) return;
  dec[warp] = MakeDecision(nd, s);
  PendingNode kids[2];
  if (!EmitNode(nd, s, sparse, used, last, st, &kids[0], &kids[1])) return;
  for (const PendingNode &k : kids) {
    if (k.end - k.start >= kSmallRefs) {
      const int at = atomicAdd(&st->next_count, 1);
      if (at < next_cap) next[at] = k;
      else atomicExch(&st->error, 2);
    } else {
      const int at = atomicAdd(&st->small_count, 1);
      if (at < small_cap) small[at] = k;
      else atomicExch(&st->error, 3);
    }
  }
}

// Block-wide exclusive scan of one int per thread (kLevelThreads threads);
// returns the thread's prefix and sets *total.
__device__ int BlockExclusiveScan(int v, int *total) {
  __shared__ int warp_sums[kLevelThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[w] = x;
  __syncthreads();
  int before = 0, all = 0;
  for (int k = 0; k < kLevelThreads / 32; ++k) {
    const int s = warp_sums[k];
    if (k < w) before += s;
    all += s;
  }
  __syncthreads();
  *total = all;
  return before + x - v;
}

constexpr int kPerThread = kChunk / kLevelThreads;

// References that go left in each work item's chunk.
__global__ void __launch_bounds__(kLevelThreads) LevelCountKernel(const float4 *box8, const int32_t *idx, int n,
                                                                   const PendingNode *level, const Decision *dec,
                                                                   const int2 *work, int *chunk_left) {
  const int2 w = work[blockIdx.x];
  const Decision d = dec[w.x];
  if (d.axis < 0) return;
  const int end = min(w.y + kChunk, level[w.x].end);
  int c = 0;
  for (int i = w.y + threadIdx.x; i < end; i += kLevelThreads) c += GoesLeft(d, box8, n, idx[i]) ? 1 : 0;
  int total = 0;
  BlockExclusiveScan(c, &total);
  if (threadIdx.x == 0) chunk_left[blockIdx.x] = total;
}

// Per level node, the exclusive prefix of its chunks' left counts (its work
// items are first[j] .. first[j + 1] - 1).
__global__ void LevelScanKernel(const Decision *dec, int m, const int *first, int *chunk_left) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m || dec[j].axis < 0) return;
  int acc = 0;
  for (int w = first[j]; w < first[j + 1]; ++w) {
    const int c = chunk_left[w];
    chunk_left[w] = acc;
    acc += c;
  }
}

// Stable partition of each chunk into tmp: thread t holds references
// [w.y + kPerThread t, + kPerThread); left and right counts packed in one
// scan (a chunk holds fewer than 65,536 references).
__global__ void __launch_bounds__(kLevelThreads) LevelScatterKernel(const float4 *box8, const int32_t *idx, int n,
                                                                     int32_t *tmp, const PendingNode *level,
                                                                     const Decision *dec, const int2 *work,
                                                                     const int *chunk_left, SahStats *st) {
  const int2 w = work[blockIdx.x];
  const Decision d = dec[w.x];
  if (d.axis < 0) return;
  const PendingNode nd = level[w.x];
  const int end = min(w.y + kChunk, nd.end);
  const int i0 = w.y + threadIdx.x * kPerThread;
  int ref[kPerThread];
  unsigned left_mask = 0;
  int nl = 0, nr = 0;
  for (int k = 0; k < kPerThread; ++k) {
    const int i = i0 + k;
    ref[k] = -1;
    if (i < end) {
      ref[k] = idx[i];
      if (GoesLeft(d, box8, n, ref[k])) left_mask |= 1u << k, ++nl;
      else ++nr;
    }
  }
  int total = 0;
  const int before = BlockExclusiveScan(nl | (nr << 16), &total);
  int l = nd.start + chunk_left[blockIdx.x] + (before & 0xffff);
  int r = d.mid + (w.y - nd.start - chunk_left[blockIdx.x]) + (before >> 16);
  for (int k = 0; k < kPerThread; ++k) {
    if (ref[k] < 0) continue;
    const bool left = (left_mask & (1u << k)) != 0;
    const int at = left ? l++ : r++;
    if (left ? (at < nd.start || at >= d.mid) : (at < d.mid || at >= nd.end)) {
      atomicExch(&st->error, 6);  // the counts and the bins disagree
      continue;
    }
    tmp[at] = ref[k];
  }
}

__global__ void __launch_bounds__(kLevelThreads) LevelCopyKernel(int32_t *idx, const int32_t *tmp,
                                                                  const PendingNode *level, const Decision *dec,
                                                                  const int2 *work) {
  const int2 w = work[blockIdx.x];
  if (dec[w.x].axis < 0) return;
  const int end = min(w.y + kChunk, level[w.x].end);
  for (int i = w.y + threadIdx.x; i < end; i += kLevelThreads) idx[i] = tmp[i];
}

// One level of the small-node phase: one warp per pending node (warps loop
// over the list), its children appended to the next level's list.
__global__ void __launch_bounds__(kSmallWarps * 32) SmallLevelKernel(const float4 *box8, int32_t *idx, int32_t *tmp,
                                                                      int n_refs, const PendingNode *in,
                                                                      const int *in_count, PendingNode *out,
                                                                      int *out_count, int cap, int max_leaf,
                                                                      BvhNode *sparse, int *used, uint8_t *last,
                                                                      SahStats *st) {
  __shared__ uint32_t bins_all[kSmallWarps][kNodeBinWords];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t *bins = bins_all[wid];
  const int count = min(*in_count, cap);
  const unsigned lt = (1u << lane) - 1u;
  for (int item = blockIdx.x * kSmallWarps + wid; item < count; item += gridDim.x * kSmallWarps) {
    const PendingNode nd = in[item];
    const int n = nd.end - nd.start;
    if (n < 1 || nd.start < 0 || nd.end > n_refs) {
      if (lane == 0) atomicExch(&st->error, 7);
      continue;
    }
    if (n == 1) {
      // Builder::Build makes a leaf of a single reference before any split
      const int ref = idx[nd.start];
      if (static_cast<unsigned>(ref) >= static_cast<unsigned>(n_refs)) {
        if (lane == 0) atomicExch(&st->error, 5);
        continue;
      }
      if (lane == 0) {
        float lo[3], hi[3];
        LoadRef(box8, ref, lo, hi);
        atomicMax(&st->max_depth, nd.depth);
        WriteSlot(sparse, nd.parent, lo, hi, ~nd.start);
        last[nd.start] = 1;
        atomicAdd(&st->leaves, 1ull);
        atomicMax(&st->max_leaf, 1);
      }
      continue;
    }
    __syncwarp();  // the previous node's bins have been read
    InitBins(bins, lane, 32);
    float scale[3];
    for (int k = 0; k < 3; ++k) scale[k] = BinScale(nd.clo[k], nd.chi[k]);
    __syncwarp();
    bool bad = false;
    for (int i = nd.start + lane; i < nd.end; i += 32) {
      const int ref = idx[i];
      if (static_cast<unsigned>(ref) >= static_cast<unsigned>(n_refs)) {
        bad = true;
        continue;
      }
      float lo[3], hi[3];
      LoadRef(box8, ref, lo, hi);
      BinRef(bins, lo, hi, nd.clo, scale);
    }
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) atomicExch(&st->error, 5);
      continue;
    }
    __syncwarp();
    const NodeSplit s = EvaluateNode(bins, nd, max_leaf, lane);
    PendingNode kids[2];
    bool split = false;
    if (lane == 0) split = EmitNode(nd, s, sparse, used, last, st, &kids[0], &kids[1]);
    split = __shfl_sync(0xffffffffu, split, 0);
    if (!split) continue;
    if (s.axis >= 0) {
      const Decision d = MakeDecision(nd, s);
      int nl = 0, nr = 0;
      for (int base = nd.start; base < nd.end; base += 32) {
        const int i = base + lane;
        const bool valid = i < nd.end;
        const int ref = valid ? idx[i] : 0;
        const bool left = valid && GoesLeft(d, box8, n_refs, ref);
        const unsigned lm = __ballot_sync(0xffffffffu, left), rm = __ballot_sync(0xffffffffu, valid && !left);
        const int at = left ? nd.start + nl + __popc(lm & lt) : d.mid + nr + __popc(rm & lt);
        if (valid) {
          if (left ? at < d.mid : at < nd.end) tmp[at] = ref;
          else atomicExch(&st->error, 6);
        }
        nl += __popc(lm);
        nr += __popc(rm);
      }
      __syncwarp();
      for (int i = nd.start + lane; i < nd.end; i += 32) idx[i] = tmp[i];
    }
    if (lane == 0) {
      const int at = atomicAdd(out_count, 2);
      if (at + 2 <= cap) {
        out[at] = kids[0];
        out[at + 1] = kids[1];
      } else {
        atomicExch(&st->error, 3);
      }
    }
  }
}

// Interior children per sparse entry (0 for positions that hold no node).
__global__ void ChildCountKernel(const BvhNode *sparse, const int *used, int n, int *kids) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n - 1) return;
  const BvhNode &nd = sparse[p];
  kids[p] = used[p] ? (nd.d.x >= 0 ? 1 : 0) + (nd.d.y >= 0 ? 1 : 0) : 0;
}

// Interior nodes into dense numbering: the root at 0, then the interior
// children of each node side by side (so one 128-byte line holds a pair of
// siblings), pairs in the order of their parents' split positions (`base`:
// exclusive scan of the child counts). Each node's thread writes its
// children; entry n - 1 of the sparse array is the root's virtual parent,
// whose slot 0 holds the root's box and link.
__global__ void DenseKernel(const BvhNode *sparse, const int *used, const int *base, int n, BvhNode *nodes) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const BvhNode &top = sparse[n - 1];
  const int root = top.d.x;
  if (root < 0) {
    // a single leaf: both slots hold it (as the host builder emits it)
    if (p == 0) {
      BvhNode nd{};
      nd.a = top.a;
      nd.b = top.a;
      nd.c = F4{top.c.x, top.c.y, top.c.x, top.c.y};
      nd.d = I4{root, root, 0, 0};
      nodes[0] = nd;
    }
    return;
  }
  auto renumbered = [&](int q) {
    BvhNode nd = sparse[q];
    int k = 0;
    if (nd.d.x >= 0) nd.d.x = 1 + base[q] + k++;
    if (nd.d.y >= 0) nd.d.y = 1 + base[q] + k++;
    nd.d.z = nd.d.w = 0;
    return nd;
  };
  if (p == 0) nodes[0] = renumbered(root);
  if (p >= n - 1 || !used[p]) return;
  const BvhNode &nd = sparse[p];
  int k = 0;
  if (nd.d.x >= 0) nodes[1 + base[p] + k++] = renumbered(nd.d.x);
  if (nd.d.y >= 0) nodes[1 + base[p] + k++] = renumbered(nd.d.y);
}

}  // namespace

namespace {

__global__ void CountKernel(const BvhNode *sparse, const int *kids, const int *base, int n, SahStats *st) {
  const int root = sparse[n - 1].d.x;
  st->root = root;
  st->next_count = root < 0 ? 1 : 1 + base[n - 2] + kids[n - 2];  // interior nodes
}

struct SahBuffers {
  float4 *box8 = nullptr;
  int32_t *tmp = nullptr;
  BvhNode *sparse = nullptr;
  int *used = nullptr, *rank = nullptr;
  PendingNode *level[2] = {nullptr, nullptr}, *small = nullptr, *small2 = nullptr;
  int *qcount = nullptr;  // the two small-node lists' lengths
  uint32_t *bins = nullptr;
  Decision *dec = nullptr;
  int2 *work = nullptr;
  int *chunk_left = nullptr, *first = nullptr;
  SahStats *st = nullptr;
  unsigned *cbounds = nullptr;
  void *scan_temp = nullptr;
  size_t scan_bytes = 0;
  int level_cap = 0, small_cap = 0, work_cap = 0;
};

// Places the buffers in `base` (nullptr: only sizes them); returns the bytes.
size_t Carve(int n, char *base, SahBuffers *b) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    char *p = base ? base + off : nullptr;
    off += (bytes + 255) / 256 * 256;
    return p;
  };
  const size_t m = static_cast<size_t>(std::max(n, 1));
  // level nodes are disjoint and hold >= kSmallRefs references each; small
  // nodes are disjoint and non-empty
  b->level_cap = n / kSmallRefs + 2;
  b->small_cap = n + 1;
  b->work_cap = n / kChunk + b->level_cap + 1;
  b->box8 = reinterpret_cast<float4 *>(take(32 * m));
  b->tmp = reinterpret_cast<int32_t *>(take(4 * m));
  b->sparse = reinterpret_cast<BvhNode *>(take(sizeof(BvhNode) * m));
  b->used = reinterpret_cast<int *>(take(4 * m));
  b->rank = reinterpret_cast<int *>(take(4 * m));
  for (int k = 0; k < 2; ++k) b->level[k] = reinterpret_cast<PendingNode *>(take(sizeof(PendingNode) * b->level_cap));
  b->small = reinterpret_cast<PendingNode *>(take(sizeof(PendingNode) * b->small_cap));
  b->small2 = reinterpret_cast<PendingNode *>(take(sizeof(PendingNode) * b->small_cap));
  b->qcount = reinterpret_cast<int *>(take(2 * sizeof(int)));
  b->bins = reinterpret_cast<uint32_t *>(take(4ull * kNodeBinWords * b->level_cap));
  b->dec = reinterpret_cast<Decision *>(take(sizeof(Decision) * b->level_cap));
  b->work = reinterpret_cast<int2 *>(take(sizeof(int2) * b->work_cap));
  b->chunk_left = reinterpret_cast<int *>(take(4ull * b->work_cap));
  b->first = reinterpret_cast<int *>(take(4ull * (b->level_cap + 1)));
  b->st = reinterpret_cast<SahStats *>(take(sizeof(SahStats)));
  b->cbounds = reinterpret_cast<unsigned *>(take(6 * sizeof(unsigned)));
  b->scan_bytes = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, b->scan_bytes, static_cast<const int *>(nullptr), static_cast<int *>(nullptr),
                                std::max(n - 1, 1));
  b->scan_temp = take(b->scan_bytes);
  return off;
}

}  // namespace

size_t GpuSahScratchBytes(int n) {
  SahBuffers b;
  return Carve(n, nullptr, &b);
}

#define SAH_TRY(expr)                      \
  do {                                     \
    const cudaError_t _e = (expr);         \
    if (_e != cudaSuccess) return _e;      \
  } while (0)

cudaError_t BuildGpuSah(const float *boxes, int n, int max_leaf, void *scratch, BvhNode *nodes, int32_t *order,
                        uint8_t *last, GpuSahResult *res, cudaStream_t st) {
  *res = GpuSahResult{};
  if (n <= 0) return cudaSuccess;
  max_leaf = std::max(max_leaf, 1);
  SahBuffers b;
  Carve(n, static_cast<char *>(scratch), &b);
  int device = 0, sms = 1;
  SAH_TRY(cudaGetDevice(&device));
  SAH_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  const unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  SAH_TRY(cudaMemcpyAsync(b.cbounds, init, sizeof(init), cudaMemcpyHostToDevice, st));
  SAH_TRY(cudaMemsetAsync(b.st, 0, sizeof(SahStats), st));
  SAH_TRY(cudaMemsetAsync(last, 0, static_cast<size_t>(n), st));
  SAH_TRY(cudaMemsetAsync(b.used, 0, 4ull * n, st));
  SAH_TRY(cudaMemsetAsync(b.sparse, 0, sizeof(BvhNode) * static_cast<size_t>(n), st));
  PackKernel<<<Blocks(n, 256), 256, 0, st>>>(boxes, n, b.box8, order, b.cbounds);
  RootKernel<<<1, 1, 0, st>>>(n, b.cbounds, b.level[0], b.small, b.st);
  SAH_TRY(cudaGetLastError());
  SahStats h{};
  SAH_TRY(cudaMemcpyAsync(&h, b.st, sizeof(h), cudaMemcpyDeviceToHost, st));
  SAH_TRY(cudaStreamSynchronize(st));
  std::vector<PendingNode> lv;
  std::vector<int2> work;
  std::vector<int> first;
  int m = h.next_count, cur = 0;
  for (int level = 0; m > 0; ++level) {
    if (level >= kMaxLevels || m > b.level_cap) {
      res->error = 1;
      return cudaSuccess;
    }
    lv.resize(m);
    SAH_TRY(cudaMemcpyAsync(lv.data(), b.level[cur], sizeof(PendingNode) * m, cudaMemcpyDeviceToHost, st));
    SAH_TRY(cudaStreamSynchronize(st));
    work.clear();
    first.assign(m + 1, 0);
    for (int j = 0; j < m; ++j) {
      first[j] = static_cast<int>(work.size());
      for (int s = lv[j].start; s < lv[j].end; s += kChunk) work.push_back(make_int2(j, s));
    }
    first[m] = static_cast<int>(work.size());
    const int nw = first[m];
    if (nw > b.work_cap) {
      res->error = 1;
      return cudaSuccess;
    }
    SAH_TRY(cudaMemcpyAsync(b.work, work.data(), sizeof(int2) * nw, cudaMemcpyHostToDevice, st));
    SAH_TRY(cudaMemcpyAsync(b.first, first.data(), sizeof(int) * (m + 1), cudaMemcpyHostToDevice, st));
    SAH_TRY(cudaMemsetAsync(&b.st->next_count, 0, sizeof(int), st));
    InitBinsKernel<<<Blocks(static_cast<int64_t>(m) * kNodeBinWords, 256), 256, 0, st>>>(b.bins, m);
    LevelBinKernel<<<nw, kLevelThreads, 0, st>>>(b.box8, order, n, b.level[cur], b.work, b.bins, b.st);
    LevelSplitKernel<<<Blocks(static_cast<int64_t>(m) * 32, 128), 128, 0, st>>>(
        b.level[cur], m, b.bins, max_leaf, b.dec, b.sparse, b.used, last, b.level[cur ^ 1], b.level_cap, b.small,
        b.small_cap, b.st);
    LevelCountKernel<<<nw, kLevelThreads, 0, st>>>(b.box8, order, n, b.level[cur], b.dec, b.work, b.chunk_left);
    LevelScanKernel<<<Blocks(m, 128), 128, 0, st>>>(b.dec, m, b.first, b.chunk_left);
    LevelScatterKernel<<<nw, kLevelThreads, 0, st>>>(b.box8, order, n, b.tmp, b.level[cur], b.dec, b.work,
                                                       b.chunk_left, b.st);
    LevelCopyKernel<<<nw, kLevelThreads, 0, st>>>(order, b.tmp, b.level[cur], b.dec, b.work);
    SAH_TRY(cudaGetLastError());
    SAH_TRY(cudaMemcpyAsync(&h, b.st, sizeof(h), cudaMemcpyDeviceToHost, st));
    SAH_TRY(cudaStreamSynchronize(st));
    if (h.error) {
      res->error = h.error;
      return cudaSuccess;
    }
    m = h.next_count;
    cur ^= 1;
  }
  // the small-node phase, level by level; the queue is read back every few
  // levels (a level with nothing to do costs one short launch)
  if (h.small_count > 0) {
    PendingNode *lists[2] = {b.small, b.small2};
    SAH_TRY(cudaMemcpyAsync(b.qcount, &b.st->small_count, sizeof(int), cudaMemcpyDeviceToDevice, st));
    const unsigned grid = static_cast<unsigned>(sms) * 8u;
    int q = 0;
    for (int level = 0;; ++level) {
      if (level >= kMaxSmallLevels) {
        res->error = 1;
        return cudaSuccess;
      }
      SAH_TRY(cudaMemsetAsync(b.qcount + (q ^ 1), 0, sizeof(int), st));
      SmallLevelKernel<<<grid, kSmallWarps * 32, 0, st>>>(b.box8, order, b.tmp, n, lists[q], b.qcount + q,
                                                          lists[q ^ 1], b.qcount + (q ^ 1), b.small_cap, max_leaf,
                                                          b.sparse, b.used, last, b.st);
      q ^= 1;
      if (level % kSmallLevelsPerCheck == kSmallLevelsPerCheck - 1) {
        int pending = 0;
        SAH_TRY(cudaGetLastError());
        SAH_TRY(cudaMemcpyAsync(&pending, b.qcount + q, sizeof(int), cudaMemcpyDeviceToHost, st));
        SAH_TRY(cudaStreamSynchronize(st));
        if (pending == 0) break;
      }
    }
  }
  // b.tmp holds the child counts, b.rank their exclusive scan
  if (n >= 2) {
    ChildCountKernel<<<Blocks(n - 1, 256), 256, 0, st>>>(b.sparse, b.used, n, b.tmp);
    SAH_TRY(cub::DeviceScan::ExclusiveSum(b.scan_temp, b.scan_bytes, b.tmp, b.rank, n - 1, st));
  }
  DenseKernel<<<Blocks(std::max(n - 1, 1), 256), 256, 0, st>>>(b.sparse, b.used, b.rank, n, nodes);
  CountKernel<<<1, 1, 0, st>>>(b.sparse, b.tmp, b.rank, n, b.st);
  SAH_TRY(cudaGetLastError());
  SAH_TRY(cudaMemcpyAsync(&h, b.st, sizeof(h), cudaMemcpyDeviceToHost, st));
  SAH_TRY(cudaStreamSynchronize(st));
  res->error = h.error;
  res->nodes = h.next_count;
  res->leaves = static_cast<int64_t>(h.leaves);
  res->max_depth = h.max_depth;
  res->max_leaf = h.max_leaf;
  return cudaSuccess;
}

}  // namespace muon_gpu
