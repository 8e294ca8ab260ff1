// BVH construction on the GPU: a linear BVH over Morton-ordered primitive
// centroids (Karras, "Maximizing Parallelism in the Construction of BVHs,
// Octrees, and k-d Trees", HPG 2012), with subtrees of at most kMaxLeaf
// primitives collapsed into leaves, emitted directly in the two-child node
// layout the traversal kernels read.
//
// Steps, all on the device: centroid bounds; 64-bit keys (30-bit Morton code
// of the centroid, primitive index below it, so keys are unique); radix sort
// of the keys (CUB); one thread per internal node finds its key range and
// split (the common-prefix search of Karras); boxes bottom-up, the second of
// two children to arrive at a node computing its box; nodes and leaf-end
// flags emitted by every internal node whose range holds more than kMaxLeaf
// primitives. Primitive records are then gathered into the sorted (leaf)
// order.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>

#include <cstdint>

#include "bvh_build.h"

namespace muon_gpu {

namespace {

constexpr int kMaxLeaf = 4;
constexpr int kThreads = 256;

inline unsigned Grid(int64_t n) { return static_cast<unsigned>((n + kThreads - 1) / kThreads); }

// Order-preserving map of a float to an unsigned integer, for atomic min/max.
__device__ __forceinline__ unsigned FloatKey(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float KeyFloat(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__global__ void BoundsKernel(const float *boxes, int n, unsigned *bounds) {
  __shared__ unsigned lo[3][kThreads], hi[3][kThreads];
  const int i = blockIdx.x * kThreads + threadIdx.x;
  for (int k = 0; k < 3; ++k) {
    unsigned l = 0xffffffffu, h = 0u;
    if (i < n) {
      const float c = 0.5f * (boxes[6 * i + k] + boxes[6 * i + 3 + k]);
      l = h = FloatKey(c);
    }
    lo[k][threadIdx.x] = l;
    hi[k][threadIdx.x] = h;
  }
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o)
      for (int k = 0; k < 3; ++k) {
        lo[k][threadIdx.x] = min(lo[k][threadIdx.x], lo[k][threadIdx.x + o]);
        hi[k][threadIdx.x] = max(hi[k][threadIdx.x], hi[k][threadIdx.x + o]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) {
      atomicMin(bounds + k, lo[k][0]);
      atomicMax(bounds + 3 + k, hi[k][0]);
    }
}

// 10 bits of v spread to every third bit.
__device__ __forceinline__ uint32_t Spread3(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void MortonKernel(const float *boxes, int n, const unsigned *bounds, uint64_t *keys) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  uint32_t q[3];
  for (int k = 0; k < 3; ++k) {
    const float lo = KeyFloat(bounds[k]), hi = KeyFloat(bounds[3 + k]);
    const float c = 0.5f * (boxes[6 * i + k] + boxes[6 * i + 3 + k]);
    const float u = hi > lo ? (c - lo) / (hi - lo) : 0.5f;
    q[k] = static_cast<uint32_t>(fminf(fmaxf(u * 1024.0f, 0.0f), 1023.0f));
  }
  const uint32_t code = (Spread3(q[0]) << 2) | (Spread3(q[1]) << 1) | Spread3(q[2]);
  keys[i] = (static_cast<uint64_t>(code) << 32) | static_cast<uint32_t>(i);
}

// Length of the common prefix of sorted keys i and j; -1 when j is out of
// range.
__device__ __forceinline__ int Delta(const uint64_t *keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(static_cast<long long>(keys[i] ^ keys[j]));
}

// Karras 2012, section 4: the range and split of internal node i. Children
// are coded as >= 0 internal node, < 0 leaf ~slot.
__global__ void HierarchyKernel(const uint64_t *keys, int n, int2 *children, int2 *range, int *parent_inner,
                                int *parent_leaf) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (Delta(keys, n, i, i + 1) - Delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = Delta(keys, n, i, i - d);
  int lmax = 2;
  while (Delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (Delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = Delta(keys, n, i, j);
  int s = 0;
  int t = l;
  do {
    t = (t + 1) >> 1;
    if (Delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int gamma = i + s * d + min(d, 0);
  const int first = min(i, j), last = max(i, j);
  const int left = (first == gamma) ? ~gamma : gamma;
  const int right = (last == gamma + 1) ? ~(gamma + 1) : gamma + 1;
  children[i] = make_int2(left, right);
  range[i] = make_int2(first, last);
  if (left >= 0) parent_inner[left] = i;
  else parent_leaf[~left] = i;
  if (right >= 0) parent_inner[right] = i;
  else parent_leaf[~right] = i;
}

__device__ __forceinline__ void LoadBox(const float *b, float *lo, float *hi) {
  for (int k = 0; k < 3; ++k) lo[k] = b[k], hi[k] = b[3 + k];
}
// Boxes another thread may have written during this kernel: read from L2.
__device__ __forceinline__ void LoadBoxCg(const float *b, float *lo, float *hi) {
  for (int k = 0; k < 3; ++k) lo[k] = __ldcg(b + k), hi[k] = __ldcg(b + 3 + k);
}

// Bottom-up boxes: each leaf climbs; at every node the second arrival
// computes the union of the two child boxes and climbs on.
__global__ void BoxesKernel(const float *boxes, const uint64_t *keys, int n, const int2 *children,
                            const int *parent_inner, const int *parent_leaf, float *inner_boxes, int *arrivals) {
  const int s = blockIdx.x * kThreads + threadIdx.x;
  if (s >= n) return;
  int node = parent_leaf[s];
  // bounded climb (the depth of a tree over 62-bit keys is below 64)
  for (int step = 0; step < 128 && node >= 0 && node < n - 1; ++step) {
    __threadfence();
    if (atomicAdd(arrivals + node, 1) == 0) return;  // the sibling is not done yet
    __threadfence();
    const int2 c = children[node];
    float lo[3], hi[3], lo2[3], hi2[3];
    if (c.x >= 0) LoadBoxCg(inner_boxes + 6 * c.x, lo, hi);
    else LoadBox(boxes + 6 * static_cast<uint32_t>(keys[~c.x]), lo, hi);
    if (c.y >= 0) LoadBoxCg(inner_boxes + 6 * c.y, lo2, hi2);
    else LoadBox(boxes + 6 * static_cast<uint32_t>(keys[~c.y]), lo2, hi2);
    float *out = inner_boxes + 6 * node;
    for (int k = 0; k < 3; ++k) {
      out[k] = fminf(lo[k], lo2[k]);
      out[3 + k] = fmaxf(hi[k], hi2[k]);
    }
    node = node == 0 ? -1 : parent_inner[node];
  }
}

// The child slot `slot` of a node: its box (padded like the host builder's)
// and its link.
__device__ __forceinline__ void SetChild(BvhNode &nd, int slot, const float *lo, const float *hi, int link) {
  float plo[3], phi[3];
  for (int k = 0; k < 3; ++k) {
    const float m = fmaxf(fabsf(lo[k]), fabsf(hi[k])) + (hi[k] - lo[k]);
    const float e = m * 4e-7f + 1e-30f;
    plo[k] = lo[k] - e;
    phi[k] = hi[k] + e;
  }
  if (slot == 0) {
    nd.a = F4{plo[0], phi[0], plo[1], phi[1]};
    nd.c.x = plo[2], nd.c.y = phi[2];
    nd.d.x = link;
  } else {
    nd.b = F4{plo[0], phi[0], plo[1], phi[1]};
    nd.c.z = plo[2], nd.c.w = phi[2];
    nd.d.y = link;
  }
}

// Nodes whose range exceeds kMaxLeaf primitives emit their two children: a
// leaf (single primitive or a whole small subtree, contiguous in sorted
// order) or an interior node. Every primitive lies in exactly one emitted
// leaf, whose last slot is flagged.
__global__ void EmitKernel(const float *boxes, const uint64_t *keys, int n, const int2 *children, const int2 *range,
                           const float *inner_boxes, BvhNode *nodes, uint8_t *last) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n - 1) return;
  const int2 r = range[i];
  if (r.y - r.x + 1 <= kMaxLeaf && i != 0) return;  // inside a collapsed leaf
  const int2 c = children[i];
  BvhNode nd{};
  const int kids[2] = {c.x, c.y};
  for (int k = 0; k < 2; ++k) {
    float lo[3], hi[3];
    int link;
    if (kids[k] < 0) {
      const int slot = ~kids[k];
      LoadBox(boxes + 6 * static_cast<uint32_t>(keys[slot]), lo, hi);
      link = ~slot;
      last[slot] = 1;
    } else {
      const int2 cr = range[kids[k]];
      LoadBox(inner_boxes + 6 * kids[k], lo, hi);
      if (cr.y - cr.x + 1 <= kMaxLeaf) {
        link = ~cr.x;
        last[cr.y] = 1;
      } else {
        link = kids[k];
      }
    }
    SetChild(nd, k, lo, hi, link);
  }
  nodes[i] = nd;
}

// Root of a tree of n <= kMaxLeaf primitives: one leaf in both slots (the
// traversal ends at an empty link, and a second test of a leaf cannot change
// a closest hit).
__global__ void SmallRootKernel(const float *boxes, int n, BvhNode *nodes, uint8_t *last) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) lo[k] = fminf(lo[k], boxes[6 * i + k]), hi[k] = fmaxf(hi[k], boxes[6 * i + 3 + k]);
  BvhNode nd{};
  SetChild(nd, 0, lo, hi, ~0);
  SetChild(nd, 1, lo, hi, ~0);
  nodes[0] = nd;
  last[n - 1] = 1;
}

__global__ void OrderKernel(const uint64_t *keys, int n, int32_t *order) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < n) order[i] = static_cast<int32_t>(keys[i] & 0xffffffffu);
}

}  // namespace

size_t GpuLbvhScratchBytes(int n) {
  size_t temp = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, temp, static_cast<const uint64_t *>(nullptr),
                                 static_cast<uint64_t *>(nullptr), n, 0, 62);
  const size_t m = static_cast<size_t>(n);
  return 256 * 16 + temp + 2 * m * 8 + m * 8 * 2 + m * 4 * 3 + m * 24 + 64;
}

void LaunchGpuLbvh(const float *boxes, int n, void *scratch, size_t scratch_bytes, BvhNode *nodes, int32_t *order,
                   uint8_t *last, cudaStream_t st) {
  char *p = static_cast<char *>(scratch);
  auto take = [&](size_t bytes) {
    char *r = p;
    p += (bytes + 255) / 256 * 256;
    return r;
  };
  const size_t m = static_cast<size_t>(n);
  unsigned *bounds = reinterpret_cast<unsigned *>(take(6 * sizeof(unsigned)));
  uint64_t *keys_in = reinterpret_cast<uint64_t *>(take(m * 8));
  uint64_t *keys = reinterpret_cast<uint64_t *>(take(m * 8));
  int2 *children = reinterpret_cast<int2 *>(take(m * 8));
  int2 *range = reinterpret_cast<int2 *>(take(m * 8));
  int *parent_inner = reinterpret_cast<int *>(take(m * 4));
  int *parent_leaf = reinterpret_cast<int *>(take(m * 4));
  int *arrivals = reinterpret_cast<int *>(take(m * 4));
  float *inner_boxes = reinterpret_cast<float *>(take(m * 24));
  size_t temp = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, temp, keys_in, keys, n, 0, 62, st);
  void *sort_temp = take(temp);
  (void)scratch_bytes;
  const unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  cudaMemcpyAsync(bounds, init, sizeof(init), cudaMemcpyHostToDevice, st);
  cudaMemsetAsync(last, 0, m, st);
  BoundsKernel<<<Grid(n), kThreads, 0, st>>>(boxes, n, bounds);
  MortonKernel<<<Grid(n), kThreads, 0, st>>>(boxes, n, bounds, keys_in);
  cub::DeviceRadixSort::SortKeys(sort_temp, temp, keys_in, keys, n, 0, 62, st);
  OrderKernel<<<Grid(n), kThreads, 0, st>>>(keys, n, order);
  if (n <= kMaxLeaf) {
    SmallRootKernel<<<1, 1, 0, st>>>(boxes, n, nodes, last);
    return;
  }
  cudaMemsetAsync(arrivals, 0, m * 4, st);
  cudaMemsetAsync(parent_inner, 0xff, m * 4, st);
  cudaMemsetAsync(parent_leaf, 0xff, m * 4, st);
  cudaMemsetAsync(nodes, 0, (m - 1) * sizeof(BvhNode), st);
  HierarchyKernel<<<Grid(n - 1), kThreads, 0, st>>>(keys, n, children, range, parent_inner, parent_leaf);
  BoxesKernel<<<Grid(n), kThreads, 0, st>>>(boxes, keys, n, children, parent_inner, parent_leaf, inner_boxes,
                                             arrivals);
  EmitKernel<<<Grid(n - 1), kThreads, 0, st>>>(boxes, keys, n, children, range, inner_boxes, nodes, last);
}

namespace {

__global__ void GatherKernel(const int32_t *order, const uint8_t *last, int n, const PrimRecord *prims_in,
                             const PrimRecord *obj_in, const ShadeRecord *shade_in, const F4 *sn_in,
                             const F4 *sno_in, PrimRecord *prims_out, PrimRecord *obj_out, ShadeRecord *shade_out,
                             F4 *sn_out, F4 *sno_out) {
  const int s = blockIdx.x * kThreads + threadIdx.x;
  if (s >= n) return;
  const int src = order[s];
  PrimRecord r = prims_in[src], ro = obj_in[src];
  uint32_t flags = __float_as_uint(r.p3.w) & ~kPrimLast;
  if (last[s]) flags |= kPrimLast;
  r.p3.w = __uint_as_float(flags);
  ro.p3.w = __uint_as_float(flags);
  prims_out[s] = r;
  obj_out[s] = ro;
  shade_out[s] = shade_in[src];
  if (sn_in) {
    for (int k = 0; k < 3; ++k) {
      sn_out[3 * s + k] = sn_in[3 * src + k];
      sno_out[3 * s + k] = sno_in[3 * src + k];
    }
  }
}

}  // namespace

void LaunchGatherPrims(const int32_t *order, const uint8_t *last, int n, const PrimRecord *prims_in,
                       const PrimRecord *obj_in, const ShadeRecord *shade_in, const F4 *sn_in, const F4 *sno_in,
                       PrimRecord *prims_out, PrimRecord *obj_out, ShadeRecord *shade_out, F4 *sn_out, F4 *sno_out,
                       cudaStream_t st) {
  if (n > 0)
    GatherKernel<<<Grid(n), kThreads, 0, st>>>(order, last, n, prims_in, obj_in, shade_in, sn_in, sno_in, prims_out,
                                                obj_out, shade_out, sn_out, sno_out);
}

}  // namespace muon_gpu
