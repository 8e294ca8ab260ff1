// Tensor-core inference of the guiding network with tcgen05 (sm_100 family).
//
// A CTA runs two independent groups of four warps. A group owns 128 rows
// (one shading point per thread), an operand buffer in shared memory and 64
// columns of tensor memory (TMEM). Per layer the group writes the layer's
// input rows as BF16 into its operand buffer; one thread issues the layer's
// chain of tcgen05.mma (M = 128, N = 64 or 48, K = 16 per instruction, BF16
// operands from shared memory, FP32 accumulation in TMEM) and commits it to
// the group's mbarrier; every thread then reads its row of the accumulator
// with tcgen05.ld and applies bias, ReLU and BF16 rounding to form the next
// layer's input. While one group encodes or runs its epilogue, the other
// group's MMAs keep the tensor core busy. The weights are one pre-arranged
// image (guide_mlp.cuh, "the inference image") that a bulk copy
// (cp.async.bulk) places in shared memory once per CTA.
//
// Every wait is bounded (about two seconds of SM cycles): a wait that gives up
// makes the group stop, and the kernel reports it through a status word
// instead of hanging.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "guide_mlp.cuh"

namespace muon_gpu {
namespace guide {

// Shared memory of a tcgen05 inference CTA: the weight image (padded to
// 66 KiB), two operand buffers of 128 rows x 256 BF16, the mbarriers (weight
// copy, group 0, group 1) and the TMEM address slot.
constexpr int kTcRows = 128;
constexpr int kTcImgSmem = 66 * 1024;
constexpr int kTcOperandBytes = kTcRows * kIn * 2;
constexpr int kTcBarOffset = kTcImgSmem + 2 * kTcOperandBytes;
constexpr int kTcSmemBytes = kTcBarOffset + 64;
constexpr int kTcThreads = 2 * kTcRows;
constexpr uint32_t kTcColumns = 128;  // TMEM columns of a CTA (64 per group)
static_assert(kImgBytes <= kTcImgSmem, "weight image larger than its shared-memory slot");

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t SmemAddr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void MbarInit(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void MbarExpectTx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// One potentially blocking test of the phase: the thread may be suspended
// for up to 0.1 ms while the phase is incomplete, rather than spinning.
__device__ __forceinline__ bool MbarTryWait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(bar), "r"(parity), "r"(100000u)
      : "memory");
  return done != 0;
}

// Waits for the phase of parity `parity` to complete; false once 4e9 SM
// cycles (about two seconds) pass without completion. The cycle counter is
// read every 64 tests.
__device__ __forceinline__ bool MbarWait(uint32_t bar, uint32_t parity) {
  if (MbarTryWait(bar, parity)) return true;
  const long long t0 = clock64();
  for (int i = 0; i < (1 << 26); ++i) {
    if (MbarTryWait(bar, parity)) return true;
    if ((i & 63) == 63 && clock64() - t0 > 4000000000ll) break;
  }
  return false;
}

// Bulk copy global -> shared memory, completing on `bar` by byte count.
__device__ __forceinline__ void BulkLoad(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void FenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void FenceBarrierInit() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void TcFenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void TcFenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Barrier over the 128 threads of a group that also ANDs a predicate.
__device__ __forceinline__ bool GroupAll(int id, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, 128, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n}"
      : "=r"(r)
      : "r"(static_cast<uint32_t>(pred)), "r"(id)
      : "memory");
  return r != 0;
}

__device__ __forceinline__ void TmemAlloc(uint32_t slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void TmemRelinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void TmemDealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// Shared-memory operand descriptor: K-major, no swizzle; core matrices 128 B
// apart along K (leading dimension) and K / 8 * 128 B apart along M or N
// (stride dimension); descriptor version 1 (bits 46-48 = 0b001).
__device__ __forceinline__ uint64_t OperandDesc(uint32_t saddr, int K) {
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(128 >> 4) << 16) |
         (static_cast<uint64_t>(((K >> 3) * 128) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major, N / 8 at bits 17-22, M / 16 at
// bits 24-28 (M = 128).
__host__ __device__ constexpr uint32_t InstrDesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
         (static_cast<uint32_t>(kTcRows >> 4) << 24);
}

__device__ __forceinline__ void MmaBf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void MmaCommit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane, waited for.
__device__ __forceinline__ void TmemLoad32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive FP32 columns of this thread's TMEM lane, waited for.
__device__ __forceinline__ void TmemLoad16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// The state of one group of a tcgen05 inference CTA.
struct TcGroup {
  uint32_t img;          // shared address of the weight image
  const float *bias;     // the image's biases (shared memory)
  unsigned char *a;      // the group's operand buffer
  uint32_t a_addr;       // its shared address
  uint32_t bar;          // the group's MMA mbarrier
  uint32_t tmem;         // the group's accumulator (lane 0, first column)
  uint32_t lane_off;     // this warp's TMEM lane quarter, as an address offset
  uint32_t phase;        // parity of the group's next MMA completion
  int bar_id;            // named barrier of the group
  int row;               // this thread's row (0..127)
  bool ok;               // false once a wait gave up
};

// CTA set-up (all kTcThreads threads): mbarriers, TMEM allocation and the
// bulk copy of the weight image `img` (global memory, kImgBytes). Returns
// false on every thread if the copy did not arrive.
__device__ __forceinline__ bool TcBegin(unsigned char *smem, const void *img, TcGroup *g) {
  const int tid = threadIdx.x, group = tid >> 7;
  const uint32_t bars = SmemAddr(smem + kTcBarOffset);  // [0] weights, [1] group 0, [2] group 1
  const uint32_t slot = bars + 24;
  if (tid == 0) {
    MbarInit(bars, 1);
    MbarInit(bars + 8, 1);
    MbarInit(bars + 16, 1);
    FenceBarrierInit();
  }
  if (tid < 32) {
    TmemAlloc(slot, kTcColumns);
    TmemRelinquish();
  }
  TcFenceBefore();
  __syncthreads();
  TcFenceAfter();
  if (tid == 0) {
    MbarExpectTx(bars, kImgBytes);
    BulkLoad(SmemAddr(smem), img, kImgBytes, bars);
  }
  const uint32_t tmem_base = *reinterpret_cast<volatile uint32_t *>(smem + kTcBarOffset + 24);
  g->img = SmemAddr(smem);
  g->bias = reinterpret_cast<const float *>(smem + kImgBiasOffset);
  g->a = smem + kTcImgSmem + group * kTcOperandBytes;
  g->a_addr = SmemAddr(g->a);
  g->bar = bars + 8 * (1 + group);
  g->tmem = tmem_base + static_cast<uint32_t>(group * 64);
  g->lane_off = static_cast<uint32_t>((tid >> 5) & 3) * 32u << 16;
  g->phase = 0;
  g->bar_id = 1 + group;
  g->row = tid & (kTcRows - 1);
  g->ok = MbarWait(bars, 0);
  return __syncthreads_and(g->ok) != 0;
}

// CTA tear-down (all threads): frees the TMEM columns; a group whose wait gave
// up sets *status.
__device__ __forceinline__ void TcEnd(unsigned char *smem, const TcGroup &g, int32_t *status) {
  if (!g.ok && status) *status = 1;
  TcFenceBefore();
  __syncthreads();
  if (threadIdx.x < 32) {
    TcFenceAfter();
    TmemDealloc(*reinterpret_cast<volatile uint32_t *>(smem + kTcBarOffset + 24), kTcColumns);
  }
}

// Runs layer l over the operand buffer: makes this thread's operand stores
// visible to the tensor core, meets the group (and votes on earlier waits),
// issues and commits the MMA chain from row 0, and waits for it. Returns
// false on every thread of the group once any wait gave up.
__device__ __forceinline__ bool TcLayer(TcGroup &g, int l) {
  FenceProxyAsync();
  TcFenceBefore();
  if (!GroupAll(g.bar_id, g.ok)) {
    g.ok = false;
    return false;
  }
  if (g.row == 0) {
    TcFenceAfter();
    const int K = In(l);
    const uint32_t idesc = InstrDesc(NPad(l));
    const uint32_t b = g.img + static_cast<uint32_t>(ImgOffset(l));
#pragma unroll 1
    for (int kk = 0; kk < K / 16; ++kk)
      MmaBf16(g.tmem, OperandDesc(g.a_addr + kk * 256, K), OperandDesc(b + kk * 256, K), idesc, kk > 0);
    MmaCommit(g.bar);
  }
  g.ok = MbarWait(g.bar, g.phase);
  g.phase ^= 1u;
  TcFenceAfter();
  return true;
}

// One-blob encoding of this thread's features into its row of the layer-0
// operand. Each block of 8 bins starts from one exponential and steps by
// exact ratios: with d = s - (k + 1/2) / 32 the value exp(-512 d^2) of bin
// k + 1 is the value of bin k times exp(32 d - 1/2), and that ratio itself
// shrinks by e^-1 per bin.
__device__ __forceinline__ void TcEncode(const TcGroup &g, const float (&f)[kFeatures]) {
  unsigned char *dst = g.a + (g.row >> 3) * (kIn / 8 * 128) + (g.row & 7) * 16;
  constexpr float kInvE = 0.36787944117144233f;
#pragma unroll
  for (int d = 0; d < kFeatures; ++d) {
    const float s = fminf(fmaxf(f[d], 0.0f), 1.0f);
#pragma unroll
    for (int q = 0; q < kBins / 8; ++q) {
      const float x = s - (static_cast<float>(8 * q) + 0.5f) * (1.0f / kBins);
      float v[8];
      v[0] = __expf(-x * x * (0.5f * kBins * kBins));
      float r = __expf(static_cast<float>(kBins) * x - 0.5f);
#pragma unroll
      for (int i = 1; i < 8; ++i) {
        v[i] = v[i - 1] * r;
        r *= kInvE;
      }
      *reinterpret_cast<uint4 *>(dst + (d * (kBins / 8) + q) * 128) =
          make_uint4(PackBf16(v[0], v[1]), PackBf16(v[2], v[3]), PackBf16(v[4], v[5]), PackBf16(v[6], v[7]));
    }
  }
}

// Hidden-layer epilogue: this thread's 64 accumulator columns + bias, ReLU,
// BF16, written as its row of the next layer's operand (K = 64).
__device__ __forceinline__ void TcHidden(const TcGroup &g, int l) {
  const float *b = g.bias + BiasOffset(l);
  unsigned char *dst = g.a + (g.row >> 3) * (kWidth / 8 * 128) + (g.row & 7) * 16;
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    TmemLoad32(g.tmem + g.lane_off + 32 * half, v);
#pragma unroll
    for (int kb = 0; kb < 4; ++kb) {
      const int c = 32 * half + 8 * kb;
      float h[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) h[i] = fmaxf(v[8 * kb + i] + b[c + i], 0.0f);
      *reinterpret_cast<uint4 *>(dst + (c / 8) * 128) =
          make_uint4(PackBf16(h[0], h[1]), PackBf16(h[2], h[3]), PackBf16(h[4], h[5]), PackBf16(h[6], h[7]));
    }
  }
}

// The network's 64 raw outputs for this thread's features. Every thread of
// the group calls it together; false (on all of them) if a wait gave up.
__device__ __forceinline__ bool TcForward(TcGroup &g, const float (&f)[kFeatures], float (&out)[kOut]) {
  TcEncode(g, f);
  if (!TcLayer(g, 0)) return false;
#pragma unroll 1
  for (int l = 1; l < kLayers; ++l) {
    TcHidden(g, l - 1);
    if (!TcLayer(g, l)) return false;
  }
  static_assert(kOut == 64, "two 32-column loads of the output layer");
  const float *b = g.bias + BiasOffset(kLayers - 1);
#pragma unroll
  for (int half = 0; half < 2; ++half) {
    float v[32];
    TmemLoad32(g.tmem + g.lane_off + 32 * half, v);
#pragma unroll
    for (int c = 0; c < 32; ++c) out[32 * half + c] = v[c] + b[32 * half + c];
  }
  return true;
}

// Stages this thread's processed mixture (kMixFloats) in its row of the
// operand buffer, which the finished network pass no longer needs; rows are
// 304 bytes (76 words) apart so that the float4 stores of 8 consecutive rows
// fall in distinct banks.
constexpr int kMixRowBytes = 304;
static_assert(kMixRowBytes >= 4 * kMixFloats && kMixRowBytes % 16 == 0, "mixture staging row");
static_assert(kTcRows * kMixRowBytes <= kTcOperandBytes, "mixture staging larger than the operand buffer");

__device__ __forceinline__ float *TcMixRow(const TcGroup &g) {
  return reinterpret_cast<float *>(g.a + g.row * kMixRowBytes);
}

// Copies the group's staged mixtures of rows [base, base + 128) to
// dst[row * 10 .. row * 10 + 9] (float4), rows below `n` only, with coalesced
// stores. Every thread of the group calls it; it meets the group before and
// after, so the operand buffer is free again on return.
__device__ __forceinline__ void TcStoreMix(const TcGroup &g, int base, int n, float4 *dst) {
  GroupAll(g.bar_id, true);
  constexpr int kVec = kMixFloats / 4;  // float4 per row
  const int rows = min(kTcRows, n - base);
  float4 *out = dst + static_cast<int64_t>(base) * kVec;
#pragma unroll 2
  for (int e = g.row; e < rows * kVec; e += kTcRows) {
    const int r = e / kVec, q = e - r * kVec;
    out[e] = *reinterpret_cast<const float4 *>(g.a + r * kMixRowBytes + 16 * q);
  }
  GroupAll(g.bar_id, true);
}

#endif  // __CUDACC__

}  // namespace guide
}  // namespace muon_gpu
