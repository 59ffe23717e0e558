// tn_gemm.cu -- batched real GEMMs of the tensor-network mode (the pairwise
// contractions of the 4M real embedding), hand-written for sm_103a.
//
//   C[b](i, j) = sum_k A[b](i, k) * B[b](j, k),  C column-major (i fastest,
//   leading dimension mr), A [mr][kr] and B [nr][kr] K-contiguous (the rows
//   the operand gathers write).
//
// FP32-accurate tensor-core path (complex64 plans): tcgen05.mma kind::tf32
// with the 3xTF32 split.  Each operand x is split in shared memory into
// hi = tf32(x) (rounded to nearest by two integer operations) and
// lo = tf32(x - hi); the accumulator in
// tensor memory receives hi*hi + hi*lo + lo*hi (the dropped lo*lo term and
// the rounding of lo are below 2^-21 relative).  The tensor cores' own
// accumulation truncates: each group of 64 K-elements is accumulated in a
// fresh tensor-memory buffer (four, in turn) and the groups are summed in
// FP32 registers with round-to-nearest, which keeps the result at FP32
// accuracy for long K.  One CTA computes a 128-row
// tile of the larger side (the "P" operand) against a BN-column tile of the
// other ("Q"), BN in {16, 32, 64, 128, 256}; persistent CTAs (one per SM) walk
// their tiles with the pipeline running on across tile boundaries; warps:
//   warp 0     TMA producer: 3-D tensor maps [batch][rows][k], 128-byte
//              swizzle, boxes of 32 K-elements (one swizzle row);
//   warp 1     allocates the tensor-memory accumulator and issues the MMAs
//              (one thread), commits each stage back to the producer;
//   warps 2-   split each landed stage into hi/lo tiles (element-wise on the
//              swizzled image, so no address arithmetic), add each K-block's
//              partial sum from tensor memory (tcgen05.ld; four warps per
//              32-lane quadrant for BN >= 32, a quarter of the columns each)
//              into registers, and store C after a tile's last K-block.
// Every mbarrier wait is bounded; a wait that gives up sets the device error
// word (read by the root kernel, which then returns NaN) and the CTA drains
// and frees its tensor memory before returning.
//
// A shared-memory-tiled SIMT kernel (FP32 or FP64 FMA) serves the complex128
// plans, the FP32 mode and the shapes too small for a 128-row tile.
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include "tn_gemm.cuh"

namespace tedq {

namespace {

// ------------------------------------------------------------------ PTX helpers

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: polls try_wait (which itself suspends the thread for a short
// time when the phase is not complete), first without sleeping -- the
// pipeline's hand-offs sit on the critical path -- then with short sleeps,
// for about a second in all; then the error word is set and false returned.
// Once any CTA has set the word, the others give up their waits at the next
// check instead of polling to their own limit.
constexpr uint32_t kWaitTries = 1u << 21;
constexpr uint32_t kSpinTries = 1u << 14;

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code, bool bail = true) {
  for (uint32_t t = 0; t < kWaitTries; ++t) {
    if (mbar_try_wait(bar, parity)) return true;
    if (t > kSpinTries) __nanosleep(256);
    if (bail && (t & 1023) == 1023 && *(volatile int*)err != 0) return false;
  }
  atomicExch(err, code);
  return false;
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1,
                                            int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Shared-memory matrix descriptor: K-major operand in the canonical swizzled
// layout whose rows are KB FP32 values (KB * 4 = 128, 64 or 32 bytes, the
// swizzle span), 8-row atoms 8 * KB * 4 bytes apart.
template <int KB>
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
  constexpr uint32_t layout = KB == 32 ? 2u : KB == 16 ? 4u : 6u;  // 128-, 64-, 32-byte swizzle
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);              // start address
  d |= (uint64_t)(1) << 16;                              // leading byte offset (unused for K-major swizzled)
  d |= (uint64_t)(((8 * KB * 4) >> 4) & 0x3FFF) << 32;   // stride byte offset: 8 rows
  d |= (uint64_t)1 << 46;                                // descriptor version (sm_100 family)
  d |= (uint64_t)layout << 61;
  return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_tf32(int n) {
  return (1u << 4)                       // D format: F32
         | (2u << 7)                     // A format: TF32
         | (2u << 10)                    // B format: TF32
         | ((uint32_t)(n >> 3) << 17)    // N / 8
         | ((uint32_t)(128 >> 4) << 24); // M / 16
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 16 / 32 consecutive accumulator columns of this thread's lane in one
// instruction (no wait: the caller waits once for all its loads)
__device__ __forceinline__ void tmem_ld16_nowait(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 8 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// x rounded to the 10 explicit mantissa bits of TF32, to nearest (ties away
// from zero) with two integer operations: add half of the dropped range to
// the magnitude bits and clear them.  A carry out of the mantissa raises the
// exponent, which is the rounded value.  Finite inputs only (the operands are
// finite whenever the parameters are).
__device__ __forceinline__ float tf32_round(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// ------------------------------------------------------------------ tensor-core kernel

// Split + epilogue warps: CG per tensor-memory lane quadrant, each owning
// BN / CG accumulator columns (at least 8); two more warps (TMA, MMA).
template <int BN>
struct TcWarps {
  static constexpr int CG = BN >= 32 ? 4 : BN / 8;
  static constexpr int kEpi = 4 * CG;
  static constexpr int kThreads = 32 * (2 + kEpi);
};

// KB: K elements per stage, one swizzle row (32, or 16 / 8 for short sums).
// Two rings: load stages (the P and Q tiles as TMA writes them) and, with the
// 3xTF32 split, operand slots (hi and lo of both, read by the MMAs).  A load
// stage is released as soon as the split has read it, so the loads in flight
// do not wait for the MMAs; without the split the MMAs read the load stages.
template <int BN, int KB, bool SPLIT>
struct TcSmem {
  static constexpr int kA = 128 * KB * 4;       // bytes of one P tile
  static constexpr int kB = BN * KB * 4;        // bytes of one Q tile
  static constexpr int kLoad = kA + kB;         // one load stage
  static constexpr int kOp = SPLIT ? 2 * kLoad : 0;  // one operand slot (hi, lo)
  static constexpr int kSlots = SPLIT ? 2 : 0;
  static constexpr int kBudget = 200 * 1024 - kSlots * kOp;
  // as many load stages as fit next to the barriers in 200 KB
  static constexpr int kStages = kBudget / kLoad > 8 ? 8 : kBudget / kLoad;
  static constexpr int kOpBase = kStages * kLoad;
  static constexpr int kBarBase = kOpBase + kSlots * kOp;
  static constexpr int kBytes = kBarBase + 1024 /* alignment */ + 512 /* barriers */;
  static_assert(kStages >= 2, "pipeline depth");
  static_assert((2 * kStages + 2 * 2 + 2 * 4 + 1) * 8 + 4 <= 512, "barrier region");
};

// Work of one launch: tiles of 128 P-rows x BN Q-columns of every batch entry,
// tile t = (batch, q tile, p tile) with the p tile fastest.
struct TcWork {
  float* c;
  int64_t sc;     // reals between batch entries of C
  int64_t ldc;    // mr
  int32_t swap;   // 0: p = i (rows of C), q = j; 1: p = j, q = i
  int32_t p_ext, q_ext;
  int32_t tiles_p, tiles_q;
  int32_t kblocks;
  int32_t p_batched, q_batched;
  int64_t tiles;  // tiles_p * tiles_q * batch
};

// Persistent: CTA b processes tiles b, b + grid, ...; its producer, MMA
// issuer and epilogue warps walk the same sequence of (tile, K-block) steps,
// so the pipeline runs on across tile boundaries.
template <int BN, bool SPLIT, int KB>
__global__ void __launch_bounds__(TcWarps<BN>::kThreads, 1)
    tn_gemm_tc_kernel(const __grid_constant__ CUtensorMap map_p, const __grid_constant__ CUtensorMap map_q,
                      const TcWork w, int* err) {
  using S = TcSmem<BN, KB, SPLIT>;
  constexpr int kStages = S::kStages;
  constexpr int kSlots = S::kSlots > 0 ? S::kSlots : 1;  // operand slots (used with the split only)
  constexpr int kEpiWarps = TcWarps<BN>::kEpi;
  // accumulator buffers (512 tensor-memory columns at most, one CTA per SM)
  // and K-blocks accumulated per buffer before the epilogue adds them up in
  // FP32 (64 K-elements: the tensor cores' truncating accumulation stays
  // short)
  constexpr int kBufs = 512 / BN < 4 ? 512 / BN : 4;
  constexpr int kGroup = 64 / KB;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + S::kBarBase);  // [kStages] TMA landed
  uint64_t* lfree = full + kStages;   // [kStages] load stage free (read by the split, or by the MMAs)
  uint64_t* opready = lfree + kStages;  // [2] operand slot written (split)
  uint64_t* opfree = opready + 2;       // [2] operand slot's MMAs complete
  uint64_t* accf = opfree + 2;          // [kBufs] group partial complete in accumulator buffer b
  uint64_t* acce = accf + kBufs;        // [kBufs] accumulator buffer b read back
  uint64_t* done = acce + kBufs;        // every MMA complete
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // kBufs accumulator buffers of BN columns: the MMAs of a group of K-blocks
  // write one while the epilogue warps add finished ones into FP32 registers
  constexpr uint32_t kCols = kBufs * BN < 32 ? 32 : kBufs * BN;
  const int64_t my_tiles = w.tiles > blockIdx.x ? (w.tiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int64_t steps = my_tiles * w.kblocks;
  // groups of up to kGroup K-blocks per accumulator buffer; a tile's last
  // group may be shorter.  Global group id of step g: tile * groups + kb / kGroup
  const int groups = (w.kblocks + kGroup - 1) / kGroup;
  auto tile_of = [&](int64_t i, int& tp, int& tq, int& b) {
    const int64_t t = blockIdx.x + i * gridDim.x;
    tp = (int)(t % w.tiles_p);
    const int64_t r = t / w.tiles_p;
    tq = (int)(r % w.tiles_q);
    b = (int)(r / w.tiles_q);
  };

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&lfree[s], SPLIT ? kEpiWarps : 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&opready[b], kEpiWarps);
      mbar_init(&opfree[b], 1);
    }
    for (int b = 0; b < kBufs; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], kEpiWarps);
    }
    mbar_init(done, 1);
    fence_proxy_async();
    prefetch_map(&map_p);
    prefetch_map(&map_q);
  }
  if (warp == 1) tmem_alloc(tmem_slot, kCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool ok = true;

  if (warp == 0) {
    if (lane == 0) {
      int64_t issued = 0;  // steps whose loads were issued
      for (int64_t g = 0; g < steps && ok; ++g) {
        const int s = (int)(g % kStages);
        if (g >= kStages) ok = mbar_wait(&lfree[s], (uint32_t)((g / kStages) - 1) & 1, err, 1);
        if (!ok) break;
        int tp, tq, b;
        tile_of(g / w.kblocks, tp, tq, b);
        const int kb = (int)(g % w.kblocks);
        unsigned char* st = smem + s * S::kLoad;
        mbar_expect_tx(&full[s], S::kA + S::kB);
        tma_load_3d(st, &map_p, &full[s], kb * KB, tp * 128, w.p_batched ? b : 0);
        tma_load_3d(st + S::kA, &map_q, &full[s], kb * KB, tq * BN, w.q_batched ? b : 0);
        issued = g + 1;
      }
      // every issued copy has landed before the CTA may exit (immediate on the
      // normal path, where the consumers waited for them already)
      for (int64_t g = issued > kStages ? issued - kStages : 0; g < issued; ++g)
        mbar_wait(&full[g % kStages], (uint32_t)(g / kStages) & 1, err, 6, false);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_tf32(BN);
      for (int64_t g = 0; g < steps && ok; ++g) {
        const int kb = (int)(g % w.kblocks);
        const int64_t gid = (g / w.kblocks) * groups + kb / kGroup;
        const int buf = (int)(gid % kBufs);
        const bool first = kb % kGroup == 0, last = kb % kGroup == kGroup - 1 || kb == w.kblocks - 1;
        if (first && gid >= kBufs)  // buffer read back
          ok = mbar_wait(&acce[buf], (uint32_t)((gid / kBufs) - 1) & 1, err, 7);
        if (!ok) break;
        uint32_t a_hi, b_hi, a_lo = 0, b_lo = 0;
        if (SPLIT) {
          const int slot = (int)(g % kSlots);
          ok = mbar_wait(&opready[slot], (uint32_t)(g / kSlots) & 1, err, 2);
          const uint32_t op = smem_u32(smem + S::kOpBase + slot * S::kOp);
          a_hi = op, b_hi = op + S::kA, a_lo = op + S::kA + S::kB, b_lo = a_lo + S::kA;
        } else {
          const int s = (int)(g % kStages);
          ok = mbar_wait(&full[s], (uint32_t)(g / kStages) & 1, err, 2);
          const uint32_t st = smem_u32(smem + s * S::kLoad);
          a_hi = st, b_hi = st + S::kA;
        }
        if (!ok) break;
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(buf * BN);
#pragma unroll
        for (int k = 0; k < KB / 8; ++k) {  // K = 8 per MMA: 32 bytes along the swizzle row
          mma_tf32(d, smem_desc<KB>(a_hi + 32 * k), smem_desc<KB>(b_hi + 32 * k), idesc,
                   (first && k == 0) ? 0u : 1u);
          if (SPLIT) {
            mma_tf32(d, smem_desc<KB>(a_hi + 32 * k), smem_desc<KB>(b_lo + 32 * k), idesc, 1u);
            mma_tf32(d, smem_desc<KB>(a_lo + 32 * k), smem_desc<KB>(b_hi + 32 * k), idesc, 1u);
          }
        }
        // frees what these MMAs read once they have read it
        mma_commit(SPLIT ? &opfree[g % kSlots] : &lfree[g % kStages]);
        if (last) mma_commit(&accf[buf]);   // the group's partial sum is ready
      }
      mma_commit(done);
    }
  } else {
    // split + epilogue warps: split each landed stage into hi / lo operand
    // tiles, and add each K-block's partial sum (tensor memory: this warp's
    // 32-lane quadrant, its group of columns) into FP32 registers with
    // round-to-nearest additions; store a tile after its last K-block
    constexpr int HALF = BN / TcWarps<BN>::CG;  // accumulator columns of this warp
    const int t = threadIdx.x - 64;  // 0 .. 32 * kEpiWarps - 1
    const int quad = warp & 3, half = (warp - 2) >> 2;  // lane quadrant, column group
    float acc[HALF];
#pragma unroll
    for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
    auto split_stage = [&](int64_t g) {
      const int s = (int)(g % kStages), slot = (int)(g % kSlots);
      ok = mbar_wait(&full[s], (uint32_t)(g / kStages) & 1, err, 3);
      // the operand slot's previous MMAs (step g - 2) have read it
      if (ok && g >= kSlots) ok = mbar_wait(&opfree[slot], (uint32_t)((g / kSlots) - 1) & 1, err, 8);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) return;
      const float4* raw = reinterpret_cast<const float4*>(smem + s * S::kLoad);  // P tile then Q tile
      float4* hi = reinterpret_cast<float4*>(smem + S::kOpBase + slot * S::kOp);  // same order
      float4* lo = reinterpret_cast<float4*>(smem + S::kOpBase + slot * S::kOp + S::kLoad);
      constexpr int n4 = S::kLoad / 16;
#pragma unroll 4
      for (int i = t; i < n4; i += 32 * kEpiWarps) {
        float4 x = raw[i], h, l;
        h.x = tf32_round(x.x); l.x = tf32_round(x.x - h.x);
        h.y = tf32_round(x.y); l.y = tf32_round(x.y - h.y);
        h.z = tf32_round(x.z); l.z = tf32_round(x.z - h.z);
        h.w = tf32_round(x.w); l.w = tf32_round(x.w - h.w);
        hi[i] = h;
        lo[i] = l;
      }
      fence_proxy_async();  // generic-proxy writes -> visible to the tensor cores
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&lfree[s]);        // the load stage may be refilled
        mbar_arrive(&opready[slot]);   // the MMAs may read the operands
      }
    };
    auto store_tile = [&](int64_t i) {
      int tp, tq, b;
      tile_of(i, tp, tq, b);
      const int p = tp * 128 + quad * 32 + lane;
      const int q0 = tq * BN + half * HALF;
      float* cb = w.c + (int64_t)b * w.sc;
      if (p < w.p_ext) {
        if (!w.swap) {
#pragma unroll
          for (int j = 0; j < HALF; ++j)
            if (q0 + j < w.q_ext) cb[(int64_t)(q0 + j) * w.ldc + p] = acc[j];
        } else {
          float* dst = cb + (int64_t)p * w.ldc + q0;
          const bool vec = q0 + HALF <= w.q_ext && ((reinterpret_cast<uintptr_t>(dst) & 15) == 0);
#pragma unroll
          for (int j = 0; j < HALF; j += 4) {
            if (vec) {
              reinterpret_cast<float4*>(dst + j)[0] = make_float4(acc[j], acc[j + 1], acc[j + 2], acc[j + 3]);
            } else {
#pragma unroll
              for (int x = 0; x < 4; ++x)
                if (q0 + j + x < w.q_ext) dst[j + x] = acc[j + x];
            }
          }
        }
      }
#pragma unroll
      for (int j = 0; j < HALF; ++j) acc[j] = 0.f;
    };
    // adds group gid of tile `tile` (buffer gid % kBufs) into the registers
    auto flush = [&](int64_t gid, int64_t tile, bool tile_end) {
      const int buf = (int)(gid % kBufs);
      ok = mbar_wait(&accf[buf], (uint32_t)(gid / kBufs) & 1, err, 4);
      ok = __all_sync(0xffffffffu, ok);  // tensor-memory loads are warp-collective
      if (!ok) return;
      tc_fence_after();
      const uint32_t base = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(buf * BN + half * HALF);
      if constexpr (HALF % 16 == 0) {
        // up to 32 columns of loads in flight together, one wait each
        constexpr int CH = HALF < 32 ? HALF : 32;
#pragma unroll
        for (int c1 = 0; c1 < HALF; c1 += CH) {
          float v[CH];
#pragma unroll
          for (int c0 = 0; c0 < CH; c0 += 16) tmem_ld16_nowait(base + (uint32_t)(c1 + c0), v + c0);
          tmem_wait_ld();
#pragma unroll
          for (int j = 0; j < CH; ++j) acc[c1 + j] += v[j];
        }
      } else {
#pragma unroll
        for (int c0 = 0; c0 < HALF; c0 += 8) {
          float v[8];
          tmem_ld8(base + (uint32_t)c0, v);
#pragma unroll
          for (int j = 0; j < 8; ++j) acc[c0 + j] += v[j];
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[buf]);
      if (tile_end) store_tile(tile);
    };
    for (int64_t g = 0; g <= steps && ok; ++g) {
      if (SPLIT && g < steps) split_stage(g);
      if (ok && g >= 1) {  // step g - 1 closed a group: add it
        const int64_t h = g - 1;
        const int kb = (int)(h % w.kblocks);
        if (kb % kGroup == kGroup - 1 || kb == w.kblocks - 1)
          flush((h / w.kblocks) * groups + kb / kGroup, h / w.kblocks, kb == w.kblocks - 1);
      }
    }
  }
  // no MMA may still write the accumulator when it is freed: the final commit
  // (already complete on the normal path) is awaited, bounded
  if (threadIdx.x == 64) mbar_wait(done, 0, err, 5, false);
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem, kCols);
  }
}

// ------------------------------------------------------------------ SIMT kernel

// Tile BM x BN of C, K in chunks of 16 through shared memory; each thread
// computes TM x TN outputs.  A [P][kr] and B [Q][kr] K-contiguous.
template <typename real, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
    tn_gemm_simt_kernel(const real* __restrict__ a, const real* __restrict__ b, real* __restrict__ c, int64_t mr,
                        int64_t nr, int64_t kr, int64_t sa, int64_t sb, int64_t sc) {
  constexpr int BK = 16;
  constexpr int T = (BM / TM) * (BN / TN);
  __shared__ real As[BK][BM + 1];
  __shared__ real Bs[BK][BN + 1];
  const int64_t bt = blockIdx.z;
  const real* A = a + bt * sa;
  const real* B = b + bt * sb;
  real* C = c + bt * sc;
  const int64_t i0 = (int64_t)blockIdx.x * BM, j0 = (int64_t)blockIdx.y * BN;
  const int tid = threadIdx.x;
  const int ti = tid % (BM / TM), tj = tid / (BM / TM);
  real acc[TM][TN];
#pragma unroll
  for (int x = 0; x < TM; ++x)
#pragma unroll
    for (int y = 0; y < TN; ++y) acc[x][y] = 0;
  for (int64_t k0 = 0; k0 < kr; k0 += BK) {
    for (int e = tid; e < BM * BK; e += T) {
      const int r = e / BK, k = e % BK;
      const int64_t gi = i0 + r, gk = k0 + k;
      As[k][r] = (gi < mr && gk < kr) ? A[gi * kr + gk] : (real)0;
    }
    for (int e = tid; e < BN * BK; e += T) {
      const int r = e / BK, k = e % BK;
      const int64_t gj = j0 + r, gk = k0 + k;
      Bs[k][r] = (gj < nr && gk < kr) ? B[gj * kr + gk] : (real)0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      real av[TM], bv[TN];
#pragma unroll
      for (int x = 0; x < TM; ++x) av[x] = As[k][ti + x * (BM / TM)];
#pragma unroll
      for (int y = 0; y < TN; ++y) bv[y] = Bs[k][tj + y * (BN / TN)];
#pragma unroll
      for (int x = 0; x < TM; ++x)
#pragma unroll
        for (int y = 0; y < TN; ++y) acc[x][y] = fma(av[x], bv[y], acc[x][y]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int y = 0; y < TN; ++y) {
    const int64_t gj = j0 + tj + y * (BN / TN);
#pragma unroll
    for (int x = 0; x < TM; ++x) {
      const int64_t gi = i0 + ti + x * (BM / TM);
      if (gi < mr && gj < nr) C[gj * mr + gi] = acc[x][y];
    }
  }
}

// Few outputs and a long sum (the network's closing contractions: a 1 x 2
// real result over thousands of terms): one CTA per batch entry, every thread
// accumulates a strided part of each output's sum, then a block reduction.
template <typename real>
__global__ void __launch_bounds__(256)
    tn_gemm_dot_kernel(const real* __restrict__ a, const real* __restrict__ b, real* __restrict__ c, int mr, int nr,
                       int64_t kr, int64_t sa, int64_t sb, int64_t sc) {
  constexpr int kMaxOut = 16;
  __shared__ real part[kMaxOut][8];
  const int64_t bt = blockIdx.x;
  const real* A = a + bt * sa;
  const real* B = b + bt * sb;
  real acc[kMaxOut];
#pragma unroll
  for (int o = 0; o < kMaxOut; ++o) acc[o] = 0;
  for (int64_t k = threadIdx.x; k < kr; k += blockDim.x) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i >= mr) break;
      const real x = A[(int64_t)i * kr + k];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (j < nr) acc[i * 4 + j] = fma(x, B[(int64_t)j * kr + k], acc[i * 4 + j]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 0; o < kMaxOut; ++o) {
    real v = acc[o];
#pragma unroll
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (lane == 0) part[o][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < mr * nr) {
    const int i = threadIdx.x / nr, j = threadIdx.x % nr;
    real v = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += part[i * 4 + j][w];
    c[bt * sc + (int64_t)j * mr + i] = v;
  }
}

// ------------------------------------------------------------------ host side

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
  static EncodeTiled fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// [batch][rows][kr] FP32, box [1][box_rows][kb], kb * 4-byte swizzle; rows
// and K beyond the extents read as zero
bool make_map(CUtensorMap* map, const float* base, int64_t rows, int64_t kr, int64_t batch, int64_t bstride,
              int box_rows, int kb) {
  EncodeTiled enc = encode_fn();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)kr, (cuuint64_t)rows, (cuuint64_t)(bstride ? batch : 1)};
  const cuuint64_t strides[2] = {(cuuint64_t)kr * 4, (cuuint64_t)(bstride ? bstride : rows * kr) * 4};
  const cuuint32_t box[3] = {(cuuint32_t)kb, (cuuint32_t)box_rows, 1};
  const CUtensorMapSwizzle sw = kb == 32 ? CU_TENSOR_MAP_SWIZZLE_128B
                                : kb == 16 ? CU_TENSOR_MAP_SWIZZLE_64B
                                           : CU_TENSOR_MAP_SWIZZLE_32B;
  const cuuint32_t estr[3] = {1, 1, 1};
  return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, bool SPLIT, int KB>
cudaError_t launch_tc(const CUtensorMap& mp, const CUtensorMap& mq, const TcWork& w, int* err, cudaStream_t s) {
  const int bytes = TcSmem<BN, KB, SPLIT>::kBytes;
  static bool attr[64] = {false};  // per device (setting it twice is harmless)
  static int sms[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (!attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(tn_gemm_tc_kernel<BN, SPLIT, KB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         bytes);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    attr[dev] = true;
  }
  // persistent: one CTA per SM (its shared memory admits one)
  const int64_t grid = w.tiles < sms[dev] ? w.tiles : sms[dev];
  tn_gemm_tc_kernel<BN, SPLIT, KB><<<(unsigned)grid, TcWarps<BN>::kThreads, bytes, s>>>(mp, mq, w, err);
  return cudaGetLastError();
}

template <int BN, bool SPLIT>
cudaError_t dispatch_kb(int kb, const CUtensorMap& mp, const CUtensorMap& mq, const TcWork& w, int* err,
                        cudaStream_t s) {
  if (kb == 8) return launch_tc<BN, SPLIT, 8>(mp, mq, w, err, s);
  if (kb == 16) return launch_tc<BN, SPLIT, 16>(mp, mq, w, err, s);
  return launch_tc<BN, SPLIT, 32>(mp, mq, w, err, s);
}

template <bool SPLIT>
cudaError_t dispatch_split(int bn, int kb, const CUtensorMap& mp, const CUtensorMap& mq, const TcWork& w, int* err,
                           cudaStream_t s) {
  if (bn == 256) return kb == 8 ? launch_tc<256, SPLIT, 8>(mp, mq, w, err, s)
                                 : launch_tc<256, SPLIT, 16>(mp, mq, w, err, s);
  if (bn == 128) return dispatch_kb<128, SPLIT>(kb, mp, mq, w, err, s);
  if (bn == 64) return dispatch_kb<64, SPLIT>(kb, mp, mq, w, err, s);
  if (bn == 32) return dispatch_kb<32, SPLIT>(kb, mp, mq, w, err, s);
  return dispatch_kb<16, SPLIT>(kb, mp, mq, w, err, s);
}

cudaError_t dispatch_bn(int bn, bool split, int kb, const CUtensorMap& mp, const CUtensorMap& mq, const TcWork& w,
                        int* err, cudaStream_t s) {
  return split ? dispatch_split<true>(bn, kb, mp, mq, w, err, s) : dispatch_split<false>(bn, kb, mp, mq, w, err, s);
}

}  // namespace

bool tn_gemm_tc_supported(const TnGemmArgs& g) {
  // FP32 rows of kr reals: 16-byte TMA strides and bases; the P side fills a
  // 128-row tile to at least a quarter, the Q side at least 8 columns
  const int64_t P = g.mr >= g.nr ? g.mr : g.nr, Q = g.mr >= g.nr ? g.nr : g.mr;
  return g.kr % 4 == 0 && g.kr >= 4 && P >= 32 && Q >= 8 && g.nbatch <= 65535 &&
         (reinterpret_cast<uintptr_t>(g.a) & 15) == 0 && (reinterpret_cast<uintptr_t>(g.b) & 15) == 0 &&
         (g.sa * 4) % 16 == 0 && (g.sb * 4) % 16 == 0 && encode_fn() != nullptr;
}

cudaError_t tn_gemm_tc(const TnGemmArgs& g, bool split, cudaStream_t s) {
  // the larger side fills the 128-row tiles
  // Which side fills the 128-row tiles: the larger one.  Tuning knob
  // TEDQ_GB300_TN_GEMM_N256=1: when both sides have at least 128 rows and one
  // at least 256, the smaller one with N = 256 MMAs on the other (twice the
  // flops per operand byte; measured slower: 64 accumulators per thread spill
  // and the operand slots leave room for K-blocks of 16 only).
  static const bool wide_ok = [] {
    const char* e = getenv("TEDQ_GB300_TN_GEMM_N256");
    return e && e[0] == '1';
  }();
  const int64_t lo_side = g.mr < g.nr ? g.mr : g.nr, hi_side = g.mr < g.nr ? g.nr : g.mr;
  const bool wide = wide_ok && lo_side >= 128 && hi_side >= 256;
  const bool swap = wide ? g.nr < g.mr : g.nr > g.mr;
  const float* P = static_cast<const float*>(swap ? g.b : g.a);
  const float* Q = static_cast<const float*>(swap ? g.a : g.b);
  const int64_t pe = swap ? g.nr : g.mr, qe = swap ? g.mr : g.nr;
  const int64_t sp = swap ? g.sb : g.sa, sq = swap ? g.sa : g.sb;
  const int bn = wide ? 256 : qe >= 128 ? 128 : qe >= 64 ? 64 : qe >= 32 ? 32 : 16;
  // K per stage: one swizzle row of 32 values, or 16 / 8 for short sums (no
  // zero-filled MMAs)
  // TEDQ_GB300_TN_GEMM_KB (8, 16 or 32) caps it: a tuning knob for measurements
  static const int kb_cap = [] {
    const char* e = getenv("TEDQ_GB300_TN_GEMM_KB");
    const int v = e ? atoi(e) : 32;
    return v == 8 || v == 16 ? v : 32;
  }();
  int kb = g.kr <= 8 ? 8 : g.kr <= 16 ? 16 : 32;
  kb = kb < kb_cap ? kb : kb_cap;
  if (bn == 256 && kb > 16) kb = 16;  // shared memory: the N = 256 operand slots
  CUtensorMap mp, mq;
  if (!make_map(&mp, P, pe, g.kr, g.nbatch, sp, 128, kb) || !make_map(&mq, Q, qe, g.kr, g.nbatch, sq, bn, kb))
    return cudaErrorInvalidValue;
  TcWork w;
  w.c = static_cast<float*>(g.c);
  w.sc = g.sc;
  w.ldc = g.mr;
  w.swap = swap ? 1 : 0;
  w.p_ext = (int32_t)pe;
  w.q_ext = (int32_t)qe;
  w.tiles_p = (int32_t)((pe + 127) / 128);
  w.tiles_q = (int32_t)((qe + bn - 1) / bn);
  w.kblocks = (int32_t)((g.kr + kb - 1) / kb);
  w.p_batched = sp != 0;
  w.q_batched = sq != 0;
  w.tiles = (int64_t)w.tiles_p * w.tiles_q * g.nbatch;
  return dispatch_bn(bn, split, kb, mp, mq, w, g.err, s);
}

template <typename real>
cudaError_t tn_gemm_simt(const TnGemmArgs& g, cudaStream_t s) {
  const real* A = static_cast<const real*>(g.a);
  const real* B = static_cast<const real*>(g.b);
  real* C = static_cast<real*>(g.c);
  if (g.mr <= 4 && g.nr <= 4 && g.kr >= 256 && g.nbatch <= 0x7fffffff) {
    tn_gemm_dot_kernel<real><<<(unsigned)g.nbatch, 256, 0, s>>>(A, B, C, (int)g.mr, (int)g.nr, g.kr, g.sa, g.sb, g.sc);
  } else if (g.mr >= 64 && g.nr >= 64) {
    dim3 grid((unsigned)((g.mr + 63) / 64), (unsigned)((g.nr + 63) / 64), (unsigned)g.nbatch);
    tn_gemm_simt_kernel<real, 64, 64, 4, 4><<<grid, 256, 0, s>>>(A, B, C, g.mr, g.nr, g.kr, g.sa, g.sb, g.sc);
  } else {
    dim3 grid((unsigned)((g.mr + 15) / 16), (unsigned)((g.nr + 15) / 16), (unsigned)g.nbatch);
    tn_gemm_simt_kernel<real, 16, 16, 1, 1><<<grid, 256, 0, s>>>(A, B, C, g.mr, g.nr, g.kr, g.sa, g.sb, g.sc);
  }
  return cudaGetLastError();
}

template cudaError_t tn_gemm_simt<float>(const TnGemmArgs&, cudaStream_t);
template cudaError_t tn_gemm_simt<double>(const TnGemmArgs&, cudaStream_t);

}  // namespace tedq
