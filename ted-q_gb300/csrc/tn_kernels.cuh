// tn_kernels.cuh -- device side of the tensor-network mode: batched gate
// tensors from the parameters, operand gathers (bit permutations into planar
// real GEMM operands) and the FP64 root accumulation.  The GEMMs themselves
// are in tn_gemm.cu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tedq {

// One parameter-dependent gate tensor (ket side, or its conjugate on the bra
// side), stored for every circuit of the batch at
// leaves + 2 * (off * batch + b * 4^k) reals.
struct TnLeafDesc {
  int32_t op;       // TEDQ_OP_*
  int32_t k;        // 1 or 2
  int32_t conj;     // 1: bra side (complex conjugate)
  int32_t pad;
  int32_t slot[4];  // parameter slots, -1 = use val
  double val[4];
  int64_t off;      // complex elements per batch entry before this tensor
};

constexpr int kTnMaxBits = 48;

// One GEMM operand: element e = f*K + k of the gather (n = F*K entries, nbits =
// log2 n, K = 2^nc) has its real part at source offset src_base +
// sum_j bit_j(e) * sw[j] (reals) and its imaginary part src_im reals further.
// Output rows of 2K reals: row f = [Re(f, 0..K), Im(f, 0..K)]; a doubled
// operand writes [Re, -Im] in row f and [Im, Re] in row F + f.
// The copy runs in tiles of 2^tb elements staged in shared memory: the tile
// holds the element bits of the lowest source offsets (read in order) and the
// 5 lowest element bits (written in order).  tile_bit lists the tile's element
// bits in write order; r2w maps read-order tile bit i to its write-order bit;
// outer_bit lists the remaining element bits.
constexpr int kTnTileBits = 10;
struct TnGatherOp {
  const void* src;
  void* dst;
  int64_t src_bstride;  // reals between batch entries of the source (0: shared)
  int64_t src_base;     // reals: slice offset
  int64_t src_im;       // reals from the real to the imaginary part
  int64_t nb;           // batch entries gathered (1 for a shared operand)
  int64_t sw[kTnMaxBits];
  int32_t nbits, nc, doubled, tb, n_outer;
  // vector access: rmode 0 = scalar reads, 1 = two adjacent elements per
  // thread (unit source weight on the lowest read bit), 2 = (re, im) pairs of
  // interleaved leaves; wpair = two adjacent elements per store (nc >= 1)
  int8_t rmode, wpair, pad[2];
  int8_t tile_bit[kTnTileBits];
  int8_t r2w[kTnTileBits];
  int8_t outer_bit[kTnMaxBits];
};

struct TnGatherArgs {
  TnGatherOp op[2];
};

// One operand of a fused contraction, read in place: element (f, k) of the
// operand's [F][K] view has its real part at src + b * bstride + base +
// sum_j bit_j(f) * wf[j] + sum_j bit_j(k) * wk[j] (reals) and its imaginary
// part `im` reals further.
struct TnFusedOp {
  const void* src;
  int64_t bstride;
  int64_t base;
  int64_t im;
  int64_t wf[kTnMaxBits];
  int64_t wk[kTnMaxBits];
};

// C[b](i, j) = sum_k A[b](i, k) B[b](k, j), written planar: Re at j * M + i,
// Im at + M * N (M = 2^lm, N = 2^ln, K = 2^lk <= 256).
struct TnFusedArgs {
  TnFusedOp a, b;
  void* dst;
  int64_t dst_bstride;
  int64_t nb;  // batch entries
  int32_t lm, ln, lk, pad;
};

template <typename real>
cudaError_t tn_fused(const TnFusedArgs& args, cudaStream_t stream);

// One fused contraction of a level launch (all fused steps of one dependency
// level run in one kernel).  Offsets are in reals from a region base (0: the
// call's workspace, 1: the plan's constant leaves), so one table serves every
// call with the same batch size.  Operand element (f, k) has its real part at
// base + b * bstride + sum_j bit_j(f) wf[j] + sum_j bit_j(k) wk[j] (+ the
// slice weights of the sliced indices set in the current slice) and its
// imaginary part `im` reals further; the result is planar (Re at j * M + i,
// Im at + M * N).
constexpr int kTnItemFree = 16, kTnItemSum = 8, kTnItemSlice = 6;
struct TnFusedItem {
  int64_t off[2];      // operand a / b
  int64_t bstride[2];  // 0: shared by all circuits
  int64_t im[2];
  int64_t dst_off, dst_bstride;
  int32_t region[2];
  int32_t nb;    // circuits computed (1: unbatched step)
  int32_t blk0;  // first CTA of the item within its level launch
  int32_t lm, ln, lk, nsl0, nsl1, pad;
  int32_t slq[2][kTnItemSlice];  // sliced index numbers
  int32_t slw[2][kTnItemSlice];  // their weights (reals)
  int32_t wf[2][kTnItemFree];
  int32_t wk[2][kTnItemSum];
};

// Items [0, n_items) of one level; grid = blk0 of the last item + its CTAs.
template <typename real>
cudaError_t tn_fused_level(const TnFusedItem* items, int n_items, int blocks, char* ws, const void* consts,
                           int64_t slice, cudaStream_t stream);

template <typename real>
cudaError_t tn_build_leaves(const TnLeafDesc* desc, int n_desc, const real* params, int n_params, int64_t batch,
                            real* leaves, cudaStream_t stream);
template <typename real>
cudaError_t tn_gather(const TnGatherArgs& args, cudaStream_t stream);
// acc[b * n_meas + m] (+)= Re(root) for every circuit b (first: assign);
// last: out[b * n_meas + m] = acc (NaN for a circuit with a non-finite
// parameter, and for every circuit when the device error word `err` is set).
template <typename real>
cudaError_t tn_root(const real* root, int64_t root_bstride, int64_t batch, double* acc, real* out, int n_meas,
                    int m, int first, int last, const real* params, int n_params, const int* err,
                    cudaStream_t stream);

}  // namespace tedq
