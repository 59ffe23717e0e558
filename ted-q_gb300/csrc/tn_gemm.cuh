// tn_gemm.cuh -- batched real GEMMs of the tensor-network mode (tn_gemm.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tedq {

// C[b](i, j) = sum_k A[b](i, k) B[b](j, k) for b < nbatch; A [mr][kr] and
// B [nr][kr] K-contiguous, C column-major [nr][mr] (i fastest).  Strides in
// reals between batch entries; 0 = the operand is shared by every entry.
struct TnGemmArgs {
  const void* a;
  const void* b;
  void* c;
  int64_t mr, nr, kr;
  int64_t sa, sb, sc;
  int64_t nbatch;
  int* err;  // device error word: set when a bounded wait of the tensor-core kernel gives up
};

// Tensor-core path (FP32 data): tcgen05 kind::tf32 MMAs from TMA-staged,
// 128-byte-swizzled shared memory, accumulators in tensor memory.
// split = true: 3xTF32 (FP32 accuracy); false: one TF32 product per term.
bool tn_gemm_tc_supported(const TnGemmArgs& g);
cudaError_t tn_gemm_tc(const TnGemmArgs& g, bool split, cudaStream_t stream);

// Shared-memory-tiled FMA kernel (float or double).
template <typename real>
cudaError_t tn_gemm_simt(const TnGemmArgs& g, cudaStream_t stream);

}  // namespace tedq
