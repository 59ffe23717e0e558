// sv_kernels.cuh -- launch interface of the state-vector kernels (sv_kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "sv_plan.h"

namespace tedq {

constexpr int kMaxTerms = 256;
constexpr int kMaxOutTerms = 512;
constexpr int kMaxProbsOut = 16;

struct TermDev {
  uint64_t x, z;
  int32_t ny;   // number of Y factors (phase (-i)^ny)
  int32_t pad;
};

struct TermTable {
  int32_t n;
  int32_t pad;
  TermDev t[kMaxTerms];
};

struct OutTermTable {  // expval outputs: out[k] = sum coef * term[s]
  int32_t n;           // entries
  int32_t n_real;      // outputs per circuit
  int32_t n_terms;
  int32_t pad;
  int32_t k[kMaxOutTerms];
  int32_t s[kMaxOutTerms];
  double coef[kMaxOutTerms];
};

struct ProbsDesc {
  int32_t offset;      // output index of bin 0
  int32_t nbits;       // measured bits
  int32_t acc_off;     // offset in the per-circuit probs accumulator (partial probs)
  int32_t full;        // 1: all logical qubits (direct write)
  uint8_t bits[kMaxStateBits];  // msb of the bin first
  uint8_t pad[6];
};

struct ProbsTable {
  int32_t n;
  int32_t n_bins;     // accumulator bins per circuit (partial probs)
  int32_t pad_bits;   // idle low-order qubits of the padded state
  int32_t pad;
  ProbsDesc p[kMaxProbsOut];
};

// Forward pass over a batch: psi [batch][2^n]; params [batch][n_params].
// Persistent grid of a pass kernel: as many CTAs as fit on the current device
// at once, at most one per tile.  `query` returns the resident CTAs per SM of
// the kernel (key) at the given block size and dynamic shared memory; its
// answer and the SM count are cached per device, so that only the first
// launch of a kernel shape makes runtime queries (later launches may run
// inside stream capture).
cudaError_t pass_grid_cached(const void* key, int threads, size_t smem, int64_t n_tiles,
                             cudaError_t (*query)(const void* key, int threads, size_t smem, int* per_sm),
                             unsigned& grid);

cudaError_t launch_fwd_pass(bool dbl, const PassParams& P, void* psi, const void* params, int n_params,
                            const void* init, int64_t batch, cudaStream_t s);
// Adjoint pass: uncomputes psi and lambda through the pass's gates and adds
// gradients into grad_acc [batch][n_params] (double).
cudaError_t launch_bwd_pass(bool dbl, const PassParams& P, void* psi, void* lam, const void* params,
                            int n_params, double* grad_acc, int64_t batch, cudaStream_t s);
// Writes |0..0> (init == nullptr) or the padded initial state into psi.
cudaError_t launch_init_state(bool dbl, int n, int pad, void* psi, const void* init, int64_t batch,
                              cudaStream_t s);
// Pauli-string expectation accumulators term_acc [batch][n_terms] (+=).
cudaError_t launch_expval(bool dbl, int n, const TermTable& T, const void* psi, double* term_acc,
                          int64_t batch, cudaStream_t s);
// Probabilities: partial ones accumulate into probs_acc, full ones are written
// straight into out_real.
cudaError_t launch_probs(bool dbl, int n, const ProbsTable& PT, const void* psi, double* probs_acc,
                         void* out_real, int n_real, int64_t batch, cudaStream_t s);
// out_real from the accumulators.
cudaError_t launch_finalize(bool dbl, const OutTermTable& O, const ProbsTable& PT, const double* term_acc,
                            const double* probs_acc, void* out_real, int64_t batch, cudaStream_t s);
// w [batch][n_terms] = sum_k dy[k] coef_{k,s}
cudaError_t launch_term_weights(bool dbl, const OutTermTable& O, const void* dy_real, double* w,
                                int64_t batch, cudaStream_t s);
// lambda = sum_s w_s P_s psi + sum_probs dy_bin psi + dy_state / 2
cudaError_t launch_lambda_init(bool dbl, int n, const TermTable& T, const ProbsTable& PT, const double* w,
                               const void* dy_real, int n_real, const void* dy_state, const void* psi,
                               void* lam, int64_t batch, cudaStream_t s);
// grad [batch][n_params] (float or double) from the double accumulators.
cudaError_t launch_grad_finalize(bool dbl, const double* grad_acc, void* grad, int64_t count, cudaStream_t s);

}  // namespace tedq
