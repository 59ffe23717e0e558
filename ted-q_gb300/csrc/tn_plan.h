// tn_plan.h -- tensor-network contraction mode: network construction and
// contraction planning (host, internal).
//
// Reference counterpart: gen_tensor_networks (tedq/tensor_network/
// tensor_network.py:850-1099) builds, per measurement, the index lists of the
// <0| U^dagger O U |0> "sandwich"; the contraction order comes from an
// external optimiser (opt_einsum in tedq/oe_wrapper/oe_wrapper.py:24-65,
// JDtensorPath or cotengra) and torch einsum executes it
// (pytorch_backend.py:242-356).  Here the same network is built natively,
// reduced to the backward light cone of the observable, ordered by a
// randomised greedy search, sliced to a memory target, and executed on the
// GPU as bit-permutation gathers plus real GEMMs (tn_kernels.cu).
//
// Network form.  The value is sum_a conj(psi_a) (O psi)_a with psi = U|0>:
// the ket side holds |0> vectors, the gate tensors U and the observable
// factors; the bra side holds <0| vectors and conj(U) in the same
// orientation; the last ket and bra index of every qubit are one index.
// Every index has dimension 2 and joins exactly two tensors.
//
// Storage of a tensor with index list L (rank r): element at flat index
// sum_t bit_t << (r-1-t), i.e. L[0] is the most significant bit.
//  * leaves: interleaved complex;
//  * intermediates: the result C (M x N, M = 2^|free_a|, N = 2^|free_b|) of
//    one real GEMM over the real embedding of the complex product -- either
//    [Re A, Im A] (M x 2K) x [[Re B, Im B], [-Im B, Re B]] (2K x 2N) = [Re C, Im C]
//    ("planar": Re C(i,j) at j*M + i, Im C at + M*N), or
//    [[Re A, -Im A], [Im A, Re A]] (2M x 2K) x [Re B; Im B] (2K x N) = [Re C; Im C]
//    ("split": Re C(i,j) at j*2M + i, Im C at + M).  The operand with the
//    smaller free dimension is the doubled one.  Index list: free_b ++ free_a
//    (i is the low part of the flat index).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "tedq_gb300.h"

namespace tedq {

enum TnLeaf : int { TL_KET0 = 0, TL_BRA0 = 1, TL_GATE = 2, TL_GATE_CONJ = 3, TL_OBS = 4 };

struct TnTensor {
  std::vector<int> full_idx;  // leaves: index list before slicing
  std::vector<int> idx;       // index list (sliced indices removed)
  int leaf = -1;              // TnLeaf, -1 for intermediates
  int gate = -1;              // TL_GATE / TL_GATE_CONJ: index into TnNet::gates
  bool batched = false;       // depends on the parameters
  int lm = 0, ln = 0;         // intermediates: |free_a|, |free_b| of the producing step
  bool split = false;         // intermediates: "split" layout (else "planar")
  // leaves: offset of the stored tensor (complex elements); batched leaves in
  // the per-call batched-leaf region (times the batch), the others in the
  // plan's constant buffer
  int64_t off = 0;
  // intermediates: offset in the batched / unbatched intermediate arena (reals)
  int64_t arena = 0;
};

struct TnGate {
  int op = 0, k = 1;
  int qubits[3] = {0, 0, 0};
  int32_t slot[3] = {-1, -1, -1};
  double val[3] = {0, 0, 0};
  bool param = false;         // some parameter is bound to a slot
  std::vector<double> fixed;  // !param: 2 * 4^k doubles (re, im), row-major
};

// Gather of one GEMM operand: element e = f*K + k (K = 2^nc) takes source bit
// src_bit[o] for bit o of e (o = 0 least significant); leaf operands with
// sliced indices add slice_bit[q] when sliced index q is 1.  Rows of 2K reals:
// [Re(f,:), Im(f,:)], and for the doubled operand F more rows
// [Im(f,:), Re(f,:)] after rows [Re(f,:), -Im(f,:)].
struct TnOperand {
  int tensor = -1;
  int nf = 0, nc = 0;
  bool doubled = false;
  std::vector<int> src_bit;
  std::vector<std::pair<int, int>> slice_bit;  // (sliced index number, source bit)
};

struct TnStep {
  int a = -1, b = -1, out = -1;
  std::vector<int> free_a, free_b, contracted;
  TnOperand opa, opb;
  bool batched = false;
  bool double_a = false;  // A is the doubled operand (result in "split" layout)
  // small contraction: one fused kernel reads both operands in place and
  // writes the planar result (no gathers, no GEMM call)
  bool fused = false;
  // dependency depth (leaf inputs only: 0).  Steps are stored by level, the
  // fused ones of a level first: one launch runs all fused steps of a level
  // together, then the level's GEMM steps run one by one.
  int level = 0;
};

struct TnNet {
  int n = 0;
  std::vector<TnGate> gates;  // ket-side gates kept by the light cone, then observable factors
  int n_circuit_gates = 0;    // gates[0 .. n_circuit_gates) are circuit gates
  std::vector<TnTensor> tensors;
  int n_leaves = 0;
  int n_index = 0;
  std::vector<TnStep> steps;
  int root = -1;
  std::vector<int> sliced;
  int max_rank = 0;            // largest intermediate (after slicing)
  double log2_flops = 0;       // real flops of one evaluation, all slices (8 per complex MAC)
  int gates_in = 0, gates_kept = 0, qubits_kept = 0;
  // sizes
  int64_t batched_leaf_elems = 0;    // complex, per batch entry
  int64_t const_elems = 0;           // complex
  int64_t batched_arena = 0;         // reals, per batch entry
  int64_t unbatched_arena = 0;       // reals
  std::vector<double> constants;     // const_elems (re, im) pairs
};

struct TnPlanOptions {
  int fused_log2 = 13;  // contractions below 2^fused_log2 complex MACs per circuit run fused
  // ... and, when >= 0, contractions over at most 2^fused_short_log2 terms
  // with up to 2^16 outputs per circuit.  Off: on the 6x6 lattice the in-place
  // kernel ran those slower than gather + GEMM (uncoalesced operand reads;
  // 258k vs 283k contractions/s with 3)
  int fused_short_log2 = -1;
  int max_rank = 27;   // slice until every intermediate has at most 2^max_rank entries
  int repeats = 64;    // randomised greedy trials (the first is plain greedy)
  uint64_t seed = 1;
};

// Builds the light-cone-reduced sandwich network of one expectation value and
// plans its contraction.  Throws std::invalid_argument / UnsupportedError.
TnNet tn_build(const tedq_gate_t* gates, int n_gates, int n_qubits, const tedq_meas_t& meas,
               const TnPlanOptions& opt);
// Planar GEMM operands of the largest step for a batch (reals).
int64_t tn_scratch_reals(const TnNet& net, int64_t batch);
std::string tn_describe(const std::vector<TnNet>& nets, int n_params, int precision);

}  // namespace tedq
