// sv_program.h -- host-side compiled program (the GB300 replacement of the
// reference's CompiledCircuit, tedq/backends/compiled_circuit.py:48-202).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "sv_plan.h"
#include "tedq_gb300.h"

namespace tedq {

// One factor of a one-qubit matrix before it is placed into a pass.
struct HFactor {
  uint8_t op = F_FIXED2;
  int32_t slot[3] = {-1, -1, -1};
  double val[3] = {0, 0, 0};
  CD m[4] = {};  // F_FIXED2: row-major 2x2; F_FIXD: m[0], m[1] = diagonal
};

// Elementary gate at global-bit level.
struct HGate {
  uint8_t kind = GK_U1;     // GateKind, or kDense
  int t0 = -1, t1 = -1;     // target bits (t1: SWAP)
  uint64_t cmask = 0;       // control bits
  std::vector<HFactor> factors;  // U1/D1
  // dense fixed k-qubit gate (applied in shared memory)
  int dk = 0;
  int dbits[3] = {-1, -1, -1};  // dbits[0] = most significant matrix bit
  std::vector<CD> dmat;         // 4^dk entries
  // adjoint gradient
  uint8_t grad = GR_NONE;
  int32_t slot = -1;
  float coef = 0.f;
  uint64_t bits() const;
};
constexpr uint8_t kDense = 15;

struct Term {            // Hermitian Pauli string (-i)^ny X^x Z^z
  uint64_t x = 0, z = 0;
};
struct OutTerm {         // out_real[k] += coef * <term s>
  int32_t k, s;
  double coef;
};
struct ProbsOut {
  int32_t offset;        // first output index in out_real
  std::vector<int> bits; // measured bits, most significant bin bit first
};

struct Schedule {
  std::vector<PassParams> passes;
  int n_phases = 0;
};

struct Program {
  int n = 0;             // logical qubits
  int ns = 0;            // state qubits (padded)
  int pad = 0;           // ns - n
  int n_params = 0;
  int precision = TEDQ_PREC_C64;
  int fuse = 1;
  int tile_qubits = 0;
  bool phase_free = false;  // forward passes may drop global phases (no state output)
  bool normalise = false;   // normalised RX / RY register gates (GK_RXN / GK_RYN)
  std::vector<HGate> elem;    // elementary gates, circuit order
  std::vector<HGate> fused;   // forward gates after fusion
  Schedule fwd, bwd;
  // measurements
  std::vector<Term> terms;
  std::vector<OutTerm> out_terms;
  std::vector<ProbsOut> probs;
  int n_real = 0;
  int n_expval = 0;
  int64_t ws_per_circuit = 0;  // bytes
  int64_t ws_terms_off = 0, ws_probs_off = 0, ws_grad_off = 0, ws_w_off = 0;
  int n_probs_bins = 0;
};

// Throws std::runtime_error / std::invalid_argument on bad input.
Program* compile_program(const tedq_gate_t* gates, int n_gates, int n_qubits,
                         const tedq_meas_t* meas, int n_meas, const tedq_options_t* opts);
std::string describe_schedule(const Program& p, bool adjoint);

struct UnsupportedError : std::exception {
  std::string msg;
  explicit UnsupportedError(std::string m) : msg(std::move(m)) {}
  const char* what() const noexcept override { return msg.c_str(); }
};

}  // namespace tedq
