// sv_program.cpp -- compiles a recorded circuit into the pass/phase schedule
// executed by sv_kernels.cu.
//
// Reference counterpart: CompiledCircuit.__init__ precomputes one tensordot
// axes pair and one inverse permutation per gate (tedq/backends/
// compiled_circuit.py:126-202) and the gate tensors are rebuilt on every call
// (compiled_circuit.py:418-440, pytorch_backend.py:579-1188).  Here the
// compile step instead
//   1. classifies every gate as diagonal / bit-flip / swap / dense one-qubit
//      matrix with control bits, or a dense multi-qubit fixed matrix;
//   2. fuses runs of uncontrolled one-qubit gates on the same qubit into one
//      2x2 matrix (forward only; the adjoint sweep needs every parameterised
//      gate separately for its gradient);
//   3. schedules the gate list greedily into HBM passes over tiles of 2^m
//      amplitudes and, inside a pass, into register phases of R bits;
//   4. expands expectation-value observables into Hermitian Pauli strings.
#include "sv_program.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>

namespace tedq {

using cplx = std::complex<double>;

static inline int popc(uint64_t v) { return __builtin_popcountll(v); }

uint64_t HGate::bits() const {
  uint64_t b = cmask;
  if (t0 >= 0) b |= 1ull << t0;
  if (t1 >= 0) b |= 1ull << t1;
  for (int i = 0; i < dk; ++i) b |= 1ull << dbits[i];
  return b;
}

// ---------------------------------------------------------------- gate model

static HFactor fixed2(cplx a, cplx b, cplx c, cplx d) {
  HFactor f;
  f.op = F_FIXED2;
  f.m[0] = {a.real(), a.imag()};
  f.m[1] = {b.real(), b.imag()};
  f.m[2] = {c.real(), c.imag()};
  f.m[3] = {d.real(), d.imag()};
  return f;
}
static HFactor fixedd(cplx a, cplx d) {
  HFactor f;
  f.op = F_FIXD;
  f.m[0] = {a.real(), a.imag()};
  f.m[1] = {d.real(), d.imag()};
  return f;
}
static HFactor paramf(uint8_t op, const tedq_gate_t& g, int i0, int i1 = -1, int i2 = -1) {
  HFactor f;
  f.op = op;
  int idx[3] = {i0, i1, i2};
  for (int j = 0; j < 3; ++j) {
    if (idx[j] < 0) continue;
    f.slot[j] = g.param_slot[idx[j]];
    f.val[j] = g.fixed[idx[j]];
  }
  return f;
}

static bool is_diag_factor(const HFactor& f) {
  return f.op == F_FIXD || f.op == F_RZ || f.op == F_PHASE;
}

static HGate one_qubit(int bit, HFactor f, uint64_t cmask = 0) {
  HGate h;
  h.kind = is_diag_factor(f) ? GK_D1 : GK_U1;
  h.t0 = bit;
  h.cmask = cmask;
  h.factors.push_back(f);
  return h;
}

static HGate bitflip(int bit, uint64_t cmask = 0) {
  HGate h;
  h.kind = GK_X;
  h.t0 = bit;
  h.cmask = cmask;
  return h;
}

static HGate swapg(int a, int b, uint64_t cmask = 0) {
  HGate h;
  h.kind = GK_SWAP;
  h.t0 = a;
  h.t1 = b;
  h.cmask = cmask;
  return h;
}

static void set_grad(HGate& h, int32_t slot, uint8_t kind, float coef) {
  if (slot < 0) return;
  h.grad = kind;
  h.slot = slot;
  h.coef = coef;
}

static const double kInvSqrt2 = 0.70710678118654752440;

// Classify a fixed k-qubit matrix (row-major, qubits[0] most significant).
static void classify_matrix(const std::vector<cplx>& M, int k, const int* bits, std::vector<HGate>& out) {
  const int d = 1 << k;
  auto at = [&](int r, int c) { return M[r * d + c]; };
  auto is0 = [](cplx v) { return v.real() == 0.0 && v.imag() == 0.0; };
  auto is1 = [](cplx v) { return v.real() == 1.0 && v.imag() == 0.0; };
  if (k == 1) {
    if (is0(at(0, 1)) && is0(at(1, 0))) {
      if (is1(at(0, 0)) && is1(at(1, 1))) return;  // identity
      out.push_back(one_qubit(bits[0], fixedd(at(0, 0), at(1, 1))));
    } else if (is0(at(0, 0)) && is0(at(1, 1)) && is1(at(0, 1)) && is1(at(1, 0))) {
      out.push_back(bitflip(bits[0]));
    } else {
      out.push_back(one_qubit(bits[0], fixed2(at(0, 0), at(0, 1), at(1, 0), at(1, 1))));
    }
    return;
  }
  // controlled-U on the last matrix bit: identity wherever the first k-1
  // matrix bits are not all 1.
  auto controlled_last = [&]() {
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) {
        bool blk = (r >> 1) == (d / 2 - 1) && (c >> 1) == (d / 2 - 1);
        if (blk) continue;
        cplx v = at(r, c);
        if (r == c ? !is1(v) : !is0(v)) return false;
      }
    return true;
  };
  if (controlled_last()) {
    uint64_t cm = 0;
    for (int i = 0; i < k - 1; ++i) cm |= 1ull << bits[i];
    std::vector<cplx> U = {at(d - 2, d - 2), at(d - 2, d - 1), at(d - 1, d - 2), at(d - 1, d - 1)};
    std::vector<HGate> tmp;
    int tb = bits[k - 1];
    classify_matrix(U, 1, &tb, tmp);
    for (auto& g : tmp) {
      g.cmask |= cm;
      out.push_back(g);
    }
    return;
  }
  if (k == 2) {
    // controlled on the second matrix bit (target = first)
    bool ok = true;
    for (int r = 0; r < 4 && ok; ++r)
      for (int c = 0; c < 4 && ok; ++c) {
        bool blk = (r & 1) && (c & 1);
        if (blk) continue;
        cplx v = at(r, c);
        ok = (r == c) ? is1(v) : is0(v);
      }
    if (ok) {
      std::vector<cplx> U = {at(1, 1), at(1, 3), at(3, 1), at(3, 3)};
      std::vector<HGate> tmp;
      int tb = bits[0];
      classify_matrix(U, 1, &tb, tmp);
      for (auto& g : tmp) {
        g.cmask |= 1ull << bits[1];
        out.push_back(g);
      }
      return;
    }
  }
  // permutation swapping the last two matrix bits (SWAP, or CSWAP for k=3)
  {
    bool ok = true;
    for (int r = 0; r < d && ok; ++r)
      for (int c = 0; c < d && ok; ++c) {
        int hi = r >> 2, a = (r >> 1) & 1, b = r & 1;
        int swapped = (k == 3 && hi == 0) ? r : ((hi << 2) | (b << 1) | a);
        if (k == 2) swapped = ((r & 1) << 1) | ((r >> 1) & 1);
        ok = (c == swapped) ? is1(at(r, c)) : is0(at(r, c));
      }
    if (ok) {
      uint64_t cm = (k == 3) ? (1ull << bits[0]) : 0;
      out.push_back(swapg(bits[k - 2], bits[k - 1], cm));
      return;
    }
  }
  HGate h;
  h.kind = kDense;
  h.dk = k;
  for (int i = 0; i < k; ++i) h.dbits[i] = bits[i];
  for (auto v : M) h.dmat.push_back({v.real(), v.imag()});
  out.push_back(h);
}

// Elementary gates of one recorded gate (global bit = ns - 1 - qubit).
static void lower_gate(const tedq_gate_t& g, int n, int ns, std::vector<HGate>& out) {
  int k = g.n_qubits;
  if (k < 1 || k > 3) throw std::invalid_argument("gate with unsupported number of qubits");
  int b[3];
  for (int i = 0; i < k; ++i) {
    if (g.qubits[i] < 0 || g.qubits[i] >= n) throw std::invalid_argument("gate qubit index out of range");
    b[i] = ns - 1 - g.qubits[i];
    for (int j = 0; j < i; ++j)
      if (b[j] == b[i]) throw std::invalid_argument("gate acts twice on one qubit");
  }
  static const int arity[] = {1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 2, 2, 2, 2};
  if (g.op < 0 || g.op > TEDQ_OP_MATRIX) throw std::invalid_argument("unknown gate opcode");
  if (g.op != TEDQ_OP_MATRIX && arity[g.op] != k) throw std::invalid_argument("gate arity mismatch");
  const cplx I(0, 1);
  switch (g.op) {
    case TEDQ_OP_I: return;
    case TEDQ_OP_H: out.push_back(one_qubit(b[0], fixed2(kInvSqrt2, kInvSqrt2, kInvSqrt2, -kInvSqrt2))); return;
    case TEDQ_OP_X: out.push_back(bitflip(b[0])); return;
    case TEDQ_OP_Y: out.push_back(one_qubit(b[0], fixed2(0, -I, I, 0))); return;
    case TEDQ_OP_Z: out.push_back(one_qubit(b[0], fixedd(1, -1))); return;
    case TEDQ_OP_S: out.push_back(one_qubit(b[0], fixedd(1, I))); return;
    case TEDQ_OP_T: out.push_back(one_qubit(b[0], fixedd(1, std::exp(I * (M_PI / 4))))); return;
    case TEDQ_OP_SX: out.push_back(one_qubit(b[0], fixed2(cplx(.5, .5), cplx(.5, -.5), cplx(.5, -.5), cplx(.5, .5)))); return;
    case TEDQ_OP_CNOT: out.push_back(bitflip(b[1], 1ull << b[0])); return;
    case TEDQ_OP_CZ: out.push_back(one_qubit(b[1], fixedd(1, -1), 1ull << b[0])); return;
    case TEDQ_OP_CY: out.push_back(one_qubit(b[1], fixed2(0, -I, I, 0), 1ull << b[0])); return;
    case TEDQ_OP_SWAP: out.push_back(swapg(b[0], b[1])); return;
    case TEDQ_OP_CSWAP: out.push_back(swapg(b[1], b[2], 1ull << b[0])); return;
    case TEDQ_OP_TOFFOLI: out.push_back(bitflip(b[2], (1ull << b[0]) | (1ull << b[1]))); return;
    case TEDQ_OP_RX: {
      HGate h = one_qubit(b[0], paramf(F_RX, g, 0));
      set_grad(h, g.param_slot[0], GR_X, 1.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_RY: {
      HGate h = one_qubit(b[0], paramf(F_RY, g, 0));
      set_grad(h, g.param_slot[0], GR_Y, 1.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_RZ: {
      HGate h = one_qubit(b[0], paramf(F_RZ, g, 0));
      set_grad(h, g.param_slot[0], GR_Z, 1.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_PHASESHIFT: {
      HGate h = one_qubit(b[0], paramf(F_PHASE, g, 0));
      set_grad(h, g.param_slot[0], GR_P1, -2.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_ROT: {
      // Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi) (qubit.py:1137-1208)
      HGate a = one_qubit(b[0], paramf(F_RZ, g, 0));
      set_grad(a, g.param_slot[0], GR_Z, 1.f);
      HGate m = one_qubit(b[0], paramf(F_RY, g, 1));
      set_grad(m, g.param_slot[1], GR_Y, 1.f);
      HGate c = one_qubit(b[0], paramf(F_RZ, g, 2));
      set_grad(c, g.param_slot[2], GR_Z, 1.f);
      out.push_back(a);
      out.push_back(m);
      out.push_back(c);
      return;
    }
    case TEDQ_OP_CPHASE: {
      HGate h = one_qubit(b[1], paramf(F_PHASE, g, 0), 1ull << b[0]);
      set_grad(h, g.param_slot[0], GR_P1, -2.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_CRX: {
      HGate h = one_qubit(b[1], paramf(F_RX, g, 0), 1ull << b[0]);
      set_grad(h, g.param_slot[0], GR_X, 1.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_CRY: {
      HGate h = one_qubit(b[1], paramf(F_RY, g, 0), 1ull << b[0]);
      set_grad(h, g.param_slot[0], GR_Y, 1.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_CRZ: {
      HGate h = one_qubit(b[1], paramf(F_RZ, g, 0), 1ull << b[0]);
      set_grad(h, g.param_slot[0], GR_Z, 1.f);
      out.push_back(h);
      return;
    }
    case TEDQ_OP_MATRIX: {
      if (!g.matrix) throw std::invalid_argument("TEDQ_OP_MATRIX without matrix");
      int d = 1 << k;
      std::vector<cplx> M(d * d);
      for (int i = 0; i < d * d; ++i) M[i] = cplx(g.matrix[2 * i], g.matrix[2 * i + 1]);
      classify_matrix(M, k, b, out);
      return;
    }
  }
}

// ---------------------------------------------------------------- fusion

static bool is_hadamard(const HGate& g);
static uint8_t normalised_kind(const HGate& g, bool norm);
static uint8_t specialised_kind(const HGate& g, bool phase_free, bool norm);

// Register-phase cost of a gate (packed FP32x2 instructions per amplitude of
// one state): the fused form is kept only where it is cheaper than its parts.
// A normalised rotation counts as 1 (one FFMA2 per component): with the tile
// pipeline, RX RY RZ as three normalised gates measured 3 % faster than the
// fused dense 2x2 in the forward passes (96.9 -> 93.8 ms per step on the
// 20-qubit VQC; with one tile per CTA the fused form had been faster, the
// kernels then being more sensitive to code size).
// TEDQ_GB300_NORM_COST=<1..4> overrides the 1 (a measurement knob).
static int norm_cost() {
  const char* env = getenv("TEDQ_GB300_NORM_COST");
  return (env && env[0] >= '1' && env[0] <= '4' && !env[1]) ? env[0] - '0' : 1;
}

static int gate_cost(const HGate& g, bool norm) {
  if (g.kind == GK_X || g.kind == GK_SWAP) return 0;
  if (normalised_kind(g, norm)) return norm_cost();
  if (g.kind == GK_D1) return (norm && g.cmask == 0) || specialised_kind(g, false, false) == GK_PH ? 1 : 2;
  if (is_hadamard(g)) return 2;
  if (g.factors.size() == 1 && (g.factors[0].op == F_RX || g.factors[0].op == F_RY)) return 2;
  return 4;
}

// Runs of uncontrolled one-qubit gates on the same qubit become one gate
// (product of their factors).  With normalised rotations (norm: the forward
// passes may drop global phases) a run whose parts cost less than the fused
// matrix stays unfused, e.g. RZ H = 1 + 2 against 4 for a dense 2x2.
static std::vector<HGate> fuse_one_qubit_runs(const std::vector<HGate>& in, int ns, bool norm) {
  std::vector<HGate> out;
  std::vector<std::vector<HGate>> parts;  // source gates of out[i]
  std::vector<int> last(ns, -1);
  const size_t kMaxRun = 8;
  for (const HGate& g : in) {
    bool single = (g.kind == GK_U1 || g.kind == GK_D1 || g.kind == GK_X) && g.cmask == 0;
    if (single) {
      int j = last[g.t0];
      if (j >= 0) {
        HGate& f = out[j];
        bool fsingle = (f.kind == GK_U1 || f.kind == GK_D1 || f.kind == GK_X) && f.cmask == 0;
        if (fsingle && f.factors.size() < kMaxRun) {
          auto add = [&](const HGate& s) {
            if (s.kind == GK_X) f.factors.push_back(fixed2(0, 1, 1, 0));
            else for (auto& x : s.factors) f.factors.push_back(x);
          };
          if (f.kind == GK_X) {
            f.factors.clear();
            f.factors.push_back(fixed2(0, 1, 1, 0));
          }
          add(g);
          bool all_diag = true;
          for (auto& x : f.factors) all_diag &= is_diag_factor(x);
          f.kind = all_diag ? GK_D1 : GK_U1;
          f.grad = GR_NONE;
          f.slot = -1;
          parts[j].push_back(g);
          continue;
        }
      }
    }
    out.push_back(g);
    parts.push_back({g});
    uint64_t b = g.bits();
    for (int i = 0; i < ns; ++i)
      if (b >> i & 1) last[i] = (int)out.size() - 1;
  }
  if (!norm) return out;
  // the parts of a run act on one qubit with nothing else on it in between:
  // they may replace the fused gate at its position
  std::vector<HGate> res;
  for (size_t i = 0; i < out.size(); ++i) {
    int sum = 0;
    for (const HGate& q : parts[i]) sum += gate_cost(q, true);
    if (parts[i].size() > 1 && sum < gate_cost(out[i], true))
      res.insert(res.end(), parts[i].begin(), parts[i].end());
    else
      res.push_back(out[i]);
  }
  return res;
}

// ---------------------------------------------------------------- scheduling

struct Geometry {
  int m, c, e, R;
};

static std::vector<int> sorted_bits(uint64_t mask) {
  std::vector<int> v;
  for (int i = 0; i < 64; ++i)
    if (mask >> i & 1) v.push_back(i);
  return v;
}

static uint64_t fill_bits(uint64_t mask, int want, int limit) {
  for (int i = 0; i < limit && popc(mask) < want; ++i) mask |= 1ull << i;
  return mask;
}

// A lone Hadamard factor (runs its own matrix-free register code).
static bool is_hadamard(const HGate& g) {
  if (g.kind != GK_U1 || g.factors.size() != 1 || g.factors[0].op != F_FIXED2) return false;
  const CD* m = g.factors[0].m;
  return m[0].re == kInvSqrt2 && m[1].re == kInvSqrt2 && m[2].re == kInvSqrt2 && m[3].re == -kInvSqrt2 &&
         m[0].im == 0.0 && m[1].im == 0.0 && m[2].im == 0.0 && m[3].im == 0.0;
}

// Register kind of a gate: structured one-factor rotations and phase-type
// diagonals get cheaper register code than a dense / general diagonal matrix.
// Uncontrolled diagonal gates whose global phase may be dropped: applied as
// diag(1, d1 / d0), multiplying only the |1> half.
static bool phase_droppable(const HGate& g, bool phase_free) {
  return phase_free && g.kind == GK_D1 && g.cmask == 0;
}

// Uncontrolled one-factor RX / RY gates that run normalised (GK_RXN / GK_RYN).
static uint8_t normalised_kind(const HGate& g, bool norm) {
  if (!norm || g.kind != GK_U1 || g.cmask != 0 || g.factors.size() != 1) return 0;
  if (g.factors[0].op == F_RX) return GK_RXN;
  if (g.factors[0].op == F_RY) return GK_RYN;
  return 0;
}

static uint8_t specialised_kind(const HGate& g, bool phase_free, bool norm) {
  if (is_hadamard(g)) return GK_H;
  if (const uint8_t k = normalised_kind(g, phase_free && norm)) return k;
  if (phase_droppable(g, phase_free)) return GK_PH;
  if (g.kind == GK_U1 && g.factors.size() == 1) {
    if (g.factors[0].op == F_RX) return GK_RXT;
    if (g.factors[0].op == F_RY) return GK_RYT;
  }
  if (g.kind == GK_D1) {
    bool phase = true;
    for (const HFactor& f : g.factors)
      phase &= f.op == F_PHASE || (f.op == F_FIXD && f.m[0].re == 1.0 && f.m[0].im == 0.0);
    if (phase) return GK_PH;
  }
  return g.kind;
}

// Capacity counters of a pass under construction.
struct Cap {
  int gates = 0, mats = 0, factors = 0, fixed = 0, grads = 0;
  bool fits(const HGate& g) const {
    if (is_hadamard(g)) return gates + 1 <= kMaxPassGates;
    int nf = (int)g.factors.size(), nfix = 0;
    for (auto& f : g.factors) nfix += (f.op == F_FIXED2) ? 4 : (f.op == F_FIXD ? 2 : 0);
    if (g.kind == kDense) nfix = (int)g.dmat.size();
    bool needs_mat = (g.kind == GK_U1 || g.kind == GK_D1);
    return gates + 1 <= kMaxPassGates && mats + (needs_mat ? 1 : 0) <= kMaxMats &&
           factors + nf <= kMaxFactors && fixed + nfix <= kMaxFixed;
  }
  void add(const HGate& g) {
    gates += 1;
    if (is_hadamard(g)) return;
    if (g.kind == GK_U1 || g.kind == GK_D1) mats += 1;
    factors += (int)g.factors.size();
    for (auto& f : g.factors) fixed += (f.op == F_FIXED2) ? 4 : (f.op == F_FIXD ? 2 : 0);
    if (g.kind == kDense) fixed += (int)g.dmat.size();
  }
};

// Register-phase construction inside one pass.  Gates that do not fit into
// kMaxPhases phases are returned in ``rejected`` (they and every gate after
// them on the same bits go to a later pass).
static void build_pass(PassParams& P, const Geometry& G, int ns, uint64_t L, const std::vector<HGate>& gl,
                       const std::vector<int>& taken, bool adjoint, bool phase_free, bool norm,
                       std::vector<int>& rejected) {
  std::vector<int> tb = sorted_bits(L);
  int pos_of[64];
  for (int i = 0; i < 64; ++i) pos_of[i] = -1;
  for (size_t i = 0; i < tb.size(); ++i) pos_of[tb[i]] = (int)i;
  auto tmask = [&](uint64_t gm) {
    uint32_t t = 0;
    for (int i = 0; i < 64; ++i)
      if (gm >> i & 1) t |= 1u << pos_of[i];
    return t;
  };
  memset(&P, 0, sizeof(P));
  P.norm_last = kNoNorm;
  P.norm_phase = kNoNorm;
  P.m = (uint8_t)G.m;
  P.c = (uint8_t)G.c;
  P.e = (uint8_t)G.e;
  P.R = (uint8_t)G.R;
  P.n = (uint8_t)ns;
  P.n_outer = (uint8_t)(ns - G.m);
  for (int i = G.c; i < G.m; ++i) P.hi[i - G.c] = (uint8_t)tb[i];
  {
    int j = 0;
    for (int b = 0; b < ns; ++b)
      if (!(L >> b & 1)) P.outer[j++] = (uint8_t)b;
  }
  // staging tables: unit bit b is tile bit b + e, i.e. global bit tb[b + e]
  {
    const int ntid = G.m - G.R, nk = 1 << (G.R - G.e);
    for (int b = 0; b < ntid; ++b) {
      P.gtid[b] = 1ull << tb[b + G.e];
      P.stid[b] = swz_unit(1u << b);
    }
    for (int k = 0; k < nk; ++k) {
      uint64_t g = 0;
      for (int j = 0; (k >> j) != 0; ++j)
        if ((k >> j) & 1) g |= 1ull << tb[ntid + j + G.e];
      P.gk[k] = g;
      P.sk[k] = swz_unit((uint32_t)k << ntid);
    }
  }
  int nfixed = 0;
  auto push_fixed = [&](const CD* v, int cnt) {
    int at = nfixed;
    for (int i = 0; i < cnt; ++i) P.fixed[nfixed++] = v[i];
    return at;
  };
  const uint32_t forced = (1u << G.e) - 1;
  std::vector<int> rem = taken;
  rejected.clear();
  // warp-index tile positions of the previous register phase (thread bits 5
  // and up; empty after a dense phase): kept as the warp bits of the next
  // phase where they stay thread bits, so that transition is warp-local
  std::vector<int> prev_warp;
  while (!rem.empty()) {
    if ((int)P.n_phases == kMaxPhases) {
      rejected = rem;
      break;
    }
    Phase& ph = P.phase[P.n_phases];
    const HGate& first = gl[rem.front()];
    if (first.kind == kDense) {
      ph.type = PH_DENSE;
      ph.dk = (uint8_t)first.dk;
      for (int i = 0; i < first.dk; ++i) ph.dpos[i] = (uint8_t)pos_of[first.dbits[i]];
      ph.dcmask = (uint16_t)tmask(first.cmask);
      ph.dagger = adjoint ? 1 : 0;
      ph.dfix = (uint16_t)push_fixed(first.dmat.data(), (int)first.dmat.size());
      P.n_phases++;
      rem.erase(rem.begin());
      prev_warp.clear();
      continue;
    }
    uint32_t Rset = forced, blocked = 0;
    std::vector<int> pg, rest;
    for (int idx : rem) {
      const HGate& g = gl[idx];
      uint32_t gb = tmask(g.bits());
      if (g.kind == kDense || (gb & blocked)) {
        blocked |= gb;
        rest.push_back(idx);
        continue;
      }
      if (popc(Rset | gb) <= G.R) {
        Rset |= gb;
        pg.push_back(idx);
      } else {
        blocked |= gb;
        rest.push_back(idx);
      }
    }
    // fill the register set: keep every residue class of (pos - e) mod 3
    // represented among the thread bits so lanes 0..2 can be conflict-free,
    // and leave the previous phase's warp bits to the threads where possible
    uint32_t pw = 0;
    for (int p : prev_warp) pw |= 1u << p;
    while (popc(Rset) < G.R) {
      int cnt[3] = {0, 0, 0};
      for (int p = G.e; p < G.m; ++p)
        if (!(Rset >> p & 1)) cnt[(p - G.e) % 3]++;
      int best = -1;
      for (int pass = 0; pass < 2 && best < 0; ++pass)
        for (int p = G.e; p < G.m; ++p) {
          if (Rset >> p & 1) continue;
          if (pass == 0 && (pw >> p & 1)) continue;
          if (best < 0 || cnt[(p - G.e) % 3] > cnt[(best - G.e) % 3]) best = p;
        }
      Rset |= 1u << best;
    }
    std::vector<int> Rpos = sorted_bits(Rset);
    int regbit_of[32];
    for (int i = 0; i < 32; ++i) regbit_of[i] = -1;
    for (size_t i = 0; i < Rpos.size(); ++i) regbit_of[Rpos[i]] = (int)i;
    // thread bits: lanes 0..2 from distinct residue classes, then the rest;
    // when the previous phase's warp bits are all thread bits here, they keep
    // their warp-index positions (bits 5 and up) and lanes 0..4 come from
    // the other positions
    auto order_tid = [&](bool keep_warp) {
      std::vector<int> t, free_pos;
      for (int p = 0; p < G.m; ++p)
        if (!(Rset >> p & 1) && !(keep_warp && (pw >> p & 1))) free_pos.push_back(p);
      for (int cls = 0; cls < 3; ++cls)
        for (size_t i = 0; i < free_pos.size(); ++i)
          if (free_pos[i] >= 0 && (free_pos[i] - G.e) % 3 == cls) {
            t.push_back(free_pos[i]);
            free_pos[i] = -1;
            break;
          }
      for (int p : free_pos)
        if (p >= 0) t.push_back(p);
      if (keep_warp) t.insert(t.end(), prev_warp.begin(), prev_warp.end());
      return t;
    };
    const int ntid_all = G.m - G.R;
    bool wl = !prev_warp.empty() && (int)prev_warp.size() == ntid_all - 5 && !(Rset & pw);
    auto classes = [&](const std::vector<int>& t) {
      int seen = 0;
      for (int b = 0; b < 3 && b < (int)t.size(); ++b) seen |= 1 << ((t[b] - G.e + 3) % 3);
      return popc(seen);
    };
    std::vector<int> tpos = order_tid(false);
    if (wl) {
      // only if lanes 0..2 cover as many residue classes as without the constraint
      std::vector<int> tw = order_tid(true);
      if (classes(tw) >= classes(tpos)) tpos = tw;
      else wl = false;
    }
    ph.wlocal = wl ? 1 : 0;
    prev_warp.assign(tpos.begin() + std::min<size_t>(5, tpos.size()), tpos.end());
    ph.type = PH_REG;
    ph.ntid = (uint8_t)tpos.size();
    for (size_t b = 0; b < tpos.size(); ++b) ph.tid_off[b] = (uint16_t)swz_unit((1u << tpos[b]) >> G.e);
    int nunits = 1 << (G.R - G.e);
    for (int j = 0; j < nunits; ++j) {
      uint32_t t = 0, reg = (uint32_t)j << G.e;
      for (int k = 0; k < G.R; ++k)
        if (reg >> k & 1) t |= 1u << Rpos[k];
      ph.reg_off[j] = (uint16_t)swz_unit(t >> G.e);
    }
    ph.g0 = P.n_gates;
    for (int idx : pg) {
      const HGate& g = gl[idx];
      RGate& r = P.gate[P.n_gates++];
      memset(&r, 0, sizeof(r));
      r.kind = specialised_kind(g, phase_free, norm);
      r.k0 = (uint8_t)regbit_of[pos_of[g.t0]];
      r.k1 = g.t1 >= 0 ? (uint8_t)regbit_of[pos_of[g.t1]] : 0;
      uint32_t cm = 0;
      for (int b = 0; b < 64; ++b)
        if (g.cmask >> b & 1) cm |= 1u << regbit_of[pos_of[b]];
      r.cmask = (uint8_t)cm;
      r.slot = -1;
      if (adjoint && g.grad != GR_NONE) {
        r.grad = g.grad;
        r.slot = g.slot;
        r.coef = g.coef;
        P.n_grad++;
      }
      if ((g.kind == GK_U1 || g.kind == GK_D1) && r.kind != GK_H) {  // (also RXT / RYT / PH)
        MatDesc& md = P.mat[P.n_mats];
        r.mat = (uint8_t)P.n_mats++;
        md.diag = g.kind != GK_D1 ? 0 : (phase_droppable(g, phase_free) ? 2 : 1);
        if (r.kind == GK_RXN || r.kind == GK_RYN) {
          md.diag = r.kind == GK_RXN ? 3 : 4;
          P.norm_last = r.mat;
          P.norm_phase = P.n_phases;
        }
        md.nf = (uint8_t)g.factors.size();
        md.f0 = (uint8_t)P.n_factors;
        md.dagger = adjoint ? 1 : 0;
        for (const HFactor& f : g.factors) {
          Factor& F = P.factor[P.n_factors++];
          memset(&F, 0, sizeof(F));
          F.op = f.op;
          for (int j = 0; j < 3; ++j) {
            F.slot[j] = f.slot[j];
            F.val[j] = f.val[j];
          }
          if (f.op == F_FIXED2) F.fix = (int16_t)push_fixed(f.m, 4);
          if (f.op == F_FIXD) F.fix = (int16_t)push_fixed(f.m, 2);
        }
      }
    }
    ph.g1 = P.n_gates;
    P.n_phases++;
    rem = rest;
  }
}

static Schedule schedule(const std::vector<HGate>& gl, int ns, const Geometry& G, bool adjoint, bool fuse,
                         bool phase_free, bool norm) {
  Schedule S;
  std::vector<int> rem(gl.size());
  for (size_t i = 0; i < gl.size(); ++i) rem[i] = (int)i;
  const uint64_t all = (ns >= 64) ? ~0ull : ((1ull << ns) - 1);
  while (!rem.empty()) {
    uint64_t L = (1ull << G.c) - 1, blocked = 0;
    Cap cap;
    std::vector<int> taken, rest;
    for (size_t ii = 0; ii < rem.size(); ++ii) {
      int idx = rem[ii];
      const HGate& g = gl[idx];
      uint64_t gb = g.bits();
      bool ok = !(gb & blocked) && popc(L | gb) <= G.m && cap.fits(g) && (fuse || taken.empty());
      if (ok) {
        L |= gb;
        taken.push_back(idx);
        cap.add(g);
      } else {
        blocked |= gb;
        rest.push_back(idx);
      }
      if ((blocked | 0) == all) {
        for (size_t jj = ii + 1; jj < rem.size(); ++jj) rest.push_back(rem[jj]);
        break;
      }
    }
    L = fill_bits(L, G.m, ns);
    PassParams P;
    std::vector<int> rejected;
    build_pass(P, G, ns, L, gl, taken, adjoint, phase_free, norm, rejected);
    if (!rejected.empty()) {
      // gates beyond the phase limit go back in circuit order
      std::vector<int> merged = rejected;
      merged.insert(merged.end(), rest.begin(), rest.end());
      std::sort(merged.begin(), merged.end());
      rest = merged;
    }
    S.n_phases += P.n_phases;
    S.passes.push_back(P);
    rem = rest;
  }
  return S;
}

// ---------------------------------------------------------------- observables

struct PTerm {  // coef * X^x Z^z
  cplx c;
  uint64_t x, z;
};

static std::vector<PTerm> pauli_expand(const tedq_obs_factor_t& f, int n, int ns) {
  int k = f.n_qubits;
  if (k < 1 || k > 3) throw std::invalid_argument("observable with unsupported number of qubits");
  if (f.obs != TEDQ_OBS_MATRIX && k != 1) throw std::invalid_argument("named observable must act on one qubit");
  int b[3];
  for (int i = 0; i < k; ++i) {
    if (f.qubits[i] < 0 || f.qubits[i] >= n) throw std::invalid_argument("observable qubit out of range");
    b[i] = ns - 1 - f.qubits[i];
  }
  std::vector<PTerm> out;
  const cplx I(0, 1);
  // X^x Z^z form: X = X, Y = i X Z, Z = Z, H = (X + Z)/sqrt2
  switch (f.obs) {
    case TEDQ_OBS_I: out.push_back({1.0, 0, 0}); return out;
    case TEDQ_OBS_X: out.push_back({1.0, 1ull << b[0], 0}); return out;
    case TEDQ_OBS_Y: out.push_back({I, 1ull << b[0], 1ull << b[0]}); return out;
    case TEDQ_OBS_Z: out.push_back({1.0, 0, 1ull << b[0]}); return out;
    case TEDQ_OBS_H:
      out.push_back({kInvSqrt2, 1ull << b[0], 0});
      out.push_back({kInvSqrt2, 0, 1ull << b[0]});
      return out;
    case TEDQ_OBS_MATRIX: break;
    default: throw std::invalid_argument("unknown observable code");
  }
  if (!f.matrix) throw std::invalid_argument("TEDQ_OBS_MATRIX without matrix");
  int d = 1 << k;
  // coefficient of X^x Z^z (local masks) is Tr((X^x Z^z)^dagger M) / d;
  // (X^x Z^z)_{w^x, w} = (-1)^{z.w}, so its dagger has entry (w, w^x) = (-1)^{z.w}.
  for (int lx = 0; lx < d; ++lx)
    for (int lz = 0; lz < d; ++lz) {
      cplx acc = 0;
      for (int w = 0; w < d; ++w) {
        int sgn = (popc((uint64_t)(lz & w)) & 1) ? -1 : 1;
        int r = w ^ lx;
        cplx Mrw(f.matrix[2 * (r * d + w)], f.matrix[2 * (r * d + w) + 1]);
        // Tr(A^dagger M) = sum_{r,w} conj(A_{r,w}) M_{r,w}; A_{w^x, w} = sgn
        acc += (double)sgn * Mrw;
      }
      acc /= (double)d;
      if (std::abs(acc) < 1e-300) continue;
      uint64_t gx = 0, gz = 0;
      for (int i = 0; i < k; ++i) {  // local bit (k-1-i) is qubit i
        if (lx >> (k - 1 - i) & 1) gx |= 1ull << b[i];
        if (lz >> (k - 1 - i) & 1) gz |= 1ull << b[i];
      }
      out.push_back({acc, gx, gz});
    }
  return out;
}

static void compile_measurements(Program& p, const tedq_meas_t* meas, int n_meas) {
  std::map<std::pair<uint64_t, uint64_t>, int> term_index;
  int out_k = 0;
  for (int mi = 0; mi < n_meas; ++mi) {
    const tedq_meas_t& m = meas[mi];
    if (m.kind == TEDQ_MEAS_EXPVAL) {
      if (m.n_factors < 1 || !m.factors) throw std::invalid_argument("expval without observable");
      // O = O_last ... O_first (factors applied in list order)
      std::vector<PTerm> acc = {{1.0, 0, 0}};
      for (int fi = 0; fi < m.n_factors; ++fi) {
        std::vector<PTerm> f = pauli_expand(m.factors[fi], p.n, p.ns), nxt;
        for (auto& a : f)
          for (auto& t : acc) {
            double sgn = (popc(a.z & t.x) & 1) ? -1.0 : 1.0;
            nxt.push_back({a.c * t.c * sgn, a.x ^ t.x, a.z ^ t.z});
          }
        std::map<std::pair<uint64_t, uint64_t>, cplx> merged;
        for (auto& t : nxt) merged[{t.x, t.z}] += t.c;
        acc.clear();
        for (auto& kv : merged) acc.push_back({kv.second, kv.first.first, kv.first.second});
      }
      for (auto& t : acc) {
        // Hermitian string P_h = i^{ny} X^x Z^z  =>  c X^x Z^z = c (-i)^{ny} P_h
        int ny = popc(t.x & t.z) & 3;
        cplx ph = 1.0;
        for (int i = 0; i < ny; ++i) ph *= cplx(0, -1);
        double coef = (t.c * ph).real();
        if (coef == 0.0) continue;
        auto key = std::make_pair(t.x, t.z);
        auto it = term_index.find(key);
        int s;
        if (it == term_index.end()) {
          s = (int)p.terms.size();
          term_index[key] = s;
          p.terms.push_back({t.x, t.z});
        } else {
          s = it->second;
        }
        p.out_terms.push_back({out_k, s, coef});
      }
      out_k += 1;
      p.n_expval += 1;
    } else if (m.kind == TEDQ_MEAS_PROBS) {
      std::vector<int> qs;
      if (m.n_qubits == 0) {
        for (int q = 0; q < p.n; ++q) qs.push_back(q);
      } else {
        if (!m.qubits) throw std::invalid_argument("probs qubits pointer is null");
        for (int i = 0; i < m.n_qubits; ++i) {
          if (m.qubits[i] < 0 || m.qubits[i] >= p.n) throw std::invalid_argument("probs qubit out of range");
          qs.push_back(m.qubits[i]);
        }
      }
      std::sort(qs.begin(), qs.end());
      qs.erase(std::unique(qs.begin(), qs.end()), qs.end());
      ProbsOut po;
      po.offset = out_k;
      for (int q : qs) po.bits.push_back(p.ns - 1 - q);
      out_k += 1 << qs.size();
      p.probs.push_back(po);
    } else if (m.kind == TEDQ_MEAS_STATE) {
      // the state output is the psi buffer itself
    } else {
      throw std::invalid_argument("unknown measurement kind");
    }
  }
  p.n_real = out_k;
}

// ---------------------------------------------------------------- entry

Program* compile_program(const tedq_gate_t* gates, int n_gates, int n_qubits, const tedq_meas_t* meas,
                         int n_meas, const tedq_options_t* opts) {
  if (n_qubits < 1 || n_qubits > 33) throw std::invalid_argument("n_qubits must be in [1, 33]");
  if (n_gates < 0 || (n_gates > 0 && !gates)) throw std::invalid_argument("bad gate list");
  if (n_meas < 0 || (n_meas > 0 && !meas)) throw std::invalid_argument("bad measurement list");
  std::unique_ptr<Program> p(new Program());
  p->n = n_qubits;
  p->precision = opts ? opts->precision : TEDQ_PREC_C64;
  p->fuse = opts ? opts->fuse : 1;
  p->tile_qubits = opts ? opts->tile_qubits : 0;
  if (p->precision != TEDQ_PREC_C64 && p->precision != TEDQ_PREC_C128)
    throw std::invalid_argument("unknown precision");
  const bool dbl = p->precision == TEDQ_PREC_C128;
  // Small circuits run on a padded state with idle low-order qubits so that
  // every tile holds at least one full warp of threads.
  p->ns = std::max(n_qubits, 10);
  p->pad = p->ns - n_qubits;
  int max_slot = -1;
  for (int i = 0; i < n_gates; ++i) {
    lower_gate(gates[i], n_qubits, p->ns, p->elem);
    int np = gates[i].op == TEDQ_OP_ROT ? 3 : 1;
    for (int j = 0; j < np; ++j) max_slot = std::max(max_slot, (int)gates[i].param_slot[j]);
  }
  p->n_params = max_slot + 1;
  p->fused = p->elem;  // fused below, once the register-gate forms are known
  Geometry gf, gb;
  int mdef_f = dbl ? 12 : 13, mdef_b = dbl ? 11 : 12;
  if (p->tile_qubits > 0) mdef_f = std::min(mdef_f, std::max(p->tile_qubits, 6));
  gf.e = gb.e = dbl ? 0 : 1;
  gf.R = dbl ? 4 : 5;
  gb.R = dbl ? 3 : 4;
  gf.m = std::min(mdef_f, p->ns);
  gb.m = std::min(mdef_b, p->ns);
  // tuning override "fwd_m,fwd_R,bwd_m,bwd_R" (0 keeps a default); tile and
  // register bits other than the defaults run on the specialised kernels only
  if (const char* env = getenv("TEDQ_GB300_GEOMETRY")) {
    int v[4] = {0, 0, 0, 0};
    if (sscanf(env, "%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3]) == 4) {
      Geometry* g2[2] = {&gf, &gb};
      for (int i = 0; i < 2; ++i) {
        Geometry& g = *g2[i];
        const int m = v[2 * i] ? std::min(v[2 * i], p->ns) : g.m, R = v[2 * i + 1] ? v[2 * i + 1] : g.R;
        if (R < 2 || R > 5 || m - R < 5 || m - R > 10 || m > kMaxTileBits)
          throw std::invalid_argument("TEDQ_GB300_GEOMETRY out of range");
        g.m = m;
        g.R = R;
      }
    }
  }
  gf.c = std::min(4, gf.m);
  gb.c = std::min(4, gb.m);
  // Global phases: every expval / probs output is invariant under them, and
  // the adjoint sweep un-applies each gate to both of its states (same phase
  // on both, so every Im <lambda|G|psi> is unchanged).  Only a state output
  // (or a caller asking for exact phases) keeps them in the forward passes.
  bool state_out = opts && opts->exact_phase;
  for (int i = 0; i < n_meas; ++i) state_out |= meas[i].kind == TEDQ_MEAS_STATE;
  p->phase_free = !state_out;
  // normalised rotations (one FMA per component).  Tuning:
  // TEDQ_GB300_NORMALISE holds the letters f (forward passes), b (adjoint
  // passes), u (runs of one-qubit gates stay unfused where their normalised
  // parts cost less); "0" = none.
  const char* norm_env = getenv("TEDQ_GB300_NORMALISE");
  const std::string norm_opt = norm_env ? norm_env : "fbu";
  const bool norm_f = norm_opt.find('f') != std::string::npos, norm_b = norm_opt.find('b') != std::string::npos,
             norm_u = norm_opt.find('u') != std::string::npos;
  p->normalise = norm_f || norm_b;
  // unfusing pays only in specialised kernels: the generic ones dispatch every
  // gate at run time (and run normalised rotations with plain matrices)
  const int jit_mode = opts ? opts->jit : 0;
  const char* jit_env = getenv("TEDQ_GB300_JIT");
  const bool jit_expected = (jit_mode > 0 || (jit_mode == 0 && p->ns >= 14)) && !(jit_env && jit_env[0] == '0');
  if (p->fuse)
    p->fused = fuse_one_qubit_runs(p->elem, p->ns, p->phase_free && norm_f && norm_u && jit_expected);
  p->fwd = schedule(p->fused, p->ns, gf, false, p->fuse != 0, p->phase_free, norm_f);
  // zero tiles of the forward sweep from |0...0>: outer bits of a pass that
  // no earlier pass had among its tile bits (TEDQ_GB300_ZERO_TILES=0 turns
  // the skipping off, a measurement knob)
  {
    const char* zt = getenv("TEDQ_GB300_ZERO_TILES");
    const bool skip = !(zt && zt[0] == '0');
    uint64_t touched = 0;
    for (PassParams& P : p->fwd.passes) {
      uint64_t tile = (1ull << P.c) - 1, outer = 0;
      for (int j = 0; j < P.m - P.c; ++j) tile |= 1ull << P.hi[j];
      for (int j = 0; j < P.n_outer; ++j) outer |= 1ull << P.outer[j];
      P.zero_outer = skip ? (outer & ~touched) : 0;
      touched |= tile;
    }
  }
  std::vector<HGate> rev(p->elem.rbegin(), p->elem.rend());
  p->bwd = schedule(rev, p->ns, gb, true, p->fuse != 0, true, norm_b);
  compile_measurements(*p, meas, n_meas);
  for (auto& pr : p->probs)
    if ((int)pr.bits.size() < p->n) p->n_probs_bins += 1 << pr.bits.size();
  p->ws_per_circuit = 8LL * (2LL * (int64_t)p->terms.size() + p->n_probs_bins + p->n_params) + 64;
  return p.release();
}

std::string describe_schedule(const Program& p, bool adjoint) {
  const Schedule& S = adjoint ? p.bwd : p.fwd;
  std::ostringstream o;
  o << std::setprecision(17);
  o << "{\"n\":" << p.n << ",\"state_qubits\":" << p.ns << ",\"adjoint\":" << (adjoint ? 1 : 0) << ",\"passes\":[";
  for (size_t i = 0; i < S.passes.size(); ++i) {
    const PassParams& P = S.passes[i];
    if (i) o << ",";
    o << "{\"m\":" << (int)P.m << ",\"c\":" << (int)P.c << ",\"e\":" << (int)P.e << ",\"R\":" << (int)P.R
      << ",\"hi\":[";
    for (int j = 0; j < P.m - P.c; ++j) o << (j ? "," : "") << (int)P.hi[j];
    o << "],\"outer\":[";
    for (int j = 0; j < P.n_outer; ++j) o << (j ? "," : "") << (int)P.outer[j];
    o << "],\"gtid\":[";
    for (int j = 0; j < P.m - P.R; ++j) o << (j ? "," : "") << P.gtid[j];
    o << "],\"stid\":[";
    for (int j = 0; j < P.m - P.R; ++j) o << (j ? "," : "") << P.stid[j];
    o << "],\"gk\":[";
    for (int j = 0; j < (1 << (P.R - P.e)); ++j) o << (j ? "," : "") << P.gk[j];
    o << "],\"sk\":[";
    for (int j = 0; j < (1 << (P.R - P.e)); ++j) o << (j ? "," : "") << P.sk[j];
    o << "],\"norm_last\":" << (P.norm_last == kNoNorm ? -1 : (int)P.norm_last)
      << ",\"norm_phase\":" << (P.norm_phase == kNoNorm ? -1 : (int)P.norm_phase);
    {
      // launch variant of the specialised kernel and its shared memory per CTA
      PassParams Q = P;
      Q.pipe = pass_pipelined(P, adjoint) ? 1 : 0;
      const int G = pipe_groups(Q, adjoint);
      const uint32_t smem = Q.pipe ? pipe_layout(Q, G, adjoint).total
                                   : tile_dynamic_smem(P, adjoint) + tile_static_smem(P, adjoint);
      o << ",\"pipelined\":" << (int)Q.pipe << ",\"groups\":" << G << ",\"cta_smem\":" << smem
        << ",\"zero_outer\":" << P.zero_outer;
    }
    o << ",\"phases\":[";
    for (int f = 0; f < P.n_phases; ++f) {
      const Phase& ph = P.phase[f];
      if (f) o << ",";
      o << "{\"type\":" << (int)ph.type << ",\"wlocal\":" << (int)ph.wlocal;
      if (ph.type == PH_REG) {
        o << ",\"reg_off\":[";
        for (int j = 0; j < (1 << (P.R - P.e)); ++j) o << (j ? "," : "") << ph.reg_off[j];
        o << "],\"tid_off\":[";
        for (int j = 0; j < ph.ntid; ++j) o << (j ? "," : "") << ph.tid_off[j];
        o << "],\"gates\":[";
        for (int g = ph.g0; g < ph.g1; ++g) {
          const RGate& r = P.gate[g];
          if (g != ph.g0) o << ",";
          o << "{\"kind\":" << (int)r.kind << ",\"k0\":" << (int)r.k0 << ",\"k1\":" << (int)r.k1
            << ",\"cmask\":" << (int)r.cmask << ",\"mat\":" << (int)r.mat << ",\"grad\":" << (int)r.grad
            << ",\"slot\":" << r.slot << ",\"coef\":" << r.coef << "}";
        }
        o << "]";
      } else {
        o << ",\"dk\":" << (int)ph.dk << ",\"dpos\":[" << (int)ph.dpos[0] << "," << (int)ph.dpos[1] << ","
          << (int)ph.dpos[2] << "],\"dcmask\":" << ph.dcmask << ",\"dagger\":" << (int)ph.dagger
          << ",\"dfix\":" << ph.dfix;
      }
      o << "}";
    }
    o << "],\"mats\":[";
    for (int j = 0; j < P.n_mats; ++j) {
      const MatDesc& md = P.mat[j];
      o << (j ? "," : "") << "{\"diag\":" << (int)md.diag << ",\"dagger\":" << (int)md.dagger << ",\"factors\":[";
      for (int f = 0; f < md.nf; ++f) {
        const Factor& F = P.factor[md.f0 + f];
        o << (f ? "," : "") << "{\"op\":" << (int)F.op << ",\"fix\":" << F.fix << ",\"slot\":[" << F.slot[0] << ","
          << F.slot[1] << "," << F.slot[2] << "],\"val\":[" << F.val[0] << "," << F.val[1] << "," << F.val[2]
          << "]}";
      }
      o << "]}";
    }
    o << "],\"fixed\":[";
    int nfix = 0;
    for (int j = 0; j < P.n_factors; ++j) {
      const Factor& F = P.factor[j];
      if (F.op == F_FIXED2) nfix = std::max(nfix, F.fix + 4);
      if (F.op == F_FIXD) nfix = std::max(nfix, F.fix + 2);
    }
    for (int f = 0; f < P.n_phases; ++f)
      if (P.phase[f].type == PH_DENSE) nfix = std::max(nfix, P.phase[f].dfix + (1 << (2 * P.phase[f].dk)));
    for (int j = 0; j < nfix; ++j) o << (j ? "," : "") << "[" << P.fixed[j].re << "," << P.fixed[j].im << "]";
    o << "]}";
  }
  o << "],\"n_real\":" << p.n_real << ",\"n_params\":" << p.n_params << ",\"terms\":[";
  for (size_t i = 0; i < p.terms.size(); ++i)
    o << (i ? "," : "") << "[" << p.terms[i].x << "," << p.terms[i].z << "]";
  o << "],\"out_terms\":[";
  for (size_t i = 0; i < p.out_terms.size(); ++i)
    o << (i ? "," : "") << "[" << p.out_terms[i].k << "," << p.out_terms[i].s << "," << p.out_terms[i].coef << "]";
  o << "],\"probs\":[";
  for (size_t i = 0; i < p.probs.size(); ++i) {
    o << (i ? "," : "") << "{\"offset\":" << p.probs[i].offset << ",\"bits\":[";
    for (size_t j = 0; j < p.probs[i].bits.size(); ++j) o << (j ? "," : "") << p.probs[i].bits[j];
    o << "]}";
  }
  o << "]}";
  return o.str();
}

}  // namespace tedq
