// tn_plan.cpp -- sandwich network, light cone, contraction path, slicing and
// workspace layout of the tensor-network mode (tn_plan.h).
//
// Reference counterpart: gen_tensor_networks (tedq/tensor_network/
// tensor_network.py:850-1099) for the network and the external path
// optimisers behind OEWrapper (tedq/oe_wrapper/oe_wrapper.py:24-65) /
// JDOptTN (compiled_circuit.py:388-393) for the order.
#include "tn_plan.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstring>
#include <iomanip>
#include <map>
#include <queue>
#include <random>
#include <set>
#include <sstream>
#include <stdexcept>
#include <tuple>

#include "sv_program.h"

namespace tedq {

using cplx = std::complex<double>;

// ------------------------------------------------------------- gate matrices

static const double kInvSqrt2 = 0.70710678118654752440;

static std::vector<cplx> eye(int d) {
  std::vector<cplx> m(d * d, 0.0);
  for (int i = 0; i < d; ++i) m[i * d + i] = 1.0;
  return m;
}

// Matrices follow tedq/QInterpreter/operators/qubit.py (RX :990-997,
// RY :1048-1055, RZ :1106-1112, Rot :1169-1189, PhaseShift :1253-1257).
static std::vector<cplx> rot1(int op, const double* a) {
  const cplx I(0, 1);
  switch (op) {
    case TEDQ_OP_RX: case TEDQ_OP_CRX: {
      double c = std::cos(a[0] / 2), s = std::sin(a[0] / 2);
      return {c, -I * s, -I * s, c};
    }
    case TEDQ_OP_RY: case TEDQ_OP_CRY: {
      double c = std::cos(a[0] / 2), s = std::sin(a[0] / 2);
      return {c, -s, s, c};
    }
    case TEDQ_OP_RZ: case TEDQ_OP_CRZ:
      return {std::exp(-I * (a[0] / 2)), 0.0, 0.0, std::exp(I * (a[0] / 2))};
    case TEDQ_OP_PHASESHIFT: case TEDQ_OP_CPHASE:
      return {1.0, 0.0, 0.0, std::exp(I * a[0])};
    default: {  // Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi)
      double c = std::cos(a[1] / 2), s = std::sin(a[1] / 2);
      cplx p = std::exp(-I * ((a[0] + a[2]) / 2)), m = std::exp(I * ((a[0] - a[2]) / 2));
      return {p * c, -m * s, std::conj(m) * s, std::conj(p) * c};
    }
  }
}

// Row-major 2^k x 2^k matrix of a gate whose parameters are all fixed
// (qubits[0] is the most significant matrix bit).
static std::vector<cplx> fixed_gate_matrix(const tedq_gate_t& g) {
  const cplx I(0, 1);
  const int k = g.n_qubits, d = 1 << k;
  std::vector<cplx> m = eye(d);
  switch (g.op) {
    case TEDQ_OP_I: break;
    case TEDQ_OP_H: m = {kInvSqrt2, kInvSqrt2, kInvSqrt2, -kInvSqrt2}; break;
    case TEDQ_OP_X: m = {0.0, 1.0, 1.0, 0.0}; break;
    case TEDQ_OP_Y: m = {0.0, -I, I, 0.0}; break;
    case TEDQ_OP_Z: m = {1.0, 0.0, 0.0, -1.0}; break;
    case TEDQ_OP_S: m = {1.0, 0.0, 0.0, I}; break;
    case TEDQ_OP_T: m = {1.0, 0.0, 0.0, std::exp(I * (M_PI / 4))}; break;
    case TEDQ_OP_SX: m = {cplx(.5, .5), cplx(.5, -.5), cplx(.5, -.5), cplx(.5, .5)}; break;
    case TEDQ_OP_CNOT: m[10] = 0.0; m[15] = 0.0; m[11] = 1.0; m[14] = 1.0; break;
    case TEDQ_OP_CZ: m[15] = -1.0; break;
    case TEDQ_OP_CY: m[10] = 0.0; m[15] = 0.0; m[11] = -I; m[14] = I; break;
    case TEDQ_OP_SWAP: m[5] = 0.0; m[10] = 0.0; m[6] = 1.0; m[9] = 1.0; break;
    case TEDQ_OP_CSWAP:
      m[5 * 8 + 5] = 0.0; m[6 * 8 + 6] = 0.0; m[5 * 8 + 6] = 1.0; m[6 * 8 + 5] = 1.0;
      break;
    case TEDQ_OP_TOFFOLI:
      m[6 * 8 + 6] = 0.0; m[7 * 8 + 7] = 0.0; m[6 * 8 + 7] = 1.0; m[7 * 8 + 6] = 1.0;
      break;
    case TEDQ_OP_RX: case TEDQ_OP_RY: case TEDQ_OP_RZ: case TEDQ_OP_ROT: case TEDQ_OP_PHASESHIFT:
      m = rot1(g.op, g.fixed);
      break;
    case TEDQ_OP_CRX: case TEDQ_OP_CRY: case TEDQ_OP_CRZ: case TEDQ_OP_CPHASE: {
      std::vector<cplx> u = rot1(g.op, g.fixed);
      m[10] = u[0]; m[11] = u[1]; m[14] = u[2]; m[15] = u[3];
      break;
    }
    case TEDQ_OP_MATRIX:
      if (!g.matrix) throw std::invalid_argument("TEDQ_OP_MATRIX without matrix");
      for (int i = 0; i < d * d; ++i) m[i] = cplx(g.matrix[2 * i], g.matrix[2 * i + 1]);
      break;
    default: throw std::invalid_argument("unknown gate opcode");
  }
  return m;
}

static std::vector<cplx> obs_matrix(const tedq_obs_factor_t& f) {
  const cplx I(0, 1);
  switch (f.obs) {
    case TEDQ_OBS_I: return eye(2);
    case TEDQ_OBS_X: return {0.0, 1.0, 1.0, 0.0};
    case TEDQ_OBS_Y: return {0.0, -I, I, 0.0};
    case TEDQ_OBS_Z: return {1.0, 0.0, 0.0, -1.0};
    case TEDQ_OBS_H: return {kInvSqrt2, kInvSqrt2, kInvSqrt2, -kInvSqrt2};
    case TEDQ_OBS_MATRIX: {
      if (!f.matrix) throw std::invalid_argument("TEDQ_OBS_MATRIX without matrix");
      int d = 1 << f.n_qubits;
      std::vector<cplx> m(d * d);
      for (int i = 0; i < d * d; ++i) m[i] = cplx(f.matrix[2 * i], f.matrix[2 * i + 1]);
      return m;
    }
    default: throw std::invalid_argument("unknown observable code");
  }
}

static bool op_has_params(int op) {
  return op == TEDQ_OP_RX || op == TEDQ_OP_RY || op == TEDQ_OP_RZ || op == TEDQ_OP_ROT ||
         op == TEDQ_OP_PHASESHIFT || op == TEDQ_OP_CPHASE || op == TEDQ_OP_CRX || op == TEDQ_OP_CRY ||
         op == TEDQ_OP_CRZ;
}
static int op_n_params(int op) { return op == TEDQ_OP_ROT ? 3 : (op_has_params(op) ? 1 : 0); }

static void check_gate(const tedq_gate_t& g, int n) {
  static const int arity[] = {1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 2, 2, 2, 2};
  if (g.op < 0 || g.op > TEDQ_OP_MATRIX) throw std::invalid_argument("unknown gate opcode");
  const int k = g.n_qubits;
  if (k < 1 || k > 3) throw std::invalid_argument("gate with unsupported number of qubits");
  if (g.op != TEDQ_OP_MATRIX && arity[g.op] != k) throw std::invalid_argument("gate arity mismatch");
  for (int i = 0; i < k; ++i) {
    if (g.qubits[i] < 0 || g.qubits[i] >= n) throw std::invalid_argument("gate qubit index out of range");
    for (int j = 0; j < i; ++j)
      if (g.qubits[j] == g.qubits[i]) throw std::invalid_argument("gate acts twice on one qubit");
  }
}

// ------------------------------------------------------------------ network

// Light-cone-reduced sandwich (tensor_network.py:850-1015 builds the full one;
// gates outside the backward light cone of the observable cancel in U^dag U).
static void build_network(TnNet& net, const tedq_gate_t* gates, int n_gates, int n, const tedq_meas_t& meas) {
  if (meas.kind != TEDQ_MEAS_EXPVAL)
    throw UnsupportedError("the tensor-network mode evaluates expectation values only");
  if (meas.n_factors < 1 || !meas.factors) throw std::invalid_argument("expval without observable factors");
  std::vector<char> active(n, 0);
  for (int f = 0; f < meas.n_factors; ++f) {
    const tedq_obs_factor_t& o = meas.factors[f];
    if (o.n_qubits < 1 || o.n_qubits > 3 || (o.obs != TEDQ_OBS_MATRIX && o.n_qubits != 1))
      throw std::invalid_argument("observable factor with unsupported number of qubits");
    for (int i = 0; i < o.n_qubits; ++i) {
      if (o.qubits[i] < 0 || o.qubits[i] >= n) throw std::invalid_argument("observable qubit out of range");
      for (int j = 0; j < i; ++j)
        if (o.qubits[j] == o.qubits[i]) throw std::invalid_argument("observable acts twice on one qubit");
      active[o.qubits[i]] = 1;
    }
  }
  std::vector<char> keep(n_gates, 0);
  for (int i = n_gates - 1; i >= 0; --i) {
    const tedq_gate_t& g = gates[i];
    bool touch = false;
    for (int j = 0; j < g.n_qubits; ++j) touch |= active[g.qubits[j]] != 0;
    if (!touch) continue;
    keep[i] = 1;
    for (int j = 0; j < g.n_qubits; ++j) active[g.qubits[j]] = 1;
  }
  net.n = n;
  net.gates_in = n_gates;
  for (int i = 0; i < n_gates; ++i) {
    if (!keep[i]) continue;
    const tedq_gate_t& g = gates[i];
    TnGate t;
    t.op = g.op;
    t.k = g.n_qubits;
    for (int j = 0; j < t.k; ++j) t.qubits[j] = g.qubits[j];
    for (int j = 0; j < op_n_params(g.op); ++j) {
      t.slot[j] = g.param_slot[j];
      t.val[j] = g.fixed[j];
      t.param |= g.param_slot[j] >= 0;
    }
    if (!t.param) {
      for (cplx v : fixed_gate_matrix(g)) {
        t.fixed.push_back(v.real());
        t.fixed.push_back(v.imag());
      }
    }
    net.gates.push_back(t);
  }
  net.n_circuit_gates = (int)net.gates.size();
  net.gates_kept = net.n_circuit_gates;
  for (int f = 0; f < meas.n_factors; ++f) {
    const tedq_obs_factor_t& o = meas.factors[f];
    TnGate t;
    t.op = -1 - o.obs;
    t.k = o.n_qubits;
    for (int j = 0; j < t.k; ++j) t.qubits[j] = o.qubits[j];
    for (cplx v : obs_matrix(o)) {
      t.fixed.push_back(v.real());
      t.fixed.push_back(v.imag());
    }
    net.gates.push_back(t);
  }

  int next = 0;
  auto leaf = [&](int kind, std::vector<int> idx, int gate, bool batched) {
    TnTensor t;
    t.full_idx = idx;
    t.idx = std::move(idx);
    t.leaf = kind;
    t.gate = gate;
    t.batched = batched;
    net.tensors.push_back(std::move(t));
  };
  std::vector<int> ket(n, -1), bra(n, -1);
  for (int q = 0; q < n; ++q) {
    if (!active[q]) continue;
    net.qubits_kept++;
    ket[q] = next++;
    leaf(TL_KET0, {ket[q]}, -1, false);
    bra[q] = next++;
    leaf(TL_BRA0, {bra[q]}, -1, false);
  }
  auto apply = [&](std::vector<int>& wire, int gi, int kind) {
    const TnGate& g = net.gates[gi];
    std::vector<int> idx(2 * g.k);
    for (int j = 0; j < g.k; ++j) {
      idx[g.k + j] = wire[g.qubits[j]];
      idx[j] = wire[g.qubits[j]] = next++;
    }
    leaf(kind, idx, gi, g.param);
  };
  for (int gi = 0; gi < net.n_circuit_gates; ++gi) {
    apply(ket, gi, TL_GATE);
    apply(bra, gi, TL_GATE_CONJ);
  }
  for (int gi = net.n_circuit_gates; gi < (int)net.gates.size(); ++gi) apply(ket, gi, TL_OBS);
  // close the sandwich: the last bra index of a qubit becomes its last ket index
  for (int q = 0; q < n; ++q) {
    if (!active[q]) continue;
    for (auto& t : net.tensors)
      for (size_t j = 0; j < t.idx.size(); ++j)
        if (t.idx[j] == bra[q]) t.idx[j] = t.full_idx[j] = ket[q];
  }
  net.n_leaves = (int)net.tensors.size();
  net.n_index = next;
}

// --------------------------------------------------------------- path search

static inline double pow2(int r) { return std::ldexp(1.0, r); }

static std::vector<int> sym_diff(const std::vector<int>& a, const std::vector<int>& b) {
  std::vector<int> out;
  std::set_symmetric_difference(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(out));
  return out;
}
static int union_size(const std::vector<int>& a, const std::vector<int>& b) {
  std::vector<int> u;
  std::set_union(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(u));
  return (int)u.size();
}

struct Path {
  std::vector<std::pair<int, int>> pairs;  // SSA ids: leaves 0..L-1, step s produces L+s
  int max_rank = 0;
  double flops = 0;  // complex multiply-adds of one slice
};

// Greedy pairwise order in the style of opt_einsum's "greedy" (cost = size of
// the result minus the sizes of the inputs), with a Boltzmann choice among the
// best few candidates for randomised trials (opt_einsum RandomGreedy).
static Path greedy_path(const std::vector<std::vector<int>>& leaves, int n_index, std::mt19937_64* rng,
                        double temp) {
  std::vector<std::vector<int>> T = leaves;
  for (auto& t : T) std::sort(t.begin(), t.end());
  std::vector<char> alive(T.size(), 1);
  std::vector<std::array<int, 2>> hold(n_index, {-1, -1});
  for (int t = 0; t < (int)T.size(); ++t)
    for (int i : T[t]) (hold[i][0] < 0 ? hold[i][0] : hold[i][1]) = t;
  typedef std::tuple<double, int, int> Cand;
  std::priority_queue<Cand, std::vector<Cand>, std::greater<Cand>> heap;
  auto cost = [&](int a, int b) {
    int r = (int)sym_diff(T[a], T[b]).size();
    return pow2(r) - pow2((int)T[a].size()) - pow2((int)T[b].size());
  };
  std::set<std::pair<int, int>> seen;
  auto push = [&](int a, int b) {
    if (a > b) std::swap(a, b);
    if (!seen.insert({a, b}).second) return;
    heap.emplace(cost(a, b), a, b);
  };
  for (int i = 0; i < n_index; ++i)
    if (hold[i][0] >= 0 && hold[i][1] >= 0) push(hold[i][0], hold[i][1]);
  Path P;
  int n_alive = (int)T.size();
  std::uniform_real_distribution<double> U(0.0, 1.0);
  auto contract = [&](int a, int b) {
    std::vector<int> out = sym_diff(T[a], T[b]);
    P.flops += pow2(union_size(T[a], T[b]));
    P.max_rank = std::max(P.max_rank, (int)out.size());
    P.pairs.push_back({a, b});
    alive[a] = alive[b] = 0;
    int c = (int)T.size();
    T.push_back(out);
    alive.push_back(1);
    n_alive--;
    for (int i : T[a])
      if (hold[i][0] == a) hold[i][0] = -1; else if (hold[i][1] == a) hold[i][1] = -1;
    for (int i : T[b])
      if (hold[i][0] == b) hold[i][0] = -1; else if (hold[i][1] == b) hold[i][1] = -1;
    for (int i : out) {
      (hold[i][0] < 0 ? hold[i][0] : hold[i][1]) = c;
      int o = hold[i][0] == c ? hold[i][1] : hold[i][0];
      if (o >= 0) push(c, o);
    }
  };
  while (n_alive > 1) {
    std::vector<Cand> best;
    while (!heap.empty() && (int)best.size() < (rng ? 8 : 1)) {
      Cand c = heap.top();
      heap.pop();
      if (alive[std::get<1>(c)] && alive[std::get<2>(c)]) best.push_back(c);
    }
    if (best.empty()) {
      // disconnected parts: outer product of the two smallest tensors
      int a = -1, b = -1;
      for (int t = 0; t < (int)T.size(); ++t) {
        if (!alive[t]) continue;
        if (a < 0 || T[t].size() < T[a].size()) { b = a; a = t; }
        else if (b < 0 || T[t].size() < T[b].size()) b = t;
      }
      contract(std::min(a, b), std::max(a, b));
      continue;
    }
    size_t pick = 0;
    if (rng && best.size() > 1) {
      double c0 = std::get<0>(best[0]), scale = temp * std::max(1.0, std::fabs(c0));
      std::vector<double> w(best.size());
      double tot = 0;
      for (size_t i = 0; i < best.size(); ++i) tot += w[i] = std::exp(-(std::get<0>(best[i]) - c0) / scale);
      double r = U(*rng) * tot;
      for (pick = 0; pick + 1 < best.size() && r > w[pick]; ++pick) r -= w[pick];
    }
    for (size_t i = 0; i < best.size(); ++i)
      if (i != pick) heap.push(best[i]);
    contract(std::get<1>(best[pick]), std::get<2>(best[pick]));
  }
  return P;
}

// Replays a path with some indices removed: intermediate index sets, largest
// rank and complex multiply-adds of one slice.
static Path replay(const std::vector<std::vector<int>>& leaves, const std::vector<std::pair<int, int>>& pairs,
                   const std::set<int>& removed, std::vector<std::vector<int>>* sets = nullptr) {
  std::vector<std::vector<int>> T;
  for (auto t : leaves) {
    std::vector<int> k;
    for (int i : t)
      if (!removed.count(i)) k.push_back(i);
    std::sort(k.begin(), k.end());
    T.push_back(k);
  }
  Path P;
  P.pairs = pairs;
  for (auto& pr : pairs) {
    P.flops += pow2(union_size(T[pr.first], T[pr.second]));
    T.push_back(sym_diff(T[pr.first], T[pr.second]));
    P.max_rank = std::max(P.max_rank, (int)T.back().size());
  }
  if (sets) *sets = std::move(T);
  return P;
}

// ------------------------------------------------------------------- layout

// First-fit arena with coalescing free list (liveness-planned intermediates).
struct Arena {
  std::map<int64_t, int64_t> free_;  // offset -> size
  int64_t top = 0;
  int64_t alloc(int64_t size) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second < size) continue;
      int64_t off = it->first, rest = it->second - size;
      free_.erase(it);
      if (rest) free_[off + size] = rest;
      return off;
    }
    // extend, merging a free block that ends at the top
    if (!free_.empty()) {
      auto last = std::prev(free_.end());
      if (last->first + last->second == top) {
        int64_t off = last->first;
        free_.erase(last);
        top = off + size;
        return off;
      }
    }
    int64_t off = top;
    top += size;
    return off;
  }
  void release(int64_t off, int64_t size) {
    auto it = free_.emplace(off, size).first;
    auto nx = std::next(it);
    if (nx != free_.end() && off + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

static int64_t inter_reals(const TnTensor& t) { return 2ll << (t.lm + t.ln); }

TnNet tn_build(const tedq_gate_t* gates, int n_gates, int n_qubits, const tedq_meas_t& meas,
               const TnPlanOptions& opt) {
  if (n_qubits < 1 || n_qubits > 100000) throw std::invalid_argument("n_qubits out of range");
  if (n_gates < 0 || (n_gates > 0 && !gates)) throw std::invalid_argument("gates is null");
  for (int i = 0; i < n_gates; ++i) check_gate(gates[i], n_qubits);
  TnNet net;
  build_network(net, gates, n_gates, n_qubits, meas);
  const int L = net.n_leaves;
  std::vector<std::vector<int>> leaves;
  for (int t = 0; t < L; ++t) leaves.push_back(net.tensors[t].idx);

  // contraction order: plain greedy, then randomised trials; fewest entries
  // in the largest intermediate first (below 2^20 all count the same), then
  // fewest multiply-adds
  auto better = [](const Path& a, const Path& b) {
    int ra = std::max(a.max_rank, 20), rb = std::max(b.max_rank, 20);
    return ra != rb ? ra < rb : a.flops < b.flops;
  };
  Path best = greedy_path(leaves, net.n_index, nullptr, 0.0);
  for (int t = 1; t < opt.repeats; ++t) {
    std::mt19937_64 rng(opt.seed * 0x9E3779B97F4A7C15ull + (uint64_t)t);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    double temp = std::exp(std::log(0.01) * (1.0 - U(rng)));
    Path p = greedy_path(leaves, net.n_index, &rng, temp);
    if (better(p, best)) best = std::move(p);
  }

  // slicing: remove the index shared by most of the largest intermediates
  // (ties: fewest multiply-adds) until the largest fits max_rank
  std::set<int> removed;
  std::vector<std::vector<int>> sets;
  Path cur = replay(leaves, best.pairs, removed, &sets);
  while (cur.max_rank > opt.max_rank) {
    std::map<int, int> count;
    for (size_t s = L; s < sets.size(); ++s)
      if ((int)sets[s].size() == cur.max_rank)
        for (int i : sets[s]) count[i]++;
    int pick = -1;
    Path pick_path;
    int pick_count = -1;
    for (auto& kv : count) {
      std::set<int> r = removed;
      r.insert(kv.first);
      Path p = replay(leaves, best.pairs, r);
      bool take = pick < 0 || p.max_rank < pick_path.max_rank ||
                  (p.max_rank == pick_path.max_rank &&
                   (kv.second > pick_count || (kv.second == pick_count && p.flops < pick_path.flops)));
      if (take) {
        pick = kv.first;
        pick_path = p;
        pick_count = kv.second;
      }
    }
    if (pick < 0) break;
    removed.insert(pick);
    net.sliced.push_back(pick);
    if (net.sliced.size() > 40) throw UnsupportedError("network needs more than 40 sliced indices");
    cur = replay(leaves, best.pairs, removed, &sets);
  }
  net.max_rank = cur.max_rank;
  net.log2_flops = std::log2(8.0 * cur.flops) + (double)net.sliced.size();

  // leaves without sliced indices; offsets and constants
  for (int t = 0; t < L; ++t) {
    TnTensor& T = net.tensors[t];
    T.idx.clear();
    for (int i : T.full_idx)
      if (!removed.count(i)) T.idx.push_back(i);
    const int64_t size = 1ll << T.full_idx.size();
    if (T.batched) {
      T.off = net.batched_leaf_elems;
      net.batched_leaf_elems += size;
      continue;
    }
    T.off = net.const_elems;
    net.const_elems += size;
    if (T.leaf == TL_KET0 || T.leaf == TL_BRA0) {
      net.constants.insert(net.constants.end(), {1.0, 0.0, 0.0, 0.0});
    } else {
      const std::vector<double>& m = net.gates[T.gate].fixed;
      for (size_t j = 0; j < m.size(); j += 2) {
        net.constants.push_back(m[j]);
        net.constants.push_back(T.leaf == TL_GATE_CONJ ? -m[j + 1] : m[j + 1]);
      }
    }
  }

  // steps, gather tables and liveness-planned arenas
  Arena ab, au;  // batched (reals per batch entry) / unbatched (reals)
  std::map<int, int> producer;  // intermediate tensor -> step
  for (auto& pr : best.pairs) {
    TnStep st;
    st.a = pr.first;
    st.b = pr.second;
    const std::vector<int>& A = net.tensors[st.a].idx;
    const std::vector<int>& B = net.tensors[st.b].idx;
    for (int i : A) (std::find(B.begin(), B.end(), i) != B.end() ? st.contracted : st.free_a).push_back(i);
    for (int i : B)
      if (std::find(A.begin(), A.end(), i) == A.end()) st.free_b.push_back(i);
    st.batched = net.tensors[st.a].batched || net.tensors[st.b].batched;
    // the doubled operand is the one with fewer stored entries (batched
    // operands count as many circuits)
    {
      const double wa = std::ldexp(net.tensors[st.a].batched ? 1048576.0 : 1.0, (int)st.free_a.size());
      const double wb = std::ldexp(net.tensors[st.b].batched ? 1048576.0 : 1.0, (int)st.free_b.size());
      st.double_a = wa < wb;
    }
    auto operand = [&](int t, const std::vector<int>& fr) {
      TnOperand o;
      o.tensor = t;
      o.doubled = (t == st.a) == st.double_a;
      o.nf = (int)fr.size();
      o.nc = (int)st.contracted.size();
      const TnTensor& T = net.tensors[t];
      const std::vector<int>& store = T.leaf >= 0 ? T.full_idx : T.idx;
      const int r = (int)store.size();
      auto pos = [&](int id) {
        for (int j = 0; j < r; ++j)
          if (store[j] == id) return r - 1 - j;
        throw std::logic_error("index not in operand");
      };
      for (int j = 0; j < o.nc; ++j) o.src_bit.push_back(pos(st.contracted[o.nc - 1 - j]));
      for (int j = 0; j < o.nf; ++j) o.src_bit.push_back(pos(fr[o.nf - 1 - j]));
      if (T.leaf >= 0)
        for (size_t q = 0; q < net.sliced.size(); ++q)
          for (int j = 0; j < r; ++j)
            if (store[j] == net.sliced[q]) o.slice_bit.push_back({(int)q, r - 1 - j});
      return o;
    };
    st.opa = operand(st.a, st.free_a);
    st.opb = operand(st.b, st.free_b);
    {
      const int lm = (int)st.free_a.size(), ln = (int)st.free_b.size(), lk = (int)st.contracted.size();
      // small contractions with enough outputs (or a short sum) per circuit
      st.fused = (lm + ln + lk < opt.fused_log2 && lk <= 8 && (lm + ln >= 5 || lk <= 6)) ||
                 (opt.fused_short_log2 >= 0 && lk <= opt.fused_short_log2 && lm + ln <= 16);
      if (st.fused) st.double_a = false;
    }
    int lv = 0;
    for (int t : {st.a, st.b})
      if (net.tensors[t].leaf < 0) lv = std::max(lv, net.steps[producer[t]].level + 1);
    st.level = lv;
    TnTensor out;
    out.idx = st.free_b;
    out.idx.insert(out.idx.end(), st.free_a.begin(), st.free_a.end());
    out.lm = (int)st.free_a.size();
    out.ln = (int)st.free_b.size();
    out.split = st.double_a;
    out.batched = st.batched;
    st.out = (int)net.tensors.size();
    net.tensors.push_back(out);
    producer[st.out] = (int)net.steps.size();
    net.steps.push_back(std::move(st));
  }
  if (net.steps.empty()) throw std::logic_error("empty contraction");
  net.root = net.steps.back().out;
  // execution order: by level, a level's fused steps (one launch) first
  std::stable_sort(net.steps.begin(), net.steps.end(), [](const TnStep& x, const TnStep& y) {
    return x.level != y.level ? x.level < y.level : (x.fused && !y.fused);
  });
  // Liveness-planned arenas in that order.  The fused steps of a level run
  // concurrently and read their inputs in place: all their outputs are placed
  // before any of their inputs is released.  A gathered step copies its
  // inputs to the operand scratch before the GEMM writes, so its output may
  // reuse their space.
  auto release_inputs = [&](const TnStep& st) {
    for (int t : {st.a, st.b}) {
      const TnTensor& T = net.tensors[t];
      if (T.leaf >= 0) continue;
      (T.batched ? ab : au).release(T.arena, inter_reals(T));
    }
  };
  auto place = [&](const TnStep& st) {
    TnTensor& T = net.tensors[st.out];
    T.arena = (T.batched ? ab : au).alloc(inter_reals(T));
  };
  for (size_t i = 0; i < net.steps.size();) {
    size_t j = i;
    while (j < net.steps.size() && net.steps[j].fused && net.steps[j].level == net.steps[i].level) ++j;
    for (size_t k = i; k < j; ++k) place(net.steps[k]);
    for (size_t k = i; k < j; ++k) release_inputs(net.steps[k]);
    if (j == i) {
      release_inputs(net.steps[i]);
      place(net.steps[i]);
      j = i + 1;
    }
    i = j;
  }
  if (!net.tensors[net.root].idx.empty()) throw std::logic_error("open indices at the root");
  net.batched_arena = ab.top;
  net.unbatched_arena = au.top;
  return net;
}

int64_t tn_scratch_reals(const TnNet& net, int64_t batch) {
  int64_t m = 0;
  for (const TnStep& s : net.steps) {
    if (s.fused) continue;
    int64_t ba = net.tensors[s.a].batched ? batch : 1, bb = net.tensors[s.b].batched ? batch : 1;
    int64_t v = ((s.opa.doubled ? 4ll : 2ll) << (s.opa.nf + s.opa.nc)) * ba +
                ((s.opb.doubled ? 4ll : 2ll) << (s.opb.nf + s.opb.nc)) * bb;
    m = std::max(m, v);
  }
  return m;
}

// ------------------------------------------------------------------ export

static void ints(std::ostringstream& o, const std::vector<int>& v) {
  o << '[';
  for (size_t i = 0; i < v.size(); ++i) o << (i ? "," : "") << v[i];
  o << ']';
}

static void operand_json(std::ostringstream& o, const TnOperand& x) {
  o << "{\"tensor\":" << x.tensor << ",\"nf\":" << x.nf << ",\"nc\":" << x.nc
    << ",\"doubled\":" << (x.doubled ? 1 : 0) << ",\"src_bit\":";
  ints(o, x.src_bit);
  o << ",\"slice_bit\":[";
  for (size_t i = 0; i < x.slice_bit.size(); ++i)
    o << (i ? "," : "") << '[' << x.slice_bit[i].first << ',' << x.slice_bit[i].second << ']';
  o << "]}";
}

std::string tn_describe(const std::vector<TnNet>& nets, int n_params, int precision) {
  std::ostringstream o;
  o << std::setprecision(17);
  o << "{\"n_params\":" << n_params << ",\"precision\":" << precision << ",\"nets\":[";
  for (size_t ni = 0; ni < nets.size(); ++ni) {
    const TnNet& n = nets[ni];
    o << (ni ? "," : "") << "{\"n\":" << n.n << ",\"n_leaves\":" << n.n_leaves << ",\"root\":" << n.root
      << ",\"max_rank\":" << n.max_rank << ",\"log2_flops\":" << n.log2_flops << ",\"gates_in\":" << n.gates_in
      << ",\"gates_kept\":" << n.gates_kept << ",\"qubits_kept\":" << n.qubits_kept
      << ",\"batched_leaf_elems\":" << n.batched_leaf_elems << ",\"const_elems\":" << n.const_elems
      << ",\"batched_arena\":" << n.batched_arena << ",\"unbatched_arena\":" << n.unbatched_arena
      << ",\"sliced\":";
    ints(o, n.sliced);
    o << ",\"gates\":[";
    for (size_t i = 0; i < n.gates.size(); ++i) {
      const TnGate& g = n.gates[i];
      o << (i ? "," : "") << "{\"op\":" << g.op << ",\"k\":" << g.k << ",\"qubits\":";
      ints(o, std::vector<int>(g.qubits, g.qubits + g.k));
      o << ",\"slot\":[" << g.slot[0] << ',' << g.slot[1] << ',' << g.slot[2] << "],\"val\":[" << g.val[0] << ','
        << g.val[1] << ',' << g.val[2] << "],\"param\":" << (g.param ? 1 : 0) << '}';
    }
    o << "],\"constants\":[";
    for (size_t i = 0; i < n.constants.size(); ++i) o << (i ? "," : "") << n.constants[i];
    o << "],\"tensors\":[";
    for (size_t i = 0; i < n.tensors.size(); ++i) {
      const TnTensor& t = n.tensors[i];
      o << (i ? "," : "") << "{\"leaf\":" << t.leaf << ",\"gate\":" << t.gate << ",\"batched\":" << (t.batched ? 1 : 0)
        << ",\"lm\":" << t.lm << ",\"ln\":" << t.ln << ",\"split\":" << (t.split ? 1 : 0) << ",\"off\":" << t.off
        << ",\"arena\":" << t.arena
        << ",\"full_idx\":";
      ints(o, t.full_idx);
      o << ",\"idx\":";
      ints(o, t.idx);
      o << '}';
    }
    o << "],\"steps\":[";
    for (size_t i = 0; i < n.steps.size(); ++i) {
      const TnStep& s = n.steps[i];
      o << (i ? "," : "") << "{\"a\":" << s.a << ",\"b\":" << s.b << ",\"out\":" << s.out
        << ",\"batched\":" << (s.batched ? 1 : 0) << ",\"double_a\":" << (s.double_a ? 1 : 0)
        << ",\"fused\":" << (s.fused ? 1 : 0) << ",\"level\":" << s.level << ",\"opa\":";
      operand_json(o, s.opa);
      o << ",\"opb\":";
      operand_json(o, s.opb);
      o << '}';
    }
    o << "]}";
  }
  o << "]}";
  return o.str();
}

}  // namespace tedq
