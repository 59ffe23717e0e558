// sv_ref.cpp -- independent complex128 CPU state-vector simulator with the
// adjoint gradient (TEST INFRASTRUCTURE ONLY: the checker for large circuits).
//
// It restates what the reference's PyTorchBackend computes for the
// state-vector branch (tedq/backends/pytorch_backend.py:358-498: gates applied
// in circuit order to the [2]*n state, qubit 0 the most significant axis;
// expectation values <psi|O|psi>) and the gradient that the reference obtains
// from torch autograd (back_prop, :142-144), for circuits too large for the
// Python oracle (24 qubits: the reference's back_prop would keep every
// intermediate state).  It shares no code with the CUDA kernels: every gate is
// a dense 2^k x 2^k complex matrix applied amplitude by amplitude, the
// gradient is the textbook adjoint sweep
//   lambda = sum_k dy_k O_k psi,
//   for g = last..first:  psi <- U_g^dag psi;
//                         grad[slot] += 2 Re <lambda| dU_g/dtheta |psi>;
//                         lambda <- U_g^dag lambda,
// and the host threads split the amplitude ranges.  Built by
// oracle/build_ref.py; called from oracle/sv_ref.py.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

using cd = std::complex<double>;

namespace {

template <typename F>
void parallel_for(int64_t count, int threads, F&& f, int64_t min_count = 4096) {
  if (threads <= 1 || count < min_count) {
    f(int64_t(0), count);
    return;
  }
  std::vector<std::thread> pool;
  const int64_t chunk = (count + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t a = t * chunk, b = std::min(count, a + chunk);
    if (a >= b) break;
    pool.emplace_back([&f, a, b] { f(a, b); });
  }
  for (auto& th : pool) th.join();
}

// bit positions of the gate's qubits, qubits[0] the most significant matrix bit
struct GateBits {
  int k = 0;
  int64_t bit[3] = {0, 0, 0};
  int64_t mask = 0;
};

GateBits gate_bits(int n, int k, const int* qubits) {
  GateBits g;
  g.k = k;
  for (int i = 0; i < k; ++i) {
    g.bit[i] = int64_t(1) << (n - 1 - qubits[i]);
    g.mask |= g.bit[i];
  }
  return g;
}

// index of the base amplitude number `t` (bits of the gate cleared)
inline int64_t base_index(int64_t t, const GateBits& g, const int64_t* sorted_bits) {
  int64_t v = t;
  for (int i = 0; i < g.k; ++i) {
    const int64_t b = sorted_bits[i];
    v = ((v & ~(b - 1)) << 1) | (v & (b - 1));
  }
  return v;
}

// out[x] = sum_y M[x][y] in[y] over every k-qubit block; in may equal out.
// dagger: use the conjugate transpose of M.
void apply(int n, int k, const int* qubits, const cd* M, bool dagger, const cd* in, cd* out, int threads) {
  const GateBits g = gate_bits(n, k, qubits);
  int64_t sorted[3] = {g.bit[0], g.bit[1], g.bit[2]};
  std::sort(sorted, sorted + k);
  const int d = 1 << k;
  int64_t off[8];
  for (int r = 0; r < d; ++r) {
    off[r] = 0;
    for (int i = 0; i < k; ++i)
      if ((r >> (k - 1 - i)) & 1) off[r] |= g.bit[i];
  }
  cd m[64];
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) m[r * d + c] = dagger ? std::conj(M[c * d + r]) : M[r * d + c];
  const int64_t blocks = (int64_t(1) << n) >> k;
  parallel_for(blocks, threads, [&](int64_t a, int64_t b) {
    cd v[8];
    for (int64_t t = a; t < b; ++t) {
      const int64_t base = base_index(t, g, sorted);
      for (int r = 0; r < d; ++r) v[r] = in[base | off[r]];
      for (int r = 0; r < d; ++r) {
        cd acc = 0;
        for (int c = 0; c < d; ++c) acc += m[r * d + c] * v[c];
        out[base | off[r]] = acc;
      }
    }
  });
}

// One step of the adjoint sweep over gate g, fused into a single pass over
// the amplitude blocks: psi <- U^dag psi; part[j] += <lambda| dU_j |psi>
// (with the uncomputed psi and the not yet updated lambda); lambda <- U^dag
// lambda.  Blocks are disjoint, so the per-block order is the sweep's order.
void backward_gate(int n, int k, const int* qubits, const cd* U, int nd, const cd* const* dU, cd* psi, cd* lam,
                   cd* part, int threads) {
  const GateBits g = gate_bits(n, k, qubits);
  int64_t sorted[3] = {g.bit[0], g.bit[1], g.bit[2]};
  std::sort(sorted, sorted + k);
  const int d = 1 << k;
  int64_t off[8];
  for (int r = 0; r < d; ++r) {
    off[r] = 0;
    for (int i = 0; i < k; ++i)
      if ((r >> (k - 1 - i)) & 1) off[r] |= g.bit[i];
  }
  cd ud[64];
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) ud[r * d + c] = std::conj(U[c * d + r]);
  const int64_t blocks = (int64_t(1) << n) >> k;
  const int T = std::max(1, threads);
  std::vector<cd> parts((size_t)T * 3, cd(0));
  const int64_t chunk = (blocks + T - 1) / T;
  parallel_for((int64_t)T, T, [&](int64_t t0, int64_t t1) {
    for (int64_t t = t0; t < t1; ++t) {
      cd acc[3] = {0, 0, 0};
      cd v[8], w[8], x[8];
      const int64_t lo = t * chunk, hi = std::min(blocks, lo + chunk);
      for (int64_t blk = lo; blk < hi; ++blk) {
        const int64_t base = base_index(blk, g, sorted);
        for (int r = 0; r < d; ++r) {
          v[r] = psi[base | off[r]];
          w[r] = lam[base | off[r]];
        }
        for (int r = 0; r < d; ++r) {
          cd a = 0;
          for (int c = 0; c < d; ++c) a += ud[r * d + c] * v[c];
          x[r] = a;
        }
        for (int j = 0; j < nd; ++j) {
          cd a = 0;
          for (int r = 0; r < d; ++r) {
            cd y = 0;
            for (int c = 0; c < d; ++c) y += dU[j][r * d + c] * x[c];
            a += std::conj(w[r]) * y;
          }
          acc[j] += a;
        }
        for (int r = 0; r < d; ++r) {
          psi[base | off[r]] = x[r];
          cd a = 0;
          for (int c = 0; c < d; ++c) a += ud[r * d + c] * w[c];
          lam[base | off[r]] = a;
        }
      }
      for (int j = 0; j < 3; ++j) parts[(size_t)t * 3 + j] = acc[j];
    }
  }, 1);
  for (int j = 0; j < nd; ++j) {
    cd s = 0;
    for (int t = 0; t < T; ++t) s += parts[(size_t)t * 3 + j];
    part[j] = s;
  }
}

// sum over x of conj(a[x]) * b[x]
cd inner(int64_t N, const cd* a, const cd* b, int threads) {
  std::vector<cd> part(std::max(1, threads));
  const int64_t chunk = (N + part.size() - 1) / part.size();
  parallel_for((int64_t)part.size(), threads, [&](int64_t p0, int64_t p1) {
    for (int64_t p = p0; p < p1; ++p) {
      cd s = 0;
      const int64_t lo = p * chunk, hi = std::min(N, lo + chunk);
      for (int64_t x = lo; x < hi; ++x) s += std::conj(a[x]) * b[x];
      part[p] = s;
    }
  }, 1);
  cd s = 0;
  for (auto& v : part) s += v;
  return s;
}

}  // namespace

extern "C" {

// Value and adjoint gradient of L = sum_k dy[k] <psi|O_k|psi>, psi = U|0...0>.
//   gates: nq[g] in 1..3, qubits[3g..3g+nq-1], matrix of gate g at
//     mats[mat_off[g] ..] (2 * 4^nq doubles, row-major re/im);
//   derivatives: n_d[g] entries per gate, slot d_slot[j] and matrix
//     dmats[d_off[j] ..] = dU_g/dtheta (same layout), j running over all
//     gates' entries in order;
//   observables: n_f[o] tensor factors each, factor f with nq_f[f] qubits
//     fq[3f..], matrix fmats[f_off[f] ..];
//   values[o] = <psi|O_o|psi> (real part); grad[n_params] accumulated.
// Returns 0, -1 when the state cannot be allocated, -2 for a gate with more
// than 3 trainable parameters.
int tedq_oracle_sv_value_and_grad(int n, int n_gates, const int* nq, const int* qubits, const double* mats,
                                  const int64_t* mat_off, const int* n_d, const int* d_slot, const double* dmats,
                                  const int64_t* d_off, int n_obs, const int* n_f, const int* nq_f, const int* fq,
                                  const double* fmats, const int64_t* f_off, const double* dy, int n_params,
                                  double* values, double* grad, int threads) {
  const int64_t N = int64_t(1) << n;
  std::vector<cd> psi, lam, tmp, acc;
  try {
    psi.assign(N, cd(0));
    lam.assign(N, cd(0));
    tmp.assign(N, cd(0));
  } catch (...) {
    return -1;
  }
  psi[0] = 1.0;
  auto M = [](const double* base, int64_t off) { return reinterpret_cast<const cd*>(base + off); };
  for (int g = 0; g < n_gates; ++g) apply(n, nq[g], qubits + 3 * g, M(mats, mat_off[g]), false, psi.data(), psi.data(), threads);
  // observables: values and lambda = sum dy_o O_o psi
  int f = 0;
  for (int o = 0; o < n_obs; ++o) {
    std::memcpy(tmp.data(), psi.data(), N * sizeof(cd));
    for (int j = 0; j < n_f[o]; ++j, ++f) apply(n, nq_f[f], fq + 3 * f, M(fmats, f_off[f]), false, tmp.data(), tmp.data(), threads);
    values[o] = inner(N, psi.data(), tmp.data(), threads).real();
    const double w = dy ? dy[o] : 0.0;
    if (w != 0.0)
      parallel_for(N, threads, [&](int64_t a, int64_t b) {
        for (int64_t x = a; x < b; ++x) lam[x] += w * tmp[x];
      });
  }
  if (!grad || n_params == 0) return 0;
  // derivative entries of each gate: first index
  std::vector<int64_t> first(n_gates + 1, 0);
  for (int g = 0; g < n_gates; ++g) first[g + 1] = first[g] + n_d[g];
  for (int g = n_gates - 1; g >= 0; --g) {
    const int nd = (int)(first[g + 1] - first[g]);
    if (nd > 3) return -2;
    const cd* dU[3] = {nullptr, nullptr, nullptr};
    for (int j = 0; j < nd; ++j) dU[j] = M(dmats, d_off[first[g] + j]);
    cd part[3];
    backward_gate(n, nq[g], qubits + 3 * g, M(mats, mat_off[g]), nd, dU, psi.data(), lam.data(), part, threads);
    for (int j = 0; j < nd; ++j) grad[d_slot[first[g] + j]] += 2.0 * part[j].real();
  }
  return 0;
}

}  // extern "C"
