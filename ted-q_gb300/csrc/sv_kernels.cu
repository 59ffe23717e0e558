// sv_kernels.cu -- sm_103a state-vector kernels of the compiled-circuit path.
//
// Reference counterpart: the per-gate ``torch.tensordot`` + ``permute`` loop
// of PyTorchBackend.execute (tedq/backends/pytorch_backend.py:365-379), the
// measurement reductions (:393-498) and, for gradients, torch autograd through
// that loop (``back_prop``, :142-144).
//
// Kernels
//   fwd_pass_kernel  one HBM pass of the forward schedule: a CTA stages one
//                    tile (2^m amplitudes, 64 KiB) in shared memory, runs the
//                    pass's register phases, writes the tile back in place.
//   bwd_pass_kernel  one pass of the adjoint sweep over psi and lambda at once:
//                    for every parameterised gate (in reverse order) it adds
//                    coef * Im<lambda|G|psi> into the gradient, then applies the
//                    inverse gate to both states.
//   expval_kernel    Pauli-string expectations, one read of the state,
//                    FP32 partial sums per thread/warp and FP64 across warps/CTAs.
//   probs kernels, lambda_init_kernel, finalize kernels.
//
// Bound: every pass kernel moves 16 B per amplitude (c64 read + write; 32 B
// for the adjoint pass) and is designed to run at HBM bandwidth; the FP32
// register work per amplitude is 4-8 FMA per gate.
#include <cuda_runtime.h>

#include "sv_kernels.cuh"

namespace tedq {
namespace {

template <typename real>
struct alignas(2 * sizeof(real)) cpx {
  real x, y;
};

template <typename real>
struct Unit;
template <>
struct alignas(16) Unit<float> {
  cpx<float> v[2];
};
template <>
struct alignas(16) Unit<double> {
  cpx<double> v[1];
};

template <typename real>
__device__ __forceinline__ cpx<real> mk(real x, real y) {
  cpx<real> r;
  r.x = x;
  r.y = y;
  return r;
}
template <typename real>
__device__ __forceinline__ cpx<real> cmul(cpx<real> a, cpx<real> b) {
  return mk<real>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// m0 * x0 + m1 * x1
template <typename real>
__device__ __forceinline__ cpx<real> cmac2(cpx<real> m0, cpx<real> x0, cpx<real> m1, cpx<real> x1) {
  real re = m0.x * x0.x;
  re = fma(-m0.y, x0.y, re);
  re = fma(m1.x, x1.x, re);
  re = fma(-m1.y, x1.y, re);
  real im = m0.x * x0.y;
  im = fma(m0.y, x0.x, im);
  im = fma(m1.x, x1.y, im);
  im = fma(m1.y, x1.x, im);
  return mk<real>(re, im);
}
template <typename real>
__device__ __forceinline__ cpx<real> cconj(cpx<real> a) {
  return mk<real>(a.x, -a.y);
}

__device__ __forceinline__ void sincos_(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_(double x, double* s, double* c) { sincos(x, s, c); }

template <typename real>
__device__ __forceinline__ real pval(const Factor& F, int j, const real* prm) {
  return F.slot[j] >= 0 ? prm[F.slot[j]] : (real)F.val[j];
}

template <typename real>
__device__ __forceinline__ cpx<real> fixed_at(const PassParams& P, int i) {
  return mk<real>((real)P.fixed[i].re, (real)P.fixed[i].im);
}

// One factor as a dense 2x2 (row-major).  Matrices follow the reference's
// gate definitions (tedq/QInterpreter/operators/qubit.py, RX :990-997, RY
// :1048-1055, RZ :1106-1112, PhaseShift :1253-1257, Rot :1169-1189).
template <typename real>
__device__ void factor_mat(const PassParams& P, const Factor& F, const real* prm, cpx<real>* m) {
  const real zero = 0, one = 1;
  switch (F.op) {
    case F_FIXED2:
      for (int k = 0; k < 4; ++k) m[k] = fixed_at<real>(P, F.fix + k);
      break;
    case F_FIXD:
      m[0] = fixed_at<real>(P, F.fix);
      m[1] = m[2] = mk<real>(zero, zero);
      m[3] = fixed_at<real>(P, F.fix + 1);
      break;
    case F_RX: {
      real s, c;
      sincos_(pval<real>(F, 0, prm) / (real)2, &s, &c);
      m[0] = m[3] = mk<real>(c, zero);
      m[1] = m[2] = mk<real>(zero, -s);
      break;
    }
    case F_RY: {
      real s, c;
      sincos_(pval<real>(F, 0, prm) / (real)2, &s, &c);
      m[0] = m[3] = mk<real>(c, zero);
      m[1] = mk<real>(-s, zero);
      m[2] = mk<real>(s, zero);
      break;
    }
    case F_RZ: {
      real s, c;
      sincos_(pval<real>(F, 0, prm) / (real)2, &s, &c);
      m[0] = mk<real>(c, -s);
      m[3] = mk<real>(c, s);
      m[1] = m[2] = mk<real>(zero, zero);
      break;
    }
    case F_PHASE: {
      real s, c;
      sincos_(pval<real>(F, 0, prm), &s, &c);
      m[0] = mk<real>(one, zero);
      m[3] = mk<real>(c, s);
      m[1] = m[2] = mk<real>(zero, zero);
      break;
    }
    default: {  // F_ROT
      real phi = pval<real>(F, 0, prm), th = pval<real>(F, 1, prm), om = pval<real>(F, 2, prm);
      real s, c, sp, cp, sm, cm;
      sincos_(th / (real)2, &s, &c);
      sincos_((phi + om) / (real)2, &sp, &cp);
      sincos_((phi - om) / (real)2, &sm, &cm);
      m[0] = mk<real>(cp * c, -sp * c);
      m[1] = mk<real>(-cm * s, -sm * s);
      m[2] = mk<real>(cm * s, -sm * s);
      m[3] = mk<real>(cp * c, sp * c);
      break;
    }
  }
}

// Matrix i of a pass: product of its factors (first factor applied first),
// conjugate-transposed for the adjoint sweep.  Diagonal matrices keep 2 entries.
template <typename real>
__device__ void compute_mat(const PassParams& P, int i, const real* prm, cpx<real>* out) {
  const MatDesc md = P.mat[i];
  cpx<real> M[4], F[4], T[4];
  factor_mat<real>(P, P.factor[md.f0], prm, M);
  for (int j = 1; j < md.nf; ++j) {
    factor_mat<real>(P, P.factor[md.f0 + j], prm, F);
    T[0] = cmac2(F[0], M[0], F[1], M[2]);
    T[1] = cmac2(F[0], M[1], F[1], M[3]);
    T[2] = cmac2(F[2], M[0], F[3], M[2]);
    T[3] = cmac2(F[2], M[1], F[3], M[3]);
    M[0] = T[0];
    M[1] = T[1];
    M[2] = T[2];
    M[3] = T[3];
  }
  if (md.dagger) {
    cpx<real> t = M[1];
    M[1] = cconj(M[2]);
    M[2] = cconj(t);
    M[0] = cconj(M[0]);
    M[3] = cconj(M[3]);
  }
  if (md.diag) {
    out[0] = M[0];
    out[1] = M[3];
  } else {
    for (int k = 0; k < 4; ++k) out[k] = M[k];
  }
}

// ---------------------------------------------------------------- register gates

template <int K, int R, typename real>
__device__ __forceinline__ void apply_u1(cpx<real>* a, const cpx<real>* M, unsigned cm) {
  const cpx<real> m0 = M[0], m1 = M[1], m2 = M[2], m3 = M[3];
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & cm) != cm) continue;
    const int j = i | (1 << K);
    const cpx<real> x0 = a[i], x1 = a[j];
    a[i] = cmac2(m0, x0, m1, x1);
    a[j] = cmac2(m2, x0, m3, x1);
  }
}

template <int K, int R, typename real>
__device__ __forceinline__ void apply_d1(cpx<real>* a, const cpx<real>* M, unsigned cm) {
  const cpx<real> d0 = M[0], d1 = M[1];
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if ((i & cm) != cm) continue;
    a[i] = cmul((i >> K) & 1 ? d1 : d0, a[i]);
  }
}

// RX-type [[c, -i s], [-i s, c]] (RX, or RX^dagger with s negated)
template <int K, int R, typename real>
__device__ __forceinline__ void apply_rxt(cpx<real>* a, const cpx<real>* M, unsigned cm) {
  const real c = M[0].x, sn = -M[1].y;
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & cm) != cm) continue;
    const int j = i | (1 << K);
    const cpx<real> x0 = a[i], x1 = a[j];
    a[i] = mk<real>(fma(c, x0.x, sn * x1.y), fma(c, x0.y, -sn * x1.x));
    a[j] = mk<real>(fma(c, x1.x, sn * x0.y), fma(c, x1.y, -sn * x0.x));
  }
}

// RY-type [[c, -s], [s, c]]
template <int K, int R, typename real>
__device__ __forceinline__ void apply_ryt(cpx<real>* a, const cpx<real>* M, unsigned cm) {
  const real c = M[0].x, sn = -M[1].x;
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & cm) != cm) continue;
    const int j = i | (1 << K);
    const cpx<real> x0 = a[i], x1 = a[j];
    a[i] = mk<real>(fma(c, x0.x, -sn * x1.x), fma(c, x0.y, -sn * x1.y));
    a[j] = mk<real>(fma(sn, x0.x, c * x1.x), fma(sn, x0.y, c * x1.y));
  }
}

// diag(1, d): multiply the |1> half only
template <int K, int R, typename real>
__device__ __forceinline__ void apply_ph(cpx<real>* a, const cpx<real>* M, unsigned cm) {
  const cpx<real> d = M[1];
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (!(i & (1 << K))) continue;
    if ((i & cm) != cm) continue;
    a[i] = cmul(d, a[i]);
  }
}

template <int K, int R, typename real>
__device__ __forceinline__ void apply_x(cpx<real>* a, unsigned cm) {
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & cm) != cm) continue;
    const int j = i | (1 << K);
    const cpx<real> t = a[i];
    a[i] = a[j];
    a[j] = t;
  }
}

template <int R, typename real, int K = 0>
__device__ __forceinline__ void dispatch_gate(int kind, int k, cpx<real>* a, const cpx<real>* M, unsigned cm) {
  if constexpr (K < R) {
    if (k == K) {
      switch (kind) {
        case GK_U1: apply_u1<K, R, real>(a, M, cm); break;
        case GK_D1: apply_d1<K, R, real>(a, M, cm); break;
        case GK_RXT: apply_rxt<K, R, real>(a, M, cm); break;
        case GK_RYT: apply_ryt<K, R, real>(a, M, cm); break;
        case GK_PH: apply_ph<K, R, real>(a, M, cm); break;
        default: apply_x<K, R, real>(a, cm); break;
      }
    } else {
      dispatch_gate<R, real, K + 1>(kind, k, a, M, cm);
    }
  }
}

template <int R, typename real>
__device__ __forceinline__ void apply_rgate(const RGate& r, cpx<real>* a, const cpx<real>* M) {
  if (r.kind == GK_SWAP) {
    const unsigned b0 = 1u << r.k0, b1 = 1u << r.k1;
    dispatch_gate<R, real>(GK_X, r.k1, a, M, r.cmask | b0);
    dispatch_gate<R, real>(GK_X, r.k0, a, M, r.cmask | b1);
    dispatch_gate<R, real>(GK_X, r.k1, a, M, r.cmask | b0);
  } else {
    dispatch_gate<R, real>(r.kind, r.k0, a, M, r.cmask);
  }
}

// Im(conj(a) b) and Re(conj(a) b)
template <typename real>
__device__ __forceinline__ real imcb(cpx<real> a, cpx<real> b) {
  return a.x * b.y - a.y * b.x;
}
template <typename real>
__device__ __forceinline__ real recb(cpx<real> a, cpx<real> b) {
  return a.x * b.x + a.y * b.y;
}

// Per-thread part of Im <lambda| G |psi> on the control subspace.
template <int G, int K, int R, typename real>
__device__ __forceinline__ real grad_part(const cpx<real>* p, const cpx<real>* l, unsigned cm) {
  real acc = 0;
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & cm) != cm) continue;
    const int j = i | (1 << K);
    if (G == GR_X) acc += imcb(l[i], p[j]) + imcb(l[j], p[i]);
    if (G == GR_Y) acc += recb(l[j], p[i]) - recb(l[i], p[j]);
    if (G == GR_Z) acc += imcb(l[i], p[i]) - imcb(l[j], p[j]);
    if (G == GR_P1) acc += imcb(l[j], p[j]);
  }
  return acc;
}

template <int R, typename real, int K = 0>
__device__ __forceinline__ real dispatch_grad(int g, int k, const cpx<real>* p, const cpx<real>* l, unsigned cm) {
  if constexpr (K < R) {
    if (k == K) {
      switch (g) {
        case GR_X: return grad_part<GR_X, K, R, real>(p, l, cm);
        case GR_Y: return grad_part<GR_Y, K, R, real>(p, l, cm);
        case GR_Z: return grad_part<GR_Z, K, R, real>(p, l, cm);
        default: return grad_part<GR_P1, K, R, real>(p, l, cm);
      }
    }
    return dispatch_grad<R, real, K + 1>(g, k, p, l, cm);
  }
  return (real)0;
}

// ---------------------------------------------------------------- tile staging

template <typename real>
constexpr int kE = sizeof(real) == 4 ? 1 : 0;  // log2 amplitudes per 16-byte unit

// Global amplitude index of the first amplitude of tile unit u.
__device__ __forceinline__ uint64_t unit_global(const PassParams& P, uint64_t base, uint32_t u, int E) {
  const uint32_t t = u << E;
  uint64_t g = base | (t & ((1u << P.c) - 1));
  uint32_t h = t >> P.c;
  for (int k = 0; h; ++k, h >>= 1)
    if (h & 1) g |= 1ull << P.hi[k];
  return g;
}

__device__ __forceinline__ uint64_t tile_base(const PassParams& P, uint32_t tile) {
  uint64_t base = 0;
  for (int k = 0; k < P.n_outer; ++k)
    if ((tile >> k) & 1) base |= 1ull << P.outer[k];
  return base;
}

template <typename real>
__device__ __forceinline__ Unit<real> load_unit(const PassParams& P, const cpx<real>* st, uint64_t g,
                                                const cpx<real>* init) {
  constexpr int E = kE<real>;
  Unit<real> v;
  if (P.init == 0) {
    v = reinterpret_cast<const Unit<real>*>(st)[g >> E];
  } else {
#pragma unroll
    for (int k = 0; k < (1 << E); ++k) {
      const uint64_t q = g + k;
      cpx<real> a = mk<real>((real)0, (real)0);
      if (P.init == 1) {
        if (q == 0) a.x = (real)1;
      } else if ((q & ((1ull << P.pad_bits) - 1)) == 0) {
        a = init[q >> P.pad_bits];
      }
      v.v[k] = a;
    }
  }
  return v;
}

// Dense fixed k-qubit matrix applied directly on the shared-memory tile.
template <typename real>
__device__ void dense_phase(const PassParams& P, const Phase& ph, Unit<real>* tile, int tid, int T) {
  constexpr int E = kE<real>;
  cpx<real>* amp = reinterpret_cast<cpx<real>*>(tile);
  const int k = ph.dk, d = 1 << k;
  uint32_t dmask = 0;
  for (int i = 0; i < k; ++i) dmask |= 1u << ph.dpos[i];
  const int ngroups = 1 << (P.m - k);
  for (int grp = tid; grp < ngroups; grp += T) {
    uint32_t base = 0, rem = grp;
    for (int p = 0; p < P.m; ++p)
      if (!((dmask >> p) & 1)) {
        if (rem & 1) base |= 1u << p;
        rem >>= 1;
      }
    if ((base & ph.dcmask) != ph.dcmask) continue;
    cpx<real> v[8], w[8];
    uint32_t addr[8];
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      if (r < d) {
        uint32_t t = base;
        for (int i = 0; i < k; ++i)
          if ((r >> (k - 1 - i)) & 1) t |= 1u << ph.dpos[i];
        addr[r] = (swz_unit(t >> E) << E) | (t & ((1u << E) - 1));
        v[r] = amp[addr[r]];
      }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      if (r < d) {
        cpx<real> acc = mk<real>((real)0, (real)0);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          if (c < d) {
            cpx<real> m = ph.dagger ? cconj(fixed_at<real>(P, ph.dfix + c * d + r)) : fixed_at<real>(P, ph.dfix + r * d + c);
            cpx<real> t = cmul(m, v[c]);
            acc.x += t.x;
            acc.y += t.y;
          }
        }
        w[r] = acc;
      }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r)
      if (r < d) amp[addr[r]] = w[r];
  }
}

// ---------------------------------------------------------------- pass kernels

template <typename real, int R>
__global__ void __launch_bounds__(256, 2)
    fwd_pass_kernel(const __grid_constant__ PassParams P, cpx<real>* __restrict__ psi,
                    const real* __restrict__ params, int n_params, const cpx<real>* __restrict__ init,
                    int64_t circ0) {
  using C = cpx<real>;
  using U = Unit<real>;
  constexpr int E = kE<real>;
  constexpr int NR = 1 << R;
  constexpr int NU = NR >> E;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  U* tile = reinterpret_cast<U*>(smem_raw);
  __shared__ C mats[kMaxMats][4];
  const int tid = threadIdx.x, T = blockDim.x;
  const int64_t circ = circ0 + blockIdx.y;
  C* st = psi + (circ << P.n);
  const real* prm = params ? params + circ * n_params : nullptr;
  for (int i = tid; i < P.n_mats; i += T) compute_mat<real>(P, i, prm, mats[i]);
  const uint64_t base = tile_base(P, blockIdx.x);
  // Stage the tile: each thread owns NU units (nunits == NU * T); all global
  // loads are issued before the first shared-memory store.
  {
    U v[NU];
#pragma unroll
    for (int k = 0; k < NU; ++k) v[k] = load_unit<real>(P, st, unit_global(P, base, tid + k * T, E), init);
#pragma unroll
    for (int k = 0; k < NU; ++k) tile[swz_unit(tid + k * T)] = v[k];
  }
  __syncthreads();
  for (int f = 0; f < P.n_phases; ++f) {
    const Phase& ph = P.phase[f];
    if (ph.type == PH_REG) {
      uint32_t bu = 0;
      for (int b = 0; b < ph.ntid; ++b)
        if ((tid >> b) & 1) bu ^= ph.tid_off[b];
      C a[NR];
#pragma unroll
      for (int j = 0; j < NU; ++j) {
        const U v = tile[bu ^ ph.reg_off[j]];
#pragma unroll
        for (int k = 0; k < (1 << E); ++k) a[(j << E) + k] = v.v[k];
      }
      for (int g = ph.g0; g < ph.g1; ++g) {
        const RGate& r = P.gate[g];
        apply_rgate<R, real>(r, a, mats[r.mat]);
      }
#pragma unroll
      for (int j = 0; j < NU; ++j) {
        U v;
#pragma unroll
        for (int k = 0; k < (1 << E); ++k) v.v[k] = a[(j << E) + k];
        tile[bu ^ ph.reg_off[j]] = v;
      }
    } else {
      dense_phase<real>(P, ph, tile, tid, T);
    }
    __syncthreads();
  }
  U* gst = reinterpret_cast<U*>(st);
#pragma unroll
  for (int k = 0; k < NU; ++k) gst[unit_global(P, base, tid + k * T, E) >> E] = tile[swz_unit(tid + k * T)];
}

template <typename real, int R>
__global__ void __launch_bounds__(256, 2)
    bwd_pass_kernel(const __grid_constant__ PassParams P, cpx<real>* __restrict__ psi, cpx<real>* __restrict__ lam,
                    const real* __restrict__ params, int n_params, double* __restrict__ grad_acc, int64_t circ0) {
  using C = cpx<real>;
  using U = Unit<real>;
  constexpr int E = kE<real>;
  constexpr int NR = 1 << R;
  constexpr int NU = NR >> E;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int nunits = 1 << (P.m - E);
  U* tp = reinterpret_cast<U*>(smem_raw);
  U* tl = tp + nunits;
  __shared__ C mats[kMaxMats][4];
  __shared__ double gacc[kMaxPassGates];
  const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31;
  const int64_t circ = circ0 + blockIdx.y;
  C* sp = psi + (circ << P.n);
  C* sl = lam + (circ << P.n);
  const real* prm = params ? params + circ * n_params : nullptr;
  for (int i = tid; i < P.n_mats; i += T) compute_mat<real>(P, i, prm, mats[i]);
  for (int i = tid; i < P.n_gates; i += T) gacc[i] = 0.0;
  const uint64_t base = tile_base(P, blockIdx.x);
  {
    U v[NU], w[NU];
#pragma unroll
    for (int k = 0; k < NU; ++k) {
      const uint64_t g = unit_global(P, base, tid + k * T, E) >> E;
      v[k] = reinterpret_cast<const U*>(sp)[g];
      w[k] = reinterpret_cast<const U*>(sl)[g];
    }
#pragma unroll
    for (int k = 0; k < NU; ++k) {
      const uint32_t s = swz_unit(tid + k * T);
      tp[s] = v[k];
      tl[s] = w[k];
    }
  }
  __syncthreads();
  for (int f = 0; f < P.n_phases; ++f) {
    const Phase& ph = P.phase[f];
    if (ph.type == PH_REG) {
      uint32_t bu = 0;
      for (int b = 0; b < ph.ntid; ++b)
        if ((tid >> b) & 1) bu ^= ph.tid_off[b];
      C a[NR], l[NR];
#pragma unroll
      for (int j = 0; j < NU; ++j) {
        const U v = tp[bu ^ ph.reg_off[j]];
        const U w = tl[bu ^ ph.reg_off[j]];
#pragma unroll
        for (int k = 0; k < (1 << E); ++k) {
          a[(j << E) + k] = v.v[k];
          l[(j << E) + k] = w.v[k];
        }
      }
      for (int g = ph.g0; g < ph.g1; ++g) {
        const RGate& r = P.gate[g];
        if (r.grad != GR_NONE) {
          real part = dispatch_grad<R, real>(r.grad, r.k0, a, l, r.cmask);
#pragma unroll
          for (int off = 16; off; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
          if (lane == 0) atomicAdd(&gacc[g], (double)part * (double)r.coef);
        }
        apply_rgate<R, real>(r, a, mats[r.mat]);
        apply_rgate<R, real>(r, l, mats[r.mat]);
      }
#pragma unroll
      for (int j = 0; j < NU; ++j) {
        U v, w;
#pragma unroll
        for (int k = 0; k < (1 << E); ++k) {
          v.v[k] = a[(j << E) + k];
          w.v[k] = l[(j << E) + k];
        }
        tp[bu ^ ph.reg_off[j]] = v;
        tl[bu ^ ph.reg_off[j]] = w;
      }
    } else {
      dense_phase<real>(P, ph, tp, tid, T);
      dense_phase<real>(P, ph, tl, tid, T);
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < NU; ++k) {
    const uint64_t g = unit_global(P, base, tid + k * T, E) >> E;
    const uint32_t s = swz_unit(tid + k * T);
    reinterpret_cast<U*>(sp)[g] = tp[s];
    reinterpret_cast<U*>(sl)[g] = tl[s];
  }
  if (P.n_grad) {
    for (int g = tid; g < P.n_gates; g += T) {
      const int32_t slot = P.gate[g].slot;
      if (slot >= 0) atomicAdd(&grad_acc[circ * n_params + slot], gacc[g]);
    }
  }
}

template <typename real>
__global__ void init_state_kernel(cpx<real>* psi, int n, int pad, const cpx<real>* init, int64_t circ0) {
  const int64_t circ = circ0 + blockIdx.y;
  const uint64_t N = 1ull << n;
  cpx<real>* st = psi + circ * (int64_t)N;
  for (uint64_t q = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; q < N; q += (uint64_t)gridDim.x * blockDim.x) {
    cpx<real> a = mk<real>((real)0, (real)0);
    if (!init) {
      if (q == 0) a.x = (real)1;
    } else if ((q & ((1ull << pad) - 1)) == 0) {
      a = init[q >> pad];
    }
    st[q] = a;
  }
}

// ---------------------------------------------------------------- measurements

constexpr int kMeasThreads = 256;
constexpr int kMeasChunk = 4096;  // amplitudes per CTA

template <typename real>
__device__ __forceinline__ real term_value(const TermDev& t, cpx<real> v, cpx<real> u) {
  // Re((-i)^ny conj(v) u)
  const real re = recb(v, u), im = imcb(v, u);
  switch (t.ny & 3) {
    case 0: return re;
    case 1: return im;
    case 2: return -re;
    default: return -im;
  }
}

template <typename real>
__global__ void __launch_bounds__(kMeasThreads)
    expval_kernel(const __grid_constant__ TermTable TT, const cpx<real>* __restrict__ psi, int n,
                  double* __restrict__ acc, int64_t circ0) {
  __shared__ double sacc[32];
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t circ = circ0 + blockIdx.y;
  const uint64_t N = 1ull << n;
  const cpx<real>* st = psi + circ * (int64_t)N;
  const uint64_t w0 = (uint64_t)blockIdx.x * kMeasChunk;
  const uint64_t w1 = w0 + kMeasChunk < N ? w0 + kMeasChunk : N;
  for (int sg = 0; sg < TT.n; sg += 32) {
    if (tid < 32) sacc[tid] = 0.0;
    __syncthreads();
    real part[32];
#pragma unroll
    for (int s = 0; s < 32; ++s) part[s] = 0;
    for (uint64_t w = w0 + tid; w < w1; w += kMeasThreads) {
      const cpx<real> v = st[w];
      const real p = v.x * v.x + v.y * v.y;
#pragma unroll
      for (int s = 0; s < 32; ++s) {
        if (sg + s < TT.n) {
          const TermDev& t = TT.t[sg + s];
          const real sgn = (__popcll(t.z & w) & 1) ? (real)-1 : (real)1;
          if (t.x == 0) part[s] += sgn * p;
          else part[s] += sgn * term_value<real>(t, v, st[w ^ t.x]);
        }
      }
    }
#pragma unroll
    for (int s = 0; s < 32; ++s) {
      if (sg + s < TT.n) {
        real x = part[s];
#pragma unroll
        for (int off = 16; off; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
        if (lane == 0) atomicAdd(&sacc[s], (double)x);
      }
    }
    __syncthreads();
    if (tid < 32 && sg + tid < TT.n) atomicAdd(&acc[circ * TT.n + sg + tid], sacc[tid]);
    __syncthreads();
  }
}

__device__ __forceinline__ uint32_t bin_of(const ProbsDesc& d, uint64_t w) {
  uint32_t b = 0;
  for (int j = 0; j < d.nbits; ++j) b = (b << 1) | (uint32_t)((w >> d.bits[j]) & 1);
  return b;
}

template <typename real>
__global__ void __launch_bounds__(kMeasThreads)
    probs_kernel(const __grid_constant__ ProbsTable PT, const cpx<real>* __restrict__ psi, int n,
                 double* __restrict__ probs_acc, real* __restrict__ out, int n_real, int64_t circ0) {
  extern __shared__ __align__(16) unsigned char hist_raw[];
  real* hist = reinterpret_cast<real*>(hist_raw);
  const int tid = threadIdx.x;
  const int64_t circ = circ0 + blockIdx.y;
  const uint64_t N = 1ull << n;
  const cpx<real>* st = psi + circ * (int64_t)N;
  const uint64_t w0 = (uint64_t)blockIdx.x * kMeasChunk;
  const uint64_t w1 = w0 + kMeasChunk < N ? w0 + kMeasChunk : N;
  const uint64_t padm = (1ull << PT.pad_bits) - 1;
  for (int pi = 0; pi < PT.n; ++pi) {
    const ProbsDesc& d = PT.p[pi];
    if (d.full) {
      for (uint64_t w = w0 + tid; w < w1; w += kMeasThreads) {
        if (w & padm) continue;
        const cpx<real> v = st[w];
        out[circ * n_real + d.offset + (w >> PT.pad_bits)] = v.x * v.x + v.y * v.y;
      }
      continue;
    }
    const int nb = 1 << d.nbits;
    const bool smem_hist = d.nbits <= 12;
    if (smem_hist) {
      for (int i = tid; i < nb; i += kMeasThreads) hist[i] = (real)0;
      __syncthreads();
    }
    double* dst = probs_acc + circ * PT.n_bins + d.acc_off;
    for (uint64_t w = w0 + tid; w < w1; w += kMeasThreads) {
      const cpx<real> v = st[w];
      const real p = v.x * v.x + v.y * v.y;
      const uint32_t b = bin_of(d, w);
      if (smem_hist) atomicAdd(&hist[b], p);
      else atomicAdd(&dst[b], (double)p);
    }
    if (smem_hist) {
      __syncthreads();
      for (int i = tid; i < nb; i += kMeasThreads)
        if (hist[i] != (real)0) atomicAdd(&dst[i], (double)hist[i]);
      __syncthreads();
    }
  }
}

template <typename real>
__global__ void finalize_kernel(const __grid_constant__ OutTermTable O, const __grid_constant__ ProbsTable PT,
                                const double* __restrict__ term_acc, const double* __restrict__ probs_acc,
                                real* __restrict__ out, int64_t batch) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch * O.n_real) return;
  const int64_t circ = i / O.n_real;
  const int k = (int)(i % O.n_real);
  double v = 0.0;
  for (int e = 0; e < O.n; ++e)
    if (O.k[e] == k) v += O.coef[e] * term_acc[circ * O.n_terms + O.s[e]];
  for (int pi = 0; pi < PT.n; ++pi) {
    const ProbsDesc& d = PT.p[pi];
    const int nb = 1 << d.nbits;
    if (k >= d.offset && k < d.offset + nb) {
      if (d.full) return;  // written by probs_kernel
      v = probs_acc[circ * PT.n_bins + d.acc_off + (k - d.offset)];
    }
  }
  out[i] = (real)v;
}

template <typename real>
__global__ void term_weights_kernel(const __grid_constant__ OutTermTable O, const real* __restrict__ dy,
                                    double* __restrict__ w, int64_t batch) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= batch * O.n_terms) return;
  const int64_t circ = i / O.n_terms;
  const int s = (int)(i % O.n_terms);
  double v = 0.0;
  if (dy)
    for (int e = 0; e < O.n; ++e)
      if (O.s[e] == s) v += O.coef[e] * (double)dy[circ * O.n_real + O.k[e]];
  w[i] = v;
}

template <typename real>
__global__ void __launch_bounds__(256)
    lambda_init_kernel(const __grid_constant__ TermTable TT, const __grid_constant__ ProbsTable PT,
                       const double* __restrict__ wts, const real* __restrict__ dy, int n_real,
                       const cpx<real>* __restrict__ dys, const cpx<real>* __restrict__ psi, cpx<real>* __restrict__ lam,
                       int n, int64_t circ0) {
  const int64_t circ = circ0 + blockIdx.y;
  const uint64_t N = 1ull << n;
  const cpx<real>* st = psi + circ * (int64_t)N;
  const uint64_t padm = (1ull << PT.pad_bits) - 1;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < N; w += (uint64_t)gridDim.x * blockDim.x) {
    const cpx<real> v = st[w];
    real d = 0;
    cpx<real> acc = mk<real>((real)0, (real)0);
    for (int s = 0; s < TT.n; ++s) {
      const real W = (real)wts[circ * TT.n + s];
      if (W == (real)0) continue;
      const TermDev& t = TT.t[s];
      const real sgn = (__popcll(t.z & w) & 1) ? -W : W;
      if (t.x == 0) {
        d += sgn;
      } else {
        const cpx<real> u = st[w ^ t.x];
        cpx<real> pu;
        switch (t.ny & 3) {
          case 0: pu = u; break;
          case 1: pu = mk<real>(u.y, -u.x); break;
          case 2: pu = mk<real>(-u.x, -u.y); break;
          default: pu = mk<real>(-u.y, u.x); break;
        }
        acc.x += sgn * pu.x;
        acc.y += sgn * pu.y;
      }
    }
    if (dy) {
      for (int pi = 0; pi < PT.n; ++pi) {
        const ProbsDesc& pd = PT.p[pi];
        if (pd.full) {
          if ((w & padm) == 0) d += dy[circ * n_real + pd.offset + (w >> PT.pad_bits)];
        } else {
          d += dy[circ * n_real + pd.offset + bin_of(pd, w)];
        }
      }
    }
    cpx<real> r = mk<real>(d * v.x + acc.x, d * v.y + acc.y);
    if (dys) {
      const cpx<real> g = dys[circ * (int64_t)N + w];
      r.x += (real)0.5 * g.x;
      r.y += (real)0.5 * g.y;
    }
    lam[circ * (int64_t)N + w] = r;
  }
}

template <typename real>
__global__ void grad_finalize_kernel(const double* __restrict__ acc, real* __restrict__ g, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) g[i] = (real)acc[i];
}

// ---------------------------------------------------------------- launch helpers

constexpr int kMaxGridY = 65535;

template <typename K>
cudaError_t ensure_smem(K kernel, size_t bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static thread_local size_t done_bytes[64] = {0};
  if (dev < 64 && done_bytes[dev] >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess && dev < 64) done_bytes[dev] = bytes;
  return e;
}

template <typename real, int R>
cudaError_t fwd_impl(const PassParams& P, void* psi, const void* params, int n_params, const void* init,
                     int64_t batch, cudaStream_t s) {
  constexpr int E = kE<real>;
  const size_t smem = (size_t)16 << (P.m - E);
  auto kern = fwd_pass_kernel<real, R>;
  cudaError_t e = ensure_smem(kern, smem);
  if (e != cudaSuccess) return e;
  const int T = 1 << (P.m - R);
  const unsigned tiles = 1u << (P.n - P.m);
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    dim3 grid(tiles, (unsigned)nb);
    kern<<<grid, T, smem, s>>>(P, static_cast<cpx<real>*>(psi), static_cast<const real*>(params), n_params,
                               static_cast<const cpx<real>*>(init), c0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename real, int R>
cudaError_t bwd_impl(const PassParams& P, void* psi, void* lam, const void* params, int n_params,
                     double* grad_acc, int64_t batch, cudaStream_t s) {
  constexpr int E = kE<real>;
  const size_t smem = (size_t)32 << (P.m - E);
  auto kern = bwd_pass_kernel<real, R>;
  cudaError_t e = ensure_smem(kern, smem);
  if (e != cudaSuccess) return e;
  const int T = 1 << (P.m - R);
  const unsigned tiles = 1u << (P.n - P.m);
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    dim3 grid(tiles, (unsigned)nb);
    kern<<<grid, T, smem, s>>>(P, static_cast<cpx<real>*>(psi), static_cast<cpx<real>*>(lam),
                               static_cast<const real*>(params), n_params, grad_acc, c0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename real>
cudaError_t init_impl(int n, int pad, void* psi, const void* init, int64_t batch, cudaStream_t s) {
  const uint64_t N = 1ull << n;
  const unsigned bx = (unsigned)((N + 255) / 256 < 4096 ? (N + 255) / 256 : 4096);
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    init_state_kernel<real><<<dim3(bx, (unsigned)nb), 256, 0, s>>>(static_cast<cpx<real>*>(psi), n, pad,
                                                                   static_cast<const cpx<real>*>(init), c0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename real>
cudaError_t expval_impl(int n, const TermTable& TT, const void* psi, double* acc, int64_t batch, cudaStream_t s) {
  const uint64_t N = 1ull << n;
  const unsigned bx = (unsigned)((N + kMeasChunk - 1) / kMeasChunk);
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    expval_kernel<real><<<dim3(bx, (unsigned)nb), kMeasThreads, 0, s>>>(TT, static_cast<const cpx<real>*>(psi), n,
                                                                         acc, c0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename real>
cudaError_t probs_impl(int n, const ProbsTable& PT, const void* psi, double* probs_acc, void* out, int n_real,
                       int64_t batch, cudaStream_t s) {
  const uint64_t N = 1ull << n;
  const unsigned bx = (unsigned)((N + kMeasChunk - 1) / kMeasChunk);
  int maxbits = 0;
  for (int i = 0; i < PT.n; ++i)
    if (!PT.p[i].full && PT.p[i].nbits <= 12 && PT.p[i].nbits > maxbits) maxbits = PT.p[i].nbits;
  const size_t smem = sizeof(real) << maxbits;
  auto kern = probs_kernel<real>;
  cudaError_t e = ensure_smem(kern, smem);
  if (e != cudaSuccess) return e;
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    kern<<<dim3(bx, (unsigned)nb), kMeasThreads, smem, s>>>(PT, static_cast<const cpx<real>*>(psi), n, probs_acc,
                                                             static_cast<real*>(out), n_real, c0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename real>
cudaError_t lambda_impl(int n, const TermTable& TT, const ProbsTable& PT, const double* w, const void* dy,
                        int n_real, const void* dys, const void* psi, void* lam, int64_t batch, cudaStream_t s) {
  const uint64_t N = 1ull << n;
  const unsigned bx = (unsigned)((N + 255) / 256 < 8192 ? (N + 255) / 256 : 8192);
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    lambda_init_kernel<real><<<dim3(bx, (unsigned)nb), 256, 0, s>>>(
        TT, PT, w, static_cast<const real*>(dy), n_real, static_cast<const cpx<real>*>(dys),
        static_cast<const cpx<real>*>(psi), static_cast<cpx<real>*>(lam), n, c0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_fwd_pass(bool dbl, const PassParams& P, void* psi, const void* params, int n_params,
                            const void* init, int64_t batch, cudaStream_t s) {
  return dbl ? fwd_impl<double, 4>(P, psi, params, n_params, init, batch, s)
             : fwd_impl<float, 5>(P, psi, params, n_params, init, batch, s);
}

cudaError_t launch_bwd_pass(bool dbl, const PassParams& P, void* psi, void* lam, const void* params,
                            int n_params, double* grad_acc, int64_t batch, cudaStream_t s) {
  return dbl ? bwd_impl<double, 3>(P, psi, lam, params, n_params, grad_acc, batch, s)
             : bwd_impl<float, 4>(P, psi, lam, params, n_params, grad_acc, batch, s);
}

cudaError_t launch_init_state(bool dbl, int n, int pad, void* psi, const void* init, int64_t batch,
                              cudaStream_t s) {
  return dbl ? init_impl<double>(n, pad, psi, init, batch, s) : init_impl<float>(n, pad, psi, init, batch, s);
}

cudaError_t launch_expval(bool dbl, int n, const TermTable& T, const void* psi, double* term_acc, int64_t batch,
                          cudaStream_t s) {
  if (T.n == 0) return cudaSuccess;
  return dbl ? expval_impl<double>(n, T, psi, term_acc, batch, s) : expval_impl<float>(n, T, psi, term_acc, batch, s);
}

cudaError_t launch_probs(bool dbl, int n, const ProbsTable& PT, const void* psi, double* probs_acc, void* out_real,
                         int n_real, int64_t batch, cudaStream_t s) {
  if (PT.n == 0) return cudaSuccess;
  return dbl ? probs_impl<double>(n, PT, psi, probs_acc, out_real, n_real, batch, s)
             : probs_impl<float>(n, PT, psi, probs_acc, out_real, n_real, batch, s);
}

cudaError_t launch_finalize(bool dbl, const OutTermTable& O, const ProbsTable& PT, const double* term_acc,
                            const double* probs_acc, void* out_real, int64_t batch, cudaStream_t s) {
  if (O.n_real == 0 || batch == 0) return cudaSuccess;
  const int64_t total = batch * O.n_real;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  if (dbl)
    finalize_kernel<double><<<blocks, 256, 0, s>>>(O, PT, term_acc, probs_acc, static_cast<double*>(out_real), batch);
  else
    finalize_kernel<float><<<blocks, 256, 0, s>>>(O, PT, term_acc, probs_acc, static_cast<float*>(out_real), batch);
  return cudaGetLastError();
}

cudaError_t launch_term_weights(bool dbl, const OutTermTable& O, const void* dy_real, double* w, int64_t batch,
                                cudaStream_t s) {
  if (O.n_terms == 0 || batch == 0) return cudaSuccess;
  const int64_t total = batch * O.n_terms;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  if (dbl)
    term_weights_kernel<double><<<blocks, 256, 0, s>>>(O, static_cast<const double*>(dy_real), w, batch);
  else
    term_weights_kernel<float><<<blocks, 256, 0, s>>>(O, static_cast<const float*>(dy_real), w, batch);
  return cudaGetLastError();
}

cudaError_t launch_lambda_init(bool dbl, int n, const TermTable& T, const ProbsTable& PT, const double* w,
                               const void* dy_real, int n_real, const void* dy_state, const void* psi, void* lam,
                               int64_t batch, cudaStream_t s) {
  return dbl ? lambda_impl<double>(n, T, PT, w, dy_real, n_real, dy_state, psi, lam, batch, s)
             : lambda_impl<float>(n, T, PT, w, dy_real, n_real, dy_state, psi, lam, batch, s);
}

cudaError_t launch_grad_finalize(bool dbl, const double* grad_acc, void* grad, int64_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((count + 255) / 256);
  if (dbl) grad_finalize_kernel<double><<<blocks, 256, 0, s>>>(grad_acc, static_cast<double*>(grad), count);
  else grad_finalize_kernel<float><<<blocks, 256, 0, s>>>(grad_acc, static_cast<float*>(grad), count);
  return cudaGetLastError();
}

}  // namespace tedq
