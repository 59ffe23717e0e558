// sv_device.cuh -- device code of the state-vector passes, shared by the
// generic pass kernels (sv_kernels.cu) and by the per-circuit kernels that
// sv_jit.cpp generates and compiles with NVRTC at program-creation time.
//
// A pass kernel is written as
//     FwdPass<real, R> c(...);          // slots, first tile fetches
//     while (c.next()) {                // next tile of this thread group
//       c.begin(f); <gates on c.a>; c.end(f);   // one register phase
//       c.finish();                     // tile back to HBM, slot refilled
//     }
//     c.close();
// In the generic kernels the gates of a phase are dispatched at run time; in
// the generated kernels every gate is a template instance with its register
// bit and control mask as compile-time constants, so control tests fold away
// and bit flips become register renames.
//
// Self-contained: compiles under nvcc and NVRTC (no host headers).
#pragma once
#include "sv_plan.h"

namespace tedq {
namespace dev {

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
struct UnitsPerAmp;
template <>
struct UnitsPerAmp<float> {
  static constexpr int E = 1;  // log2 amplitudes per 16-byte unit
};
template <>
struct UnitsPerAmp<double> {
  static constexpr int E = 0;
};

// Compile-time control mask (generated kernels) -- converts to unsigned so the
// same gate templates accept a run-time mask (generic kernels).
template <unsigned V>
struct CM {
  __device__ __forceinline__ constexpr operator unsigned() const { return V; }
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
// Im(conj(a) b), Re(conj(a) b)
template <typename real>
__device__ __forceinline__ real imcb(cpx<real> a, cpx<real> b) {
  return a.x * b.y - a.y * b.x;
}
template <typename real>
__device__ __forceinline__ real recb(cpx<real> a, cpx<real> b) {
  return a.x * b.x + a.y * b.y;
}

// ---------------------------------------------------------------- register sets
// A thread's 2^R amplitudes of a phase.  complex128: one cpx per amplitude.
// complex64: amplitudes 2g and 2g+1 (register bit 0 is the "pair bit") are
// packed per group g as float2 (re_2g, re_2g+1) and (im_2g, im_2g+1), so one
// packed FP32x2 instruction (FFMA2) updates two amplitudes.
template <typename real, int R>
struct Regs;
template <int R>
struct Regs<double, R> {
  cpx<double> a[1 << R];
};
template <int R>
struct Regs<float, R> {
  float2 re[1 << (R - 1)], im[1 << (R - 1)];
};

// Shared-memory image of a 16-byte unit: complex64 units hold their two
// amplitudes pair-planar (re0, re1, im0, im1), complex128 units one amplitude.
template <typename real>
struct SUnit;
template <>
struct alignas(16) SUnit<float> {
  float2 re, im;
};
template <>
struct alignas(16) SUnit<double> {
  cpx<double> v;
};

__device__ __forceinline__ SUnit<float> to_s(const Unit<float>& u) {
  SUnit<float> s;
  s.re = make_float2(u.v[0].x, u.v[1].x);
  s.im = make_float2(u.v[0].y, u.v[1].y);
  return s;
}
__device__ __forceinline__ Unit<float> from_s(const SUnit<float>& s) {
  Unit<float> u;
  u.v[0] = mk<float>(s.re.x, s.im.x);
  u.v[1] = mk<float>(s.re.y, s.im.y);
  return u;
}
__device__ __forceinline__ SUnit<double> to_s(const Unit<double>& u) {
  SUnit<double> s;
  s.v = u.v[0];
  return s;
}
__device__ __forceinline__ Unit<double> from_s(const SUnit<double>& s) {
  Unit<double> u;
  u.v[0] = s.v;
  return u;
}

// Amplitude `addr` (unit << E | amplitude-in-unit) of a shared-memory image.
__device__ __forceinline__ cpx<float> amp_ld(const SUnit<float>* t, uint32_t addr) {
  const float* f = reinterpret_cast<const float*>(t + (addr >> 1));
  return mk<float>(f[addr & 1], f[2 + (addr & 1)]);
}
__device__ __forceinline__ void amp_st(SUnit<float>* t, uint32_t addr, cpx<float> v) {
  float* f = reinterpret_cast<float*>(t + (addr >> 1));
  f[addr & 1] = v.x;
  f[2 + (addr & 1)] = v.y;
}
__device__ __forceinline__ cpx<double> amp_ld(const SUnit<double>* t, uint32_t addr) { return t[addr].v; }
__device__ __forceinline__ void amp_st(SUnit<double>* t, uint32_t addr, cpx<double> v) { t[addr].v = v; }

// unit j of a register set <-> shared-memory unit
template <int R>
__device__ __forceinline__ void regs_ld(Regs<float, R>& A, int j, const SUnit<float>& s) {
  A.re[j] = s.re;
  A.im[j] = s.im;
}
template <int R>
__device__ __forceinline__ SUnit<float> regs_st(const Regs<float, R>& A, int j) {
  SUnit<float> s;
  s.re = A.re[j];
  s.im = A.im[j];
  return s;
}
template <int R>
__device__ __forceinline__ void regs_ld(Regs<double, R>& A, int j, const SUnit<double>& s) {
  A.a[j] = s.v;
}
template <int R>
__device__ __forceinline__ SUnit<double> regs_st(const Regs<double, R>& A, int j) {
  SUnit<double> s;
  s.v = A.a[j];
  return s;
}

// The same for a unit still in HBM order (complex64: re0, im0, re1, im1): the
// tile as the asynchronous copies leave it and as it goes back to HBM.
template <int R>
__device__ __forceinline__ void regs_ld_raw(Regs<float, R>& A, int j, const SUnit<float>& s) {
  A.re[j] = make_float2(s.re.x, s.im.x);
  A.im[j] = make_float2(s.re.y, s.im.y);
}
template <int R>
__device__ __forceinline__ SUnit<float> regs_st_raw(const Regs<float, R>& A, int j) {
  SUnit<float> s;
  s.re = make_float2(A.re[j].x, A.im[j].x);
  s.im = make_float2(A.re[j].y, A.im[j].y);
  return s;
}
template <int R>
__device__ __forceinline__ void regs_ld_raw(Regs<double, R>& A, int j, const SUnit<double>& s) {
  A.a[j] = s.v;
}
template <int R>
__device__ __forceinline__ SUnit<double> regs_st_raw(const Regs<double, R>& A, int j) {
  SUnit<double> s;
  s.v = A.a[j];
  return s;
}

// HBM order <-> pair-planar order of one shared-memory unit.
__device__ __forceinline__ SUnit<float> raw_to_s(const SUnit<float>& r) {
  SUnit<float> s;
  s.re = make_float2(r.re.x, r.im.x);
  s.im = make_float2(r.re.y, r.im.y);
  return s;
}
__device__ __forceinline__ SUnit<double> raw_to_s(const SUnit<double>& r) { return r; }
__device__ __forceinline__ SUnit<float> s_to_raw(const SUnit<float>& s) { return raw_to_s(s); }
__device__ __forceinline__ SUnit<double> s_to_raw(const SUnit<double>& s) { return s; }

// packed FP32x2 helpers
__device__ __forceinline__ float2 bc2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 swp(float2 a) { return make_float2(a.y, a.x); }
// a gate controlled on the pair bit changes only the odd half
__device__ __forceinline__ float2 odd_only(bool c0, float2 old, float2 nw) {
  return c0 ? make_float2(old.x, nw.y) : nw;
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

// One factor as a dense 2x2 (row-major).  Gate definitions follow the
// reference (tedq/QInterpreter/operators/qubit.py: RX :990-997, RY :1048-1055,
// RZ :1106-1112, PhaseShift :1253-1257, Rot :1169-1189).
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
// norm = false (generic kernels): normalised rotations keep their plain
// entries and run as GK_RXT / GK_RYT.
template <typename real>
__device__ void compute_mat(const PassParams& P, int i, const real* prm, cpx<real>* out, bool norm = true) {
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
  if (md.diag >= 3 && norm) {  // normalised rotation: divide by the larger of |c|, |s|
    const real c = M[0].x, sn = md.diag == 3 ? -M[1].y : -M[1].x;
    const bool f0 = fabs(c) >= fabs(sn);
    out[0] = mk<real>(f0 ? sn / c : c / sn, f0 ? (real)0 : (real)1);
    out[1] = mk<real>(f0 ? fabs(c) : fabs(sn), (real)0);
    out[2] = mk<real>((real)1, (real)0);  // running scale: norm_scan
    return;
  }
  if (md.diag == 2) {  // unit-modulus diagonal: d1 / d0 = d1 conj(d0)
    out[0] = mk<real>((real)1, (real)0);
    out[1] = cmul(M[3], cconj(M[0]));
  } else if (md.diag == 1) {
    out[0] = M[0];
    out[1] = M[3];
  } else {
    for (int k = 0; k < 4; ++k) out[k] = M[k];
  }
}

// Running scale of the normalised rotations of a pass: entry [2].x of
// normalised matrix i becomes the product of the scales of matrices 0..i
// (matrices are numbered in application order), accumulated in double by
// warp 0 with a shuffle scan.
template <typename real>
__device__ void norm_scan(const PassParams& P, cpx<real> (*mats)[4], int tid) {
  if (tid >= 32) return;
  double carry = 1.0;
  const int n = P.norm_last + 1;
  for (int base = 0; base < n; base += 32) {
    const int i = base + tid;
    const bool on = i < n && P.mat[i].diag >= 3;
    double v = on ? (double)mats[i][1].x : 1.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double u = __shfl_up_sync(0xffffffffu, v, o);
      if (tid >= o) v *= u;
    }
    v *= carry;
    if (on) mats[i][2].x = (real)v;
    carry = __shfl_sync(0xffffffffu, v, 31);
  }
}

template <typename real>
__device__ __forceinline__ real sq(real x) { return x * x; }

// ---------------------------------------------------------------- register gates
// Complex-array forms (complex128 register sets): bit k of the register index
// is register bit k.  Ctl is an unsigned run-time mask or a CM<> constant.

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_u1_c(cpx<real>* a, const cpx<real>* M, Ctl cm) {
  const cpx<real> m0 = M[0], m1 = M[1], m2 = M[2], m3 = M[3];
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    const int j = i | (1 << K);
    const cpx<real> x0 = a[i], x1 = a[j];
    a[i] = cmac2(m0, x0, m1, x1);
    a[j] = cmac2(m2, x0, m3, x1);
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_d1_c(cpx<real>* a, const cpx<real>* M, Ctl cm) {
  const cpx<real> d0 = M[0], d1 = M[1];
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    a[i] = cmul((i >> K) & 1 ? d1 : d0, a[i]);
  }
}

// RX-type [[c, -i s], [-i s, c]] (RX, or RX^dagger with s negated)
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_rxt_c(cpx<real>* a, const cpx<real>* M, Ctl cm) {
  const real c = M[0].x, sn = -M[1].y;
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    const int j = i | (1 << K);
    const cpx<real> x0 = a[i], x1 = a[j];
    a[i] = mk<real>(fma(c, x0.x, sn * x1.y), fma(c, x0.y, -sn * x1.x));
    a[j] = mk<real>(fma(c, x1.x, sn * x0.y), fma(c, x1.y, -sn * x0.x));
  }
}

// RY-type [[c, -s], [s, c]]
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_ryt_c(cpx<real>* a, const cpx<real>* M, Ctl cm) {
  const real c = M[0].x, sn = -M[1].x;
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    const int j = i | (1 << K);
    const cpx<real> x0 = a[i], x1 = a[j];
    a[i] = mk<real>(fma(c, x0.x, -sn * x1.x), fma(c, x0.y, -sn * x1.y));
    a[j] = mk<real>(fma(sn, x0.x, c * x1.x), fma(sn, x0.y, c * x1.y));
  }
}

// diag(1, d): multiply the |1> half only
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_ph_c(cpx<real>* a, const cpx<real>* M, Ctl cm) {
  const cpx<real> d = M[1];
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (!(i & (1 << K))) continue;
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    a[i] = cmul(d, a[i]);
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_x_c(cpx<real>* a, Ctl cm) {
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    const int j = i | (1 << K);
    const cpx<real> t = a[i];
    a[i] = a[j];
    a[j] = t;
  }
}

// Hadamard: (x0 + x1, x0 - x1) / sqrt(2)
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_h_c(cpx<real>* a, Ctl cm) {
  const real s = (real)0.70710678118654752440;
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    const int j = i | (1 << K);
    const cpx<real> x0 = a[i], x1 = a[j];
    a[i] = mk<real>(s * (x0.x + x1.x), s * (x0.y + x1.y));
    a[j] = mk<real>(s * (x0.x - x1.x), s * (x0.y - x1.y));
  }
}

// Normalised rotations (uncontrolled; matrix entries as for GK_RXN / GK_RYN).
// The form is the same for every thread of the CTA (one circuit): the branch
// does not diverge.
template <int K, int R, typename real>
__device__ __forceinline__ void apply_rxn_c(cpx<real>* a, const cpx<real>* M) {
  const real w = M[0].x;
  if (M[0].y == (real)0) {  // [[1, -i t], [-i t, 1]]
#pragma unroll
    for (int i = 0; i < (1 << R); ++i) {
      if (i & (1 << K)) continue;
      const int j = i | (1 << K);
      const cpx<real> x0 = a[i], x1 = a[j];
      a[i] = mk<real>(fma(w, x1.y, x0.x), fma(-w, x1.x, x0.y));
      a[j] = mk<real>(fma(w, x0.y, x1.x), fma(-w, x0.x, x1.y));
    }
  } else {  // [[i u, 1], [1, i u]]
#pragma unroll
    for (int i = 0; i < (1 << R); ++i) {
      if (i & (1 << K)) continue;
      const int j = i | (1 << K);
      const cpx<real> x0 = a[i], x1 = a[j];
      a[i] = mk<real>(fma(-w, x0.y, x1.x), fma(w, x0.x, x1.y));
      a[j] = mk<real>(fma(-w, x1.y, x0.x), fma(w, x1.x, x0.y));
    }
  }
}

template <int K, int R, typename real>
__device__ __forceinline__ void apply_ryn_c(cpx<real>* a, const cpx<real>* M) {
  const real w = M[0].x;
  if (M[0].y == (real)0) {  // [[1, -t], [t, 1]]
#pragma unroll
    for (int i = 0; i < (1 << R); ++i) {
      if (i & (1 << K)) continue;
      const int j = i | (1 << K);
      const cpx<real> x0 = a[i], x1 = a[j];
      a[i] = mk<real>(fma(-w, x1.x, x0.x), fma(-w, x1.y, x0.y));
      a[j] = mk<real>(fma(w, x0.x, x1.x), fma(w, x0.y, x1.y));
    }
  } else {  // [[u, -1], [1, u]]
#pragma unroll
    for (int i = 0; i < (1 << R); ++i) {
      if (i & (1 << K)) continue;
      const int j = i | (1 << K);
      const cpx<real> x0 = a[i], x1 = a[j];
      a[i] = mk<real>(fma(w, x0.x, -x1.x), fma(w, x0.y, -x1.y));
      a[j] = mk<real>(fma(w, x1.x, x0.x), fma(w, x1.y, x0.y));
    }
  }
}

// Per-thread part of Im <lambda| G |psi> on the control subspace
// (G = X, Y, Z or P1 = |1><1| on register bit K).
template <int G, int K, int R, typename real, typename Ctl>
__device__ __forceinline__ real grad_part_c(const cpx<real>* p, const cpx<real>* l, Ctl cm) {
  real acc = 0;
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) {
    if (i & (1 << K)) continue;
    if ((i & (unsigned)cm) != (unsigned)cm) continue;
    const int j = i | (1 << K);
    if (G == GR_X) acc += imcb(l[i], p[j]) + imcb(l[j], p[i]);
    if (G == GR_Y) acc += recb(l[j], p[i]) - recb(l[i], p[j]);
    if (G == GR_Z) acc += imcb(l[i], p[i]) - imcb(l[j], p[j]);
    if (G == GR_P1) acc += imcb(l[j], p[j]);
  }
  return acc;
}

// complex128 register sets
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_u1(Regs<double, R>& A, const cpx<double>* M, Ctl cm) {
  apply_u1_c<K, R, double>(A.a, M, cm);
}
template <int K, int R, typename real>
__device__ __forceinline__ void apply_rxn(Regs<double, R>& A, const cpx<double>* M) {
  apply_rxn_c<K, R, double>(A.a, M);
}
template <int K, int R, typename real>
__device__ __forceinline__ void apply_ryn(Regs<double, R>& A, const cpx<double>* M) {
  apply_ryn_c<K, R, double>(A.a, M);
}
template <int R>
__device__ __forceinline__ void rescale(Regs<double, R>& A, double k) {
#pragma unroll
  for (int i = 0; i < (1 << R); ++i) A.a[i] = mk<double>(k * A.a[i].x, k * A.a[i].y);
}
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_d1(Regs<double, R>& A, const cpx<double>* M, Ctl cm) {
  apply_d1_c<K, R, double>(A.a, M, cm);
}
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_rxt(Regs<double, R>& A, const cpx<double>* M, Ctl cm) {
  apply_rxt_c<K, R, double>(A.a, M, cm);
}
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_ryt(Regs<double, R>& A, const cpx<double>* M, Ctl cm) {
  apply_ryt_c<K, R, double>(A.a, M, cm);
}
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_ph(Regs<double, R>& A, const cpx<double>* M, Ctl cm) {
  apply_ph_c<K, R, double>(A.a, M, cm);
}
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_x(Regs<double, R>& A, Ctl cm) {
  apply_x_c<K, R, double>(A.a, cm);
}
template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_h(Regs<double, R>& A, Ctl cm) {
  apply_h_c<K, R, double>(A.a, cm);
}
template <int G, int K, int R, typename real, typename Ctl>
__device__ __forceinline__ double grad_part(const Regs<double, R>& p, const Regs<double, R>& l, Ctl cm) {
  return grad_part_c<G, K, R, double>(p.a, l.a, cm);
}

// complex64 register sets (packed pairs): group g holds amplitudes 2g and
// 2g+1; a gate on register bit K >= 1 pairs group g with g | 1 << (K-1) and
// runs on FP32x2 instructions; a gate on bit 0 mixes the halves of a group.
// A control on bit 0 restricts a gate to the odd halves.
#define TEDQ_GROUPS                                  \
  constexpr int NG = 1 << (R - 1);                   \
  const unsigned cg = (unsigned)cm >> 1;             \
  const bool c0 = ((unsigned)cm & 1u) != 0u;         \
  (void)c0;

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_u1(Regs<float, R>& A, const cpx<float>* M, Ctl cm) {
  TEDQ_GROUPS
  if constexpr (K == 0) {
    const cpx<float> m0 = M[0], m1 = M[1], m2 = M[2], m3 = M[3];
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if ((g & cg) != cg) continue;
      const cpx<float> x0 = mk<float>(A.re[g].x, A.im[g].x), x1 = mk<float>(A.re[g].y, A.im[g].y);
      const cpx<float> y0 = cmac2(m0, x0, m1, x1), y1 = cmac2(m2, x0, m3, x1);
      A.re[g] = make_float2(y0.x, y1.x);
      A.im[g] = make_float2(y0.y, y1.y);
    }
  } else {
    const float2 m0r = bc2(M[0].x), m0i = bc2(M[0].y), n0i = bc2(-M[0].y);
    const float2 m1r = bc2(M[1].x), m1i = bc2(M[1].y), n1i = bc2(-M[1].y);
    const float2 m2r = bc2(M[2].x), m2i = bc2(M[2].y), n2i = bc2(-M[2].y);
    const float2 m3r = bc2(M[3].x), m3i = bc2(M[3].y), n3i = bc2(-M[3].y);
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if (g & (1 << (K - 1))) continue;
      if ((g & cg) != cg) continue;
      const int h = g | (1 << (K - 1));
      const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
      float2 yr0 = mul2(m0r, xr0);
      yr0 = fma2(n0i, xi0, yr0);
      yr0 = fma2(m1r, xr1, yr0);
      yr0 = fma2(n1i, xi1, yr0);
      float2 yi0 = mul2(m0r, xi0);
      yi0 = fma2(m0i, xr0, yi0);
      yi0 = fma2(m1r, xi1, yi0);
      yi0 = fma2(m1i, xr1, yi0);
      float2 yr1 = mul2(m2r, xr0);
      yr1 = fma2(n2i, xi0, yr1);
      yr1 = fma2(m3r, xr1, yr1);
      yr1 = fma2(n3i, xi1, yr1);
      float2 yi1 = mul2(m2r, xi0);
      yi1 = fma2(m2i, xr0, yi1);
      yi1 = fma2(m3r, xi1, yi1);
      yi1 = fma2(m3i, xr1, yi1);
      A.re[g] = odd_only(c0, xr0, yr0);
      A.im[g] = odd_only(c0, xi0, yi0);
      A.re[h] = odd_only(c0, xr1, yr1);
      A.im[h] = odd_only(c0, xi1, yi1);
    }
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_d1(Regs<float, R>& A, const cpx<float>* M, Ctl cm) {
  TEDQ_GROUPS
  float2 dr0, di0, dr1, di1;  // multipliers of a group whose bit K-1 is 0 / 1
  if constexpr (K == 0) {
    dr0 = dr1 = make_float2(M[0].x, M[1].x);
    di0 = di1 = make_float2(M[0].y, M[1].y);
  } else {
    dr0 = bc2(M[0].x);
    di0 = bc2(M[0].y);
    dr1 = bc2(M[1].x);
    di1 = bc2(M[1].y);
  }
  const float2 nd0 = make_float2(-di0.x, -di0.y), nd1 = make_float2(-di1.x, -di1.y);
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    if ((g & cg) != cg) continue;
    const bool hi = K > 0 && ((g >> (K > 0 ? K - 1 : 0)) & 1);
    const float2 dr = hi ? dr1 : dr0, di = hi ? di1 : di0, nd = hi ? nd1 : nd0;
    const float2 xr = A.re[g], xi = A.im[g];
    const float2 yr = fma2(nd, xi, mul2(dr, xr));
    const float2 yi = fma2(di, xr, mul2(dr, xi));
    A.re[g] = odd_only(c0, xr, yr);
    A.im[g] = odd_only(c0, xi, yi);
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_rxt(Regs<float, R>& A, const cpx<float>* M, Ctl cm) {
  TEDQ_GROUPS
  const float2 C = bc2(M[0].x), S = bc2(-M[1].y), NS = bc2(M[1].y);
  if constexpr (K == 0) {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if ((g & cg) != cg) continue;
      const float2 xr = A.re[g], xi = A.im[g];
      A.re[g] = fma2(C, xr, mul2(S, swp(xi)));
      A.im[g] = fma2(C, xi, mul2(NS, swp(xr)));
    }
  } else {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if (g & (1 << (K - 1))) continue;
      if ((g & cg) != cg) continue;
      const int h = g | (1 << (K - 1));
      const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
      A.re[g] = odd_only(c0, xr0, fma2(C, xr0, mul2(S, xi1)));
      A.im[g] = odd_only(c0, xi0, fma2(C, xi0, mul2(NS, xr1)));
      A.re[h] = odd_only(c0, xr1, fma2(C, xr1, mul2(S, xi0)));
      A.im[h] = odd_only(c0, xi1, fma2(C, xi1, mul2(NS, xr0)));
    }
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_ryt(Regs<float, R>& A, const cpx<float>* M, Ctl cm) {
  TEDQ_GROUPS
  const float c = M[0].x, sn = -M[1].x;
  const float2 C = bc2(c), S = bc2(sn), NS = bc2(-sn);
  if constexpr (K == 0) {
    const float2 W = make_float2(-sn, sn);
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if ((g & cg) != cg) continue;
      const float2 xr = A.re[g], xi = A.im[g];
      A.re[g] = fma2(C, xr, mul2(W, swp(xr)));
      A.im[g] = fma2(C, xi, mul2(W, swp(xi)));
    }
  } else {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if (g & (1 << (K - 1))) continue;
      if ((g & cg) != cg) continue;
      const int h = g | (1 << (K - 1));
      const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
      A.re[g] = odd_only(c0, xr0, fma2(C, xr0, mul2(NS, xr1)));
      A.im[g] = odd_only(c0, xi0, fma2(C, xi0, mul2(NS, xi1)));
      A.re[h] = odd_only(c0, xr1, fma2(S, xr0, mul2(C, xr1)));
      A.im[h] = odd_only(c0, xi1, fma2(S, xi0, mul2(C, xi1)));
    }
  }
}

// Normalised rotations on packed registers: one FFMA2 per float2 component.
template <int K, int R, typename real>
__device__ __forceinline__ void apply_rxn(Regs<float, R>& A, const cpx<float>* M) {
  constexpr int NG = 1 << (R - 1);
  const float2 W = bc2(M[0].x), NW = bc2(-M[0].x);
  if (M[0].y == 0.f) {  // [[1, -i t], [-i t, 1]]
    if constexpr (K == 0) {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float2 xr = A.re[g], xi = A.im[g];
        A.re[g] = fma2(W, swp(xi), xr);
        A.im[g] = fma2(NW, swp(xr), xi);
      }
    } else {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        if (g & (1 << (K - 1))) continue;
        const int h = g | (1 << (K - 1));
        const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
        A.re[g] = fma2(W, xi1, xr0);
        A.im[g] = fma2(NW, xr1, xi0);
        A.re[h] = fma2(W, xi0, xr1);
        A.im[h] = fma2(NW, xr0, xi1);
      }
    }
  } else {  // [[i u, 1], [1, i u]]
    if constexpr (K == 0) {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        const float2 xr = A.re[g], xi = A.im[g];
        A.re[g] = fma2(NW, xi, swp(xr));
        A.im[g] = fma2(W, xr, swp(xi));
      }
    } else {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        if (g & (1 << (K - 1))) continue;
        const int h = g | (1 << (K - 1));
        const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
        A.re[g] = fma2(NW, xi0, xr1);
        A.im[g] = fma2(W, xr0, xi1);
        A.re[h] = fma2(NW, xi1, xr0);
        A.im[h] = fma2(W, xr1, xi0);
      }
    }
  }
}

template <int K, int R, typename real>
__device__ __forceinline__ void apply_ryn(Regs<float, R>& A, const cpx<float>* M) {
  constexpr int NG = 1 << (R - 1);
  const float w = M[0].x;
  const float2 W = bc2(w), NW = bc2(-w);
  if (M[0].y == 0.f) {  // [[1, -t], [t, 1]]
    if constexpr (K == 0) {
      const float2 V = make_float2(-w, w);
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        A.re[g] = fma2(V, swp(A.re[g]), A.re[g]);
        A.im[g] = fma2(V, swp(A.im[g]), A.im[g]);
      }
    } else {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        if (g & (1 << (K - 1))) continue;
        const int h = g | (1 << (K - 1));
        const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
        A.re[g] = fma2(NW, xr1, xr0);
        A.im[g] = fma2(NW, xi1, xi0);
        A.re[h] = fma2(W, xr0, xr1);
        A.im[h] = fma2(W, xi0, xi1);
      }
    }
  } else {  // [[u, -1], [1, u]]
    if constexpr (K == 0) {
      const float2 V = make_float2(-1.f, 1.f);
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        A.re[g] = fma2(V, swp(A.re[g]), mul2(W, A.re[g]));
        A.im[g] = fma2(V, swp(A.im[g]), mul2(W, A.im[g]));
      }
    } else {
#pragma unroll
      for (int g = 0; g < NG; ++g) {
        if (g & (1 << (K - 1))) continue;
        const int h = g | (1 << (K - 1));
        const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
        A.re[g] = fma2(W, xr0, make_float2(-xr1.x, -xr1.y));
        A.im[g] = fma2(W, xi0, make_float2(-xi1.x, -xi1.y));
        A.re[h] = fma2(W, xr1, xr0);
        A.im[h] = fma2(W, xi1, xi0);
      }
    }
  }
}

// Multiply a register set by the pass's scale (after its last normalised gate).
template <int R>
__device__ __forceinline__ void rescale(Regs<float, R>& A, float k) {
  const float2 K2 = bc2(k);
#pragma unroll
  for (int g = 0; g < (1 << (R - 1)); ++g) {
    A.re[g] = mul2(K2, A.re[g]);
    A.im[g] = mul2(K2, A.im[g]);
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_ph(Regs<float, R>& A, const cpx<float>* M, Ctl cm) {
  TEDQ_GROUPS
  float2 dr, di;
  if constexpr (K == 0) {
    dr = make_float2(1.f, M[1].x);
    di = make_float2(0.f, M[1].y);
  } else {
    dr = bc2(M[1].x);
    di = bc2(M[1].y);
  }
  const float2 nd = make_float2(-di.x, -di.y);
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    if (K > 0 && !((g >> (K > 0 ? K - 1 : 0)) & 1)) continue;
    if ((g & cg) != cg) continue;
    const float2 xr = A.re[g], xi = A.im[g];
    A.re[g] = odd_only(c0, xr, fma2(nd, xi, mul2(dr, xr)));
    A.im[g] = odd_only(c0, xi, fma2(di, xr, mul2(dr, xi)));
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_x(Regs<float, R>& A, Ctl cm) {
  TEDQ_GROUPS
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    if ((g & cg) != cg) continue;
    if constexpr (K == 0) {
      A.re[g] = swp(A.re[g]);
      A.im[g] = swp(A.im[g]);
    } else {
      if (g & (1 << (K - 1))) continue;
      const int h = g | (1 << (K - 1));
      const float2 r0 = A.re[g], i0 = A.im[g], r1 = A.re[h], i1 = A.im[h];
      A.re[g] = odd_only(c0, r0, r1);
      A.im[g] = odd_only(c0, i0, i1);
      A.re[h] = odd_only(c0, r1, r0);
      A.im[h] = odd_only(c0, i1, i0);
    }
  }
}

template <int K, int R, typename real, typename Ctl>
__device__ __forceinline__ void apply_h(Regs<float, R>& A, Ctl cm) {
  TEDQ_GROUPS
  const float s = 0.70710678118654752440f;
  if constexpr (K == 0) {
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if ((g & cg) != cg) continue;
      const float2 xr = A.re[g], xi = A.im[g];
      A.re[g] = make_float2(s * (xr.x + xr.y), s * (xr.x - xr.y));
      A.im[g] = make_float2(s * (xi.x + xi.y), s * (xi.x - xi.y));
    }
  } else {
    const float2 S = bc2(s), NS = bc2(-s);
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if (g & (1 << (K - 1))) continue;
      if ((g & cg) != cg) continue;
      const int h = g | (1 << (K - 1));
      const float2 xr0 = A.re[g], xi0 = A.im[g], xr1 = A.re[h], xi1 = A.im[h];
      A.re[g] = odd_only(c0, xr0, fma2(S, xr0, mul2(S, xr1)));
      A.im[g] = odd_only(c0, xi0, fma2(S, xi0, mul2(S, xi1)));
      A.re[h] = odd_only(c0, xr1, fma2(S, xr0, mul2(NS, xr1)));
      A.im[h] = odd_only(c0, xi1, fma2(S, xi0, mul2(NS, xi1)));
    }
  }
}

template <int G, int K, int R, typename real, typename Ctl>
__device__ __forceinline__ float grad_part(const Regs<float, R>& p, const Regs<float, R>& l, Ctl cm) {
  TEDQ_GROUPS
  float2 ap = make_float2(0.f, 0.f), an = make_float2(0.f, 0.f);
  if constexpr (K == 0) {
    float acc = 0.f;
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if ((g & cg) != cg) continue;
      const float2 pr = p.re[g], pi = p.im[g], lr = l.re[g], li = l.im[g];
      if (G == GR_X) acc += (lr.x * pi.y - li.x * pr.y) + (lr.y * pi.x - li.y * pr.x);
      if (G == GR_Y) acc += (lr.y * pr.x + li.y * pi.x) - (lr.x * pr.y + li.x * pi.y);
      if (G == GR_Z || G == GR_P1) {
        ap = fma2(lr, pi, ap);
        an = fma2(li, pr, an);
      }
    }
    if (G == GR_Z) acc += (ap.x - an.x) - (ap.y - an.y);
    if (G == GR_P1) acc += ap.y - an.y;
    return acc;
  } else {
    // two accumulator pairs alternate between group pairs: half-length chains
    float2 bp = make_float2(0.f, 0.f), bn = make_float2(0.f, 0.f);
    int par = 0;
#pragma unroll
    for (int g = 0; g < NG; ++g) {
      if (g & (1 << (K - 1))) continue;
      if ((g & cg) != cg) continue;
      const int h = g | (1 << (K - 1));
      float2& xp = par ? bp : ap;
      float2& xn = par ? bn : an;
      par ^= 1;
      if (G == GR_X) {
        xp = fma2(l.re[g], p.im[h], xp);
        xn = fma2(l.im[g], p.re[h], xn);
        xp = fma2(l.re[h], p.im[g], xp);
        xn = fma2(l.im[h], p.re[g], xn);
      }
      if (G == GR_Y) {
        xp = fma2(l.re[h], p.re[g], xp);
        xp = fma2(l.im[h], p.im[g], xp);
        xn = fma2(l.re[g], p.re[h], xn);
        xn = fma2(l.im[g], p.im[h], xn);
      }
      if (G == GR_Z) {
        xp = fma2(l.re[g], p.im[g], xp);
        xn = fma2(l.im[g], p.re[g], xn);
        xn = fma2(l.re[h], p.im[h], xn);
        xp = fma2(l.im[h], p.re[h], xp);
      }
      if (G == GR_P1) {
        xp = fma2(l.re[h], p.im[h], xp);
        xn = fma2(l.im[h], p.re[h], xn);
      }
    }
    const float dx = (ap.x - an.x) + (bp.x - bn.x), dy = (ap.y - an.y) + (bp.y - bn.y);
    return c0 ? dy : dx + dy;
  }
}
#undef TEDQ_GROUPS

// ---------------------------------------------------------------- run-time dispatch

template <int R, typename real, int K = 0>
__device__ __forceinline__ void dispatch_gate(int kind, int k, Regs<real, R>& a, const cpx<real>* M, unsigned cm) {
  if constexpr (K < R) {
    if (k == K) {
      switch (kind) {
        case GK_U1: apply_u1<K, R, real>(a, M, cm); break;
        case GK_D1: apply_d1<K, R, real>(a, M, cm); break;
        case GK_RXT: apply_rxt<K, R, real>(a, M, cm); break;
        case GK_RYT: apply_ryt<K, R, real>(a, M, cm); break;
        case GK_PH: apply_ph<K, R, real>(a, M, cm); break;
        case GK_H: apply_h<K, R, real>(a, cm); break;
        default: apply_x<K, R, real>(a, cm); break;
      }
    } else {
      dispatch_gate<R, real, K + 1>(kind, k, a, M, cm);
    }
  }
}

// Generic kernels: normalised rotations arrive with plain entries
// (compute_mat with norm = false) and run as RX / RY-type gates.
template <int R, typename real>
__device__ __forceinline__ void apply_rgate(const RGate& r, Regs<real, R>& a, const cpx<real>* M) {
  if (r.kind == GK_RXN || r.kind == GK_RYN) {
    dispatch_gate<R, real>(r.kind == GK_RXN ? GK_RXT : GK_RYT, r.k0, a, M, r.cmask);
  } else if (r.kind == GK_SWAP) {
    const unsigned b0 = 1u << r.k0, b1 = 1u << r.k1;
    dispatch_gate<R, real>(GK_X, r.k1, a, M, r.cmask | b0);
    dispatch_gate<R, real>(GK_X, r.k0, a, M, r.cmask | b1);
    dispatch_gate<R, real>(GK_X, r.k1, a, M, r.cmask | b0);
  } else {
    dispatch_gate<R, real>(r.kind, r.k0, a, M, r.cmask);
  }
}

template <int R, typename real, int K = 0>
__device__ __forceinline__ real dispatch_grad(int g, int k, const Regs<real, R>& p, const Regs<real, R>& l,
                                              unsigned cm) {
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

__device__ __forceinline__ uint64_t tile_base(const PassParams& P, uint32_t tile) {
  uint64_t base = 0;
  for (int k = 0; k < P.n_outer; ++k)
    if ((tile >> k) & 1) base |= 1ull << P.outer[k];
  return base;
}

template <typename real>
__device__ __forceinline__ Unit<real> load_unit(const PassParams& P, const cpx<real>* st, uint64_t g,
                                                const cpx<real>* init) {
  constexpr int E = UnitsPerAmp<real>::E;
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
__device__ void dense_phase(const PassParams& P, const Phase& ph, SUnit<real>* tile, int tid, int T) {
  constexpr int E = UnitsPerAmp<real>::E;
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
        v[r] = amp_ld(tile, addr[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      if (r < d) {
        cpx<real> acc = mk<real>((real)0, (real)0);
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          if (c < d) {
            cpx<real> m = ph.dagger ? cconj(fixed_at<real>(P, ph.dfix + c * d + r))
                                    : fixed_at<real>(P, ph.dfix + r * d + c);
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
      if (r < d) amp_st(tile, addr[r], w[r]);
  }
}

// Thread part of the staging addresses: thread-index bits map to fixed
// global-offset and shared-memory-unit contributions (tables of the pass).
__device__ __forceinline__ void thread_offsets(const PassParams& P, int tid, int ntid, uint64_t& g, uint32_t& s) {
  for (int b = 0; b < ntid; ++b)
    if ((tid >> b) & 1) {
      g |= P.gtid[b];
      s ^= P.stid[b];
    }
}

// ---------------------------------------------------------------- tile pipeline
// The pipelined variant of a specialised pass kernel is persistent: CTA b
// takes a contiguous range of the launch's tiles (tile index = circuit *
// 2^(n-m) + tile of the circuit) and runs it in G thread groups that take the
// range's tiles in turn (group k % G takes tile k).  Tile k lives in slot
// k % (G + 1).  When a group has written tile k back to HBM it issues the
// asynchronous copies (cp.async, 16 bytes a thread) of tile k + G + 1 into the
// slot it just freed, so HBM reads run while the groups compute; the copies
// arrive on the slot's mbarrier, which the group owning the tile waits on.
// Groups synchronise with their own named barrier and never wait on each
// other except through the slot mbarriers, so one group's shared-memory
// transitions overlap the other's arithmetic.  The matrices are built once
// per circuit and group; adjoint gradient partials are summed per warp in
// FP32 over at most 8 tiles, folded into per-gate FP64 sums and added to HBM
// once per circuit and group.  All-zero tiles of a forward sweep from
// |0...0> (PassParams::zero_outer) are skipped.

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}

// One bounded wait step: the thread is suspended until the mbarrier phase of
// the given parity completes or about a microsecond has passed.
__device__ __forceinline__ bool mbar_try(uint64_t* b, unsigned parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(smem_addr(b)), "r"(parity), "r"(1000u)
      : "memory");
  return done != 0;
}

// Waits for the completion of the mbarrier phase of the given parity; gives
// up after 2^20 steps (about a second) and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity) {
  for (uint32_t i = 0; i < (1u << 20); ++i)
    if (mbar_try(b, parity)) return true;
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_addr(b)) : "memory");
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}

// The mbarrier counts one arrival of this thread once all its earlier
// cp.async copies have landed.
__device__ __forceinline__ void cp_async_arrive(uint64_t* b) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_addr(b)) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void group_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

template <typename real>
__device__ __forceinline__ Unit<real> nan_unit() {
  Unit<real> v;
  const real q = (real)__int_as_float(0x7fc00000);
#pragma unroll
  for (int k = 0; k < (1 << UnitsPerAmp<real>::E); ++k) v.v[k] = mk<real>(q, q);
  return v;
}

// Tile bookkeeping shared by the forward and the adjoint pass.
template <typename real, int R, bool ADJ>
struct Pipe {
  using C = cpx<real>;
  using U = Unit<real>;
  using S = SUnit<real>;
  static constexpr int E = UnitsPerAmp<real>::E;
  static constexpr int NR = 1 << R;
  static constexpr int NU = NR >> E;
  const PassParams& P;
  S* slots;
  uint32_t su;     // units per slot
  uint32_t half;   // adjoint: offset of lambda inside a slot (units)
  S* tile;         // slot of the current tile
  C (*mats)[4];    // this group's matrices
  uint64_t* mbar;  // one per slot
  C* psi;
  C* lam;
  const real* params;
  int n_params;
  int G, g, T, tid, bar, nslots;
  int64_t t0, cnt, k, circ;
  C* st;           // current circuit's psi
  C* sl;           // current circuit's lambda
  bool ok;         // false once a slot wait gave up (outputs become NaN)
  bool norm;

  __device__ __forceinline__ Pipe(const PassParams& P_, unsigned char* smem, C* psi_, C* lam_, const real* params_,
                                  int n_params_, int64_t n_tiles, bool norm_)
      : P(P_), psi(psi_), lam(lam_), params(params_), n_params(n_params_), norm(norm_) {
    T = 1 << (P.m - R);
    G = (int)blockDim.x / T;
    g = (int)threadIdx.x / T;
    tid = (int)threadIdx.x - g * T;
    bar = 1 + g;
    nslots = pipe_slots(P, G);
    const PipeLayout L = pipe_layout(P, G, ADJ);
    slots = reinterpret_cast<S*>(smem);
    su = L.slot_bytes >> 4;
    half = su >> 1;
    const int nm = P.n_mats > 0 ? P.n_mats : 1;
    mats = reinterpret_cast<C(*)[4]>(smem + L.mats_off) + g * nm;
    mbar = reinterpret_cast<uint64_t*>(smem + L.mbar_off);
    const int64_t per = n_tiles / gridDim.x, rem = n_tiles % gridDim.x, b = blockIdx.x;
    t0 = b * per + (b < rem ? b : rem);
    cnt = per + (b < rem ? 1 : 0);
    if (threadIdx.x == 0)
      for (int s = 0; s < nslots; ++s) mbar_init(&mbar[s], (unsigned)T);
    k = g - G;
    circ = -1;
    ok = true;
    tile = slots;
    st = sl = nullptr;
  }

  // First tiles: tile j < nslots is fetched by group (j + G - 1) % G, the
  // group that fetches every later tile of its slot.  Call after the CTA
  // barrier that publishes the mbarrier initialisation.
  __device__ __forceinline__ void start(const C* init) {
    for (int j = 0; j < nslots && j < cnt; ++j)
      if ((j + G - 1) % G == g) fetch(j, init);
  }

  __device__ __forceinline__ void fetch(int64_t kk, const C* init) {
    const int s = (int)(kk % nslots);
    S* dst = slots + (size_t)s * su;
    const int64_t gt = t0 + kk;
    const int64_t c = gt >> (P.n - P.m);
    const uint32_t tic = (uint32_t)(gt & ((1ll << (P.n - P.m)) - 1));
    // staging offsets are recomputed per tile (not kept in registers across
    // the register phases)
    const uint64_t tb = tile_base(P, tic);
    if (tb & P.zero_outer) {  // all-zero tile: nothing to copy
      mbar_arrive(&mbar[s]);
      return;
    }
    uint64_t gth = 0;
    uint32_t sthr = 0;
    thread_offsets(P, tid, P.m - R, gth, sthr);
    const uint64_t gb = tb | gth;
    const C* src = psi + (c << P.n);
    if (ADJ || P.init == 0) {
#pragma unroll
      for (int q = 0; q < NU; ++q) cp_async16(dst + (sthr ^ P.sk[q]), reinterpret_cast<const U*>(src) + ((gb | P.gk[q]) >> E));
      if (ADJ) {
        const C* srl = lam + (c << P.n);
#pragma unroll
        for (int q = 0; q < NU; ++q)
          cp_async16(dst + half + (sthr ^ P.sk[q]), reinterpret_cast<const U*>(srl) + ((gb | P.gk[q]) >> E));
      }
      cp_async_arrive(&mbar[s]);
    } else {
#pragma unroll
      for (int q = 0; q < NU; ++q)
        *reinterpret_cast<U*>(dst + (sthr ^ P.sk[q])) = load_unit<real>(P, src, gb | P.gk[q], init);
      mbar_arrive(&mbar[s]);
    }
  }

  // Next tile of this group (slot not yet waited for): on a new circuit the
  // caller rebuilds the matrices (returns 2) -- while the tile may still be
  // arriving -- else returns 1; 0 = no tile left.
  __device__ __forceinline__ int advance() {
    k += G;
    if (k >= cnt) return 0;
    tile = slots + (size_t)(k % nslots) * su;
    const int64_t gt = t0 + k;
    const int64_t c = gt >> (P.n - P.m);
    if (c == circ) return 1;
    circ = c;
    st = psi + (c << P.n);
    if (ADJ) sl = lam + (c << P.n);
    return 2;
  }

  // The current tile is all zero (forward sweep from |0...0>, qubits not yet
  // touched): it stays zero and is neither computed nor written.
  __device__ __forceinline__ bool zero_tile() const {
    return (tile_base(P, (uint32_t)((t0 + k) & ((1ll << (P.n - P.m)) - 1))) & P.zero_outer) != 0;
  }

  // Releases a zero tile's slot: its (copy-free) phase must complete before
  // the slot is refilled.
  __device__ __forceinline__ void skip(const C* init) {
    arrive_wait();
    const int64_t kk = k + nslots;
    if (kk < cnt) fetch(kk, init);
  }

  // Waits for the current tile's copies.
  __device__ __forceinline__ void arrive_wait() {
    if (ok && !mbar_wait(&mbar[k % nslots], (unsigned)((k / nslots) & 1))) ok = false;
  }

  // Matrices of the current circuit (the previous tile's last group barrier
  // guarantees no thread of the group still reads the old ones).
  __device__ __forceinline__ void build_mats() {
    const real* prm = params ? params + circ * n_params : nullptr;
    for (int i = tid; i < P.n_mats; i += T) compute_mat<real>(P, i, prm, mats[i], norm);
    group_sync(bar, T);
    if (norm && P.norm_last != kNoNorm) {
      norm_scan<real>(P, mats, tid);
      group_sync(bar, T);
    }
  }

  // Converts the current tile between HBM order and pair-planar order (needed
  // around a dense phase that opens or closes a pass), then syncs the group.
  __device__ __forceinline__ void convert(bool to_planar) {
    for (uint32_t u = (uint32_t)tid; u < su; u += (uint32_t)T) tile[u] = to_planar ? raw_to_s(tile[u]) : s_to_raw(tile[u]);
    group_sync(bar, T);
  }

  // Writes the current tile back and refills its slot with tile k + nslots
  // (pipelined launches: the slot's next tile, k + G + 1).
  __device__ __forceinline__ void write_back(const C* init) {
    uint64_t gthr = 0;
    uint32_t sthr = 0;
    thread_offsets(P, tid, P.m - R, gthr, sthr);
    gthr |= tile_base(P, (uint32_t)((t0 + k) & ((1ll << (P.n - P.m)) - 1)));
    U* gp = reinterpret_cast<U*>(st);
#pragma unroll
    for (int q = 0; q < NU; ++q) {
      U v = *reinterpret_cast<const U*>(tile + (sthr ^ P.sk[q]));
      if (!ok) v = nan_unit<real>();
      gp[(gthr | P.gk[q]) >> E] = v;
    }
    if (ADJ) {
      U* gl = reinterpret_cast<U*>(sl);
#pragma unroll
      for (int q = 0; q < NU; ++q) {
        U v = *reinterpret_cast<const U*>(tile + half + (sthr ^ P.sk[q]));
        if (!ok) v = nan_unit<real>();
        gl[(gthr | P.gk[q]) >> E] = v;
      }
    }
    group_sync(bar, T);
    const int64_t kk = k + nslots;
    if (kk < cnt) fetch(kk, init);
  }
};

// ---------------------------------------------------------------- forward pass

template <typename real, int R>
struct FwdPass {
  using C = cpx<real>;
  using S = SUnit<real>;
  static constexpr int E = UnitsPerAmp<real>::E;
  static constexpr int NR = 1 << R;
  static constexpr int NU = NR >> E;
  Pipe<real, R, false> p;
  const C* init;
  C (*mats)[4];
  int64_t mats_circ;  // circuit whose matrices are built (-1: none)
  uint32_t bu;
  Regs<real, R> a;

  __device__ __forceinline__ FwdPass(const PassParams& P_, unsigned char* smem, C* psi, const real* params,
                                     int n_params, const C* init_, int64_t n_tiles, bool norm = true)
      : p(P_, smem, psi, nullptr, params, n_params, n_tiles, norm), init(init_), mats_circ(-1) {
    mats = p.mats;
    __syncthreads();
    p.start(init);
  }

  // next tile of this thread's group (false: none left); all-zero tiles are
  // skipped, the matrices built for the circuit of the first one computed
  __device__ __forceinline__ bool next() {
    for (;;) {
      if (!p.advance()) return false;
      if (p.P.zero_outer && p.zero_tile()) {
        p.skip(init);
        continue;
      }
      if (p.circ != mats_circ) {
        p.build_mats();
        mats_circ = p.circ;
      }
      p.arrive_wait();
      return true;
    }
  }

  // Register phases read the tile in pair-planar order, except the first,
  // which reads it as the copies left it (HBM order); the last writes it back
  // in HBM order.
  __device__ __forceinline__ void load(int f, bool raw) {
    const Phase& ph = p.P.phase[f];
    bu = 0;
    for (int b = 0; b < ph.ntid; ++b)
      if ((p.tid >> b) & 1) bu ^= ph.tid_off[b];
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      if (raw) regs_ld_raw(a, j, p.tile[bu ^ ph.reg_off[j]]);
      else regs_ld(a, j, p.tile[bu ^ ph.reg_off[j]]);
    }
  }

  __device__ __forceinline__ void store(int f, bool raw) {
    const Phase& ph = p.P.phase[f];
#pragma unroll
    for (int j = 0; j < NU; ++j) p.tile[bu ^ ph.reg_off[j]] = raw ? regs_st_raw(a, j) : regs_st(a, j);
  }

  __device__ __forceinline__ void begin(int f) { load(f, false); }
  __device__ __forceinline__ void begin_first(int f) { load(f, true); }

  __device__ __forceinline__ void end(int f) {
    store(f, false);
    group_sync(p.bar, p.T);
  }

  __device__ __forceinline__ void end_last(int f) {
    store(f, true);
    group_sync(p.bar, p.T);
  }

  // end of a phase whose successor is warp-local (Phase::wlocal)
  __device__ __forceinline__ void end_w(int f) {
    store(f, false);
    __syncwarp();
  }

  // dense phases work in pair-planar order: to_planar() before one that opens
  // the pass, to_raw() after one that closes it
  __device__ __forceinline__ void dense(int f) {
    dense_phase<real>(p.P, p.P.phase[f], p.tile, p.tid, p.T);
    group_sync(p.bar, p.T);
  }
  __device__ __forceinline__ void to_planar() { p.convert(true); }
  __device__ __forceinline__ void to_raw() { p.convert(false); }

  __device__ __forceinline__ void finish() { p.write_back(init); }

  __device__ __forceinline__ void close() { cp_async_wait_all(); }
};

// ---------------------------------------------------------------- adjoint pass

template <typename real, int R>
struct BwdPass {
  using C = cpx<real>;
  using S = SUnit<real>;
  static constexpr int E = UnitsPerAmp<real>::E;
  static constexpr int NR = 1 << R;
  static constexpr int NU = NR >> E;
  Pipe<real, R, true> p;
  C (*mats)[4];
  real* gacc;     // this group's per-warp gradient partials [warp][gate] (a few tiles)
  double* gsum;   // this group's FP64 gradient sums [gate] of the current circuit
  double* grad_acc;
  int ng;
  int since_fold;  // tiles whose partials are still in gacc
  uint32_t bu;
  Regs<real, R> a;
  Regs<real, R> l;

  // tiles a warp's partials stay in the state's precision before they are
  // folded into the FP64 sums
  static constexpr int kFoldTiles = 8;

  __device__ __forceinline__ BwdPass(const PassParams& P_, unsigned char* smem, C* psi, C* lam,
                                     const real* params, int n_params, double* grad_acc_, int64_t n_tiles,
                                     bool norm = true)
      : p(P_, smem, psi, lam, params, n_params, n_tiles, norm), grad_acc(grad_acc_) {
    mats = p.mats;
    ng = p.P.n_gates > 0 ? p.P.n_gates : 1;
    since_fold = 0;
    const int W = p.T >= 32 ? p.T / 32 : 1;
    const PipeLayout L = pipe_layout(p.P, p.G, true);
    gsum = reinterpret_cast<double*>(smem + L.gacc_off) + (size_t)p.g * ng;
    gacc = reinterpret_cast<real*>(smem + L.gacc_off + (size_t)p.G * ng * 8) + (size_t)p.g * W * ng;
    for (int i = p.tid; i < W * ng; i += p.T) gacc[i] = (real)0;
    for (int i = p.tid; i < ng; i += p.T) gsum[i] = 0.0;
    __syncthreads();
    p.start(nullptr);
  }

  // Folds the warps' partials into the FP64 sums.  Thread t owns gates
  // t, t + T, ...; called where every warp of the group has passed a group
  // barrier since its last partial and before the next tile's partials.
  __device__ __forceinline__ void fold() {
    const int W = p.T >= 32 ? p.T / 32 : 1;
    for (int gi = p.tid; gi < p.P.n_gates; gi += p.T) {
      double sum = 0.0;
      for (int w = 0; w < W; ++w) {
        sum += (double)gacc[w * ng + gi];
        gacc[w * ng + gi] = (real)0;
      }
      gsum[gi] += sum;
    }
    since_fold = 0;
  }

  // Adds this group's gradient sums of the current circuit to HBM and clears
  // them (one FP64 atomic per gate and group).
  __device__ __forceinline__ void flush() {
    fold();
    for (int gi = p.tid; gi < p.P.n_gates; gi += p.T) {
      const double sum = gsum[gi];
      gsum[gi] = 0.0;
      const int32_t slot = p.P.gate[gi].slot;
      if (slot >= 0 && sum != 0.0)
        atomicAdd(&grad_acc[p.circ * p.n_params + slot], sum * (double)p.P.gate[gi].coef);
    }
  }

  __device__ __forceinline__ bool next() {
    const int64_t prev = p.circ;
    const int r = p.advance();
    if (r == 0) return false;
    if (r == 2) {
      if (prev >= 0 && p.P.n_grad) {
        const int64_t c = p.circ;
        p.circ = prev;
        flush();
        p.circ = c;
      }
      p.build_mats();
    }
    p.arrive_wait();
    return true;
  }

  // tile orders as in FwdPass
  __device__ __forceinline__ void load(int f, bool raw) {
    const Phase& ph = p.P.phase[f];
    bu = 0;
    for (int b = 0; b < ph.ntid; ++b)
      if ((p.tid >> b) & 1) bu ^= ph.tid_off[b];
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      if (raw) {
        regs_ld_raw(a, j, p.tile[bu ^ ph.reg_off[j]]);
        regs_ld_raw(l, j, p.tile[p.half + (bu ^ ph.reg_off[j])]);
      } else {
        regs_ld(a, j, p.tile[bu ^ ph.reg_off[j]]);
        regs_ld(l, j, p.tile[p.half + (bu ^ ph.reg_off[j])]);
      }
    }
  }

  __device__ __forceinline__ void store(int f, bool raw) {
    const Phase& ph = p.P.phase[f];
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      p.tile[bu ^ ph.reg_off[j]] = raw ? regs_st_raw(a, j) : regs_st(a, j);
      p.tile[p.half + (bu ^ ph.reg_off[j])] = raw ? regs_st_raw(l, j) : regs_st(l, j);
    }
  }

  __device__ __forceinline__ void begin(int f) { load(f, false); }
  __device__ __forceinline__ void begin_first(int f) { load(f, true); }

  __device__ __forceinline__ void end(int f) {
    store(f, false);
    group_sync(p.bar, p.T);
  }

  __device__ __forceinline__ void end_last(int f) {
    store(f, true);
    group_sync(p.bar, p.T);
  }

  // end of a phase whose successor is warp-local (Phase::wlocal)
  __device__ __forceinline__ void end_w(int f) {
    store(f, false);
    __syncwarp();
  }

  // Warp-reduce one gate's partial gradient into this warp's sum of gate g
  // (each sum is updated by one lane of one warp: no atomics).
  __device__ __forceinline__ void grad(int g, real part) {
#pragma unroll
    for (int off = 16; off; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((p.tid & 31) == 0) gacc[(p.tid >> 5) * ng + g] += part;
  }

  // Eight gates at once: a transposed butterfly leaves the warp sum of value
  // j on lanes 4j..4j+3 after 9 shuffles (instead of 8 x 5); gate index < 0
  // marks an unused value.
  __device__ __forceinline__ void grad8(real v0, real v1, real v2, real v3, real v4, real v5, real v6, real v7,
                                        int g0, int g1, int g2, int g3, int g4, int g5, int g6, int g7) {
    const unsigned lane = p.tid & 31;
    real v[8] = {v0, v1, v2, v3, v4, v5, v6, v7};
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const real send = b4 ? v[j] : v[j + 4];
      const real keep = b4 ? v[j + 4] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const real send = b3 ? v[j] : v[j + 2];
      const real keep = b3 ? v[j + 2] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    {
      const real send = b2 ? v[0] : v[1];
      const real keep = b2 ? v[1] : v[0];
      v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
    if ((lane & 3) == 0) {
      const int which = (b4 ? 4 : 0) + (b3 ? 2 : 0) + (b2 ? 1 : 0);
      const int gs[8] = {g0, g1, g2, g3, g4, g5, g6, g7};
      int g = gs[0];
#pragma unroll
      for (int j = 1; j < 8; ++j)
        if (which == j) g = gs[j];
      if (g >= 0) gacc[(p.tid >> 5) * ng + g] += v[0];
    }
  }

  __device__ __forceinline__ void dense(int f) {
    dense_phase<real>(p.P, p.P.phase[f], p.tile, p.tid, p.T);
    dense_phase<real>(p.P, p.P.phase[f], p.tile + p.half, p.tid, p.T);
    group_sync(p.bar, p.T);
  }
  __device__ __forceinline__ void to_planar() { p.convert(true); }
  __device__ __forceinline__ void to_raw() { p.convert(false); }

  // the last phase ended with a group barrier: the partials may be folded
  __device__ __forceinline__ void finish() {
    if (p.P.n_grad && ++since_fold == kFoldTiles) fold();
    p.write_back(nullptr);
  }

  __device__ __forceinline__ void close() {
    if (p.circ >= 0 && p.P.n_grad) flush();
    cp_async_wait_all();
  }
};

// ---------------------------------------------------------------- one tile per CTA
// The launch variant without the tile pipeline: CTA b owns tile b (tile index
// = circuit * 2^(n-m) + tile of the circuit), stages it from HBM through
// registers into shared memory (converting to pair-planar order), builds the
// pass matrices while its loads are in flight, runs the register phases and
// writes the tile back.  Passes with many gates run faster this way (their
// long unrolled phase code is shared by fewer instruction streams per SM).
// The interface matches FwdPass / BwdPass: next() yields the CTA's one tile.

template <typename real, int R>
struct FwdTile {
  using C = cpx<real>;
  using U = Unit<real>;
  using S = SUnit<real>;
  static constexpr int E = UnitsPerAmp<real>::E;
  static constexpr int NR = 1 << R;
  static constexpr int NU = NR >> E;
  const PassParams& P;
  S* tile;
  C (*mats)[4];
  C* st;
  int tid;
  uint64_t gthr;
  uint32_t sthr;
  uint32_t bu;
  Regs<real, R> a;

  bool first;

  __device__ __forceinline__ FwdTile(const PassParams& P_, S* tile_, C (*mats_)[4], C* psi, const real* params,
                                     int n_params, const C* init, int64_t n_tiles, bool norm = true)
      : P(P_), tile(tile_), mats(mats_), first(true) {
    (void)n_tiles;
    tid = threadIdx.x;
    const int T = blockDim.x;
    const int64_t circ = (int64_t)(blockIdx.x >> (P.n - P.m));
    st = psi + (circ << P.n);
    const real* prm = params ? params + circ * n_params : nullptr;
    gthr = tile_base(P, blockIdx.x & ((1u << (P.n - P.m)) - 1));
    // an all-zero tile (untouched qubits set, forward sweep from |0...0>)
    // stays zero: nothing to read, compute or write
    if (gthr & P.zero_outer) {
      first = false;
      return;
    }
    sthr = 0;
    thread_offsets(P, tid, P.m - R, gthr, sthr);
    U v[NU];
#pragma unroll
    for (int k = 0; k < NU; ++k) v[k] = load_unit<real>(P, st, gthr | P.gk[k], init);
    // matrices while the tile loads are in flight
    for (int i = tid; i < P.n_mats; i += T) compute_mat<real>(P, i, prm, mats[i], norm);
    if (norm && P.norm_last != kNoNorm) {
      __syncthreads();
      norm_scan<real>(P, mats, tid);
    }
#pragma unroll
    for (int k = 0; k < NU; ++k) tile[sthr ^ P.sk[k]] = to_s(v[k]);
    __syncthreads();
  }

  __device__ __forceinline__ void begin(int f) {
    const Phase& ph = P.phase[f];
    bu = 0;
    for (int b = 0; b < ph.ntid; ++b)
      if ((tid >> b) & 1) bu ^= ph.tid_off[b];
#pragma unroll
    for (int j = 0; j < NU; ++j) regs_ld(a, j, tile[bu ^ ph.reg_off[j]]);
  }

  __device__ __forceinline__ void end(int f) {
    const Phase& ph = P.phase[f];
#pragma unroll
    for (int j = 0; j < NU; ++j) tile[bu ^ ph.reg_off[j]] = regs_st(a, j);
    __syncthreads();
  }

  // end of a phase whose successor is warp-local (Phase::wlocal)
  __device__ __forceinline__ void end_w(int f) {
    const Phase& ph = P.phase[f];
#pragma unroll
    for (int j = 0; j < NU; ++j) tile[bu ^ ph.reg_off[j]] = regs_st(a, j);
    __syncwarp();
  }

  __device__ __forceinline__ void dense(int f) {
    dense_phase<real>(P, P.phase[f], tile, tid, blockDim.x);
    __syncthreads();
  }


  // the CTA's one tile
  __device__ __forceinline__ bool next() {
    const bool r = first;
    first = false;
    return r;
  }
  // the tile is staged in pair-planar order: the first and last register
  // phases need no conversion, nor do dense phases
  __device__ __forceinline__ void begin_first(int f) { begin(f); }
  __device__ __forceinline__ void end_last(int f) { end(f); }
  __device__ __forceinline__ void to_planar() {}
  __device__ __forceinline__ void to_raw() {}
  __device__ __forceinline__ void close() {}

  __device__ __forceinline__ void finish() {
    U* gst = reinterpret_cast<U*>(st);
#pragma unroll
    for (int k = 0; k < NU; ++k) gst[(gthr | P.gk[k]) >> E] = from_s(tile[sthr ^ P.sk[k]]);
  }
};

// ---------------------------------------------------------------- adjoint pass

template <typename real, int R>
struct BwdTile {
  using C = cpx<real>;
  using U = Unit<real>;
  using S = SUnit<real>;
  static constexpr int E = UnitsPerAmp<real>::E;
  static constexpr int NR = 1 << R;
  static constexpr int NU = NR >> E;
  const PassParams& P;
  S* tp;
  S* tl;
  C (*mats)[4];
  real* gacc;  // per-warp gradient partials (the warp sums, in the state's precision)
  C* sp;
  C* sl;
  double* grad_acc;
  int64_t circ;
  int n_params;
  int tid;
  uint64_t gthr;
  uint32_t sthr;
  uint32_t bu;
  Regs<real, R> a;
  Regs<real, R> l;

  bool first;

  __device__ __forceinline__ BwdTile(const PassParams& P_, S* smem, C (*mats_)[4], real* gacc_, C* psi, C* lam,
                                     const real* params, int n_params_, double* grad_acc_, int64_t n_tiles,
                                     bool norm = true)
      : P(P_), mats(mats_), gacc(gacc_), grad_acc(grad_acc_), n_params(n_params_), first(true) {
    (void)n_tiles;
    tid = threadIdx.x;
    const int T = blockDim.x;
    tp = smem;
    tl = smem + (1 << (P.m - E));
    circ = (int64_t)(blockIdx.x >> (P.n - P.m));
    sp = psi + (circ << P.n);
    sl = lam + (circ << P.n);
    const real* prm = params ? params + circ * n_params : nullptr;
    for (int i = tid; i < P.n_mats; i += T) compute_mat<real>(P, i, prm, mats[i], norm);
    if (norm && P.norm_last != kNoNorm) {
      __syncthreads();
      norm_scan<real>(P, mats, tid);
    }
    gthr = tile_base(P, blockIdx.x & ((1u << (P.n - P.m)) - 1));
    sthr = 0;
    thread_offsets(P, tid, P.m - R, gthr, sthr);
    U v[NU], w[NU];
#pragma unroll
    for (int k = 0; k < NU; ++k) {
      const uint64_t g = (gthr | P.gk[k]) >> E;
      v[k] = reinterpret_cast<const U*>(sp)[g];
      w[k] = reinterpret_cast<const U*>(sl)[g];
    }
#pragma unroll
    for (int k = 0; k < NU; ++k) {
      tp[sthr ^ P.sk[k]] = to_s(v[k]);
      tl[sthr ^ P.sk[k]] = to_s(w[k]);
    }
    __syncthreads();
  }

  __device__ __forceinline__ void begin(int f) {
    const Phase& ph = P.phase[f];
    bu = 0;
    for (int b = 0; b < ph.ntid; ++b)
      if ((tid >> b) & 1) bu ^= ph.tid_off[b];
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      regs_ld(a, j, tp[bu ^ ph.reg_off[j]]);
      regs_ld(l, j, tl[bu ^ ph.reg_off[j]]);
    }
  }

  __device__ __forceinline__ void end(int f) {
    const Phase& ph = P.phase[f];
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      tp[bu ^ ph.reg_off[j]] = regs_st(a, j);
      tl[bu ^ ph.reg_off[j]] = regs_st(l, j);
    }
    __syncthreads();
  }

  // end of a phase whose successor is warp-local (Phase::wlocal)
  __device__ __forceinline__ void end_w(int f) {
    const Phase& ph = P.phase[f];
#pragma unroll
    for (int j = 0; j < NU; ++j) {
      tp[bu ^ ph.reg_off[j]] = regs_st(a, j);
      tl[bu ^ ph.reg_off[j]] = regs_st(l, j);
    }
    __syncwarp();
  }

  // Warp-reduce one gate's partial gradient into this warp's slot of gate g
  // (each slot is written by one lane of one warp: no atomics).
  __device__ __forceinline__ void grad(int g, real part) {
#pragma unroll
    for (int off = 16; off; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((tid & 31) == 0) gacc[(tid >> 5) * kMaxPassGates + g] = part;
  }

  // Eight gates at once: a transposed butterfly leaves the warp sum of value
  // j on lanes 4j..4j+3 after 9 shuffles (instead of 8 x 5); gate index < 0
  // marks an unused value.
  __device__ __forceinline__ void grad8(real v0, real v1, real v2, real v3, real v4, real v5, real v6, real v7,
                                        int g0, int g1, int g2, int g3, int g4, int g5, int g6, int g7) {
    const unsigned lane = tid & 31;
    real v[8] = {v0, v1, v2, v3, v4, v5, v6, v7};
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const real send = b4 ? v[j] : v[j + 4];
      const real keep = b4 ? v[j + 4] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const real send = b3 ? v[j] : v[j + 2];
      const real keep = b3 ? v[j + 2] : v[j];
      v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    {
      const real send = b2 ? v[0] : v[1];
      const real keep = b2 ? v[1] : v[0];
      v[0] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 2);
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
    if ((lane & 3) == 0) {
      const int which = (b4 ? 4 : 0) + (b3 ? 2 : 0) + (b2 ? 1 : 0);
      const int gs[8] = {g0, g1, g2, g3, g4, g5, g6, g7};
      int g = gs[0];
#pragma unroll
      for (int j = 1; j < 8; ++j)
        if (which == j) g = gs[j];
      if (g >= 0) gacc[(tid >> 5) * kMaxPassGates + g] = v[0];
    }
  }

  __device__ __forceinline__ void dense(int f) {
    dense_phase<real>(P, P.phase[f], tp, tid, blockDim.x);
    dense_phase<real>(P, P.phase[f], tl, tid, blockDim.x);
    __syncthreads();
  }


  // the CTA's one tile
  __device__ __forceinline__ bool next() {
    const bool r = first;
    first = false;
    return r;
  }
  // the tile is staged in pair-planar order: the first and last register
  // phases need no conversion, nor do dense phases
  __device__ __forceinline__ void begin_first(int f) { begin(f); }
  __device__ __forceinline__ void end_last(int f) { end(f); }
  __device__ __forceinline__ void to_planar() {}
  __device__ __forceinline__ void to_raw() {}
  __device__ __forceinline__ void close() {}

  __device__ __forceinline__ void finish() {
#pragma unroll
    for (int k = 0; k < NU; ++k) {
      const uint64_t g = (gthr | P.gk[k]) >> E;
      reinterpret_cast<U*>(sp)[g] = from_s(tp[sthr ^ P.sk[k]]);
      reinterpret_cast<U*>(sl)[g] = from_s(tl[sthr ^ P.sk[k]]);
    }
    if (P.n_grad) {
      __syncthreads();
      const int nw = blockDim.x >> 5;
      for (int g = tid; g < P.n_gates; g += blockDim.x) {
        const int32_t slot = P.gate[g].slot;
        if (slot < 0) continue;
        double sum = 0.0;
        for (int w = 0; w < nw; ++w) sum += (double)gacc[w * kMaxPassGates + g];
        atomicAdd(&grad_acc[circ * n_params + slot], sum * (double)P.gate[g].coef);
      }
    }
  }
};

}  // namespace dev
}  // namespace tedq

// Kernel prologues shared by the generic and the generated pass kernels.
// Generic (interpreted) kernels: plain matrices for the normalised rotations.
// One tile per CTA (FwdTile / BwdTile): matrices and gradient slots in static
// shared memory, the tile in dynamic shared memory.
#define TEDQ_FWD_TILE_PROLOGUE_IMPL(REAL, RB, NORM)                                                     \
  extern __shared__ __align__(16) unsigned char tedq_smem_raw[];                                        \
  __shared__ tedq::dev::cpx<REAL> tedq_mats[tedq::kMaxMats][4];                                         \
  tedq::dev::FwdTile<REAL, RB> c(P, reinterpret_cast<tedq::dev::SUnit<REAL>*>(tedq_smem_raw), tedq_mats,   \
                                 psi, params, n_params, init, n_tiles, NORM);
#define TEDQ_BWD_TILE_PROLOGUE_IMPL(REAL, RB, NORM)                                                     \
  extern __shared__ __align__(16) unsigned char tedq_smem_raw[];                                        \
  __shared__ tedq::dev::cpx<REAL> tedq_mats[tedq::kMaxMats][4];                                         \
  __shared__ REAL tedq_gacc[8 * tedq::kMaxPassGates];                                                   \
  tedq::dev::BwdTile<REAL, RB> c(P, reinterpret_cast<tedq::dev::SUnit<REAL>*>(tedq_smem_raw), tedq_mats,   \
                                 tedq_gacc, psi, lam, params, n_params, grad_acc, n_tiles, NORM);
#define TEDQ_FWD_TILE_PROLOGUE_GENERIC(REAL, RB) TEDQ_FWD_TILE_PROLOGUE_IMPL(REAL, RB, false)
#define TEDQ_BWD_TILE_PROLOGUE_GENERIC(REAL, RB) TEDQ_BWD_TILE_PROLOGUE_IMPL(REAL, RB, false)
#define TEDQ_FWD_TILE_PROLOGUE(REAL, RB) TEDQ_FWD_TILE_PROLOGUE_IMPL(REAL, RB, true)
#define TEDQ_BWD_TILE_PROLOGUE(REAL, RB) TEDQ_BWD_TILE_PROLOGUE_IMPL(REAL, RB, true)

// Tile pipeline (FwdPass / BwdPass, specialised kernels only): everything in
// dynamic shared memory.
#define TEDQ_FWD_PROLOGUE(REAL, RB)                                                                     \
  extern __shared__ __align__(16) unsigned char tedq_smem_raw[];                                        \
  tedq::dev::FwdPass<REAL, RB> c(P, tedq_smem_raw, psi, params, n_params, init, n_tiles);
#define TEDQ_BWD_PROLOGUE(REAL, RB)                                                                     \
  extern __shared__ __align__(16) unsigned char tedq_smem_raw[];                                        \
  tedq::dev::BwdPass<REAL, RB> c(P, tedq_smem_raw, psi, lam, params, n_params, grad_acc, n_tiles);
