// sv_kernels.cu -- sm_103a state-vector kernels of the compiled-circuit path.
//
// Reference counterpart: the per-gate ``torch.tensordot`` + ``permute`` loop
// of PyTorchBackend.execute (tedq/backends/pytorch_backend.py:365-379), the
// measurement reductions (:393-498) and, for gradients, torch autograd through
// that loop (``back_prop``, :142-144).
//
// Kernels
//   fwd_pass_kernel  one HBM pass of the forward schedule, gates dispatched at
//                    run time (until the circuit's specialised kernels are
//                    compiled, and for small circuits): a CTA stages one tile
//                    (2^m amplitudes) in shared memory, runs the pass's
//                    register phases, writes the tile back in place.
//   bwd_pass_kernel  one pass of the adjoint sweep over psi and lambda at once:
//                    for every parameterised gate (in reverse order) it adds
//                    coef * Im<lambda|G|psi> into the gradient, then applies the
//                    inverse gate to both states.
// The specialised kernels (sv_jit.cpp) add the tile pipeline (sv_device.cuh).
//   expval_kernel    Pauli-string expectations, one read of the state,
//                    FP32 partial sums per thread/warp and FP64 across warps/CTAs.
//   probs kernels, lambda_init_kernel, finalize kernels.
//
// Bound: every pass kernel moves 16 B per amplitude (c64 read + write; 32 B
// for the adjoint pass) and is designed to run at HBM bandwidth; the FP32
// register work per amplitude is 4-8 FMA per gate.
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <utility>

#include "sv_device.cuh"
#include "sv_kernels.cuh"
#include "launch.cuh"

namespace tedq {
namespace {

using dev::cconj;
using dev::cmul;
using dev::cpx;
using dev::imcb;
using dev::mk;
using dev::recb;
using dev::Unit;

template <typename real>
constexpr int kE = dev::UnitsPerAmp<real>::E;

// ---------------------------------------------------------------- pass kernels
// Generic pass kernels: the gates of each phase are dispatched at run time
// from the PassParams tables (used when no specialised kernel was generated).
// Normalised rotations run with their plain matrices here (no pass scale).

template <typename real, int R>
__global__ void __launch_bounds__(256, 2)
    fwd_pass_kernel(const __grid_constant__ PassParams P, cpx<real>* __restrict__ psi,
                    const real* __restrict__ params, int n_params, const cpx<real>* __restrict__ init,
                    int64_t n_tiles) {
  TEDQ_FWD_TILE_PROLOGUE_GENERIC(real, R)
  while (c.next()) {
    for (int f = 0; f < P.n_phases; ++f) {
      const Phase& ph = P.phase[f];
      const bool last = f + 1 == P.n_phases;
      if (ph.type == PH_REG) {
        if (f == 0) c.begin_first(f);
        else c.begin(f);
        for (int g = ph.g0; g < ph.g1; ++g) {
          const RGate& r = P.gate[g];
          dev::apply_rgate<R, real>(r, c.a, c.mats[r.mat]);
        }
        if (last) c.end_last(f);
        else if (P.phase[f + 1].type == PH_REG && P.phase[f + 1].wlocal) c.end_w(f);
        else c.end(f);
      } else {
        if (f == 0) c.to_planar();
        c.dense(f);
        if (last) c.to_raw();
      }
    }
    c.finish();
  }
  c.close();
}

template <typename real, int R>
__global__ void __launch_bounds__(256, 2)
    bwd_pass_kernel(const __grid_constant__ PassParams P, cpx<real>* __restrict__ psi, cpx<real>* __restrict__ lam,
                    const real* __restrict__ params, int n_params, double* __restrict__ grad_acc,
                    int64_t n_tiles) {
  TEDQ_BWD_TILE_PROLOGUE_GENERIC(real, R)
  while (c.next()) {
    for (int f = 0; f < P.n_phases; ++f) {
      const Phase& ph = P.phase[f];
      const bool last = f + 1 == P.n_phases;
      if (ph.type == PH_REG) {
        if (f == 0) c.begin_first(f);
        else c.begin(f);
        for (int g = ph.g0; g < ph.g1; ++g) {
          const RGate& r = P.gate[g];
          if (r.grad != GR_NONE) c.grad(g, dev::dispatch_grad<R, real>(r.grad, r.k0, c.a, c.l, r.cmask));
          dev::apply_rgate<R, real>(r, c.a, c.mats[r.mat]);
          dev::apply_rgate<R, real>(r, c.l, c.mats[r.mat]);
        }
        if (last) c.end_last(f);
        else if (P.phase[f + 1].type == PH_REG && P.phase[f + 1].wlocal) c.end_w(f);
        else c.end(f);
      } else {
        if (f == 0) c.to_planar();
        c.dense(f);
        if (last) c.to_raw();
      }
    }
    c.finish();
  }
  c.close();
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

// 16-point Walsh-Hadamard transform in registers: h[k] <- sum_j h[j] (-1)^{popc(k & j)}.
template <typename real>
__device__ __forceinline__ void wht16(real* h) {
#pragma unroll
  for (int len = 1; len < 16; len <<= 1)
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (!(i & len)) {
        const real a = h[i], b = h[i | len];
        h[i] = a + b;
        h[i | len] = a - b;
      }
}

// 16 consecutive amplitudes starting at a multiple of 16 (vector loads).
template <typename real>
__device__ __forceinline__ void load16(const cpx<real>* st, uint64_t w0, cpx<real>* v) {
  constexpr int E = kE<real>;
  const Unit<real>* u = reinterpret_cast<const Unit<real>*>(st + w0);
  Unit<real> x[16 >> E];
#pragma unroll
  for (int k = 0; k < (16 >> E); ++k) x[k] = u[k];
#pragma unroll
  for (int k = 0; k < (16 >> E); ++k)
#pragma unroll
    for (int e = 0; e < (1 << E); ++e) v[(k << E) + e] = x[k].v[e];
}

// Pauli-string expectations.  Each thread takes 16 consecutive amplitudes
// w0..w0+15; for a diagonal string Z^z the chunk contributes
// (-1)^{popc(z & w0)} * WHT(|psi|^2)[z & 15], one shared-memory lookup per
// string after one 16-point transform.  Off-diagonal strings (X/Y factors)
// read the partner amplitudes directly.  FP32 per thread and warp, FP64 across.
template <typename real>
__global__ void __launch_bounds__(kMeasThreads)
    expval_kernel(const __grid_constant__ TermTable TT, const cpx<real>* __restrict__ psi, int n,
                  double* __restrict__ acc, int64_t circ0) {
  __shared__ real hs[16][kMeasThreads];
  __shared__ double sacc[32];
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t circ = circ0 + blockIdx.y;
  const uint64_t N = 1ull << n;
  const cpx<real>* st = psi + circ * (int64_t)N;
  // each thread walks 16-amplitude chunks of its circuit with a grid stride and
  // keeps FP32 partial sums; one FP64 reduction per CTA and group of 32 strings
  const uint64_t stride = (uint64_t)gridDim.x * kMeasThreads * 16;
  for (int sg = 0; sg < TT.n; sg += 32) {
    real part[32];
#pragma unroll
    for (int s = 0; s < 32; ++s) part[s] = 0;
    for (uint64_t w0 = ((uint64_t)blockIdx.x * kMeasThreads + tid) * 16; w0 < N; w0 += stride) {
      cpx<real> v[16];
      load16<real>(st, w0, v);
      {
        real h[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) h[j] = v[j].x * v[j].x + v[j].y * v[j].y;
        wht16<real>(h);
#pragma unroll
        for (int j = 0; j < 16; ++j) hs[j][tid] = h[j];  // own column: no barrier needed
      }
#pragma unroll
      for (int s = 0; s < 32; ++s) {
        if (sg + s < TT.n) {
          const TermDev& t = TT.t[sg + s];
          if (t.x == 0) {
            const real hv = hs[t.z & 15][tid];
            part[s] += (__popcll(t.z & w0) & 1) ? -hv : hv;
          } else {
            real q = 0;
            for (int j = 0; j < 16; ++j) {
              const uint64_t w = w0 + j;
              const real tv = term_value<real>(t, v[j], st[w ^ t.x]);
              q += (__popcll(t.z & w) & 1) ? -tv : tv;
            }
            part[s] += q;
          }
        }
      }
    }
    if (tid < 32) sacc[tid] = 0.0;
    __syncthreads();
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

// lambda = sum_s w_s P_s psi + (probs weights) psi + dy_state / 2, in chunks of
// 16 consecutive amplitudes: the diagonal strings' weights are scattered to
// D[z & 15] with the sign of the chunk's high bits, and one inverse 16-point
// Walsh-Hadamard transform gives the diagonal multiplier of every amplitude.
template <typename real>
__global__ void __launch_bounds__(256)
    lambda_init_kernel(const __grid_constant__ TermTable TT, const __grid_constant__ ProbsTable PT,
                       const double* __restrict__ wts, const real* __restrict__ dy, int n_real,
                       const cpx<real>* __restrict__ dys, const cpx<real>* __restrict__ psi, cpx<real>* __restrict__ lam,
                       int n, int64_t circ0) {
  constexpr int E = kE<real>;
  __shared__ real ds[16][256];
  __shared__ real wsm[kMaxTerms];
  const int tid = threadIdx.x;
  const int64_t circ = circ0 + blockIdx.y;
  const uint64_t N = 1ull << n;
  const cpx<real>* st = psi + circ * (int64_t)N;
  cpx<real>* lt = lam + circ * (int64_t)N;
  const uint64_t padm = (1ull << PT.pad_bits) - 1;
  for (int s = tid; s < TT.n; s += blockDim.x) wsm[s] = (real)wts[circ * TT.n + s];
  __syncthreads();
  for (uint64_t w0 = ((uint64_t)blockIdx.x * blockDim.x + tid) * 16; w0 < N;
       w0 += (uint64_t)gridDim.x * blockDim.x * 16) {
    cpx<real> v[16];
    load16<real>(st, w0, v);
#pragma unroll
    for (int j = 0; j < 16; ++j) ds[j][tid] = 0;
    for (int s = 0; s < TT.n; ++s) {
      const TermDev& t = TT.t[s];
      const real W = wsm[s];
      if (t.x == 0 && W != (real)0) ds[t.z & 15][tid] += (__popcll(t.z & w0) & 1) ? -W : W;
    }
    real d[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) d[j] = ds[j][tid];
    wht16<real>(d);
    if (dy) {
      for (int pi = 0; pi < PT.n; ++pi) {
        const ProbsDesc& pd = PT.p[pi];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const uint64_t w = w0 + j;
          if (pd.full) {
            if ((w & padm) == 0) d[j] += dy[circ * n_real + pd.offset + (w >> PT.pad_bits)];
          } else {
            d[j] += dy[circ * n_real + pd.offset + bin_of(pd, w)];
          }
        }
      }
    }
    cpx<real> r[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) r[j] = mk<real>(d[j] * v[j].x, d[j] * v[j].y);
    for (int s = 0; s < TT.n; ++s) {
      const TermDev& t = TT.t[s];
      const real W = wsm[s];
      if (t.x == 0 || W == (real)0) continue;
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const uint64_t w = w0 + j;
        const cpx<real> u = st[w ^ t.x];
        cpx<real> pu;
        switch (t.ny & 3) {
          case 0: pu = u; break;
          case 1: pu = mk<real>(u.y, -u.x); break;
          case 2: pu = mk<real>(-u.x, -u.y); break;
          default: pu = mk<real>(-u.y, u.x); break;
        }
        const real sgn = (__popcll(t.z & w) & 1) ? -W : W;
        r[j].x += sgn * pu.x;
        r[j].y += sgn * pu.y;
      }
    }
    if (dys) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const cpx<real> g = dys[circ * (int64_t)N + w0 + j];
        r[j].x += (real)0.5 * g.x;
        r[j].y += (real)0.5 * g.y;
      }
    }
    Unit<real>* out = reinterpret_cast<Unit<real>*>(lt + w0);
#pragma unroll
    for (int k = 0; k < (16 >> E); ++k) {
      Unit<real> x;
#pragma unroll
      for (int e = 0; e < (1 << E); ++e) x.v[e] = r[(k << E) + e];
      out[k] = x;
    }
  }
}

template <typename real>
__global__ void grad_finalize_kernel(const double* __restrict__ acc, real* __restrict__ g, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) g[i] = (real)acc[i];
}

// ---------------------------------------------------------------- launch helpers

constexpr int kMaxGridY = 65535;

// Raises a kernel's dynamic shared-memory limit to at least `bytes`.  The limit
// is a property of the function (shared by all host threads), so the record of
// what was set is process-wide per device and the limit is never lowered.
template <typename K>
cudaError_t ensure_smem(K kernel, size_t bytes) {
  static std::mutex mu;
  static size_t done_bytes[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  std::lock_guard<std::mutex> lock(mu);
  if (done_bytes[dev] >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) done_bytes[dev] = bytes;
  return e;
}

// Generic kernels run one tile per CTA (FwdTile / BwdTile).
template <typename real, int R>
cudaError_t fwd_impl(const PassParams& P, void* psi, const void* params, int n_params, const void* init,
                     int64_t batch, cudaStream_t s) {
  const size_t smem = tile_dynamic_smem(P, false);
  auto kern = fwd_pass_kernel<real, R>;
  cudaError_t e = ensure_smem(kern, smem);
  if (e != cudaSuccess) return e;
  const int threads = 1 << (P.m - R);
  const int64_t n_tiles = batch << (P.n - P.m);
  return launch_kernel(kern, dim3((unsigned)n_tiles), dim3(threads), smem, s, P, static_cast<cpx<real>*>(psi),
                       static_cast<const real*>(params), n_params, static_cast<const cpx<real>*>(init), n_tiles);
}

template <typename real, int R>
cudaError_t bwd_impl(const PassParams& P, void* psi, void* lam, const void* params, int n_params,
                     double* grad_acc, int64_t batch, cudaStream_t s) {
  const size_t smem = tile_dynamic_smem(P, true);
  auto kern = bwd_pass_kernel<real, R>;
  cudaError_t e = ensure_smem(kern, smem);
  if (e != cudaSuccess) return e;
  const int threads = 1 << (P.m - R);
  const int64_t n_tiles = batch << (P.n - P.m);
  return launch_kernel(kern, dim3((unsigned)n_tiles), dim3(threads), smem, s, P, static_cast<cpx<real>*>(psi),
                       static_cast<cpx<real>*>(lam), static_cast<const real*>(params), n_params, grad_acc, n_tiles);
}

template <typename real>
cudaError_t init_impl(int n, int pad, void* psi, const void* init, int64_t batch, cudaStream_t s) {
  const uint64_t N = 1ull << n;
  const unsigned bx = (unsigned)((N + 255) / 256 < 4096 ? (N + 255) / 256 : 4096);
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    cudaError_t e = launch_kernel(init_state_kernel<real>, dim3(bx, (unsigned)nb), dim3(256), 0, s,
                                  static_cast<cpx<real>*>(psi), n, pad, static_cast<const cpx<real>*>(init), c0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename real>
cudaError_t expval_impl(int n, const TermTable& TT, const void* psi, double* acc, int64_t batch, cudaStream_t s) {
  const uint64_t N = 1ull << n;
  // 16 CTAs per circuit (fewer for small states): each thread sums 16-amplitude
  // chunks with a grid stride
  uint64_t bx64 = (N + kMeasChunk - 1) / kMeasChunk;
  if (bx64 > 16) bx64 = 16;
  const unsigned bx = (unsigned)bx64;
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    cudaError_t e = launch_kernel(expval_kernel<real>, dim3(bx, (unsigned)nb), dim3(kMeasThreads), 0, s, TT,
                                  static_cast<const cpx<real>*>(psi), n, acc, c0);
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
    e = launch_kernel(kern, dim3(bx, (unsigned)nb), dim3(kMeasThreads), smem, s, PT,
                      static_cast<const cpx<real>*>(psi), n, probs_acc, static_cast<real*>(out), n_real, c0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename real>
cudaError_t lambda_impl(int n, const TermTable& TT, const ProbsTable& PT, const double* w, const void* dy,
                        int n_real, const void* dys, const void* psi, void* lam, int64_t batch, cudaStream_t s) {
  const uint64_t N = 1ull << n;
  const uint64_t chunks = (N + 16 * 256 - 1) / (16 * 256);
  const unsigned bx = (unsigned)(chunks < 32 ? chunks : 32);  // grid stride: several chunks per thread
  for (int64_t c0 = 0; c0 < batch; c0 += kMaxGridY) {
    const int64_t nb = batch - c0 < kMaxGridY ? batch - c0 : kMaxGridY;
    cudaError_t e = launch_kernel(lambda_init_kernel<real>, dim3(bx, (unsigned)nb), dim3(256), 0, s, TT, PT, w,
                                  static_cast<const real*>(dy), n_real, static_cast<const cpx<real>*>(dys),
                                  static_cast<const cpx<real>*>(psi), static_cast<cpx<real>*>(lam), n, c0);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t pass_grid_cached(const void* key, int threads, size_t smem, int64_t n_tiles,
                             cudaError_t (*query)(const void* key, int threads, size_t smem, int* per_sm),
                             unsigned& grid) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, int, size_t>, int> resident;  // (kernel, device, threads, smem)
  static int sm_count[64] = {0};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int per_sm = 0, sms = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = resident.find(std::make_tuple(key, dev, threads, smem));
    if (it != resident.end()) per_sm = it->second;
    if (dev >= 0 && dev < 64) sms = sm_count[dev];
  }
  if (sms == 0) {
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
  }
  if (per_sm == 0) {
    e = query(key, threads, smem, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
  }
  {
    std::lock_guard<std::mutex> lock(mu);
    resident[std::make_tuple(key, dev, threads, smem)] = per_sm;
    if (dev >= 0 && dev < 64) sm_count[dev] = sms;
  }
  const int64_t want = (int64_t)sms * per_sm;
  grid = (unsigned)(n_tiles < want ? n_tiles : want);
  return cudaSuccess;
}

cudaError_t launch_fwd_pass(bool dbl, const PassParams& P, void* psi, const void* params, int n_params,
                            const void* init, int64_t batch, cudaStream_t s) {
  // the generic kernels exist for the default register bits only
  if (P.R != (dbl ? 4 : 5)) return cudaErrorNotSupported;
  return dbl ? fwd_impl<double, 4>(P, psi, params, n_params, init, batch, s)
             : fwd_impl<float, 5>(P, psi, params, n_params, init, batch, s);
}

cudaError_t launch_bwd_pass(bool dbl, const PassParams& P, void* psi, void* lam, const void* params,
                            int n_params, double* grad_acc, int64_t batch, cudaStream_t s) {
  if (P.R != (dbl ? 3 : 4)) return cudaErrorNotSupported;
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
    return launch_kernel(finalize_kernel<double>, dim3(blocks), dim3(256), 0, s, O, PT, term_acc, probs_acc,
                         static_cast<double*>(out_real), batch);
  return launch_kernel(finalize_kernel<float>, dim3(blocks), dim3(256), 0, s, O, PT, term_acc, probs_acc,
                       static_cast<float*>(out_real), batch);
}

cudaError_t launch_term_weights(bool dbl, const OutTermTable& O, const void* dy_real, double* w, int64_t batch,
                                cudaStream_t s) {
  if (O.n_terms == 0 || batch == 0) return cudaSuccess;
  const int64_t total = batch * O.n_terms;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  if (dbl)
    return launch_kernel(term_weights_kernel<double>, dim3(blocks), dim3(256), 0, s, O,
                         static_cast<const double*>(dy_real), w, batch);
  return launch_kernel(term_weights_kernel<float>, dim3(blocks), dim3(256), 0, s, O,
                       static_cast<const float*>(dy_real), w, batch);
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
  if (dbl)
    return launch_kernel(grad_finalize_kernel<double>, dim3(blocks), dim3(256), 0, s, grad_acc,
                         static_cast<double*>(grad), count);
  return launch_kernel(grad_finalize_kernel<float>, dim3(blocks), dim3(256), 0, s, grad_acc,
                       static_cast<float*>(grad), count);
}

}  // namespace tedq
