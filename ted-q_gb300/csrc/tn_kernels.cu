// tn_kernels.cu -- kernels of the tensor-network mode (tn_kernels.cuh).
//
// Work per pairwise contraction of A (M x K) and B (K x N), complex:
//  * small contractions (the planner's `fused` steps): one tn_fused_kernel
//    launch reads both operands in place through additive per-bit offsets and
//    writes the planar complex result;
//  * large ones: one gather launch writes both operands as rows of the real
//    embedding ([Re, Im], and [Re, -Im] / [Im, Re] for the doubled operand),
//    then one real GEMM over the batch (tn_gemm.cu: tcgen05 tensor cores with
//    the 3xTF32 split, or FP32 / FP64 FMA) produces [Re C, Im C] -- the 4M
//    decomposition in one product.
// Gather traffic per operand entry (c64): 8 B read, 8 B written (16 B for the
// doubled operand).
#include <cuda_runtime.h>

#include <type_traits>

#include "launch.cuh"
#include "tedq_gb300.h"
#include "tn_kernels.cuh"

namespace tedq {
namespace {

__device__ __forceinline__ void sc(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sc(double x, double* s, double* c) { sincos(x, s, c); }

// Row-major 2x2 of a parameterised one-qubit rotation, (re, im) pairs.
// Definitions: tedq/QInterpreter/operators/qubit.py (RX :990-997,
// RY :1048-1055, RZ :1106-1112, Rot :1169-1189, PhaseShift :1253-1257).
template <typename real>
__device__ void rot_2x2(int op, const real* a, real* m) {
  real s, c;
  for (int i = 0; i < 8; ++i) m[i] = 0;
  switch (op) {
    case TEDQ_OP_RX: case TEDQ_OP_CRX:
      sc(a[0] / 2, &s, &c);
      m[0] = c; m[3] = -s; m[5] = -s; m[6] = c;
      break;
    case TEDQ_OP_RY: case TEDQ_OP_CRY:
      sc(a[0] / 2, &s, &c);
      m[0] = c; m[2] = -s; m[4] = s; m[6] = c;
      break;
    case TEDQ_OP_RZ: case TEDQ_OP_CRZ:
      sc(a[0] / 2, &s, &c);
      m[0] = c; m[1] = -s; m[6] = c; m[7] = s;
      break;
    case TEDQ_OP_PHASESHIFT: case TEDQ_OP_CPHASE:
      sc(a[0], &s, &c);
      m[0] = 1; m[6] = c; m[7] = s;
      break;
    default: {  // Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi)
      real sp, cp, sm, cm;
      sc(a[1] / 2, &s, &c);
      sc((a[0] + a[2]) / 2, &sp, &cp);
      sc((a[0] - a[2]) / 2, &sm, &cm);
      m[0] = cp * c; m[1] = -sp * c;
      m[2] = -cm * s; m[3] = -sm * s;
      m[4] = cm * s; m[5] = -sm * s;
      m[6] = cp * c; m[7] = sp * c;
      break;
    }
  }
}

// One thread per (tensor, circuit): consecutive threads write consecutive
// circuits of one tensor (contiguous 4^k-entry blocks).
template <typename real>
__global__ void __launch_bounds__(256) tn_leaf_kernel(const TnLeafDesc* __restrict__ desc, int n_desc,
                                                      const real* __restrict__ prm, int n_params,
                                                      int64_t batch, real* __restrict__ leaves) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (int64_t)n_desc * batch) return;
  const int64_t b = t % batch;
  const TnLeafDesc d = desc[t / batch];
  real a[3];
  for (int j = 0; j < 3; ++j) a[j] = d.slot[j] >= 0 ? prm[b * n_params + d.slot[j]] : (real)d.val[j];
  real m[8];
  rot_2x2<real>(d.op, a, m);
  const real sgn = d.conj ? (real)-1 : (real)1;
  if (d.k == 1) {
    real* o = leaves + 2 * (d.off * batch + b * 4);
    for (int i = 0; i < 4; ++i) {
      o[2 * i] = m[2 * i];
      o[2 * i + 1] = sgn * m[2 * i + 1];
    }
  } else {  // controlled: identity on the control-0 block, m on the control-1 block
    real* o = leaves + 2 * (d.off * batch + b * 16);
    for (int r = 0; r < 4; ++r)
      for (int cidx = 0; cidx < 4; ++cidx) {
        real re = (r == cidx) ? (real)1 : (real)0, im = 0;
        if (r >= 2 && cidx >= 2) {
          re = m[2 * ((r - 2) * 2 + (cidx - 2))];
          im = m[2 * ((r - 2) * 2 + (cidx - 2)) + 1];
        }
        o[2 * (r * 4 + cidx)] = re;
        o[2 * (r * 4 + cidx) + 1] = sgn * im;
      }
  }
}

// Tiled bit-permutation copy (one operand per blockIdx.y, 256 threads): per
// tile, source elements are read in source order into shared memory (padded
// one word per 32) and written out in destination order, so both sides are
// coalesced.  Tile-local offsets are tabulated once per CTA in the order each
// phase uses them (32-bit: the host limits operands to 2^28 entries), the
// low 8 outer element bits likewise; the next tile's loads are issued before
// the current tile is written out.
template <typename real>
__global__ void __launch_bounds__(256) tn_gather_kernel(const __grid_constant__ TnGatherArgs A) {
  constexpr int TS_MAX = 1 << kTnTileBits, PER = TS_MAX / 256;
  __shared__ real sre[TS_MAX + TS_MAX / 32], sim[TS_MAX + TS_MAX / 32];
  __shared__ int32_t ld_off[TS_MAX], st_off[TS_MAX];  // read order: source offset; write order: row offset
  __shared__ int16_t ld_slot[TS_MAX];                 // read order: padded shared-memory slot
  __shared__ int64_t olo_s[256], olo_d[256];
  const int op = blockIdx.y;
  const int tb = A.op[op].tb, TS = 1 << tb, nc = A.op[op].nc, nbits = A.op[op].nbits;
  const int n_outer = A.op[op].n_outer, doubled = A.op[op].doubled;
  const int64_t K = 1ll << nc, n = 1ll << nbits, src_im = A.op[op].src_im;
  const int64_t src_bstride = A.op[op].src_bstride, src_base = A.op[op].src_base;
  const int64_t* sw = A.op[op].sw;
  const int8_t* tile_bit = A.op[op].tile_bit;
  const int8_t* r2w = A.op[op].r2w;
  const int8_t* outer_bit = A.op[op].outer_bit;
  auto dw = [nc, K](int j) -> int64_t { return j < nc ? (1ll << j) : ((2 * K) << (j - nc)); };
  // tables by doubling: entry x | 2^i = entry x + weight of bit i
  __shared__ int16_t wr[TS_MAX];  // read-order index -> write-order index
  if (threadIdx.x == 0) {
    ld_off[0] = 0;
    st_off[0] = 0;
    wr[0] = 0;
  }
  __syncthreads();
  for (int i = 0; i < tb; ++i) {
    const int h = 1 << i;
    const int32_t wsrc = (int32_t)sw[tile_bit[r2w[i]]], wdst = (int32_t)dw(tile_bit[i]);
    for (int x = threadIdx.x; x < h; x += blockDim.x) {
      ld_off[h + x] = ld_off[x] + wsrc;
      st_off[h + x] = st_off[x] + wdst;
      wr[h + x] = (int16_t)(wr[x] | (1 << r2w[i]));
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < TS; r += blockDim.x) {
    const int w = wr[r];
    ld_slot[r] = (int16_t)(w + (w >> 5));
  }
  const int nlo = n_outer < 8 ? n_outer : 8;
  for (int u = threadIdx.x; u < (1 << nlo); u += blockDim.x) {
    int64_t so = 0, dof = 0;
    for (int q = 0; q < nlo; ++q)
      if ((u >> q) & 1) {
        so += sw[outer_bit[q]];
        dof += dw(outer_bit[q]);
      }
    olo_s[u] = so;
    olo_d[u] = dof;
  }
  __syncthreads();
  const int outer = nbits - tb;
  const int64_t total = A.op[op].nb << outer;
  const int64_t dstride = (doubled ? 4 : 2) * n;
  const real* __restrict__ src = static_cast<const real*>(A.op[op].src);
  real* __restrict__ dst = static_cast<real*>(A.op[op].dst);
  const int lomask = (1 << nlo) - 1;
  real vr[PER], vi[PER];
  int64_t tile = blockIdx.x, dcur = 0;
  using V2 = typename std::conditional<sizeof(real) == 4, float2, double2>::type;
  const int rmode = A.op[op].rmode, wpair = A.op[op].wpair;
  auto load = [&](int64_t t) {
    const int64_t b = t >> outer, ou = t & ((1ll << outer) - 1);
    int64_t so = src_base + b * src_bstride + olo_s[ou & lomask];
    int64_t dof = b * dstride + olo_d[ou & lomask];
    for (int q = nlo; q < n_outer; ++q)
      if ((ou >> q) & 1) {
        so += sw[outer_bit[q]];
        dof += dw(outer_bit[q]);
      }
    const real* sp = src + so;
    if (rmode == 1) {
#pragma unroll
      for (int q = 0; q < PER / 2; ++q) {
        const int r = 2 * (threadIdx.x + q * 256);
        if (r < TS) {
          const int32_t at = ld_off[r];
          const V2 a = *reinterpret_cast<const V2*>(sp + at);
          const V2 c = *reinterpret_cast<const V2*>(sp + at + src_im);
          vr[2 * q] = a.x;
          vr[2 * q + 1] = a.y;
          vi[2 * q] = c.x;
          vi[2 * q + 1] = c.y;
        }
      }
    } else if (rmode == 2) {
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int r = threadIdx.x + q * 256;
        if (r < TS) {
          const V2 a = *reinterpret_cast<const V2*>(sp + ld_off[r]);
          vr[q] = a.x;
          vi[q] = a.y;
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int r = threadIdx.x + q * 256;
        if (r < TS) {
          const int32_t at = ld_off[r];
          vr[q] = sp[at];
          vi[q] = sp[at + src_im];
        }
      }
    }
    return dof;
  };
  if (tile < total) dcur = load(tile);
  for (; tile < total; tile += gridDim.x) {
    if (rmode == 1) {
#pragma unroll
      for (int q = 0; q < PER / 2; ++q) {
        const int r = 2 * (threadIdx.x + q * 256);
        if (r < TS) {
          const int s0 = ld_slot[r], s1 = ld_slot[r + 1];
          sre[s0] = vr[2 * q];
          sim[s0] = vi[2 * q];
          sre[s1] = vr[2 * q + 1];
          sim[s1] = vi[2 * q + 1];
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int r = threadIdx.x + q * 256;
        if (r < TS) {
          const int slot = ld_slot[r];
          sre[slot] = vr[q];
          sim[slot] = vi[q];
        }
      }
    }
    __syncthreads();
    real* d = dst + dcur;
    if (tile + gridDim.x < total) dcur = load(tile + gridDim.x);
    if (wpair) {
#pragma unroll
      for (int q = 0; q < PER / 2; ++q) {
        const int w = 2 * (threadIdx.x + q * 256);
        if (w < TS) {
          const int s0 = w + (w >> 5), s1 = (w + 1) + ((w + 1) >> 5);
          const real r0 = sre[s0], r1 = sre[s1], i0 = sim[s0], i1 = sim[s1];
          real* row = d + st_off[w];
          *reinterpret_cast<V2*>(row) = V2{r0, r1};
          if (!doubled) {
            *reinterpret_cast<V2*>(row + K) = V2{i0, i1};
          } else {
            *reinterpret_cast<V2*>(row + K) = V2{-i0, -i1};
            *reinterpret_cast<V2*>(row + 2 * n) = V2{i0, i1};  // row F + f
            *reinterpret_cast<V2*>(row + 2 * n + K) = V2{r0, r1};
          }
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < PER; ++q) {
        const int w = threadIdx.x + q * 256;
        if (w < TS) {
          const real re = sre[w + (w >> 5)], im = sim[w + (w >> 5)];
          real* row = d + st_off[w];
          row[0] = re;
          if (!doubled) {
            row[K] = im;
          } else {
            row[K] = -im;
            row[2 * n] = im;  // row F + f
            row[2 * n + K] = re;
          }
        }
      }
    }
    __syncthreads();
  }
}

// One thread per (circuit, output element); the contracted-index offsets of
// both operands are tabulated once per CTA in shared memory.
template <typename real>
__global__ void __launch_bounds__(256) tn_fused_kernel(const __grid_constant__ TnFusedArgs A) {
  __shared__ int64_t koff[2][256];
  const int K = 1 << A.lk;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    int64_t oa = 0, ob = 0;
    for (int j = 0; j < A.lk; ++j)
      if ((k >> j) & 1) {
        oa += A.a.wk[j];
        ob += A.b.wk[j];
      }
    koff[0][k] = oa;
    koff[1][k] = ob;
  }
  __syncthreads();
  const int lmn = A.lm + A.ln;
  const int64_t MN = 1ll << lmn, total = MN * A.nb, imask = (1ll << A.lm) - 1;
  const real* sa = static_cast<const real*>(A.a.src);
  const real* sb = static_cast<const real*>(A.b.src);
  real* dst = static_cast<real*>(A.dst);
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t >> lmn, idx = t & (MN - 1);
    const int64_t i = idx & imask, j = idx >> A.lm;
    int64_t oa = A.a.base + b * A.a.bstride, ob = A.b.base + b * A.b.bstride;
    for (int q = 0; q < A.lm; ++q)
      if ((i >> q) & 1) oa += A.a.wf[q];
    for (int q = 0; q < A.ln; ++q)
      if ((j >> q) & 1) ob += A.b.wf[q];
    const real* pa = sa + oa;
    const real* pb = sb + ob;
    real re = 0, im = 0;
    for (int k = 0; k < K; ++k) {
      const real ar = pa[koff[0][k]], ai = pa[koff[0][k] + A.a.im];
      const real br = pb[koff[1][k]], bi = pb[koff[1][k] + A.b.im];
      re = fma(ar, br, fma(-ai, bi, re));
      im = fma(ar, bi, fma(ai, br, im));
    }
    real* d = dst + b * A.dst_bstride;
    d[idx] = re;
    d[MN + idx] = im;
  }
}

// One CTA = 256 outputs of one item; the item is found by binary search on
// blk0.  Contracted-index offsets of both operands are tabulated in shared
// memory first (every thread reaches the barrier before any exits).
template <typename real>
__global__ void __launch_bounds__(256) tn_fused_level_kernel(const TnFusedItem* __restrict__ items, int n_items,
                                                             char* __restrict__ ws, const char* __restrict__ consts,
                                                             int64_t slice) {
  __shared__ int32_t koff[2][256];
  int lo = 0, hi = n_items - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (items[mid].blk0 <= (int)blockIdx.x) lo = mid;
    else hi = mid - 1;
  }
  const TnFusedItem& it = items[lo];
  const int lk = it.lk, K = 1 << lk;
  for (int k = threadIdx.x; k < K; k += blockDim.x) {
    int32_t oa = 0, ob = 0;
    for (int j = 0; j < lk; ++j)
      if ((k >> j) & 1) {
        oa += it.wk[0][j];
        ob += it.wk[1][j];
      }
    koff[0][k] = oa;
    koff[1][k] = ob;
  }
  __syncthreads();
  const int lm = it.lm, lmn = lm + it.ln;
  const int64_t MN = 1ll << lmn, total = MN * it.nb;
  const int64_t t = (int64_t)(blockIdx.x - it.blk0) * blockDim.x + threadIdx.x;
  if (t >= total) return;
  const int64_t b = t >> lmn, idx = t & (MN - 1);
  const int64_t i = idx & ((1ll << lm) - 1), j = idx >> lm;
  int64_t oa = it.off[0] + b * it.bstride[0], ob = it.off[1] + b * it.bstride[1];
  for (int q = 0; q < it.nsl0; ++q)
    if ((slice >> it.slq[0][q]) & 1) oa += it.slw[0][q];
  for (int q = 0; q < it.nsl1; ++q)
    if ((slice >> it.slq[1][q]) & 1) ob += it.slw[1][q];
  for (int q = 0; q < lm; ++q)
    if ((i >> q) & 1) oa += it.wf[0][q];
  for (int q = 0; q < it.ln; ++q)
    if ((j >> q) & 1) ob += it.wf[1][q];
  const real* pa = reinterpret_cast<const real*>(it.region[0] ? consts : ws) + oa;
  const real* pb = reinterpret_cast<const real*>(it.region[1] ? consts : ws) + ob;
  const int64_t ima = it.im[0], imb = it.im[1];
  real re = 0, im = 0;
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    const real ar = pa[koff[0][k]], ai = pa[koff[0][k] + ima];
    const real br = pb[koff[1][k]], bi = pb[koff[1][k] + imb];
    re = fma(ar, br, fma(-ai, bi, re));
    im = fma(ar, bi, fma(ai, br, im));
  }
  real* d = reinterpret_cast<real*>(ws) + it.dst_off + b * it.dst_bstride;
  d[idx] = re;
  d[MN + idx] = im;
}

// One warp per circuit: lane 0 accumulates the root; on the last slice the
// warp checks the circuit's parameters (coalesced) and a circuit with a
// non-finite parameter returns NaN (the emulated GEMMs run without
// special-value handling, so such inputs are not propagated there).
template <typename real>
__global__ void tn_root_kernel(const real* __restrict__ root, int64_t bstride, int64_t batch, double* acc,
                               real* out, int n_meas, int m, int first, int last, const real* __restrict__ prm,
                               int n_params, const int* err) {
  const int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (b >= batch) return;
  bool finite = true;
  if (last)
    for (int j = lane; j < n_params; j += 32) finite &= isfinite(prm[b * n_params + j]);
  finite = __all_sync(0xffffffffu, finite);
  // a contraction kernel that gave up a bounded wait leaves every result invalid
  if (last && err && *(volatile const int*)err != 0) finite = false;
  if (lane) return;
  const real* p = root + b * bstride;
  double v = (double)p[0];
  double* a = acc + b * n_meas + m;
  if (!first) v += *a;
  *a = v;
  if (last) out[b * n_meas + m] = finite ? (real)v : (real)NAN;
}

}  // namespace

template <typename real>
cudaError_t tn_build_leaves(const TnLeafDesc* desc, int n_desc, const real* params, int n_params, int64_t batch,
                            real* leaves, cudaStream_t stream) {
  const int64_t total = (int64_t)n_desc * batch;
  if (total == 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((total + 255) / 256);
  return launch_kernel(tn_leaf_kernel<real>, dim3(blocks), dim3(256), 0, stream, desc, n_desc, params, n_params,
                       batch, leaves);
}

template <typename real>
cudaError_t tn_gather(const TnGatherArgs& args, cudaStream_t stream) {
  int64_t most = 0;
  for (int i = 0; i < 2; ++i) {
    const TnGatherOp& o = args.op[i];
    if (o.tb < 0 || o.tb > kTnTileBits || o.tb > o.nbits || o.n_outer != o.nbits - o.tb) return cudaErrorInvalidValue;
    if (o.nbits > 28) return cudaErrorInvalidValue;  // 32-bit tile tables
    const int64_t t = o.nb << (o.nbits - o.tb);
    most = t > most ? t : most;
  }
  // several CTAs per SM per operand: each keeps one tile of loads in flight
  // (fewer, longer-lived CTAs measured slower)
  int64_t blocks = most;
  if (blocks > 152 * 8) blocks = 152 * 8;
  return launch_kernel(tn_gather_kernel<real>, dim3((unsigned)blocks, 2), dim3(256), 0, stream, args);
}

template <typename real>
cudaError_t tn_fused(const TnFusedArgs& args, cudaStream_t stream) {
  if (args.lk > 8) return cudaErrorInvalidValue;
  const int64_t total = (1ll << (args.lm + args.ln)) * args.nb;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  return launch_kernel(tn_fused_kernel<real>, dim3((unsigned)blocks), dim3(256), 0, stream, args);
}

template <typename real>
cudaError_t tn_fused_level(const TnFusedItem* items, int n_items, int blocks, char* ws, const void* consts,
                           int64_t slice, cudaStream_t stream) {
  if (n_items <= 0 || blocks <= 0) return cudaErrorInvalidValue;
  return launch_kernel(tn_fused_level_kernel<real>, dim3((unsigned)blocks), dim3(256), 0, stream, items, n_items, ws,
                       static_cast<const char*>(consts), slice);
}

template <typename real>
cudaError_t tn_root(const real* root, int64_t root_bstride, int64_t batch, double* acc, real* out, int n_meas,
                    int m, int first, int last, const real* params, int n_params, const int* err,
                    cudaStream_t stream) {
  const unsigned blocks = (unsigned)((batch * 32 + 255) / 256);
  return launch_kernel(tn_root_kernel<real>, dim3(blocks), dim3(256), 0, stream, root, root_bstride, batch, acc, out,
                       n_meas, m, first, last, params, n_params, err);
}

template cudaError_t tn_build_leaves<float>(const TnLeafDesc*, int, const float*, int, int64_t, float*, cudaStream_t);
template cudaError_t tn_build_leaves<double>(const TnLeafDesc*, int, const double*, int, int64_t, double*,
                                             cudaStream_t);
template cudaError_t tn_gather<float>(const TnGatherArgs&, cudaStream_t);
template cudaError_t tn_gather<double>(const TnGatherArgs&, cudaStream_t);
template cudaError_t tn_fused<float>(const TnFusedArgs&, cudaStream_t);
template cudaError_t tn_fused<double>(const TnFusedArgs&, cudaStream_t);
template cudaError_t tn_fused_level<float>(const TnFusedItem*, int, int, char*, const void*, int64_t, cudaStream_t);
template cudaError_t tn_fused_level<double>(const TnFusedItem*, int, int, char*, const void*, int64_t,
                                            cudaStream_t);
template cudaError_t tn_root<float>(const float*, int64_t, int64_t, double*, float*, int, int, int, int,
                                    const float*, int, const int*, cudaStream_t);
template cudaError_t tn_root<double>(const double*, int64_t, int64_t, double*, double*, int, int, int, int,
                                     const double*, int, const int*, cudaStream_t);

}  // namespace tedq
