// tn_capi.cpp -- extern "C" entry points of the tensor-network mode
// (include/tedq_gb300.h, "tensor-network mode").
//
// Reference counterpart: the TN branch of PyTorchBackend.execute
// (tedq/backends/pytorch_backend.py:242-356), which rebuilds the operand list
// per call (compiled_circuit.py:442-467, pytorch_backend.py:524-546) and hands
// it to the path object's contract().  Here the plan is built once; a call
// builds the parameter-dependent gate tensors of the whole batch on the device
// and runs the planned pairwise contractions: the small ones in level
// launches that read their operands in place, the large ones as one gather
// launch and one batched real GEMM of this library (tn_gemm.cu: tcgen05
// tensor cores, 3xTF32 for FP32 accuracy) over the batch.  A CUDA graph of a
// call's launches can be replayed when the same buffers are used again.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "sv_program.h"
#include "tedq_gb300.h"
#include "tn_gemm.cuh"
#include "tn_kernels.cuh"
#include "tn_plan.h"

using namespace tedq;

int32_t tedq_record_error(int32_t status, const char* msg);

namespace {

inline size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

// ---------------------------------------------------------------------- plan

// One level launch: the fused steps [step0, step1) of a network (same level).
struct TnLevelRun {
  int step0 = 0, step1 = 0;
  int item0 = 0, n_items = 0;
  int blocks = 0;
  double flops = 0;
};

struct TnDevice {
  bool ready = false;
  int* err = nullptr;           // error word of the tensor-core GEMMs (bounded waits)
  void* consts = nullptr;       // constants of all networks (plan precision)
  TnLeafDesc* desc = nullptr;   // batched-leaf descriptors of all networks
  // graph of the last call, replayed while its arguments repeat
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr;
  const void* g_params = nullptr;
  void* g_out = nullptr;
  void* g_ws = nullptr;
  int64_t g_batch = -1;
  // fused-step items of the level launches for batch `items_batch`
  TnFusedItem* items = nullptr;
  size_t items_cap = 0;
  int64_t items_batch = -1;
  std::vector<std::vector<TnLevelRun>> runs;  // per network, for items_batch
};

struct tedq_tn_plan {
  std::vector<TnNet> nets;
  int n = 0, n_params = 0, precision = TEDQ_PREC_C64, gemm = TEDQ_TN_GEMM_FP32;
  bool graphs = false;
  std::vector<std::vector<TnLeafDesc>> descs;
  std::vector<int64_t> const_base;  // reals, per network
  std::vector<int64_t> desc_base;   // descriptors, per network
  int64_t const_total = 0, desc_total = 0;
  std::mutex mu;
  TnDevice dev[64];
  // kernel timing (tedq_tn_profile_*)
  struct Ev {
    cudaEvent_t a, b;
    int family;  // 0 leaf, 1 gather, 2 contraction (FMA), 3 root, 4 tensor-core GEMM
    double work;
  };
  bool profiling = false;
  std::vector<Ev> events;
  std::mutex prof_mu;
};

namespace {

int64_t elem_bytes(const tedq_tn_plan* p) { return p->precision == TEDQ_PREC_C128 ? 8 : 4; }

struct Layout {
  size_t acc, leaves, arena_b, arena_u, scratch, total;
};

// acc (FP64 sums) | per network (reused): batched leaves, batched arena,
// unbatched arena, GEMM operand scratch
Layout layout(const tedq_tn_plan* p, int64_t batch) {
  const size_t es = (size_t)elem_bytes(p);
  Layout L{};
  L.acc = 0;
  size_t region = align256((size_t)batch * p->nets.size() * sizeof(double));
  size_t most = 0, mleaves = 0, mab = 0, mau = 0;
  for (const TnNet& n : p->nets) {
    size_t lv = align256(2 * (size_t)n.batched_leaf_elems * batch * es);
    size_t ab = align256((size_t)n.batched_arena * batch * es);
    size_t au = align256((size_t)n.unbatched_arena * es);
    size_t sc = align256((size_t)tn_scratch_reals(n, batch) * es);
    mleaves = std::max(mleaves, lv);
    mab = std::max(mab, ab);
    mau = std::max(mau, au);
    most = std::max(most, sc);
  }
  L.leaves = region;
  L.arena_b = L.leaves + mleaves;
  L.arena_u = L.arena_b + mab;
  L.scratch = L.arena_u + mau;
  L.total = L.scratch + most;
  return L;
}

int32_t fail(int32_t status, const std::string& msg) { return tedq_record_error(status, msg.c_str()); }

int32_t cuda_fail(const char* where, cudaError_t e) {
  return fail(TEDQ_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}


#define TEDQ_CUDA(where, expr)                    \
  do {                                            \
    cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return cuda_fail(where, e_); \
  } while (0)

// Device-resident constants, descriptors and the error word (first use).
int32_t ensure_device(tedq_tn_plan* p, int dev) {
  TnDevice& D = p->dev[dev];
  if (D.ready) return TEDQ_OK;
  if (!D.err) {
    TEDQ_CUDA("tedq_tn_contract: cudaMalloc", cudaMalloc(&D.err, sizeof(int)));
    TEDQ_CUDA("tedq_tn_contract: cudaMemset", cudaMemset(D.err, 0, sizeof(int)));
  }
  const size_t es = (size_t)elem_bytes(p);
  if (!D.consts) {
    std::vector<char> host(std::max<int64_t>(p->const_total, 1) * es);
    int64_t k = 0;
    for (const TnNet& n : p->nets)
      for (double v : n.constants) {
        if (es == 8) reinterpret_cast<double*>(host.data())[k++] = v;
        else reinterpret_cast<float*>(host.data())[k++] = (float)v;
      }
    TEDQ_CUDA("tedq_tn_contract: cudaMalloc", cudaMalloc(&D.consts, host.size()));
    TEDQ_CUDA("tedq_tn_contract: cudaMemcpy", cudaMemcpy(D.consts, host.data(), host.size(), cudaMemcpyHostToDevice));
  }
  if (!D.desc && p->desc_total) {
    std::vector<TnLeafDesc> all;
    for (auto& d : p->descs) all.insert(all.end(), d.begin(), d.end());
    TEDQ_CUDA("tedq_tn_contract: cudaMalloc", cudaMalloc(&D.desc, all.size() * sizeof(TnLeafDesc)));
    TEDQ_CUDA("tedq_tn_contract: cudaMemcpy",
              cudaMemcpy(D.desc, all.data(), all.size() * sizeof(TnLeafDesc), cudaMemcpyHostToDevice));
  }
  if (p->graphs && !D.capture)
    TEDQ_CUDA("tedq_tn_contract: cudaStreamCreate", cudaStreamCreateWithFlags(&D.capture, cudaStreamNonBlocking));
  D.ready = true;
  return TEDQ_OK;
}

// Item table of the level launches for `batch` (uploaded when the batch size
// changes; offsets are relative to the workspace or the constants, so the
// table does not depend on the buffers of a call).
int32_t prepare_items(tedq_tn_plan* p, TnDevice& D, int64_t batch) {
  if (D.items_batch == batch) return TEDQ_OK;
  const Layout L = layout(p, batch);
  const int64_t es = elem_bytes(p);
  std::vector<TnFusedItem> items;
  D.runs.assign(p->nets.size(), {});
  for (size_t m = 0; m < p->nets.size(); ++m) {
    const TnNet& net = p->nets[m];
    const int64_t cb = p->const_base[m];
    auto tensor_off = [&](const TnTensor& T, int& region) -> int64_t {
      region = 0;
      if (T.leaf >= 0) {
        if (!T.batched) {
          region = 1;
          return cb + 2 * T.off;
        }
        return (int64_t)L.leaves / es + 2 * T.off * batch;
      }
      return T.batched ? (int64_t)L.arena_b / es + T.arena * batch : (int64_t)L.arena_u / es + T.arena;
    };
    size_t i = 0;
    while (i < net.steps.size()) {
      if (!net.steps[i].fused) {
        ++i;
        continue;
      }
      size_t j = i;
      TnLevelRun run;
      run.step0 = (int)i;
      run.item0 = (int)items.size();
      int64_t blocks = 0;
      bool ok = true;
      while (j < net.steps.size() && net.steps[j].fused && net.steps[j].level == net.steps[i].level) {
        const TnStep& st = net.steps[j];
        TnFusedItem it;
        std::memset(&it, 0, sizeof(it));
        it.lm = st.opa.nf;
        it.ln = st.opb.nf;
        it.lk = st.opa.nc;
        it.nb = st.batched ? (int32_t)batch : 1;
        ok &= it.lm <= kTnItemFree && it.ln <= kTnItemFree && it.lk <= kTnItemSum;
        const TnOperand* ops[2] = {&st.opa, &st.opb};
        for (int x = 0; x < 2 && ok; ++x) {
          const TnOperand& op = *ops[x];
          const TnTensor& T = net.tensors[op.tensor];
          it.off[x] = tensor_off(T, it.region[x]);
          const int64_t M = 1ll << T.lm, N = 1ll << T.ln, sj = T.split ? 2 * M : M;
          it.bstride[x] = !T.batched ? 0 : (T.leaf >= 0 ? (2ll << T.full_idx.size()) : (2ll << (T.lm + T.ln)));
          it.im[x] = T.leaf >= 0 ? 1 : (T.split ? M : M * N);
          auto w = [&](int sbit) -> int64_t {
            if (T.leaf >= 0) return 2ll << sbit;
            return sbit < T.lm ? (1ll << sbit) : (sj << (sbit - T.lm));
          };
          if ((int)op.slice_bit.size() > kTnItemSlice) ok = false;
          for (size_t q = 0; q < op.slice_bit.size() && ok; ++q) {
            it.slq[x][q] = op.slice_bit[q].first;
            it.slw[x][q] = (int32_t)w(op.slice_bit[q].second);
          }
          (x ? it.nsl1 : it.nsl0) = (int32_t)op.slice_bit.size();
          for (int k = 0; k < op.nc && ok; ++k) it.wk[x][k] = (int32_t)w(op.src_bit[k]);
          for (int k = 0; k < op.nf && ok; ++k) it.wf[x][k] = (int32_t)w(op.src_bit[op.nc + k]);
        }
        const TnTensor& O = net.tensors[st.out];
        int reg = 0;
        it.dst_off = tensor_off(O, reg);
        it.dst_bstride = O.batched ? (2ll << (O.lm + O.ln)) : 0;
        it.blk0 = (int32_t)blocks;
        blocks += ((int64_t)it.nb << (it.lm + it.ln)) / 256 + ((((int64_t)it.nb << (it.lm + it.ln)) % 256) ? 1 : 0);
        run.flops += 8.0 * std::ldexp(1.0, it.lm + it.ln + it.lk) * (double)it.nb;
        items.push_back(it);
        ++j;
      }
      if (!ok || blocks > 0x7fffffffll) {
        // outside the item limits: these steps run one launch each
        items.resize(run.item0);
        for (size_t k = i; k < j; ++k) {
          TnLevelRun one;
          one.step0 = (int)k;
          one.step1 = (int)k + 1;
          one.n_items = 0;
          D.runs[m].push_back(one);
        }
      } else {
        run.step1 = (int)j;
        run.n_items = (int)(j - i);
        run.blocks = (int)blocks;
        D.runs[m].push_back(run);
      }
      i = j;
    }
  }
  const size_t bytes = std::max<size_t>(items.size(), 1) * sizeof(TnFusedItem);
  if (bytes > D.items_cap) {
    if (D.items) cudaFree(D.items);
    D.items = nullptr;
    D.items_cap = 0;
    TEDQ_CUDA("tedq_tn_contract: cudaMalloc", cudaMalloc(&D.items, bytes));
    D.items_cap = bytes;
  }
  if (!items.empty()) {
    // launches of earlier calls may still read the previous table
    TEDQ_CUDA("tedq_tn_contract: cudaDeviceSynchronize", cudaDeviceSynchronize());
    TEDQ_CUDA("tedq_tn_contract: cudaMemcpy",
              cudaMemcpy(D.items, items.data(), items.size() * sizeof(TnFusedItem), cudaMemcpyHostToDevice));
  }
  D.items_batch = batch;
  return TEDQ_OK;
}

// Runs one launch; with profiling on, brackets it with events on its stream.
template <typename F>
int32_t timed(tedq_tn_plan* p, cudaStream_t s, int family, double work, F&& launch) {
  if (!p->profiling) return launch();
  tedq_tn_plan::Ev ev{nullptr, nullptr, family, work};
  TEDQ_CUDA("tedq_tn_contract: cudaEventCreate", cudaEventCreate(&ev.a));
  TEDQ_CUDA("tedq_tn_contract: cudaEventCreate", cudaEventCreate(&ev.b));
  TEDQ_CUDA("tedq_tn_contract: cudaEventRecord", cudaEventRecord(ev.a, s));
  int32_t rc = launch();
  TEDQ_CUDA("tedq_tn_contract: cudaEventRecord", cudaEventRecord(ev.b, s));
  std::lock_guard<std::mutex> lk(p->prof_mu);
  p->events.push_back(ev);
  return rc;
}

// Enqueues one call: batched gate tensors, then per network and slice the
// gathers and GEMMs of every step and the FP64 root accumulation.
template <typename real>
int32_t enqueue(tedq_tn_plan* p, TnDevice& D, const real* params, int64_t batch, real* out, char* ws,
                cudaStream_t s) {
  const Layout L = layout(p, batch);
  double* acc = reinterpret_cast<double*>(ws + L.acc);
  real* leaves = reinterpret_cast<real*>(ws + L.leaves);
  real* arena_b = reinterpret_cast<real*>(ws + L.arena_b);
  real* arena_u = reinterpret_cast<real*>(ws + L.arena_u);
  real* scratch = reinterpret_cast<real*>(ws + L.scratch);
  const bool dbl = sizeof(real) == 8;
  // AUTO: the FP32-accurate tensor-core GEMM for contractions of at least
  // 2^auto_log2 real flops per circuit, FMA below
  int auto_log2 = 16;
  if (const char* env = getenv("TEDQ_GB300_TN_AUTO_LOG2")) auto_log2 = atoi(env);
  const int n_meas = (int)p->nets.size();
  for (int m = 0; m < n_meas; ++m) {
    const TnNet& net = p->nets[m];
    const real* consts = static_cast<const real*>(D.consts) + p->const_base[m];
    if (!p->descs[m].empty()) {
      int32_t rc = timed(p, s, 0, 0.0, [&]() -> int32_t {
        TEDQ_CUDA("tedq_tn_contract: leaf kernel",
                  tn_build_leaves<real>(D.desc + p->desc_base[m], (int)p->descs[m].size(), params, p->n_params,
                                        batch, leaves, s));
        return TEDQ_OK;
      });
      if (rc != TEDQ_OK) return rc;
    }
    // gather operand: source weights of the element bits, slice offset and
    // the copy tiles (lowest source offsets and lowest element bits)
    auto gather_op = [&](const TnOperand& op, int64_t sl, TnGatherOp& o) {
      const TnTensor& T = net.tensors[op.tensor];
      std::memset(&o, 0, sizeof(o));
      o.nbits = op.nf + op.nc;
      const int64_t M = 1ll << T.lm, N = 1ll << T.ln, sj = T.split ? 2 * M : M;
      auto w = [&](int sbit) -> int64_t {
        if (T.leaf >= 0) return 2ll << sbit;
        return sbit < T.lm ? (1ll << sbit) : (sj << (sbit - T.lm));
      };
      if (T.leaf >= 0) {
        o.src = T.batched ? leaves + 2 * T.off * batch : consts + 2 * T.off;
        o.src_bstride = T.batched ? (2ll << T.full_idx.size()) : 0;
        o.src_im = 1;
        for (auto& qb : op.slice_bit) o.src_base += ((sl >> qb.first) & 1) ? w(qb.second) : 0;
      } else {
        o.src = T.batched ? arena_b + T.arena * batch : arena_u + T.arena;
        o.src_bstride = T.batched ? (2ll << (T.lm + T.ln)) : 0;
        o.src_im = T.split ? M : M * N;
      }
      for (int j = 0; j < o.nbits; ++j) o.sw[j] = w(op.src_bit[j]);
      o.nb = T.batched ? batch : 1;
      o.nc = op.nc;
      o.doubled = op.doubled ? 1 : 0;
      std::vector<int> by_src(o.nbits);
      for (int j = 0; j < o.nbits; ++j) by_src[j] = j;
      std::sort(by_src.begin(), by_src.end(), [&](int x, int y) { return o.sw[x] < o.sw[y]; });
      const int nlow = std::min(5, o.nbits);
      std::vector<int> tile, rd;
      for (int j = 0; j < nlow; ++j) tile.push_back(j);                       // written in order
      for (int q = 0; q < nlow; ++q)
        if (by_src[q] >= nlow) tile.push_back(by_src[q]);                     // read in order
      for (int q = 0; q < nlow; ++q) rd.push_back(by_src[q]);
      for (int j = 0; j < nlow; ++j)
        if (std::find(rd.begin(), rd.end(), j) == rd.end()) rd.push_back(j);
      o.tb = (int32_t)tile.size();
      for (int i = 0; i < o.tb; ++i) {
        o.tile_bit[i] = (int8_t)tile[i];
        o.r2w[i] = (int8_t)(std::find(tile.begin(), tile.end(), rd[i]) - tile.begin());
      }
      for (int j = 0; j < o.nbits; ++j)
        if (std::find(tile.begin(), tile.end(), j) == tile.end()) o.outer_bit[o.n_outer++] = (int8_t)j;
      // vector access (every offset involved is even, see TnGatherOp)
      o.rmode = T.leaf >= 0 ? 2 : ((o.tb >= 1 && o.sw[rd[0]] == 1 && T.lm >= 1) ? 1 : 0);
      o.wpair = (o.nc >= 1 && o.tb >= 1) ? 1 : 0;
    };
    // fused operand: per-bit offsets (reals) of the source storage
    auto fused_op = [&](const TnOperand& op, int64_t sl, TnFusedOp& o) {
      const TnTensor& T = net.tensors[op.tensor];
      const int64_t M = 1ll << T.lm, N = 1ll << T.ln;
      const int64_t sj = T.split ? 2 * M : M;
      auto w = [&](int sbit) -> int64_t {
        if (T.leaf >= 0) return 2ll << sbit;
        return sbit < T.lm ? (1ll << sbit) : (sj << (sbit - T.lm));
      };
      std::memset(&o, 0, sizeof(o));
      if (T.leaf >= 0) {
        o.src = T.batched ? leaves + 2 * T.off * batch : consts + 2 * T.off;
        o.bstride = T.batched ? (2ll << T.full_idx.size()) : 0;
        o.im = 1;
        for (auto& qb : op.slice_bit) o.base += ((sl >> qb.first) & 1) ? w(qb.second) : 0;
      } else {
        o.src = T.batched ? arena_b + T.arena * batch : arena_u + T.arena;
        o.bstride = T.batched ? (2ll << (T.lm + T.ln)) : 0;
        o.im = T.split ? M : M * N;
      }
      for (int j = 0; j < op.nc; ++j) o.wk[j] = w(op.src_bit[j]);
      for (int j = 0; j < op.nf; ++j) o.wf[j] = w(op.src_bit[op.nc + j]);
    };
    const int64_t n_slices = 1ll << net.sliced.size();
    const std::vector<TnLevelRun>& runs = D.runs[m];
    for (int64_t sl = 0; sl < n_slices; ++sl) {
      size_t next_run = 0;
      for (size_t si = 0; si < net.steps.size(); ++si) {
        const TnStep& stp = net.steps[si];
        if (stp.fused && next_run < runs.size() && runs[next_run].step0 == (int)si && runs[next_run].n_items > 0) {
          const TnLevelRun& run = runs[next_run++];
          int32_t rc = timed(p, s, 2, run.flops, [&]() -> int32_t {
            TEDQ_CUDA("tedq_tn_contract: fused level kernel",
                      tn_fused_level<real>(D.items + run.item0, run.n_items, run.blocks, ws, D.consts, sl, s));
            return TEDQ_OK;
          });
          if (rc != TEDQ_OK) return rc;
          si = run.step1 - 1;
          continue;
        }
        if (stp.fused) {
          if (next_run < runs.size() && runs[next_run].step0 == (int)si) ++next_run;
          const TnTensor& T = net.tensors[stp.out];
          TnFusedArgs F;
          std::memset(&F, 0, sizeof(F));
          fused_op(stp.opa, sl, F.a);
          fused_op(stp.opb, sl, F.b);
          F.lm = stp.opa.nf;
          F.ln = stp.opb.nf;
          F.lk = stp.opa.nc;
          if (F.lm > kTnMaxBits || F.ln > kTnMaxBits)
            return fail(TEDQ_ERR_UNSUPPORTED, "tedq_tn_contract: fused operand above 2^48 entries");
          F.nb = stp.batched ? batch : 1;
          F.dst = T.batched ? arena_b + T.arena * batch : arena_u + T.arena;
          F.dst_bstride = T.batched ? (2ll << (T.lm + T.ln)) : 0;
          const double flops = 8.0 * std::ldexp(1.0, F.lm + F.ln + F.lk) * (double)F.nb;
          int32_t rc = timed(p, s, 2, flops, [&]() -> int32_t {
            TEDQ_CUDA("tedq_tn_contract: fused kernel", tn_fused<real>(F, s));
            return TEDQ_OK;
          });
          if (rc != TEDQ_OK) return rc;
          continue;
        }
        TnGatherArgs A;
        std::memset(&A, 0, sizeof(A));
        const TnOperand* ops[2] = {&stp.opa, &stp.opb};
        for (int x = 0; x < 2; ++x) {
          if (ops[x]->nf + ops[x]->nc > 28)
            return fail(TEDQ_ERR_UNSUPPORTED, "tedq_tn_contract: GEMM operand above 2^28 entries (lower max_rank)");
          gather_op(*ops[x], sl, A.op[x]);
        }
        A.op[0].dst = scratch;
        A.op[1].dst = scratch + ((A.op[0].doubled ? 4ll : 2ll) << A.op[0].nbits) * A.op[0].nb;
        double gbytes = 0;
        for (int x = 0; x < 2; ++x) {
          const TnGatherOp& o = A.op[x];
          gbytes += (double)o.nb * (double)(1ll << o.nbits) * sizeof(real) * (o.doubled ? 6.0 : 4.0);
        }
        int32_t rc = timed(p, s, 1, gbytes, [&]() -> int32_t {
          TEDQ_CUDA("tedq_tn_contract: gather kernel", tn_gather<real>(A, s));
          return TEDQ_OK;
        });
        if (rc != TEDQ_OK) return rc;
        const TnTensor& T = net.tensors[stp.out];
        const long long M = 1ll << stp.opa.nf, N = 1ll << stp.opb.nf, K = 1ll << stp.opa.nc;
        real* C = T.batched ? arena_b + T.arena * batch : arena_u + T.arena;
        const int nbatch = stp.batched ? (int)batch : 1;
        // real embedding: [Re A, Im A] x [[Re B, Im B], [-Im B, Re B]] (B doubled) or
        // [[Re A, -Im A], [Im A, Re A]] x [Re B; Im B] (A doubled); K is doubled either way
        const long long mr = stp.double_a ? 2 * M : M, nr = stp.double_a ? N : 2 * N;
        TnGemmArgs G;
        G.a = A.op[0].dst;
        G.b = A.op[1].dst;
        G.c = C;
        G.mr = mr;
        G.nr = nr;
        G.kr = 2 * K;
        G.sa = A.op[0].nb > 1 ? mr * 2 * K : 0;
        G.sb = A.op[1].nb > 1 ? nr * 2 * K : 0;
        G.sc = 2 * M * N;
        G.nbatch = nbatch;
        G.err = D.err;
        // GEMM arithmetic: FP64 FMA (complex128); FP32 FMA; tensor cores with
        // one TF32 product (TF32) or the 3xTF32 split (TC32, AUTO above the
        // threshold) where the shape fills the tensor-core tiles
        int path = 0;  // 0 FMA, 1 3xTF32, 2 TF32
        if (!dbl && tn_gemm_tc_supported(G)) {
          if (p->gemm == TEDQ_TN_GEMM_TC32) path = 1;
          else if (p->gemm == TEDQ_TN_GEMM_TF32) path = 2;
          else if (p->gemm == TEDQ_TN_GEMM_AUTO && 8.0 * M * N * K >= std::ldexp(1.0, auto_log2)) path = 1;
        }
        rc = timed(p, s, path ? 4 : 2, 8.0 * M * N * K * nbatch, [&]() -> int32_t {
          TEDQ_CUDA("tedq_tn_contract: GEMM kernel",
                    path ? tn_gemm_tc(G, path == 1, s) : tn_gemm_simt<real>(G, s));
          return TEDQ_OK;
        });
        if (rc != TEDQ_OK) return rc;
      }
      const TnTensor& R = net.tensors[net.root];
      const real* root = R.batched ? arena_b + R.arena * batch : arena_u + R.arena;
      int32_t rc = timed(p, s, 3, 0.0, [&]() -> int32_t {
        TEDQ_CUDA("tedq_tn_contract: root kernel",
                  tn_root<real>(root, R.batched ? 2 : 0, batch, acc, out, n_meas, m, sl == 0, sl == n_slices - 1,
                                params, p->n_params, D.err, s));
        return TEDQ_OK;
      });
      if (rc != TEDQ_OK) return rc;
    }
  }
  return TEDQ_OK;
}

template <typename real>
int32_t contract(tedq_tn_plan* p, TnDevice& D, const void* params, int64_t batch, void* out, char* ws,
                 cudaStream_t s) {
  const real* prm = static_cast<const real*>(params);
  real* o = static_cast<real*>(out);
  const int32_t prc = prepare_items(p, D, batch);
  if (prc != TEDQ_OK) return prc;
  if (!p->graphs || p->profiling) return enqueue<real>(p, D, prm, batch, o, ws, s);
  const bool same = D.g_params == params && D.g_out == out && D.g_ws == ws && D.g_batch == batch;
  if (!same) {
    // new arguments: run eagerly, capture on the next call with the same ones
    if (D.exec) cudaGraphExecDestroy(D.exec);
    D.exec = nullptr;
    D.g_params = params;
    D.g_out = out;
    D.g_ws = ws;
    D.g_batch = batch;
    return enqueue<real>(p, D, prm, batch, o, ws, s);
  }
  if (!D.exec) {
    cudaGraph_t g = nullptr;
    TEDQ_CUDA("tedq_tn_contract: cudaStreamBeginCapture",
              cudaStreamBeginCapture(D.capture, cudaStreamCaptureModeThreadLocal));
    int32_t rc = enqueue<real>(p, D, prm, batch, o, ws, D.capture);
    cudaError_t e = cudaStreamEndCapture(D.capture, &g);
    if (rc != TEDQ_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail("tedq_tn_contract: cudaStreamEndCapture", e);
    e = cudaGraphInstantiate(&D.exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      D.exec = nullptr;
      return cuda_fail("tedq_tn_contract: cudaGraphInstantiate", e);
    }
  }
  TEDQ_CUDA("tedq_tn_contract: cudaGraphLaunch", cudaGraphLaunch(D.exec, s));
  return TEDQ_OK;
}

void release_devices(tedq_tn_plan* p) {
  int cur = 0;
  cudaGetDevice(&cur);
  for (int d = 0; d < 64; ++d) {
    TnDevice& D = p->dev[d];
    if (!D.err && !D.consts && !D.desc && !D.exec && !D.capture && !D.items) continue;
    cudaSetDevice(d);
    if (D.exec) cudaGraphExecDestroy(D.exec);
    if (D.capture) cudaStreamDestroy(D.capture);
    if (D.consts) cudaFree(D.consts);
    if (D.desc) cudaFree(D.desc);
    if (D.items) cudaFree(D.items);
    if (D.err) cudaFree(D.err);
    D = TnDevice();
  }
  cudaSetDevice(cur);
}

}  // namespace

extern "C" {

int32_t tedq_tn_plan_create(const tedq_gate_t* gates, int32_t n_gates, int32_t n_qubits, const tedq_meas_t* meas,
                            int32_t n_meas, const tedq_tn_options_t* opts, tedq_tn_plan_t** out) {
  if (!out) return fail(TEDQ_ERR_ARG, "tedq_tn_plan_create: out is null");
  *out = nullptr;
  if (n_meas < 1 || !meas) return fail(TEDQ_ERR_ARG, "tedq_tn_plan_create: no measurements");
  tedq_tn_plan* p = nullptr;
  try {
    p = new tedq_tn_plan();
    TnPlanOptions po;
    if (opts) {
      if (opts->precision != TEDQ_PREC_C64 && opts->precision != TEDQ_PREC_C128)
        throw std::invalid_argument("unknown precision");
      if (opts->gemm < TEDQ_TN_GEMM_FP32 || opts->gemm > TEDQ_TN_GEMM_AUTO)
        throw std::invalid_argument("unknown GEMM mode");
      // at most 2^28 entries per intermediate (32-bit tile offsets of the gathers)
      if (opts->max_rank < 0 || opts->max_rank > 28) throw std::invalid_argument("max_rank out of range [0, 28]");
      p->precision = opts->precision;
      p->gemm = opts->gemm;
      p->graphs = opts->graphs != 0;
      if (opts->max_rank) po.max_rank = opts->max_rank;
      if (opts->repeats > 0) po.repeats = opts->repeats;
      if (opts->seed) po.seed = opts->seed;
    }
    // tuning; at most 13 keeps every fused operand within the level-launch
    // item limits (16 free, 8 contracted bits)
    if (const char* env = getenv("TEDQ_GB300_TN_FUSED_LOG2")) po.fused_log2 = std::max(0, std::min(13, atoi(env)));
    if (const char* env = getenv("TEDQ_GB300_TN_SHORT_LOG2"))  // tuning, -1 = off
      po.fused_short_log2 = std::max(-1, std::min(8, atoi(env)));
    p->n = n_qubits;
    for (int i = 0; i < n_gates && gates; ++i)
      for (int j = 0; j < 3; ++j) p->n_params = std::max(p->n_params, gates[i].param_slot[j] + 1);
    for (int m = 0; m < n_meas; ++m) {
      p->nets.push_back(tn_build(gates, n_gates, n_qubits, meas[m], po));
      const TnNet& net = p->nets.back();
      std::vector<TnLeafDesc> d;
      for (int t = 0; t < net.n_leaves; ++t) {
        const TnTensor& T = net.tensors[t];
        if (!T.batched) continue;
        const TnGate& g = net.gates[T.gate];
        TnLeafDesc x;
        std::memset(&x, 0, sizeof(x));
        x.op = g.op;
        x.k = g.k;
        x.conj = T.leaf == TL_GATE_CONJ;
        for (int j = 0; j < 3; ++j) {
          x.slot[j] = g.slot[j];
          x.val[j] = g.val[j];
        }
        x.slot[3] = -1;
        x.off = T.off;
        d.push_back(x);
      }
      p->const_base.push_back(p->const_total);
      p->const_total += (int64_t)net.constants.size();
      p->desc_base.push_back(p->desc_total);
      p->desc_total += (int64_t)d.size();
      p->descs.push_back(std::move(d));
    }
    *out = p;
    return TEDQ_OK;
  } catch (const UnsupportedError& e) {
    delete p;
    return fail(TEDQ_ERR_UNSUPPORTED, std::string("tedq_tn_plan_create: ") + e.what());
  } catch (const std::bad_alloc&) {
    delete p;
    return fail(TEDQ_ERR_OOM, "tedq_tn_plan_create: out of host memory");
  } catch (const std::exception& e) {
    delete p;
    return fail(TEDQ_ERR_ARG, std::string("tedq_tn_plan_create: ") + e.what());
  }
}

int32_t tedq_tn_plan_destroy(tedq_tn_plan_t* plan) {
  if (!plan) return TEDQ_OK;
  release_devices(plan);
  delete plan;
  return TEDQ_OK;
}

int32_t tedq_tn_plan_info(const tedq_tn_plan_t* plan, tedq_tn_info_t* info) {
  if (!plan || !info) return fail(TEDQ_ERR_ARG, "tedq_tn_plan_info: null argument");
  std::memset(info, 0, sizeof(*info));
  info->n_qubits = plan->n;
  info->n_params = plan->n_params;
  info->n_meas = (int32_t)plan->nets.size();
  info->precision = plan->precision;
  double flops = 0;
  for (const TnNet& n : plan->nets) {
    info->n_steps += (int32_t)n.steps.size();
    info->max_rank = std::max(info->max_rank, n.max_rank);
    info->n_sliced = std::max(info->n_sliced, (int32_t)n.sliced.size());
    info->gates_kept += n.gates_kept;
    flops += std::exp2(n.log2_flops);
  }
  info->log2_flops = std::log2(flops);
  const Layout L1 = layout(plan, 1), L2 = layout(plan, 2);
  info->workspace_per_circuit = (int64_t)(L2.total - L1.total);
  info->workspace_fixed = (int64_t)L1.total - info->workspace_per_circuit;
  return TEDQ_OK;
}

int64_t tedq_tn_plan_describe(const tedq_tn_plan_t* plan, char* buf, int64_t len) {
  if (!plan) {
    fail(TEDQ_ERR_ARG, "tedq_tn_plan_describe: plan is null");
    return -1;
  }
  try {
    std::string s = tn_describe(plan->nets, plan->n_params, plan->precision);
    if (buf && len > 0) {
      int64_t k = std::min<int64_t>((int64_t)s.size(), len - 1);
      std::memcpy(buf, s.data(), (size_t)k);
      buf[k] = 0;
    }
    return (int64_t)s.size() + 1;
  } catch (const std::exception& e) {
    fail(TEDQ_ERR_OOM, std::string("tedq_tn_plan_describe: ") + e.what());
    return -1;
  }
}

int64_t tedq_tn_workspace_bytes(const tedq_tn_plan_t* plan, int64_t batch) {
  if (!plan || batch < 1) {
    fail(TEDQ_ERR_ARG, "tedq_tn_workspace_bytes: invalid argument");
    return -1;
  }
  return (int64_t)layout(plan, batch).total;
}

int32_t tedq_tn_contract(tedq_tn_plan_t* plan, const void* params, int64_t batch, void* out, void* workspace,
                         size_t workspace_bytes, void* stream) {
  if (!plan) return fail(TEDQ_ERR_ARG, "tedq_tn_contract: plan is null");
  if (batch < 1 || batch > (1ll << 30)) return fail(TEDQ_ERR_ARG, "tedq_tn_contract: batch out of range");
  if (plan->n_params > 0 && !params) return fail(TEDQ_ERR_ARG, "tedq_tn_contract: params is null");
  if (!out || !workspace) return fail(TEDQ_ERR_ARG, "tedq_tn_contract: out or workspace is null");
  if (reinterpret_cast<uintptr_t>(workspace) & 255)
    return fail(TEDQ_ERR_ARG, "tedq_tn_contract: workspace is not 256-byte aligned");
  const Layout L = layout(plan, batch);
  if (workspace_bytes < L.total)
    return fail(TEDQ_ERR_ARG, "tedq_tn_contract: workspace too small (" + std::to_string(L.total) + " bytes needed)");
  try {
    int dev = 0;
    TEDQ_CUDA("tedq_tn_contract: cudaGetDevice", cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(TEDQ_ERR_UNSUPPORTED, "tedq_tn_contract: device index above 63");
    std::lock_guard<std::mutex> lk(plan->mu);
    int32_t rc = ensure_device(plan, dev);
    if (rc != TEDQ_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    char* ws = static_cast<char*>(workspace);
    return plan->precision == TEDQ_PREC_C128
               ? contract<double>(plan, plan->dev[dev], params, batch, out, ws, s)
               : contract<float>(plan, plan->dev[dev], params, batch, out, ws, s);
  } catch (const std::bad_alloc&) {
    return fail(TEDQ_ERR_OOM, "tedq_tn_contract: out of host memory");
  } catch (const std::exception& e) {
    return fail(TEDQ_ERR_ARG, std::string("tedq_tn_contract: ") + e.what());
  }
}

int32_t tedq_tn_profile_enable(tedq_tn_plan_t* plan, int32_t on) {
  if (!plan) return fail(TEDQ_ERR_ARG, "tedq_tn_profile_enable: plan is null");
  std::lock_guard<std::mutex> lk(plan->mu);
  plan->profiling = on != 0;
  return TEDQ_OK;
}

int32_t tedq_tn_gemm(int32_t precision, int32_t gemm, const void* a, const void* b, void* c, int64_t mr, int64_t nr,
                     int64_t kr, int64_t sa, int64_t sb, int64_t sc, int64_t nbatch, int32_t* err_word, void* stream) {
  if (!a || !b || !c) return fail(TEDQ_ERR_ARG, "tedq_tn_gemm: null operand");
  if (mr < 1 || nr < 1 || kr < 1 || nbatch < 1 || nbatch > 65535 || sa < 0 || sb < 0 || sc < 0)
    return fail(TEDQ_ERR_ARG, "tedq_tn_gemm: sizes out of range");
  if (precision != TEDQ_PREC_C64 && precision != TEDQ_PREC_C128)
    return fail(TEDQ_ERR_ARG, "tedq_tn_gemm: unknown precision");
  if (gemm < TEDQ_TN_GEMM_FP32 || gemm > TEDQ_TN_GEMM_AUTO) return fail(TEDQ_ERR_ARG, "tedq_tn_gemm: unknown mode");
  TnGemmArgs G;
  G.a = a;
  G.b = b;
  G.c = c;
  G.mr = mr;
  G.nr = nr;
  G.kr = kr;
  G.sa = sa;
  G.sb = sb;
  G.sc = sc;
  G.nbatch = nbatch;
  G.err = err_word;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (precision == TEDQ_PREC_C128) {
    e = tn_gemm_simt<double>(G, s);
  } else if (gemm == TEDQ_TN_GEMM_FP32) {
    e = tn_gemm_simt<float>(G, s);
  } else {
    const bool tc = err_word && tn_gemm_tc_supported(G);
    if (!tc && gemm != TEDQ_TN_GEMM_AUTO)
      return fail(TEDQ_ERR_UNSUPPORTED, "tedq_tn_gemm: shape, alignment or missing error word rules out the "
                                        "tensor-core kernel");
    e = tc ? tn_gemm_tc(G, gemm != TEDQ_TN_GEMM_TF32, s) : tn_gemm_simt<float>(G, s);
  }
  if (e != cudaSuccess) return cuda_fail("tedq_tn_gemm", e);
  return TEDQ_OK;
}

int32_t tedq_tn_profile_read(tedq_tn_plan_t* plan, tedq_tn_profile_t* out) {
  if (!plan || !out) return fail(TEDQ_ERR_ARG, "tedq_tn_profile_read: null argument");
  std::vector<tedq_tn_plan::Ev> evs;
  {
    std::lock_guard<std::mutex> lk(plan->prof_mu);
    evs.swap(plan->events);
  }
  std::memset(out, 0, sizeof(*out));
  int32_t rc = TEDQ_OK;
  for (auto& e : evs) {
    float ms = 0;
    cudaError_t err = cudaEventSynchronize(e.b);
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e.a, e.b);
    if (err != cudaSuccess && rc == TEDQ_OK) rc = cuda_fail("tedq_tn_profile_read", err);
    switch (e.family) {
      case 0: out->leaf_launches++; out->leaf_ms += ms; break;
      case 1: out->gather_launches++; out->gather_ms += ms; out->gather_bytes += e.work; break;
      case 2: out->gemm_launches++; out->gemm_ms += ms; out->gemm_flops += e.work; break;
      case 4:
        out->gemm_launches++; out->gemm_ms += ms; out->gemm_flops += e.work;
        out->tc_launches++; out->tc_ms += ms; out->tc_flops += e.work;
        break;
      default: out->root_launches++; out->root_ms += ms; break;
    }
    cudaEventDestroy(e.a);
    cudaEventDestroy(e.b);
  }
  // error word of the tensor-core GEMMs on the current device
  int dev = 0;
  if (rc == TEDQ_OK && cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64 && plan->dev[dev].err) {
    int word = 0;
    cudaError_t e = cudaMemcpy(&word, plan->dev[dev].err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail("tedq_tn_profile_read", e);
    out->gemm_error = word;
    if (word) rc = fail(TEDQ_ERR_TIMEOUT, "tedq_tn_profile_read: a tensor-core GEMM gave up a bounded wait (code " +
                                             std::to_string(word) + "); its results are NaN");
  }
  return rc;
}

}  // extern "C"
