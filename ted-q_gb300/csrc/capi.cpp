// capi.cpp -- the extern "C" boundary (include/tedq_gb300.h).
//
// Every entry point validates its arguments, converts C++ exceptions into a
// tedq_status and records a message retrievable with tedq_last_error()
// (thread-local).  Kernels are launched asynchronously on the caller's stream;
// launch errors are reported, execution errors surface at the caller's next
// synchronisation.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <future>
#include <mutex>
#include <new>
#include <tuple>
#include <stdexcept>
#include <string>
#include <vector>

#include "sv_jit.h"
#include "sv_kernels.cuh"
#include "sv_program.h"
#include "tedq_gb300.h"

using namespace tedq;

struct ProfEvent {
  cudaEvent_t a, b;
  int family;  // 0 fwd, 1 bwd, 2 meas, 3 lambda
  int64_t amp_passes;
};

struct tedq_program {
  Program* p = nullptr;
  TermTable terms;
  OutTermTable outs;
  ProbsTable probs;
  bool profiling = false;
  std::vector<ProfEvent> events;
  // specialised kernels: compiled in the background from program creation,
  // loaded per device on first use
  bool jit_on = false;
  bool jit_background = false;  // use the generic kernels until compiled
  int jit_state = 0;  // 0 off, 1 compiling, 2 compiled, 3 loaded, -1 failed
  std::future<std::tuple<bool, std::vector<std::string>, std::string>> jit_future;
  std::vector<JitSource> jit_srcs;
  std::vector<std::string> jit_cubins;
  std::string jit_err;
  std::mutex jit_mu;
  JitKernels jit_dev[64];
  bool jit_tried[64] = {false};
};

namespace {

thread_local std::string g_err;

int32_t fail(int32_t status, const std::string& msg) {
  g_err = msg;
  return status;
}

int32_t cuda_fail(cudaError_t e, const char* where) {
  std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess && pending != e)
    msg += std::string(" (earlier error pending in this thread: ") + cudaGetErrorString(pending) + ")";
  return fail(TEDQ_ERR_CUDA, msg);
}

// Launch wrapper: with profiling on, brackets the launch with an event pair.
template <typename F>
cudaError_t timed(tedq_program* h, int family, int64_t amp_passes, cudaStream_t s, F&& launch) {
  if (!h->profiling) return launch();
  ProfEvent ev{nullptr, nullptr, family, amp_passes};
  cudaError_t e = cudaEventCreate(&ev.a);
  if (e != cudaSuccess) return e;
  e = cudaEventCreate(&ev.b);
  if (e != cudaSuccess) return e;
  cudaEventRecord(ev.a, s);
  e = launch();
  cudaEventRecord(ev.b, s);
  h->events.push_back(ev);
  return e;
}

// Waits for the background compile; returns true when a cubin is available.
bool jit_compiled(tedq_program* h, bool block = true) {
  if (!h->jit_on) return false;
  if (h->jit_state == 1 && !block &&
      h->jit_future.wait_for(std::chrono::seconds(0)) != std::future_status::ready)
    return false;
  if (h->jit_state == 1) {
    auto r = h->jit_future.get();
    if (std::get<0>(r)) {
      h->jit_cubins = std::move(std::get<1>(r));
      h->jit_state = 2;
    } else {
      h->jit_err = std::get<2>(r);
      h->jit_state = -1;
      fprintf(stderr, "tedq_gb300: specialised kernels unavailable, using generic kernels: %s\n",
              h->jit_err.substr(0, 300).c_str());
    }
  }
  return h->jit_state >= 2;
}

// The specialised kernels of the current device, or nullptr (generic kernels).
JitKernels* jit_kernels(tedq_program* h) {
  if (!h->jit_on) return nullptr;
  std::lock_guard<std::mutex> lock(h->jit_mu);
  if (!jit_compiled(h, !h->jit_background)) return nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!h->jit_tried[dev]) {
    h->jit_tried[dev] = true;
    std::string err;
    if (jit_load(h->jit_cubins, h->jit_srcs, (int)h->p->fwd.passes.size(), (int)h->p->bwd.passes.size(),
                 h->jit_dev[dev], err)) {
      h->jit_state = 3;
    } else {
      h->jit_dev[dev] = JitKernels();
      fprintf(stderr, "tedq_gb300: loading specialised kernels failed, using generic kernels: %s\n", err.c_str());
    }
  }
  JitKernels& k = h->jit_dev[dev];
  return k.modules.empty() ? nullptr : &k;
}

// The specialised kernels of the current device if an earlier call has
// already loaded them, else nullptr: never waits for the compile and never
// loads a module (loading allocates device memory for the code).
JitKernels* jit_kernels_if_loaded(tedq_program* h) {
  if (!h->jit_on) return nullptr;
  std::lock_guard<std::mutex> lock(h->jit_mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!h->jit_tried[dev]) return nullptr;
  JitKernels& k = h->jit_dev[dev];
  return k.modules.empty() ? nullptr : &k;
}

int64_t align256(int64_t v) { return (v + 255) & ~int64_t(255); }

struct WsLayout {
  int64_t terms, w, probs, grad, total;
};

WsLayout ws_layout(const Program& p, int64_t batch) {
  WsLayout L;
  const int64_t S = (int64_t)p.terms.size();
  L.terms = 0;
  L.w = align256(L.terms + batch * S * 8);
  L.probs = align256(L.w + batch * S * 8);
  L.grad = align256(L.probs + batch * (int64_t)p.n_probs_bins * 8);
  L.total = align256(L.grad + batch * (int64_t)p.n_params * 8);
  return L;
}

void build_tables(tedq_program* h) {
  const Program& p = *h->p;
  std::memset(&h->terms, 0, sizeof(h->terms));
  std::memset(&h->outs, 0, sizeof(h->outs));
  std::memset(&h->probs, 0, sizeof(h->probs));
  if ((int)p.terms.size() > kMaxTerms)
    throw UnsupportedError("more than " + std::to_string(kMaxTerms) + " distinct Pauli strings measured");
  if ((int)p.out_terms.size() > kMaxOutTerms)
    throw UnsupportedError("observable expansion exceeds " + std::to_string(kMaxOutTerms) + " terms");
  if ((int)p.probs.size() > kMaxProbsOut)
    throw UnsupportedError("more than " + std::to_string(kMaxProbsOut) + " probs measurements");
  h->terms.n = (int)p.terms.size();
  for (size_t i = 0; i < p.terms.size(); ++i) {
    h->terms.t[i].x = p.terms[i].x;
    h->terms.t[i].z = p.terms[i].z;
    h->terms.t[i].ny = __builtin_popcountll(p.terms[i].x & p.terms[i].z);
  }
  h->outs.n = (int)p.out_terms.size();
  h->outs.n_real = p.n_real;
  h->outs.n_terms = (int)p.terms.size();
  for (size_t i = 0; i < p.out_terms.size(); ++i) {
    h->outs.k[i] = p.out_terms[i].k;
    h->outs.s[i] = p.out_terms[i].s;
    h->outs.coef[i] = p.out_terms[i].coef;
  }
  h->probs.n = (int)p.probs.size();
  h->probs.n_bins = p.n_probs_bins;
  h->probs.pad_bits = p.pad;
  int acc = 0;
  for (size_t i = 0; i < p.probs.size(); ++i) {
    ProbsDesc& d = h->probs.p[i];
    d.offset = p.probs[i].offset;
    d.nbits = (int)p.probs[i].bits.size();
    d.full = d.nbits == p.n ? 1 : 0;
    d.acc_off = d.full ? 0 : acc;
    if (!d.full) acc += 1 << d.nbits;
    for (int j = 0; j < d.nbits; ++j) d.bits[j] = (uint8_t)p.probs[i].bits[j];
  }
}

}  // namespace

extern "C" {

int32_t tedq_abi_version(void) { return TEDQ_ABI_VERSION; }

int32_t tedq_last_error(char* buf, size_t len) {
  if (buf && len) {
    size_t n = g_err.size() < len - 1 ? g_err.size() : len - 1;
    std::memcpy(buf, g_err.data(), n);
    buf[n] = 0;
  }
  return (int32_t)g_err.size();
}

int32_t tedq_program_create(const tedq_gate_t* gates, int32_t n_gates, int32_t n_qubits, const tedq_meas_t* meas,
                            int32_t n_meas, const tedq_options_t* opts, tedq_program_t** out) {
  if (!out) return fail(TEDQ_ERR_ARG, "tedq_program_create: out is null");
  *out = nullptr;
  tedq_program* h = nullptr;
  try {
    h = new tedq_program();
    h->p = compile_program(gates, n_gates, n_qubits, meas, n_meas, opts);
    build_tables(h);
    const char* env = getenv("TEDQ_GB300_JIT");
    const int mode = opts ? opts->jit : 0;
    h->jit_on = mode > 0 || (mode == 0 && h->p->ns >= 14);
    h->jit_background = mode == 2;
    if (env && env[0] == '0') h->jit_on = false;
    if (h->jit_on) {
      h->jit_state = 1;
      h->jit_srcs = jit_sources(*h->p);
      const std::vector<JitSource>* srcs = &h->jit_srcs;
      h->jit_future = std::async(std::launch::async, [srcs]() {
        std::vector<std::string> cubins;
        std::string err;
        bool ok = jit_compile_all(*srcs, cubins, err);
        return std::make_tuple(ok, std::move(cubins), std::move(err));
      });
    }
    *out = h;
    return TEDQ_OK;
  } catch (const UnsupportedError& e) {
    if (h) delete h->p;
    delete h;
    return fail(TEDQ_ERR_UNSUPPORTED, std::string("tedq_program_create: ") + e.what());
  } catch (const std::bad_alloc&) {
    if (h) delete h->p;
    delete h;
    return fail(TEDQ_ERR_OOM, "tedq_program_create: out of host memory");
  } catch (const std::exception& e) {
    if (h) delete h->p;
    delete h;
    return fail(TEDQ_ERR_ARG, std::string("tedq_program_create: ") + e.what());
  }
}

int32_t tedq_program_destroy(tedq_program_t* prog) {
  if (!prog) return TEDQ_OK;
  if (prog->jit_future.valid()) prog->jit_future.wait();
  for (auto& ev : prog->events) {
    cudaEventDestroy(ev.a);
    cudaEventDestroy(ev.b);
  }
  delete prog->p;
  delete prog;
  return TEDQ_OK;
}

int32_t tedq_program_info(const tedq_program_t* prog, tedq_program_info_t* info) {
  if (!prog || !info) return fail(TEDQ_ERR_ARG, "tedq_program_info: null argument");
  const Program& p = *prog->p;
  std::memset(info, 0, sizeof(*info));
  info->n_qubits = p.n;
  info->state_qubits = p.ns;
  info->n_params = p.n_params;
  info->n_real_outputs = p.n_real;
  info->n_terms = (int32_t)p.terms.size();
  info->n_fwd_passes = (int32_t)p.fwd.passes.size();
  info->n_bwd_passes = (int32_t)p.bwd.passes.size();
  info->n_fwd_phases = p.fwd.n_phases;
  info->n_bwd_phases = p.bwd.n_phases;
  info->n_fused_gates = (int32_t)p.fused.size();
  info->n_elem_gates = (int32_t)p.elem.size();
  info->precision = p.precision;
  info->workspace_per_circuit = ws_layout(p, 1).total;
  info->jit_state = prog->jit_state;
  int64_t loaded = 0;
  for (const JitKernels& k : prog->jit_dev) loaded += (int64_t)k.modules.size();
  info->jit_modules_loaded = loaded;
  return TEDQ_OK;
}

int32_t tedq_program_jit_wait(tedq_program_t* prog) {
  if (!prog) return fail(TEDQ_ERR_ARG, "tedq_program_jit_wait: program is null");
  if (!prog->jit_on) return fail(TEDQ_ERR_UNSUPPORTED, "tedq_program_jit_wait: specialised kernels are off");
  std::lock_guard<std::mutex> lock(prog->jit_mu);
  if (!jit_compiled(prog)) return fail(TEDQ_ERR_UNSUPPORTED, "tedq_program_jit_wait: " + prog->jit_err);
  return TEDQ_OK;
}

int64_t tedq_program_workspace_bytes(const tedq_program_t* prog, int64_t batch) {
  if (!prog || batch < 0) return -1;
  return ws_layout(*prog->p, batch).total;
}

int64_t tedq_program_describe(const tedq_program_t* prog, int32_t adjoint, char* buf, int64_t len) {
  if (!prog) return -1;
  std::string s = describe_schedule(*prog->p, adjoint != 0);
  if (buf && len > 0) {
    int64_t n = (int64_t)s.size() < len - 1 ? (int64_t)s.size() : len - 1;
    std::memcpy(buf, s.data(), (size_t)n);
    buf[n] = 0;
  }
  return (int64_t)s.size() + 1;
}

}  // extern "C"

namespace {

// The forward of tedq_run.  forward_only: the workspace needs only the
// forward accumulators (Pauli terms and probability bins, the layout's bytes
// before the gradient region) and the specialised kernels are used only when
// already loaded on this device (no compile wait, no module load: the
// allocation-free entry point).
int32_t run_forward(tedq_program_t* prog, const void* params, int64_t batch, void* psi, void* out_real,
                    const void* init, void* workspace, size_t workspace_bytes, void* stream, bool forward_only) {
  if (!prog) return fail(TEDQ_ERR_ARG, "tedq_run: program is null");
  const Program& p = *prog->p;
  if (batch < 0) return fail(TEDQ_ERR_ARG, "tedq_run: negative batch");
  if (batch == 0) return TEDQ_OK;
  if (!psi) return fail(TEDQ_ERR_ARG, "tedq_run: psi is null");
  if (p.n_params > 0 && !params) return fail(TEDQ_ERR_ARG, "tedq_run: params is null");
  if (p.n_real > 0 && !out_real) return fail(TEDQ_ERR_ARG, "tedq_run: out_real is null");
  const WsLayout L = ws_layout(p, batch);
  const bool need_ws = !p.terms.empty() || p.n_probs_bins > 0;
  const int64_t ws_need = forward_only ? L.grad : L.total;
  if (need_ws && (!workspace || (int64_t)workspace_bytes < ws_need))
    return fail(TEDQ_ERR_ARG, "tedq_run: workspace smaller than tedq_program_workspace_bytes(batch) = " +
                                  std::to_string(L.total));
  if (workspace && (reinterpret_cast<uintptr_t>(workspace) & 255))
    return fail(TEDQ_ERR_ARG, "tedq_run: workspace must be 256-byte aligned");
  if (reinterpret_cast<uintptr_t>(psi) & 15) return fail(TEDQ_ERR_ARG, "tedq_run: psi must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool dbl = p.precision == TEDQ_PREC_C128;
  cudaError_t e;
  if (p.fwd.passes.empty()) {
    e = timed(prog, 0, 0, s, [&] { return launch_init_state(dbl, p.ns, p.pad, psi, init, batch, s); });
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run/init");
  }
  JitKernels* jk = p.fwd.passes.empty() ? nullptr : forward_only ? jit_kernels_if_loaded(prog) : jit_kernels(prog);
  // From |0...0> the passes skip all-zero tiles (PassParams::zero_outer): the
  // state is cleared first so that the skipped amplitudes read as zero.  A
  // given initial state has no zero tiles to count on.
  if (!init && !p.fwd.passes.empty() && p.fwd.passes[0].zero_outer) {
    e = cudaMemsetAsync(psi, 0, (size_t)(batch << p.ns) * (dbl ? 16 : 8), s);
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run/memset");
  }
  for (size_t i = 0; i < p.fwd.passes.size(); ++i) {
    PassParams P = p.fwd.passes[i];
    if (init) P.zero_outer = 0;
    if (i == 0) {
      P.init = init ? 2 : 1;
      P.pad_bits = (uint8_t)p.pad;
    }
    const void* ini = i == 0 ? init : nullptr;
    e = timed(prog, 0, batch << p.ns, s, [&] {
      return jk ? jit_launch_fwd(jk->fwd[i], dbl, P, psi, params, p.n_params, ini, batch, s)
                : launch_fwd_pass(dbl, P, psi, params, p.n_params, ini, batch, s);
    });
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run/pass");
  }
  char* ws = static_cast<char*>(workspace);
  double* term_acc = need_ws ? reinterpret_cast<double*>(ws + L.terms) : nullptr;
  double* probs_acc = need_ws ? reinterpret_cast<double*>(ws + L.probs) : nullptr;
  if (!p.terms.empty()) {
    e = cudaMemsetAsync(term_acc, 0, (size_t)batch * p.terms.size() * 8, s);
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run/memset");
    e = timed(prog, 2, 0, s, [&] { return launch_expval(dbl, p.ns, prog->terms, psi, term_acc, batch, s); });
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run/expval");
  }
  if (!p.probs.empty()) {
    if (p.n_probs_bins > 0) {
      e = cudaMemsetAsync(probs_acc, 0, (size_t)batch * p.n_probs_bins * 8, s);
      if (e != cudaSuccess) return cuda_fail(e, "tedq_run/memset");
    }
    e = timed(prog, 2, 0, s,
              [&] { return launch_probs(dbl, p.ns, prog->probs, psi, probs_acc, out_real, p.n_real, batch, s); });
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run/probs");
  }
  if (p.n_real > 0) {
    e = timed(prog, 2, 0, s,
              [&] { return launch_finalize(dbl, prog->outs, prog->probs, term_acc, probs_acc, out_real, batch, s); });
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run/finalize");
  }
  return TEDQ_OK;
}

}  // namespace

extern "C" {

int32_t tedq_run(tedq_program_t* prog, const void* params, int64_t batch, void* psi, void* out_real,
                 const void* init, void* workspace, size_t workspace_bytes, void* stream) {
  return run_forward(prog, params, batch, psi, out_real, init, workspace, workspace_bytes, stream, false);
}

int32_t tedq_run_adjoint(tedq_program_t* prog, const void* params, int64_t batch, const void* dy_real,
                         const void* dy_state, void* psi, void* lambda_, void* grad, void* workspace,
                         size_t workspace_bytes, void* stream) {
  if (!prog) return fail(TEDQ_ERR_ARG, "tedq_run_adjoint: program is null");
  const Program& p = *prog->p;
  if (batch < 0) return fail(TEDQ_ERR_ARG, "tedq_run_adjoint: negative batch");
  if (batch == 0 || p.n_params == 0) return TEDQ_OK;
  if (!psi || !lambda_ || !grad || !params) return fail(TEDQ_ERR_ARG, "tedq_run_adjoint: null buffer");
  const WsLayout L = ws_layout(p, batch);
  if (!workspace || (int64_t)workspace_bytes < L.total)
    return fail(TEDQ_ERR_ARG, "tedq_run_adjoint: workspace smaller than tedq_program_workspace_bytes(batch) = " +
                                  std::to_string(L.total));
  if (reinterpret_cast<uintptr_t>(workspace) & 255)
    return fail(TEDQ_ERR_ARG, "tedq_run_adjoint: workspace must be 256-byte aligned");
  if ((reinterpret_cast<uintptr_t>(psi) | reinterpret_cast<uintptr_t>(lambda_)) & 15)
    return fail(TEDQ_ERR_ARG, "tedq_run_adjoint: psi/lambda must be 16-byte aligned");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const bool dbl = p.precision == TEDQ_PREC_C128;
  char* ws = static_cast<char*>(workspace);
  double* w = reinterpret_cast<double*>(ws + L.w);
  double* grad_acc = reinterpret_cast<double*>(ws + L.grad);
  cudaError_t e = cudaMemsetAsync(grad_acc, 0, (size_t)batch * p.n_params * 8, s);
  if (e != cudaSuccess) return cuda_fail(e, "tedq_run_adjoint/memset");
  if (!p.terms.empty()) {
    e = timed(prog, 3, 0, s, [&] { return launch_term_weights(dbl, prog->outs, dy_real, w, batch, s); });
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run_adjoint/weights");
  }
  e = timed(prog, 3, 0, s, [&] {
    return launch_lambda_init(dbl, p.ns, prog->terms, prog->probs, w, dy_real, p.n_real, dy_state, psi, lambda_,
                              batch, s);
  });
  if (e != cudaSuccess) return cuda_fail(e, "tedq_run_adjoint/lambda");
  JitKernels* jk = jit_kernels(prog);
  for (size_t i = 0; i < p.bwd.passes.size(); ++i) {
    const PassParams& P = p.bwd.passes[i];
    e = timed(prog, 1, batch << p.ns, s, [&] {
      return jk ? jit_launch_bwd(jk->bwd[i], dbl, P, psi, lambda_, params, p.n_params, grad_acc, batch, s)
                : launch_bwd_pass(dbl, P, psi, lambda_, params, p.n_params, grad_acc, batch, s);
    });
    if (e != cudaSuccess) return cuda_fail(e, "tedq_run_adjoint/pass");
  }
  e = timed(prog, 3, 0, s, [&] { return launch_grad_finalize(dbl, grad_acc, grad, batch * p.n_params, s); });
  if (e != cudaSuccess) return cuda_fail(e, "tedq_run_adjoint/finalize");
  return TEDQ_OK;
}

int32_t tedq_profile_enable(tedq_program_t* prog, int32_t on) {
  if (!prog) return fail(TEDQ_ERR_ARG, "tedq_profile_enable: program is null");
  prog->profiling = on != 0;
  return TEDQ_OK;
}

int32_t tedq_profile_read(tedq_program_t* prog, tedq_profile_t* out) {
  if (!prog || !out) return fail(TEDQ_ERR_ARG, "tedq_profile_read: null argument");
  std::memset(out, 0, sizeof(*out));
  int32_t status = TEDQ_OK;
  for (auto& ev : prog->events) {
    float ms = 0.f;
    cudaError_t e = cudaEventSynchronize(ev.b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ev.a, ev.b);
    if (e != cudaSuccess) status = cuda_fail(e, "tedq_profile_read");
    switch (ev.family) {
      case 0: out->fwd_launches++; out->fwd_ms += ms; out->fwd_amp_passes += ev.amp_passes; break;
      case 1: out->bwd_launches++; out->bwd_ms += ms; out->bwd_amp_passes += ev.amp_passes; break;
      case 2: out->meas_launches++; out->meas_ms += ms; break;
      default: out->lam_launches++; out->lam_ms += ms; break;
    }
    cudaEventDestroy(ev.a);
    cudaEventDestroy(ev.b);
  }
  prog->events.clear();
  return status;
}

}  // extern "C"

// Records an error message for tedq_last_error from other translation units
// of this library (C++ linkage, not part of the public ABI).
int32_t tedq_record_error(int32_t status, const char* msg) { return fail(status, msg ? msg : ""); }

// Forward workspace (bytes before the gradient region of the layout) and the
// forward that never loads kernels, for the allocation-free entry point
// (C++ linkage, not part of the public ABI).
int64_t tedq_forward_workspace_bytes(const tedq_program_t* prog, int64_t batch) {
  if (!prog || batch < 0) return -1;
  return ws_layout(*prog->p, batch).grad;
}
int32_t tedq_run_forward_loaded_only(tedq_program_t* prog, const void* params, int64_t batch, void* psi,
                                     void* out_real, const void* init, void* workspace, size_t workspace_bytes,
                                     void* stream) {
  return run_forward(prog, params, batch, psi, out_real, init, workspace, workspace_bytes, stream, true);
}
