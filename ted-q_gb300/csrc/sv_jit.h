// sv_jit.h -- per-circuit specialised pass kernels (internal).
//
// For a compiled program, jit_source() emits one CUDA kernel per pass of the
// forward and adjoint schedules in which every gate is a template instance of
// sv_device.cuh with its register bit, control mask and kind fixed at compile
// time.  jit_compile() builds them for sm_103a with NVRTC (loaded with dlopen,
// results cached on disk), jit_load() loads the cubin on the current device
// through the driver entry points the CUDA runtime exposes.  When any step is
// unavailable the caller keeps using the generic pass kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "sv_plan.h"

namespace tedq {

struct Program;

// One translation unit per pass kernel: tedq_fwd_<i> / tedq_bwd_<i>.
struct JitSource {
  std::string name;
  std::string src;
};
std::vector<JitSource> jit_sources(const Program& p);

// NVRTC compile of one source to a cubin for sm_103a; uses the on-disk cache.
// Returns false (with a message in `err`) when NVRTC is missing or fails.
bool jit_compile(const std::string& src, std::string& cubin, std::string& err);
// All sources, compiled on parallel host threads.
bool jit_compile_all(const std::vector<JitSource>& srcs, std::vector<std::string>& cubins, std::string& err);

struct JitKernels {
  std::vector<void*> modules;
  std::vector<void*> fwd, bwd;  // CUfunction per pass
};

// Loads the cubins on the current device and resolves the pass kernels.
bool jit_load(const std::vector<std::string>& cubins, const std::vector<JitSource>& srcs, int n_fwd, int n_bwd,
              JitKernels& out, std::string& err);

// One launch per pass: grid = (tiles of a state, circuits), chunked by the
// grid's y limit.
cudaError_t jit_launch_fwd(void* fn, bool dbl, const PassParams& P, void* psi, const void* params, int n_params,
                           const void* init, int64_t batch, cudaStream_t s);
cudaError_t jit_launch_bwd(void* fn, bool dbl, const PassParams& P, void* psi, void* lam, const void* params,
                           int n_params, double* grad_acc, int64_t batch, cudaStream_t s);

}  // namespace tedq
