// noalloc.cu -- forward entry point that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they run a
// circuit: code inside a CUDA stream capture, allocator or memory-pool
// callbacks, real-time loops that must not touch the allocator, or embedders
// whose device memory is owned by another runtime.  tedq_run_noalloc serves
// them: it is tedq_run with its workspace (the Pauli-term and probability
// accumulators) taken from a fixed static device array instead of a caller
// buffer.  The caller still passes parameters, the state buffer and the
// output buffer.
//
// Limits and rules:
//   * the static scratch is kStaticScratchBytes (1 MiB) per device; every GPU
//     that loads this library holds it until the process exits;
//   * the limit applies to the forward part of the workspace layout (the
//     Pauli-term and probability-bin accumulators, 8 bytes per term or bin
//     and circuit, each region rounded up to 256 bytes); the gradient region
//     that tedq_program_workspace_bytes also counts is not used here.  A call
//     whose batch needs more is rejected with TEDQ_ERR_ARG;
//   * the device address of the array is looked up with cudaGetSymbolAddress
//     on the first call on each device (with that device current); make that
//     first call before any stream capture;
//   * the per-circuit specialised pass kernels are used only when an earlier
//     tedq_run or tedq_run_adjoint of the program has loaded them on this
//     device; otherwise the generic pass kernels run.  This call never waits
//     for their compile and never loads a module (loading allocates device
//     memory for the code);
//   * every call shares the one array: accumulators are cleared on the stream
//     at the start of each call, and calls that overlap on the GPU (concurrent
//     streams, several host threads) race on it.
// No cudaMalloc, cudaFree or allocating library routine is called here.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "tedq_gb300.h"

int32_t tedq_record_error(int32_t status, const char* msg);
int64_t tedq_forward_workspace_bytes(const tedq_program_t* prog, int64_t batch);
int32_t tedq_run_forward_loaded_only(tedq_program_t* prog, const void* params, int64_t batch, void* psi,
                                     void* out_real, const void* init, void* workspace, size_t workspace_bytes,
                                     void* stream);

namespace {

constexpr size_t kStaticScratchBytes = size_t(1) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {nullptr};

}  // namespace

extern "C" int32_t tedq_run_noalloc(tedq_program_t* prog, const void* params, int64_t batch, void* psi,
                                    void* out_real, const void* init, void* stream) {
  if (!prog) return tedq_record_error(TEDQ_ERR_ARG, "tedq_run_noalloc: program is null");
  if (batch < 0) return tedq_record_error(TEDQ_ERR_ARG, "tedq_run_noalloc: negative batch");
  const int64_t need = tedq_forward_workspace_bytes(prog, batch);
  if (need < 0 || need > (int64_t)kStaticScratchBytes)
    return tedq_record_error(TEDQ_ERR_ARG, ("tedq_run_noalloc: batch of " + std::to_string(batch) + " needs " +
                                            std::to_string(need) + " bytes of forward workspace, more than the static " +
                                            std::to_string(kStaticScratchBytes) + " bytes")
                                               .c_str());
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return tedq_record_error(TEDQ_ERR_CUDA, (std::string("tedq_run_noalloc: cudaGetDevice: ") +
                                             cudaGetErrorString(e)).c_str());
  if (dev < 0 || dev >= kMaxDevices) return tedq_record_error(TEDQ_ERR_ARG, "tedq_run_noalloc: device index too large");
  void* ptr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      e = cudaGetSymbolAddress(&ptr, g_static_scratch);
      if (e != cudaSuccess)
        return tedq_record_error(TEDQ_ERR_CUDA, (std::string("tedq_run_noalloc: cudaGetSymbolAddress: ") +
                                                 cudaGetErrorString(e)).c_str());
      g_scratch_ptr[dev] = ptr;
    }
    ptr = g_scratch_ptr[dev];
  }
  return tedq_run_forward_loaded_only(prog, params, batch, psi, out_real, init, ptr, kStaticScratchBytes, stream);
}
