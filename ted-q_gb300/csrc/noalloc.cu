// noalloc.cu -- forward entry point that allocates nothing.
//
// Some callers cannot allocate device memory at the point where they run a
// circuit: code inside a CUDA stream capture, allocator or memory-pool
// callbacks, real-time loops that must not touch the allocator, or embedders
// whose device memory is owned by another runtime.  tedq_run_noalloc serves
// them: it is tedq_run with its workspace (the Pauli-term, probability and
// gradient accumulators) taken from a fixed static device array instead of a
// caller buffer.  The caller still passes parameters, the state buffer and the
// output buffer.
//
// Limits and rules:
//   * the static scratch is kStaticScratchBytes (1 MiB) per device; every GPU
//     that loads this library holds it until the process exits;
//   * a call whose batch needs more workspace than that is rejected with
//     TEDQ_ERR_ARG (tedq_program_workspace_bytes(prog, batch) tells the need);
//   * the device address of the array is looked up with cudaGetSymbolAddress
//     on the first call on each device (with that device current); make that
//     first call before any stream capture;
//   * every call shares the one array: accumulators are cleared on the stream
//     at the start of each call, and calls that overlap on the GPU (concurrent
//     streams, several host threads) race on it.
// No cudaMalloc, cudaFree or allocating library routine is called here.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "tedq_gb300.h"

int32_t tedq_record_error(int32_t status, const char* msg);

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
  const int64_t need = tedq_program_workspace_bytes(prog, batch < 0 ? 0 : batch);
  if (need < 0 || need > (int64_t)kStaticScratchBytes)
    return tedq_record_error(TEDQ_ERR_ARG, ("tedq_run_noalloc: batch of " + std::to_string(batch) + " needs " +
                                            std::to_string(need) + " bytes of workspace, more than the static " +
                                            std::to_string(kStaticScratchBytes) + " bytes")
                                               .c_str());
  return tedq_run(prog, params, batch, psi, out_real, init, ptr, kStaticScratchBytes, stream);
}
