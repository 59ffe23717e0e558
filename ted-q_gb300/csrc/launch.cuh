// launch.cuh -- kernel launches through cudaLaunchKernel, so the status
// returned is the launch's own (cudaGetLastError after <<<>>> also reports
// stale errors of earlier calls).
#pragma once
#include <cuda_runtime.h>

#include <tuple>
#include <type_traits>
#include <utility>

namespace tedq {

template <typename... KArgs, size_t... I, typename Tup>
cudaError_t launch_with(void (*k)(KArgs...), dim3 g, dim3 b, size_t smem, cudaStream_t s, Tup& t,
                        std::index_sequence<I...>) {
  void* ptrs[sizeof...(KArgs) > 0 ? sizeof...(KArgs) : 1] = {static_cast<void*>(&std::get<I>(t))...};
  return cudaLaunchKernel(reinterpret_cast<const void*>(k), g, b, ptrs, smem, s);
}

template <typename... KArgs, typename... Actual>
cudaError_t launch_kernel(void (*k)(KArgs...), dim3 g, dim3 b, size_t smem, cudaStream_t s, Actual&&... a) {
  std::tuple<typename std::decay<KArgs>::type...> t(std::forward<Actual>(a)...);
  return launch_with(k, g, b, smem, s, t, std::index_sequence_for<KArgs...>{});
}

}  // namespace tedq
