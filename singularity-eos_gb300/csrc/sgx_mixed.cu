// Dispatch of the mixed-precision PTE kernels (one instantiation per
// material count, built from sgx_pte_mixed_n.cu): pass 1 for every material
// count, then pass 2 over the compacted retry queue.
//
// The queue (one int per cell plus a counter) is stream-ordered scratch from
// the device's default memory pool (cudaMallocAsync / cudaFreeAsync on the
// caller's stream), so concurrent calls on different streams never share it.
#include <cuda_runtime.h>

#include "sgx_internal.h"

namespace sgx {

template <int N> cudaError_t launch_pte_mixed_n(const PteArgs &a, cudaStream_t stream);
template <int N> cudaError_t launch_pte_retry_n(const PteArgs &a, cudaStream_t stream);

namespace {

template <bool RETRY> cudaError_t launch_n(const int n, const PteArgs &a, cudaStream_t s) {
  switch (n) {
  case 1: return RETRY ? launch_pte_retry_n<1>(a, s) : launch_pte_mixed_n<1>(a, s);
  case 2: return RETRY ? launch_pte_retry_n<2>(a, s) : launch_pte_mixed_n<2>(a, s);
  case 3: return RETRY ? launch_pte_retry_n<3>(a, s) : launch_pte_mixed_n<3>(a, s);
  case 4: return RETRY ? launch_pte_retry_n<4>(a, s) : launch_pte_mixed_n<4>(a, s);
  case 5: return RETRY ? launch_pte_retry_n<5>(a, s) : launch_pte_mixed_n<5>(a, s);
  case 6: return RETRY ? launch_pte_retry_n<6>(a, s) : launch_pte_mixed_n<6>(a, s);
  }
  return cudaSuccess;
}

} // namespace

cudaError_t launch_pte_mixed_with(const PteArgs &args, cudaStream_t stream) {
  const int lo = args.eos_idx ? 1 : args.nmat;
  const int hi = args.nmat < PTE_MAX_N ? args.nmat : PTE_MAX_N;
  cudaError_t e = cudaMemsetAsync(args.retry_count, 0, sizeof(unsigned), stream);
  for (int n = lo; n <= hi && e == cudaSuccess; ++n)
    e = launch_n<false>(n, args, stream);
  for (int n = lo; n <= hi && e == cudaSuccess; ++n)
    e = launch_n<true>(n, args, stream);
  return e;
}

cudaError_t launch_pte_mixed(const PteArgs &a, cudaStream_t stream) {
  if (a.ncell <= 0) return cudaSuccess;
  if (a.solver != SGX_PTE_RHOT) return cudaErrorNotSupported;
  if (a.ncell > 0x7fffffffLL) return cudaErrorInvalidValue; // queue holds int32 cell ids
  PteArgs args = a;
  void *scratch = nullptr;
  const size_t bytes = 256 + static_cast<size_t>(a.ncell) * sizeof(int);
  cudaError_t e = cudaMallocAsync(&scratch, bytes, stream);
  if (e != cudaSuccess) return e;
  args.retry_count = static_cast<unsigned *>(scratch);
  args.retry_idx = reinterpret_cast<int *>(static_cast<char *>(scratch) + 256);
  e = launch_pte_mixed_with(args, stream);
  const cudaError_t f = cudaFreeAsync(scratch, stream);
  return e != cudaSuccess ? e : f;
}

} // namespace sgx
