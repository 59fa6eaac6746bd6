// Dispatch of the mixed-precision PTE kernels (one instantiation per
// material count, built from sgx_pte_mixed_n.cu).
#include <cuda_runtime.h>

#include "sgx_internal.h"

namespace sgx {

template <int N> cudaError_t launch_pte_mixed_n(const PteArgs &a, cudaStream_t stream);

cudaError_t launch_pte_mixed(const PteArgs &a, cudaStream_t stream) {
  if (a.ncell <= 0) return cudaSuccess;
  if (a.solver != SGX_PTE_RHOT) return cudaErrorNotSupported;
  const int lo = a.eos_idx ? 1 : a.nmat;
  const int hi = a.nmat < PTE_MAX_N ? a.nmat : PTE_MAX_N;
  cudaError_t e = cudaSuccess;
  for (int n = lo; n <= hi && e == cudaSuccess; ++n) {
    switch (n) {
    case 1: e = launch_pte_mixed_n<1>(a, stream); break;
    case 2: e = launch_pte_mixed_n<2>(a, stream); break;
    case 3: e = launch_pte_mixed_n<3>(a, stream); break;
    case 4: e = launch_pte_mixed_n<4>(a, stream); break;
    case 5: e = launch_pte_mixed_n<5>(a, stream); break;
    case 6: e = launch_pte_mixed_n<6>(a, stream); break;
    }
  }
  return e;
}

} // namespace sgx
