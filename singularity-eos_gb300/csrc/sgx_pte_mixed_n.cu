// One instantiation of the mixed-precision per-cell PTE kernel: SGX_PTE_N
// materials per cell (set by the build, one object per value).
#include "sgx_pte_mixed.cuh"

#ifndef SGX_PTE_N
#error "SGX_PTE_N must be defined"
#endif

namespace sgx {
template cudaError_t launch_pte_mixed_n<SGX_PTE_N>(const PteArgs &, cudaStream_t);
template cudaError_t launch_pte_retry_n<SGX_PTE_N>(const PteArgs &, cudaStream_t);
} // namespace sgx
