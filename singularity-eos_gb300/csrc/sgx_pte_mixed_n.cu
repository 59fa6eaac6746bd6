// One instantiation of the mixed-precision PTE kernels of pass 1 (one
// thread per cell, and one lane group per cell): SGX_PTE_N materials per
// cell (set by the build, one object per value).
// Pass 2 (the FP64 re-solve) is instantiated in sgx_pte_retry_n.cu.
// a mixed-precision path: bare models only (see sgx_dispatch.cuh)
#define SGX_BARE_MODELS
#include "sgx_pte_group.cuh"
#include "sgx_pte_mixed.cuh"

#ifndef SGX_PTE_N
#error "SGX_PTE_N must be defined"
#endif

namespace sgx {
template cudaError_t launch_pte_mixed_n<SGX_PTE_N>(const PteArgs &, cudaStream_t);
template cudaError_t launch_pte_group_n<SGX_PTE_N>(const PteArgs &, cudaStream_t);
} // namespace sgx
