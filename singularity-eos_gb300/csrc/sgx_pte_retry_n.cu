// One instantiation of pass 2 of the mixed-precision PTE path, the FP64
// re-solve of the cells pass 1 queued: SGX_PTE_N materials per cell.
// Compiled with --fmad=false, like the plain path, so that its FP64
// iteration rounds as the reference does: a cell that does not converge
// then stops where the reference stops (most within 50 iterations) instead
// of wandering to the iteration cap.
// a mixed-precision path: bare models only (see sgx_dispatch.cuh)
#define SGX_BARE_MODELS
#include "sgx_pte_mixed.cuh"

#ifndef SGX_PTE_N
#error "SGX_PTE_N must be defined"
#endif

namespace sgx {
template cudaError_t launch_pte_retry_n<SGX_PTE_N>(const PteArgs &, cudaStream_t);
} // namespace sgx
