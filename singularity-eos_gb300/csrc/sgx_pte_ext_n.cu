// One instantiation of the FP64 per-cell kernels of PTESolverFixedT,
// PTESolverFixedP and PTESolverRhoU: SGX_PTE_N materials per cell (set by
// the build, one object per value). Compiled with --fmad=false.
#include "sgx_pte_kernel.cuh"

#ifndef SGX_PTE_N
#error "SGX_PTE_N must be defined"
#endif

namespace sgx {
template cudaError_t SGX_PTE_LAUNCHER(launch_pte_ext_n)<SGX_PTE_N>(const PteArgs &,
                                                          cudaStream_t);
} // namespace sgx
