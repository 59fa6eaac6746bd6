// Mixed-precision kernels (FP32 iterations, FP64 refinement).
#include <cuda_runtime.h>

#include "sgx_internal.h"

namespace sgx {

cudaError_t launch_pte_mixed(const PteArgs &, cudaStream_t) { return cudaErrorNotSupported; }

} // namespace sgx
