// Stream-ordered scratch memory from a memory pool the library owns, one per
// device; and the launch-shape knobs an autotuner or a benchmark sets.
//
// Scratch: The pool keeps what it has reserved between calls (release
// threshold at its maximum), so a call that needs the same scratch as the
// one before it takes it from the pool instead of mapping device memory
// again; the device's default pool, whose threshold is zero, may return its
// memory at every synchronisation.
#include <atomic>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "sgx_internal.h"

namespace sgx {

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[MAX_DEVICES] = {};

cudaError_t pool_for(int dev, cudaMemPool_t *out) {
  if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pools[dev]) {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    cudaError_t e = cudaMemPoolCreate(&p, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) {
      cudaMemPoolDestroy(p);
      return e;
    }
    g_pools[dev] = p;
  }
  *out = g_pools[dev];
  return cudaSuccess;
}

} // namespace

cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t stream) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  cudaMemPool_t pool = nullptr;
  e = pool_for(dev, &pool);
  if (e != cudaSuccess) return e;
  return cudaMallocFromPoolAsync(p, bytes, pool, stream);
}

cudaError_t scratch_free(void *p, cudaStream_t stream) { return cudaFreeAsync(p, stream); }

namespace {
// knob -> {value, lowest, highest}
struct Knob {
  std::atomic<int> value;
  int lo, hi;
};
Knob g_knobs[] = {
    {{0}, 0, 0},
    {{5}, 4, 6}, // SGX_TUNE_LOOKUP_BLOCKS_PER_SM
    {{2}, 0, 2}, // SGX_TUNE_LOOKUP_STAGE
    {{0}, 0, 1}, // SGX_TUNE_L2_PERSIST
    {{0}, 0, 1}, // SGX_TUNE_HOST_FILL_STAGED
    {{8}, 2, 64},  // SGX_TUNE_PTE_FP32_ITERS
    {{8}, 4, 128},  // SGX_TUNE_PTE_RETRY_ITERS
};
constexpr int NKNOBS = sizeof(g_knobs) / sizeof(g_knobs[0]);
} // namespace

int tune_get(int knob) { return (knob > 0 && knob < NKNOBS) ? g_knobs[knob].value.load() : 0; }

} // namespace sgx

extern "C" int sgx_tune_set(int knob, int value) {
  using namespace sgx;
  if (knob <= 0 || knob >= NKNOBS) return set_error(SGX_ERR_INVALID, "sgx_tune_set: bad knob");
  if (value < g_knobs[knob].lo || value > g_knobs[knob].hi)
    return set_error(SGX_ERR_INVALID, "sgx_tune_set: value out of range");
  g_knobs[knob].value.store(value);
  return SGX_OK;
}

extern "C" int sgx_tune_get(int knob, int *value) {
  using namespace sgx;
  if (knob <= 0 || knob >= NKNOBS || !value)
    return set_error(SGX_ERR_INVALID, "sgx_tune_get: bad knob");
  *value = g_knobs[knob].value.load();
  return SGX_OK;
}
