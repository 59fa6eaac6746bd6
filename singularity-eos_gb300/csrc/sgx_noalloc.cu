// The mixed-precision PTE dispatch of sgx_mixed.cu with its scratch in a
// fixed device array of this module instead of pool memory.
//
// Who needs it: host codes that reserve, at start-up, all the device memory
// they will ever use for their own allocator and forbid allocations after
// that. For them the stream-ordered pool allocation inside the mixed path of
// sgx_pte_solve can fail, or break the memory budget they planned. Here the
// scratch -- the counter block with the signature histogram (153 KiB), the
// cell ids binned by material count and the retry queue, 8 bytes per cell --
// is a static __device__ array sized for SGX_PTE_NOALLOC_MAX_CELLS cells
// (8 MiB + 153 KiB), part of the module's image. No call here allocates device or pinned memory.
//
// The array's device address is looked up with the device current and
// cached per CUDA context: the first call in a context does the look-up
// (which also loads this module into that context) and should come before
// any stream capture begins. The cache is keyed on the context's unique id
// (cuCtxGetId), not on the device ordinal, so after cudaDeviceReset, or with
// another driver context made current on the same device, the next call looks
// the address up again instead of using one from a destroyed module image.
// There is one array per context, so calls that overlap in time on one device
// -- from two streams or two host threads -- race on it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "sgx_internal.h"

namespace {

constexpr size_t NOALLOC_IDS_BYTES =
    (static_cast<size_t>(SGX_PTE_NOALLOC_MAX_CELLS) * sizeof(int) + 255) / 256 * 256;
constexpr size_t NOALLOC_BINS = (sgx::PTE_BINS_BYTES + 255) / 256 * 256;
constexpr size_t NOALLOC_BYTES = NOALLOC_BINS + 2 * NOALLOC_IDS_BYTES;

} // namespace

static __device__ __align__(256) unsigned char sgx_pte_noalloc_scratch[NOALLOC_BYTES];

namespace sgx {

namespace {

// The current context's unique id through the driver entry points the
// runtime hands out (no link against libcuda); 0 when there is no current
// context yet.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

cudaError_t current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<CtxGetIdFn>(f);
  });
  if (!get_current || !get_id) return cudaErrorNotSupported;
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  *id = 0;
  if (ctx && get_id(ctx, id) != CUDA_SUCCESS) return cudaErrorDeviceUninitialized;
  return cudaSuccess;
}

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_scratch_mu;
struct ScratchEntry {
  unsigned long long ctx_id; // 0: not looked up
  char *ptr;
};
ScratchEntry g_scratch[NOALLOC_MAX_DEVICES];

cudaError_t scratch_on_current_device(char **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  unsigned long long id = 0;
  e = current_context_id(&id);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (id == 0 || g_scratch[dev].ctx_id != id) {
    // a new context (or none yet: the runtime creates the primary one
    // here), so the module image and its array are new too
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, sgx_pte_noalloc_scratch);
    if (e != cudaSuccess) return e;
    e = current_context_id(&id);
    if (e != cudaSuccess) return e;
    g_scratch[dev] = {id, static_cast<char *>(p)};
  }
  *out = g_scratch[dev].ptr;
  return cudaSuccess;
}

} // namespace

cudaError_t launch_pte_mixed_noalloc(const PteArgs &a, cudaStream_t stream) {
  if (a.ncell <= 0) return cudaSuccess;
  if (a.solver != SGX_PTE_RHOT) return cudaErrorNotSupported;
  if (a.ncell > SGX_PTE_NOALLOC_MAX_CELLS) return cudaErrorInvalidValue;
  char *p = nullptr;
  const cudaError_t e = scratch_on_current_device(&p);
  if (e != cudaSuccess) return e;
  PteArgs args = a;
  // launch_pte_mixed_with zeroes the counter block (bin counts, scatter
  // cursors, queue lengths) on the stream before its first kernel; the id
  // arrays are written before they are read and need no clearing.
  args.bins = reinterpret_cast<unsigned *>(p);
  args.retry_idx = reinterpret_cast<int *>(p + NOALLOC_BINS);
  int *perm = a.eos_idx ? reinterpret_cast<int *>(p + NOALLOC_BINS + NOALLOC_IDS_BYTES) : nullptr;
  return launch_pte_mixed_with(args, perm, stream);
}

} // namespace sgx
