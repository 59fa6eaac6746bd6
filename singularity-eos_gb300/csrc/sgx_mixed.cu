// Dispatch of the mixed-precision PTE kernels (one instantiation per
// material count, built from sgx_pte_mixed_n.cu).
//
// With an index map (cells holding different numbers of materials), the
// cells are first binned by material count and, within a count, by the
// ordered EOS kinds of their materials -- a counting kernel, a scan of the
// signature histogram and a scatter of cell ids into perm[] -- so that each
// per-count kernel runs full warps whose lanes take the same EOS branches.
// Then, for each count N in turn: pass 1 (FP32 solve + FP64
// refinement) over the N-bin on the caller's stream, and pass 2 (FP64
// re-solve) over the cells pass 1 queued on a side stream, overlapping the
// next counts' pass 1.
//
// The scratch (the counter block, perm[ncell], retry_idx[ncell]) is
// stream-ordered memory from the library's pool (scratch_alloc /
// scratch_free on the caller's stream), so calls on different streams never
// share it.
// a mixed-precision path: bare models only (see sgx_dispatch.cuh)
#define SGX_BARE_MODELS
#include <mutex>

#include <cuda_runtime.h>

#include "sgx_internal.h"

namespace sgx {

template <int N> cudaError_t launch_pte_mixed_n(const PteArgs &a, cudaStream_t stream);
template <int N> cudaError_t launch_pte_retry_n(const PteArgs &a, cudaStream_t stream);
template <int N> cudaError_t launch_pte_group_n(const PteArgs &a, cudaStream_t stream);

namespace {

constexpr int BIN_BLOCK = 256;

// The cell's material count and signature key: the ordered EOS kinds of
// its present materials, base 5, offset by the keys of smaller counts (a
// count above PTE_MAX_N gets key -1 and is left out, as the solve skips it).
__device__ __forceinline__ int pte_key(const PteArgs &a, const sgx_eos *eos, const long long i,
                                       int &n) {
  int sig = 0, pw = 1;
  n = 0;
  for (int m = 0; m < a.nmat; ++m) {
    const int ie = a.eos_idx[static_cast<long long>(m) * a.ncell + i];
    if (ie < 0 || ie >= a.neos) continue;
    int kind = eos[ie].type - SGX_IDEAL_GAS;
    kind = kind < 0 ? 0 : (kind >= PTE_SIG_KINDS ? PTE_SIG_KINDS - 1 : kind);
    sig += kind * pw;
    pw *= PTE_SIG_KINDS;
    ++n;
  }
  if (n < 1 || n > PTE_MAX_N) return -1;
  // keys of counts 1..n-1: 5 + 25 + ... = (5^n - 5) / 4
  return (pw - PTE_SIG_KINDS) / (PTE_SIG_KINDS - 1) + sig;
}

// bins[n] = cells with n materials; hist[key] = cells with that signature.
__global__ void __launch_bounds__(BIN_BLOCK) pte_bin_count(const PteArgs a) {
  __shared__ unsigned h[PTE_BINS];
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  if (threadIdx.x < PTE_BINS) h[threadIdx.x] = 0;
  __syncthreads();
  unsigned *hist = a.bins + 256 / sizeof(unsigned);
  const unsigned lane = threadIdx.x & 31u;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  // warp-uniform trip count: every lane runs every round
  for (long long base = static_cast<long long>(blockIdx.x) * blockDim.x; base < a.ncell;
       base += stride) {
    const long long i = base + threadIdx.x;
    int n = 0;
    const int key = i < a.ncell ? pte_key(a, s_eos, i, n) : -1;
    if (i < a.ncell) atomicAdd(&h[n < PTE_BINS ? n : 0], 1u);
    // one atomic per distinct key in the warp
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && static_cast<int>(lane) == __ffs(peers) - 1)
      atomicAdd(&hist[key], static_cast<unsigned>(__popc(peers)));
  }
  __syncthreads();
  if (threadIdx.x < PTE_BINS && h[threadIdx.x]) atomicAdd(&a.bins[threadIdx.x], h[threadIdx.x]);
}

// Exclusive scan of the signature histogram into the cursors (one block):
// cursor[key] = first position of that key's cells in perm. Keys are
// count-major, so the cells of each count stay one contiguous segment, at
// the offset the per-count kernels compute from bins[].
constexpr int SCAN_BLOCK = 1024;
__global__ void __launch_bounds__(SCAN_BLOCK) pte_sig_scan(const PteArgs a) {
  __shared__ unsigned part[SCAN_BLOCK];
  const unsigned *hist = a.bins + 256 / sizeof(unsigned);
  unsigned *cursor = a.bins + 256 / sizeof(unsigned) + PTE_SIG_KEYS;
  constexpr int PER = (PTE_SIG_KEYS + SCAN_BLOCK - 1) / SCAN_BLOCK;
  const int k0 = threadIdx.x * PER;
  unsigned sum = 0;
  for (int k = k0; k < k0 + PER && k < PTE_SIG_KEYS; ++k)
    sum += hist[k];
  part[threadIdx.x] = sum;
  __syncthreads();
  // Hillis-Steele inclusive scan of the partial sums
  for (int d = 1; d < SCAN_BLOCK; d <<= 1) {
    const unsigned v = threadIdx.x >= static_cast<unsigned>(d) ? part[threadIdx.x - d] : 0u;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  // cells without a material (count 0) come first in the count order but
  // have no signature: the keyed segments start after them
  unsigned run = a.bins[0] + (threadIdx.x ? part[threadIdx.x - 1] : 0u);
  for (int k = k0; k < k0 + PER && k < PTE_SIG_KEYS; ++k) {
    cursor[k] = run;
    run += hist[k];
  }
}

// perm[cursor[key]++] = cell id, one atomic per distinct key in a warp
// (ascending within a warp, so neighbouring lanes of the solve kernels
// mostly touch nearby cells).
__global__ void __launch_bounds__(BIN_BLOCK) pte_bin_scatter(const PteArgs a, int *perm) {
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  unsigned *cursor = a.bins + 256 / sizeof(unsigned) + PTE_SIG_KEYS;
  const unsigned lane = threadIdx.x & 31u;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long base = static_cast<long long>(blockIdx.x) * blockDim.x; base < a.ncell;
       base += stride) {
    const long long i = base + threadIdx.x;
    int n = 0;
    const int key = i < a.ncell ? pte_key(a, s_eos, i, n) : -1;
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    const int leader = __ffs(peers) - 1;
    unsigned pos = 0;
    if (key >= 0 && static_cast<int>(lane) == leader)
      pos = atomicAdd(&cursor[key], static_cast<unsigned>(__popc(peers)));
    pos = __shfl_sync(0xffffffffu, pos, leader);
    if (key >= 0) perm[pos + __popc(peers & ((1u << lane) - 1u))] = static_cast<int>(i);
  }
}

// The side streams of pass 2, a few per device, taken in turn (a stream in
// one graph capture cannot join another); null if they cannot be created.
cudaStream_t side_stream() {
  constexpr int PER_DEV = 8, MAX_DEV = 64;
  static std::mutex mu;
  static cudaStream_t pool[MAX_DEV][PER_DEV] = {};
  static unsigned next[MAX_DEV] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEV) return nullptr;
  std::lock_guard<std::mutex> lk(mu);
  const unsigned k = next[dev]++ % PER_DEV;
  if (!pool[dev][k] && cudaStreamCreateWithFlags(&pool[dev][k], cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    pool[dev][k] = nullptr;
  }
  return pool[dev][k];
}

template <bool RETRY> cudaError_t launch_n(const int n, const PteArgs &a, cudaStream_t s) {
  // pass 1 of counts from SGX_TUNE_PTE_GROUP_MIN_N up: a lane group per cell
  if (!RETRY && n >= 2 && n >= tune_get(SGX_TUNE_PTE_GROUP_MIN_N)) {
    switch (n) {
    case 2: return launch_pte_group_n<2>(a, s);
    case 3: return launch_pte_group_n<3>(a, s);
    case 4: return launch_pte_group_n<4>(a, s);
    case 5: return launch_pte_group_n<5>(a, s);
    case 6: return launch_pte_group_n<6>(a, s);
    }
  }
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

// The count, scan and scatter kernels of the binning (a.bins zeroed).
cudaError_t launch_pte_binning(const PteArgs &a, int *perm, cudaStream_t stream) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (a.ncell + BIN_BLOCK - 1) / BIN_BLOCK;
  const long long cap = 4LL * sms;
  const int grid = static_cast<int>(want < cap ? want : cap);
  pte_bin_count<<<grid, BIN_BLOCK, 0, stream>>>(a);
  pte_sig_scan<<<1, SCAN_BLOCK, 0, stream>>>(a);
  pte_bin_scatter<<<grid, BIN_BLOCK, 0, stream>>>(a, perm);
  return cudaGetLastError();
}

// Runs the binning and both passes with caller-provided scratch: bins (the
// 3 * PTE_BINS counters), and perm (when eos_idx is set) and retry_idx of
// ncell ints each.
cudaError_t launch_pte_mixed_with(const PteArgs &args, int *perm, cudaStream_t stream,
                                  cudaStream_t side_given) {
  PteArgs a = args;
  a.perm = nullptr;
  a.fp32_iters = tune_get(SGX_TUNE_PTE_FP32_ITERS);
  a.fp32_tol_exp = tune_get(SGX_TUNE_PTE_FP32_TOL);
  a.retry_iters = tune_get(SGX_TUNE_PTE_RETRY_ITERS);
  cudaError_t e = cudaMemsetAsync(a.bins, 0, a.eos_idx ? PTE_BINS_BYTES : 256, stream);
  if (e != cudaSuccess) return e;
  const int lo = a.eos_idx ? 1 : a.nmat;
  const int hi = a.nmat < PTE_MAX_N ? a.nmat : PTE_MAX_N;
  if (a.eos_idx) {
    if ((e = launch_pte_binning(a, perm, stream)) != cudaSuccess) return e;
    a.perm = perm;
  }
  // Pass 1 of every count on the caller's stream; pass 2 of count n on a
  // side stream once pass 1 of n is done. Pass 2 re-solves few cells but
  // runs long (FP64 at the reference's iteration counts, up to the cap for
  // cells that do not converge), so it overlaps pass 1 of the next counts
  // instead of idling the GPU after each.
  cudaStream_t side = side_given ? side_given : side_stream();
  if (!side) {
    for (int n = lo; n <= hi && e == cudaSuccess; ++n) {
      e = launch_n<false>(n, a, stream);
      if (e == cudaSuccess) e = launch_n<true>(n, a, stream);
    }
    return e;
  }
  const bool down = tune_get(SGX_TUNE_PTE_COUNT_ORDER) != 0;
  for (int i = 0; i <= hi - lo && e == cudaSuccess; ++i) {
    const int n = down ? hi - i : lo + i;
    e = launch_n<false>(n, a, stream);
    cudaEvent_t ev = nullptr;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev, stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(side, ev, 0);
    if (ev) cudaEventDestroy(ev);
    if (e == cudaSuccess) e = launch_n<true>(n, a, side);
  }
  // the caller's stream resumes after the last pass 2
  cudaEvent_t join = nullptr;
  cudaError_t j = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
  if (j == cudaSuccess) j = cudaEventRecord(join, side);
  if (j == cudaSuccess) j = cudaStreamWaitEvent(stream, join, 0);
  if (join) cudaEventDestroy(join);
  return e != cudaSuccess ? e : j;
}

cudaError_t launch_pte_mixed(const PteArgs &a, cudaStream_t stream) {
  if (a.ncell <= 0) return cudaSuccess;
  if (a.solver != SGX_PTE_RHOT) return cudaErrorNotSupported;
  if (a.ncell > 0x7fffffffLL) return cudaErrorInvalidValue; // int32 cell ids in perm / queue
  PteArgs args = a;
  void *scratch = nullptr;
  const size_t n4 = ((static_cast<size_t>(a.ncell) * sizeof(int) + 255) / 256) * 256;
  const size_t nb = (PTE_BINS_BYTES + 255) / 256 * 256;
  const size_t bytes = nb + (a.eos_idx ? 2 : 1) * n4;
  cudaError_t e = scratch_alloc(&scratch, bytes, stream);
  if (e != cudaSuccess) return e;
  char *p = static_cast<char *>(scratch);
  args.bins = reinterpret_cast<unsigned *>(p);
  args.retry_idx = reinterpret_cast<int *>(p + nb);
  int *perm = a.eos_idx ? reinterpret_cast<int *>(p + nb + n4) : nullptr;
  e = launch_pte_mixed_with(args, perm, stream);
  const cudaError_t f = scratch_free(scratch, stream);
  return e != cudaSuccess ? e : f;
}

} // namespace sgx
