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
    {{0}, 0, 1},    // SGX_TUNE_PTE_COUNT_ORDER
    {{128}, 32, 128}, // SGX_TUNE_PTE_MIXED_BLOCK
    {{3}, 2, 7},      // SGX_TUNE_PTE_GROUP_MIN_N
    {{4}, 3, 6},      // SGX_TUNE_PTE_FP32_TOL
    {{0}, 0, 100},    // SGX_TUNE_HELM_PASS1_STEPS (0: the precision's default)
    {{0}, 0, 100},    // SGX_TUNE_HELM_MID_STEPS
    {{0}, 0, 100},    // SGX_TUNE_HELM_MID2_STEPS
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

// The autotuner of the lookup's launch shape: every (blocks per SM, staging)
// pair on the caller's own batch, through the public call, timed with events
// on the caller's stream; the fastest pair stays set. These two knobs change
// how the work is spread and staged, never what a lookup returns, so the
// choice is free to follow the hardware and the batch. Each trial is an
// ordinary call: its outputs, and a lambda cache if given, are written.
extern "C" int sgx_tune_autotune_fill(const sgx_eos *eos, int64_t n, double *rho, double *temp,
                                      double *sie, double *press, double *cv, double *bmod,
                                      double *cs, uint32_t output, double *lambda,
                                      int lambda_stride, int reps, int *blocks_per_sm,
                                      int *stage, sgx_stream_t stream) {
  using namespace sgx;
  static const char *who = "sgx_tune_autotune_fill";
  if (!eos || n <= 0 || reps < 1 || reps > 1000)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const int keep_b = g_knobs[SGX_TUNE_LOOKUP_BLOCKS_PER_SM].value.load();
  const int keep_s = g_knobs[SGX_TUNE_LOOKUP_STAGE].value.load();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  float best = 0.0f;
  int best_b = keep_b, best_s = keep_s, rc = SGX_OK;
  for (int b = g_knobs[SGX_TUNE_LOOKUP_BLOCKS_PER_SM].lo;
       ce == cudaSuccess && rc == SGX_OK && b <= g_knobs[SGX_TUNE_LOOKUP_BLOCKS_PER_SM].hi; ++b)
    for (int st = g_knobs[SGX_TUNE_LOOKUP_STAGE].lo;
         ce == cudaSuccess && rc == SGX_OK && st <= g_knobs[SGX_TUNE_LOOKUP_STAGE].hi; ++st) {
      g_knobs[SGX_TUNE_LOOKUP_BLOCKS_PER_SM].value.store(b);
      g_knobs[SGX_TUNE_LOOKUP_STAGE].value.store(st);
      // one untimed call (first use of this shape), then reps timed
      rc = sgx_eos_fill_ex(eos, n, rho, temp, sie, press, cv, bmod, cs, output, lambda,
                           lambda_stride, SGX_PREC_MIXED, stream);
      if (rc == SGX_OK) ce = cudaEventRecord(e0, s);
      for (int r = 0; r < reps && rc == SGX_OK && ce == cudaSuccess; ++r)
        rc = sgx_eos_fill_ex(eos, n, rho, temp, sie, press, cv, bmod, cs, output, lambda,
                             lambda_stride, SGX_PREC_MIXED, stream);
      if (rc == SGX_OK && ce == cudaSuccess) ce = cudaEventRecord(e1, s);
      if (rc == SGX_OK && ce == cudaSuccess) ce = cudaEventSynchronize(e1);
      float ms = 0.0f;
      if (rc == SGX_OK && ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
      if (rc == SGX_OK && ce == cudaSuccess && (best == 0.0f || ms < best)) {
        best = ms;
        best_b = b;
        best_s = st;
      }
    }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  // keep the winner, or the previous setting if a trial failed
  const bool ok = rc == SGX_OK && ce == cudaSuccess;
  g_knobs[SGX_TUNE_LOOKUP_BLOCKS_PER_SM].value.store(ok ? best_b : keep_b);
  g_knobs[SGX_TUNE_LOOKUP_STAGE].value.store(ok ? best_s : keep_s);
  if (rc != SGX_OK) return rc;
  if (ce != cudaSuccess)
    return set_error(SGX_ERR_CUDA, std::string(who) + ": " + cudaGetErrorString(ce));
  if (blocks_per_sm) *blocks_per_sm = best_b;
  if (stage) *stage = best_s;
  return SGX_OK;
}

// The autotuner of the mixed PTE launch: every combination of the pass-1
// block size (32, 64, 128 threads), the order of the material counts and,
// when allowed, the material count from which pass 1 runs a lane group per
// cell, timed on the caller's own batch through sgx_pte_solve. The caller's
// starting state is kept in a device copy and restored before every trial,
// so each trial solves the same problem and the arrays end holding the
// solve of the winning setting.
extern "C" int sgx_tune_autotune_pte(int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                                     const int32_t *eos_idx, const double *vfrac_tot,
                                     const double *sie_tot, double *rho, double *vfrac,
                                     double *sie, double *temp, double *press, double *lambda,
                                     const sgx_mix_params *params, sgx_pte_status *status,
                                     int reps, int tune_group, int *chosen,
                                     sgx_stream_t stream) {
  using namespace sgx;
  static const char *who = "sgx_tune_autotune_pte";
  if (nmat < 1 || ncell <= 0 || reps < 1 || reps > 100 || !rho || !vfrac || !sie || !temp ||
      !press)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": bad arguments");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const size_t arr = static_cast<size_t>(nmat) * static_cast<size_t>(ncell) * sizeof(double);
  const size_t lam_bytes = lambda ? 3 * arr : 0;
  double *io[5] = {rho, vfrac, sie, temp, press};
  void *keep = nullptr;
  cudaError_t ce = scratch_alloc(&keep, 5 * arr + lam_bytes, s);
  if (ce != cudaSuccess) return set_error(SGX_ERR_CUDA, std::string(who) + ": scratch");
  char *kp = static_cast<char *>(keep);
  for (int k = 0; k < 5 && ce == cudaSuccess; ++k)
    ce = cudaMemcpyAsync(kp + k * arr, io[k], arr, cudaMemcpyDeviceToDevice, s);
  if (ce == cudaSuccess && lambda)
    ce = cudaMemcpyAsync(kp + 5 * arr, lambda, lam_bytes, cudaMemcpyDeviceToDevice, s);
  auto restore = [&]() {
    cudaError_t r = cudaSuccess;
    for (int k = 0; k < 5 && r == cudaSuccess; ++k)
      r = cudaMemcpyAsync(io[k], kp + k * arr, arr, cudaMemcpyDeviceToDevice, s);
    if (r == cudaSuccess && lambda)
      r = cudaMemcpyAsync(lambda, kp + 5 * arr, lam_bytes, cudaMemcpyDeviceToDevice, s);
    return r;
  };
  const int keep_b = g_knobs[SGX_TUNE_PTE_MIXED_BLOCK].value.load();
  const int keep_o = g_knobs[SGX_TUNE_PTE_COUNT_ORDER].value.load();
  const int keep_g = g_knobs[SGX_TUNE_PTE_GROUP_MIN_N].value.load();
  const int blocks[3] = {32, 64, 128};
  // (thresholds of 3 and up: with lane groups for two-material cells a few
  // stiff cells of the uneven batch ended 1e-9 from the tight FP64 solve in
  // T, against 1e-10 with the thread-per-cell kernel)
  const int groups[4] = {keep_g, 3, 4, 7};
  const int ng = tune_group ? 4 : 1;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
  if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
  float best = 0.0f;
  int best_b = keep_b, best_o = keep_o, best_g = keep_g, rc = SGX_OK;
  for (int gi = 0; gi < ng; ++gi)
    for (int bi = 0; bi < 3; ++bi)
      for (int o = 0; o < 2 && ce == cudaSuccess && rc == SGX_OK; ++o) {
        g_knobs[SGX_TUNE_PTE_MIXED_BLOCK].value.store(blocks[bi]);
        g_knobs[SGX_TUNE_PTE_COUNT_ORDER].value.store(o);
        g_knobs[SGX_TUNE_PTE_GROUP_MIN_N].value.store(groups[gi]);
        float total = 0.0f;
        for (int r = 0; r <= reps && ce == cudaSuccess && rc == SGX_OK; ++r) {
          ce = restore();
          if (ce == cudaSuccess) ce = cudaEventRecord(e0, s);
          if (ce == cudaSuccess)
            rc = sgx_pte_solve(SGX_PTE_RHOT, nmat, ncell, eos_list, neos, eos_idx, vfrac_tot,
                               sie_tot, rho, vfrac, sie, temp, press, lambda, params, status,
                               SGX_PREC_MIXED, stream);
          if (rc == SGX_OK && ce == cudaSuccess) ce = cudaEventRecord(e1, s);
          if (rc == SGX_OK && ce == cudaSuccess) ce = cudaEventSynchronize(e1);
          float ms = 0.0f;
          if (rc == SGX_OK && ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
          if (r > 0) total += ms; // the first run of a setting is untimed
        }
        if (rc == SGX_OK && ce == cudaSuccess && (best == 0.0f || total < best)) {
          best = total;
          best_b = blocks[bi];
          best_o = o;
          best_g = groups[gi];
        }
      }
  const bool ok = rc == SGX_OK && ce == cudaSuccess;
  g_knobs[SGX_TUNE_PTE_MIXED_BLOCK].value.store(ok ? best_b : keep_b);
  g_knobs[SGX_TUNE_PTE_COUNT_ORDER].value.store(ok ? best_o : keep_o);
  g_knobs[SGX_TUNE_PTE_GROUP_MIN_N].value.store(ok ? best_g : keep_g);
  // leave the arrays holding the winner's solve
  if (ok) {
    ce = restore();
    if (ce == cudaSuccess)
      rc = sgx_pte_solve(SGX_PTE_RHOT, nmat, ncell, eos_list, neos, eos_idx, vfrac_tot, sie_tot,
                         rho, vfrac, sie, temp, press, lambda, params, status, SGX_PREC_MIXED,
                         stream);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  const cudaError_t f = scratch_free(keep, s);
  if (ce == cudaSuccess) ce = f;
  if (rc != SGX_OK) return rc;
  if (ce != cudaSuccess)
    return set_error(SGX_ERR_CUDA, std::string(who) + ": " + cudaGetErrorString(ce));
  if (chosen) {
    chosen[0] = best_b;
    chosen[1] = best_o;
    chosen[2] = best_g;
  }
  return SGX_OK;
}
