// Internal interfaces between the C-ABI layer (sgx_capi.cu) and the kernel
// translation units (sgx_fp64.cu, sgx_mixed.cu).
#pragma once

#include <string>

#include <cuda_runtime.h>

#include "../../include/sgx.h"

namespace sgx {

constexpr int MAX_EOS = 16;
// Models the PTE solvers evaluate (Helmholtz is a lookup-only model here).
inline bool pte_model(const int t) {
  return (t >= SGX_IDEAL_GAS && t <= SGX_SPINER_RHOT) || t == SGX_SPINER_RHOSIE;
}
constexpr int MAX_NMAT = 8;  // material slots per cell
constexpr int PTE_MAX_N = 6; // materials present per cell (Jacobian up to 6x6)

// Launch arguments of the per-cell PTE kernels (passed by value: about 2.4 KB
// of kernel parameter space).
struct PteArgs {
  int solver;
  int nmat;
  long long ncell;
  int neos;
  int pad;
  sgx_eos eos[MAX_EOS];
  const int32_t *eos_idx;
  const double *vfrac_tot, *sie_tot;
  double *rho, *vfrac, *sie, *temp, *press, *lambda;
  sgx_pte_status *status;
  sgx_mix_params params;
  // Mixed path only (device scratch):
  //  - perm: cell ids grouped by material count, the cells with n materials
  //    at perm[sum(bins[0..n)) ...] (null when every cell holds nmat);
  //  - bins[0..8): cells per material count; bins[8..16): unused;
  //    bins[16..24): retry-queue length per material count; from byte 256
  //    the signature histogram and cursors (PTE_BINS_BYTES in all);
  //  - retry_idx: cells whose FP32 solve + FP64 refinement failed, queued for
  //    a second, FP64 pass (ncell entries; the cells with n materials queue
  //    at the same offset as their segment of perm).
  const int *perm;
  unsigned *bins;
  int *retry_idx;
  // iteration limits per material of pass 1 (FP32) and pass 2 (FP64)
  int fp32_iters, retry_iters;
  // the FP32 phase's relative residual tolerance, 10^-fp32_tol_exp
  int fp32_tol_exp;
};
constexpr int PTE_BINS = 8;
// Cells are binned by material count and by the ordered EOS types of their
// materials (5 kinds that take part in PTE): 5^n signatures for n
// materials, n-major, sum over n = 1..6.
constexpr int PTE_SIG_KINDS = 5;
constexpr int PTE_SIG_KEYS = 5 + 25 + 125 + 625 + 3125 + 15625;
// The counter block of the mixed path: 3 * PTE_BINS counters (256 bytes),
// then the signature histogram and its scatter cursors.
constexpr size_t PTE_BINS_BYTES = 256 + 2 * PTE_SIG_KEYS * sizeof(unsigned);

// The argument checks of sgx_pte_solve and the PteArgs they describe;
// empty is set when there is nothing to launch (ncell 0).
int pte_prepare(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
                double *rho, double *vfrac, double *sie, double *temp, double *press,
                double *lambda, const sgx_mix_params *params, sgx_pte_status *status,
                int precision, PteArgs &a, bool &empty);
// Sets the calling thread's sgx_last_error() message; returns code.
int set_error(int code, const std::string &msg);
// SGX_OK, or the error (with its message set) for an EOS whose modifier bits
// are unknown, that is Helmholtz with modifiers, or that has modifiers on a
// mixed-precision path.
int check_eos_mods(const sgx_eos &e, bool mixed, const char *who);

// Tuning knobs (sgx_tune_set); the value a launcher uses now.
int tune_get(int knob);

// Stream-ordered scratch from the library's per-device memory pool
// (sgx_pool.cu); freed with scratch_free on a stream.
cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t stream);
cudaError_t scratch_free(void *p, cudaStream_t stream);

// Per-cell PTE, FP64, following the reference iteration exactly.
cudaError_t launch_pte_fp64(const PteArgs &a, cudaStream_t stream);
// The same with caller-provided binning scratch when a.eos_idx is set: bins
// (PTE_BINS_BYTES) and perm (ncell ints).
cudaError_t launch_pte_fp64_with(const PteArgs &a, unsigned *bins, int *perm,
                                 cudaStream_t stream);
// Bins the cells of a (eos_idx set; a.bins zeroed, PTE_BINS_BYTES) by
// material count and EOS-kind signature into perm (ncell ints).
cudaError_t launch_pte_binning(const PteArgs &a, int *perm, cudaStream_t stream);
// Per-cell PTE, FP32 iterations then FP64 refinement.
cudaError_t launch_pte_mixed(const PteArgs &a, cudaStream_t stream);
// The same with caller-provided scratch: a.bins (PTE_BINS_BYTES), a.retry_idx
// and, when a.eos_idx is set, perm (ncell ints each). Pass 2 runs on `side`
// when given, else on a stream of the library's per-device pool.
cudaError_t launch_pte_mixed_with(const PteArgs &a, int *perm, cudaStream_t stream,
                                  cudaStream_t side = nullptr);
// The same with the scratch in a static device array (sgx_noalloc.cu).
cudaError_t launch_pte_mixed_noalloc(const PteArgs &a, cudaStream_t stream);

struct EvalArgs {
  sgx_eos eos;
  int fn;
  long long n;
  const double *in1, *in2;
  double *out, *lambda;
  int lambda_stride;
};
cudaError_t launch_eval_fp64(const EvalArgs &a, cudaStream_t stream);
cudaError_t launch_bounds_fp64(const sgx_eos &e, int what, long long n, const double *x,
                               double *out, cudaStream_t stream);

struct FillArgs {
  sgx_eos eos;
  long long n;
  double *rho, *temp, *sie, *press, *cv, *bmod, *lambda;
  double *cs; // optional sound speed sqrt(bmod / rho)
  unsigned output;
  int lambda_stride;
  int *err; // device flag: set to 1 on an undefined input/output combination
};
cudaError_t launch_fill_fp64(const FillArgs &a, cudaStream_t stream);
// SpinerEOSDependsRhoSie FillEos from (rho, sie) in float-float
// (sgx_lookup_sie.cu); the table must carry its float-float cells.
cudaError_t launch_fill_sie_mixed(const FillArgs &a, cudaStream_t stream);
// PTDerivativesFromPreferred per element: d[0..3] = dedP_T, drdP_T, dedT_P,
// drdT_P.
struct PtDerivArgs {
  sgx_eos eos;
  long long n;
  const double *rho, *sie, *press, *temp;
  double *d[4];
  double *lambda;
  int lambda_stride;
};
cudaError_t launch_pt_derivs(const PtDerivArgs &a, cudaStream_t stream);
// Tabulated rho-T FillEos from (rho, sie): FP32 bracket search + FP64 solve.
cudaError_t launch_fill_mixed(const FillArgs &a, cudaStream_t stream);
// The reference's FP64 tabulated FillEos for the elements whose bit is set
// in `left` (one bit per element, 32 per word).
cudaError_t launch_fill_ref(const FillArgs &a, const unsigned *left, cudaStream_t stream);
// Helmholtz vector lookups and FillEos (lambda rows [Abar, Zbar, lT]).
cudaError_t launch_helm_eval(const EvalArgs &a, cudaStream_t stream);
// mixed: the inversion's Newton iteration starts from an FP32 Newton phase
// (T(rho, sie) outputs only; everything else is the FP64 path).
cudaError_t launch_helm_fill(const FillArgs &a, cudaStream_t stream, bool mixed = false);

} // namespace sgx
