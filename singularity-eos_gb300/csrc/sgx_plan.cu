// PTE plans: one sgx_pte_solve bound to fixed device arrays, captured once
// into a CUDA graph and replayed.
//
// A hydro code calls the closure on the same arrays every cycle. A plain
// sgx_pte_solve issues up to 16 operations per call: a memset, the three
// binning kernels, pass 1 and pass 2 per material count, and the events of
// the side stream. A plan captures that sequence once, with its scratch
// allocated up front, and each run is one cudaGraphLaunch. The graph reads
// the bound arrays when it runs, so the caller refills them in place
// between runs. The iteration knobs are read when the plan is made.
//
// Capture runs on the plan's own stream; pass 2 of the mixed path forks to
// the plan's own side stream and joins back, so capture never touches a
// stream that other calls use. No reference counterpart: the reference's
// closure is a per-cell loop the caller runs each cycle
// (get_sg_eos_rho_e.cpp:30-88).
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "sgx_internal.h"

struct sgx_pte_plan {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t capture = nullptr, side = nullptr;
  void *scratch = nullptr;
  int device = 0;
  long long ncell = 0;
};

namespace {

void release(sgx_pte_plan *p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->capture) cudaStreamDestroy(p->capture);
  if (p->side) cudaStreamDestroy(p->side);
  if (p->scratch) cudaFree(p->scratch);
  delete p;
}

int cuda_error(const cudaError_t e, const char *what) {
  return sgx::set_error(SGX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

} // namespace

extern "C" {

int sgx_pte_plan_create(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                        const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
                        double *rho, double *vfrac, double *sie, double *temp, double *press,
                        double *lambda, const sgx_mix_params *params, sgx_pte_status *status,
                        int precision, sgx_pte_plan **out) {
  static const char *who = "sgx_pte_plan_create";
  if (!out) return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": null out");
  *out = nullptr;
  sgx::PteArgs a;
  bool empty = false;
  if (const int rc = sgx::pte_prepare(solver, nmat, ncell, eos_list, neos, eos_idx, vfrac_tot,
                                      sie_tot, rho, vfrac, sie, temp, press, lambda, params,
                                      status, precision, a, empty))
    return rc;
  if (ncell > 0x7fffffffLL)
    return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": ncell above 2^31 - 1");
  auto *p = new sgx_pte_plan;
  p->ncell = ncell;
  cudaError_t e = cudaGetDevice(&p->device);
  // scratch: the counter block, then perm and the retry queue (ncell ints)
  const size_t nb = (sgx::PTE_BINS_BYTES + 255) / 256 * 256;
  const size_t n4 = ((static_cast<size_t>(ncell > 0 ? ncell : 1) * sizeof(int) + 255) / 256) * 256;
  if (e == cudaSuccess) e = cudaMalloc(&p->scratch, nb + 2 * n4);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->capture, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    release(p);
    return cuda_error(e, who);
  }
  char *s = static_cast<char *>(p->scratch);
  unsigned *bins = reinterpret_cast<unsigned *>(s);
  int *perm = eos_idx ? reinterpret_cast<int *>(s + nb) : nullptr;
  a.bins = bins;
  a.retry_idx = reinterpret_cast<int *>(s + nb + n4);
  // relaxed mode: the launchers query device attributes while capturing
  e = cudaStreamBeginCapture(p->capture, cudaStreamCaptureModeRelaxed);
  cudaError_t launch = cudaSuccess;
  if (e == cudaSuccess && !empty) {
    if (precision == SGX_PREC_MIXED)
      launch = sgx::launch_pte_mixed_with(a, perm, p->capture, p->side);
    else
      launch = sgx::launch_pte_fp64_with(a, bins, perm, p->capture);
  }
  if (e == cudaSuccess) e = cudaStreamEndCapture(p->capture, &p->graph);
  if (e == cudaSuccess && launch != cudaSuccess) e = launch;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  if (e != cudaSuccess) {
    cudaGetLastError();
    release(p);
    return cuda_error(e, who);
  }
  *out = p;
  return SGX_OK;
}

int sgx_pte_plan_run(sgx_pte_plan *plan, sgx_stream_t stream) {
  if (!plan) return sgx::set_error(SGX_ERR_INVALID, "sgx_pte_plan_run: null plan");
  int dev = -1;
  cudaGetDevice(&dev);
  if (dev != plan->device)
    return sgx::set_error(SGX_ERR_INVALID, "sgx_pte_plan_run: plan made on another device");
  const cudaError_t e = cudaGraphLaunch(plan->exec, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_error(e, "sgx_pte_plan_run");
  return SGX_OK;
}

int sgx_pte_plan_destroy(sgx_pte_plan *plan) {
  if (!plan) return SGX_OK;
  // a run still in flight finishes first: cudaGraphExecDestroy defers to
  // it, and cudaFree of the scratch waits for the device
  release(plan);
  return SGX_OK;
}

} // extern "C"
