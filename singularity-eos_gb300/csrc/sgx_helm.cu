// Vector lookups and FillEos of the Helmholtz EOS (sgx_helm.cuh), one thread
// per element. The table header is staged in shared memory once per block;
// the per-cell Hermite records are read straight from the L2-resident
// table image.
#include <cuda_runtime.h>

#include "sgx_helm.cuh"
#include "sgx_internal.h"

namespace sgx {

namespace {

constexpr int HELM_BLOCK = 128;

// The scalar member functions of Helmholtz (eos_helmholtz.hpp:513-650): each
// is a FillEos with one output bit, except the Gruneisen parameter (Gamma3 - 1).
__device__ double helm_eval(const HelmTable &t, const int opt, const int fn, const double rho,
                            const double x, double *lam) {
  using namespace helm;
  double temp = 0.0, sie = 0.0, p = 0.0, cv = 0.0, bmod = 0.0;
  int err = 0;
  switch (fn) {
  case SGX_FN_T_FROM_RHO_SIE:
    sie = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_TEMPERATURE, lam, &err);
    return temp;
  case SGX_FN_SIE_FROM_RHO_T:
    temp = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_SIE, lam, &err);
    return sie;
  case SGX_FN_P_FROM_RHO_T:
    temp = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_PRESSURE, lam, &err);
    return p;
  case SGX_FN_P_FROM_RHO_SIE:
    sie = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_PRESSURE | Q_TEMPERATURE, lam, &err);
    return p;
  case SGX_FN_CV_FROM_RHO_T:
    temp = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_CV, lam, &err);
    return cv;
  case SGX_FN_CV_FROM_RHO_SIE:
    sie = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_CV | Q_TEMPERATURE, lam, &err);
    return cv;
  case SGX_FN_B_FROM_RHO_T:
    temp = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_BMOD, lam, &err);
    return bmod;
  case SGX_FN_B_FROM_RHO_SIE:
    sie = x;
    helm_fill(t, opt, rho, temp, sie, p, cv, bmod, Q_BMOD | Q_TEMPERATURE, lam, &err);
    return bmod;
  case SGX_FN_G_FROM_RHO_T: {
    // GetFromDensityTemperature_ reads the lT cache but does not use it
    const Cell c = cell(rho, lam[0], lam[1]);
    double pp[5], e[5], s[5], eta[5], nep[5];
    evaluate(t, opt, c, x, pp, e, s, eta, nep, false);
    return gamma3(rho, x, pp, e) - 1.0;
  }
  case SGX_FN_G_FROM_RHO_SIE: {
    const Cell c = cell(rho, lam[0], lam[1]);
    const double lT = lT_from_rho_sie(t, opt, c, x, lam);
    const double T = pow10e(lT);
    double pp[5], e[5], s[5], eta[5], nep[5];
    evaluate(t, opt, c, T, pp, e, s, eta, nep, false);
    return gamma3(rho, T, pp, e) - 1.0;
  }
  }
  return NAN;
}

__global__ void __launch_bounds__(HELM_BLOCK) helm_eval_kernel(const EvalArgs a) {
  __shared__ HelmTable st;
  if (threadIdx.x == 0) st = *reinterpret_cast<const HelmTable *>(a.eos.table);
  __syncthreads();
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += stride)
    a.out[i] = helm_eval(st, a.eos.flags, a.fn, a.in1[i], a.in2[i],
                         a.lambda + i * a.lambda_stride);
}

__global__ void __launch_bounds__(HELM_BLOCK) helm_fill_kernel(const FillArgs a) {
  __shared__ HelmTable st;
  if (threadIdx.x == 0) st = *reinterpret_cast<const HelmTable *>(a.eos.table);
  __syncthreads();
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  const unsigned output = a.output | (a.cs ? Q_BMOD : 0u);
  int bad = 0;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += stride) {
    const double rho = a.rho[i];
    double temp = a.temp ? a.temp[i] : 0.0;
    double sie = a.sie ? a.sie[i] : 0.0;
    double press = 0.0, cv = 0.0, bmod = 0.0;
    int err = 0;
    helm_fill(st, a.eos.flags, rho, temp, sie, press, cv, bmod, output,
              a.lambda + i * a.lambda_stride, &err);
    bad |= err;
    if (a.cs) a.cs[i] = sqrt(bmod / rho);
    if ((a.output & Q_TEMPERATURE) && a.temp) a.temp[i] = temp;
    if ((a.output & Q_SIE) && a.sie) a.sie[i] = sie;
    if ((a.output & Q_PRESSURE) && a.press) a.press[i] = press;
    if ((a.output & Q_CV) && a.cv) a.cv[i] = cv;
    if ((a.output & Q_BMOD) && a.bmod) a.bmod[i] = bmod;
  }
  if (bad && a.err) atomicOr(a.err, 1);
}

// Staged inversion FillEos (outputs include T, inputs rho and sie): pass 1
// runs every element's Newton iteration for at most a few steps and
// finishes the ones that stop; the others are queued with their exact
// iteration state (x, iteration count) and resumed over the compacted queue
// by up to three more passes (the last up to the reference's 100
// iterations), then its fallbacks. Each element's result is the one a single
// pass gives; the hard elements (hundreds of evaluations where e(T) is not
// monotone) no longer hold up the warps of the easy ones, nor the ones that
// wander to the iteration limit those that converge on the way. The step
// caps are launch knobs (SGX_TUNE_HELM_PASS1_STEPS, SGX_TUNE_HELM_MID_STEPS,
// SGX_TUNE_HELM_MID2_STEPS).

// An iteration-state queue between two passes.
struct HelmQueue {
  int *id;
  double *x;
  int *iter;
  unsigned *count;
};

__device__ __forceinline__ void store_fill(const FillArgs &a, const long long i, const double rho,
                                           const double temp, const double sie,
                                           const double press, const double cv,
                                           const double bmod) {
  if (a.cs) a.cs[i] = sqrt(bmod / rho);
  if ((a.output & Q_TEMPERATURE) && a.temp) a.temp[i] = temp;
  if ((a.output & Q_SIE) && a.sie) a.sie[i] = sie;
  if ((a.output & Q_PRESSURE) && a.press) a.press[i] = press;
  if ((a.output & Q_CV) && a.cv) a.cv[i] = cv;
  if ((a.output & Q_BMOD) && a.bmod) a.bmod[i] = bmod;
}

// An element whose iteration stopped at `cap` steps: queued for the next
// pass with its state, or, at the reference's 100, for the regula falsi of
// pass 3 (id only).
__device__ __forceinline__ void queue_unfinished(const HelmQueue &next, const HelmQueue &rf,
                                                 const long long i, const double x,
                                                 const int iter) {
  if (iter < helm::NEWTON_MAX_ITER) {
    const unsigned pos = atomicAdd(next.count, 1u);
    next.id[pos] = static_cast<int>(i);
    next.x[pos] = x;
    next.iter[pos] = iter;
  } else {
    rf.id[atomicAdd(rf.count, 1u)] = static_cast<int>(i);
  }
}

// MIXED: the Newton iteration starts from the FP32 phase's root (newton_e32,
// FP32 e(T) to 1e-6) instead of the reference's guess, so the FP64 steps
// that follow are the reference's last one or two.
template <bool MIXED>
__global__ void __launch_bounds__(HELM_BLOCK)
    helm_invert_pass1(const FillArgs a, HelmQueue next, HelmQueue rf, const int cap) {
  using namespace helm;
  __shared__ HelmTable st;
  if (threadIdx.x == 0) st = *reinterpret_cast<const HelmTable *>(a.eos.table);
  __syncthreads();
  const int opt = a.eos.flags;
  const unsigned output = a.output | (a.cs ? Q_BMOD : 0u);
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += stride) {
    const double rho = a.rho[i];
    const double sie = a.sie[i];
    double *lam = a.lambda + i * a.lambda_stride;
    const Cell c = cell(rho, lam[0], lam[1]);
    Inversion v = inversion_begin(st, opt, c, sie, lam);
    if (MIXED) {
      double x32 = v.x;
      if (newton_e32(st, opt, cell32(c), sie, v.Ta, v.Tb, x32)) v.x = x32;
    }
    const bool done = newton_e_steps(st, opt, c, sie, v.Ta, v.Tb, HELM_EOS_EPS, v.x, v.iter, cap);
    if (!done) {
      queue_unfinished(next, rf, i, v.x, v.iter);
      continue;
    }
    const double temp = pow10e(inversion_end(st, opt, c, v, true, lam));
    double e_out = sie, press = 0.0, cv = 0.0, bmod = 0.0;
    helm_fill_tail(st, opt, c, temp, e_out, press, cv, bmod, output);
    store_fill(a, i, rho, temp, e_out, press, cv, bmod);
  }
}

// The elements of `in` resumed from their saved state, up to `cap` steps
// in all; those still running are queued on (next, or rf at 100 steps).
__global__ void __launch_bounds__(HELM_BLOCK)
    helm_invert_pass2(const FillArgs a, const HelmQueue in, HelmQueue next, HelmQueue rf,
                      const int cap) {
  using namespace helm;
  __shared__ HelmTable st;
  if (threadIdx.x == 0) st = *reinterpret_cast<const HelmTable *>(a.eos.table);
  __syncthreads();
  const int opt = a.eos.flags;
  const unsigned output = a.output | (a.cs ? Q_BMOD : 0u);
  const unsigned count = *in.count;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < count;
       k += gridDim.x * blockDim.x) {
    const long long i = in.id[k];
    const double rho = a.rho[i];
    const double sie = a.sie[i];
    double *lam = a.lambda + i * a.lambda_stride;
    const Cell c = cell(rho, lam[0], lam[1]);
    Inversion v = inversion_begin(st, opt, c, sie, lam);
    v.x = in.x[k];
    v.iter = in.iter[k];
    const bool done = newton_e_steps(st, opt, c, sie, v.Ta, v.Tb, HELM_EOS_EPS, v.x, v.iter, cap);
    if (!done) {
      queue_unfinished(next, rf, i, v.x, v.iter);
      continue;
    }
    const double temp = pow10e(inversion_end(st, opt, c, v, true, lam));
    double e_out = sie, press = 0.0, cv = 0.0, bmod = 0.0;
    helm_fill_tail(st, opt, c, temp, e_out, press, cv, bmod, output);
    store_fill(a, i, rho, temp, e_out, press, cv, bmod);
  }
}

// Pass 3: the elements whose Newton iteration used all 100 steps go on to
// the reference's regula falsi (up to 1000 more evaluations) and, failing
// that, the analytic estimate.
__global__ void __launch_bounds__(HELM_BLOCK) helm_invert_pass3(const FillArgs a, const HelmQueue rf) {
  using namespace helm;
  __shared__ HelmTable st;
  if (threadIdx.x == 0) st = *reinterpret_cast<const HelmTable *>(a.eos.table);
  __syncthreads();
  const int opt = a.eos.flags;
  const unsigned output = a.output | (a.cs ? Q_BMOD : 0u);
  const unsigned count = *rf.count;
  for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < count;
       k += gridDim.x * blockDim.x) {
    const long long i = rf.id[k];
    const double rho = a.rho[i];
    const double sie = a.sie[i];
    double *lam = a.lambda + i * a.lambda_stride;
    const Cell c = cell(rho, lam[0], lam[1]);
    const Inversion v = inversion_begin(st, opt, c, sie, lam);
    const double temp = pow10e(inversion_end(st, opt, c, v, false, lam));
    double e_out = sie, press = 0.0, cv = 0.0, bmod = 0.0;
    helm_fill_tail(st, opt, c, temp, e_out, press, cv, bmod, output);
    store_fill(a, i, rho, temp, e_out, press, cv, bmod);
  }
}

int helm_grid(const long long n) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (n + HELM_BLOCK - 1) / HELM_BLOCK;
  const long long cap = static_cast<long long>(sms) * 16;
  return static_cast<int>(want < cap ? want : cap);
}

} // namespace

cudaError_t launch_helm_eval(const EvalArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  helm_eval_kernel<<<helm_grid(a.n), HELM_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_helm_fill(const FillArgs &a, cudaStream_t stream, const bool mixed) {
  if (a.n <= 0) return cudaSuccess;
  const int opt = a.eos.flags;
  const bool iterate = (opt & HELM_RAD) || (opt & HELM_ELE) || (opt & HELM_COUL);
  const bool two_pass = (a.output & Q_TEMPERATURE) && iterate && !(opt & HELM_REGULA_FALSI) &&
                        a.n <= 0x7fffffffLL;
  if (!two_pass) {
    helm_fill_kernel<<<helm_grid(a.n), HELM_BLOCK, 0, stream>>>(a);
    return cudaGetLastError();
  }
  // queues: a 256 B counter block, then two state queues (x, id, iter) that
  // the passes hand on alternately, and the ids for pass 3
  const size_t n = static_cast<size_t>(a.n);
  const size_t ids = (n * sizeof(int) + 255) / 256 * 256;
  const size_t xs = (n * sizeof(double) + 255) / 256 * 256;
  void *scratch = nullptr;
  cudaError_t e = scratch_alloc(&scratch, 256 + 2 * (xs + 2 * ids) + ids, stream);
  if (e != cudaSuccess) return e;
  char *p = static_cast<char *>(scratch);
  HelmQueue qa, qb, rf;
  qa.count = reinterpret_cast<unsigned *>(p);
  qb.count = reinterpret_cast<unsigned *>(p + 64);
  rf.count = reinterpret_cast<unsigned *>(p + 128);
  char *o = p + 256;
  for (HelmQueue *q : {&qa, &qb}) {
    q->x = reinterpret_cast<double *>(o);
    q->id = reinterpret_cast<int *>(o + xs);
    q->iter = reinterpret_cast<int *>(o + xs + ids);
    o += xs + 2 * ids;
  }
  rf.id = reinterpret_cast<int *>(o);
  rf.x = nullptr;
  rf.iter = nullptr;
  // the step caps: a knob left at 0 takes its precision's default schedule,
  // measured on 2^20 cells of the benchmark's distribution (FP64 10, 20,
  // 40: 59 ms against 91 ms for 12 and 100; mixed 3, 12, 40: 47 ms against
  // 72 ms -- after the FP32 phase most elements need one to three FP64 steps)
  int cap1 = tune_get(SGX_TUNE_HELM_PASS1_STEPS);
  int mid = tune_get(SGX_TUNE_HELM_MID_STEPS);
  int mid2 = tune_get(SGX_TUNE_HELM_MID2_STEPS);
  if (cap1 == 0) cap1 = mixed ? 3 : 10;
  if (mid == 0) mid = mixed ? 12 : 20;
  if (mid2 == 0) mid2 = 40;
  e = cudaMemsetAsync(p, 0, 256, stream);
  if (e == cudaSuccess) {
    if (mixed)
      helm_invert_pass1<true><<<helm_grid(a.n), HELM_BLOCK, 0, stream>>>(a, qa, rf, cap1);
    else
      helm_invert_pass1<false><<<helm_grid(a.n), HELM_BLOCK, 0, stream>>>(a, qa, rf, cap1);
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess)
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (a.n + HELM_BLOCK - 1) / HELM_BLOCK;
    const int grid2 = static_cast<int>(want < 4LL * sms ? want : 4LL * sms);
    // the resumed passes, each to a higher cap, the last to the reference's
    // 100; the state queues alternate (a pass reads one, fills the other,
    // whose counter it has cleared)
    int caps[3], nst = 0, prev = cap1;
    for (const int c : {mid, mid2})
      if (c > prev && c < helm::NEWTON_MAX_ITER) caps[nst++] = prev = c;
    caps[nst++] = helm::NEWTON_MAX_ITER;
    HelmQueue *in = &qa, *nx = &qb;
    for (int k = 0; k < nst && e == cudaSuccess; ++k) {
      if (k > 0) e = cudaMemsetAsync(nx->count, 0, sizeof(unsigned), stream);
      if (e != cudaSuccess) break;
      helm_invert_pass2<<<grid2, HELM_BLOCK, 0, stream>>>(a, *in, *nx, rf, caps[k]);
      HelmQueue *t = in;
      in = nx;
      nx = t;
    }
    helm_invert_pass3<<<grid2, HELM_BLOCK, 0, stream>>>(a, rf);
    e = cudaGetLastError();
  }
  const cudaError_t f = scratch_free(scratch, stream);
  return e != cudaSuccess ? e : f;
}

} // namespace sgx
