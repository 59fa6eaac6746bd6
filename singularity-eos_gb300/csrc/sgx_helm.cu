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

cudaError_t launch_helm_fill(const FillArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  helm_fill_kernel<<<helm_grid(a.n), HELM_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

} // namespace sgx
