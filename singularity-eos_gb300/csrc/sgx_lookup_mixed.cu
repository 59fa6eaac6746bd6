// Tabulated rho-T lookups with an FP32 bracket search and FP64 refinement.
//
// FillEos of SpinerEOSDependsRhoT (eos/eos_spiner_rho_temp.hpp:1052-1101)
// inverts sie(lRho, lT) for lT by regula falsi over the bilinear table
// (lTFromlRhoSie_, :1192-1250): tens of FP64 iterations, each with a
// division. At fixed lRho the bilinear interpolant is piecewise linear in lT,
// so when sie increases along T (checked per table at load) its root is
// unique and lies in the one grid cell whose density-blended end values
// bracket the target. This kernel:
//   1. classifies the element exactly as the reference does (FP64);
//   2. finds the bracketing cell by binary search over the FP32 corner-packed
//      copy of sie (8 probes for 256 nodes, one 16-byte load each);
//   3. solves the cell's linear interpolant for lT in FP64, moving to a
//      neighbour cell if FP32 rounding picked the wrong one;
//   4. evaluates T, P, bmod, cv (and cs = sqrt(bmod/rho)) from lT in FP64
//      exactly as the reference does.
// The root differs from the reference's regula-falsi endpoint midpoint only
// by the reference's own tolerance (1e-14 in lT). Elements whose target is
// not bracketed by the table row, tables that are not monotone, and off-table
// states take the reference's FP64 iteration unchanged.
#include <cuda_runtime.h>

#include "sgx_dispatch.cuh"
#include "sgx_internal.h"

namespace sgx {

namespace {

constexpr int LOOKUP_BLOCK = 256;

__device__ __forceinline__ bool fast_lT(const SpinerTable &t, const double lRho, const double sie,
                                        double &lT) {
  int j;
  double b0, b1;
  t.gRho.weights(lRho, j, b0, b1);
  if (!(b0 >= 0.0 && b1 >= 0.0)) return false; // extrapolated rows may not be monotone
  const int nc = t.nT - 1;
  const fq4 *row32 = t.sie4f + static_cast<long long>(j) * nc;
  const dq4 *row64 = t.sie4 + static_cast<long long>(j) * nc;
  // Bracket check against the exact end values of the row blend.
  const dq4 first = row64[0], last = row64[nc - 1];
  const double r_lo = b0 * first.x + b1 * first.z;
  const double r_hi = b0 * last.y + b1 * last.w;
  if (!(sie >= r_lo && sie <= r_hi)) return false;
  // FP32 binary search: largest node k in [0, nc-1] with blend(k) <= sie.
  const float b0f = static_cast<float>(b0), b1f = static_cast<float>(b1);
  const float ef = static_cast<float>(sie);
  int lo = 0, hi = nc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const fq4 q = row32[mid];
    const float rm = fmaf(b1f, q.z, b0f * q.x);
    if (rm <= ef)
      lo = mid;
    else
      hi = mid - 1;
  }
  // FP64 solve of the cell's linear interpolant, with neighbour correction.
  int i = lo;
  double a1 = 0.0;
  for (int k = 0; k < 4; ++k) {
    const dq4 c = row64[i];
    const double r0 = b0 * c.x + b1 * c.z;
    const double r1 = b0 * c.y + b1 * c.w;
    a1 = (sie - r0) / (r1 - r0);
    if (a1 < 0.0 && i > 0) {
      --i;
      continue;
    }
    if (a1 > 1.0 && i < nc - 1) {
      ++i;
      continue;
    }
    break;
  }
  if (!(a1 >= 0.0 && a1 <= 1.0)) return false;
  lT = t.gT.min + (i + a1) * t.gT.dx;
  return true;
}

__global__ void __launch_bounds__(LOOKUP_BLOCK) spiner_fill_mixed(const FillArgs a) {
  __shared__ SpinerTable st;
  if (threadIdx.x == 0) st = sp_table(a.eos);
  __syncthreads();
  const SpinerTable &t = st;
  const unsigned out = a.output;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < a.n;
       i += stride) {
    const double rho = a.rho[i];
    const double sie = a.sie[i];
    double *lam = a.lambda ? a.lambda + i * a.lambda_stride : nullptr;
    const double lRho = sp_lRho(t, rho);
    double lT;
    TableStatus w = sp_loc_rho_sie(t, lRho, sie);
    if (!(w == TableStatus::OnTable && t.sie_monotone_T && fast_lT(t, lRho, sie, lT)))
      lT = sp_lT_from_lRho_sie(t, lRho, sie, w, lam);
    const double temp = sp_T(t, lT);
    w = sp_loc_rho_T(t, lRho, lT);
    if ((out & Q_TEMPERATURE) && a.temp) a.temp[i] = temp;
    if ((out & Q_PRESSURE) && a.press) a.press[i] = sp_P_from(t, rho, lRho, temp, lT, w);
    if ((out & Q_CV) && a.cv) a.cv[i] = sp_cv_from(t, lRho, lT, w);
    if ((out & Q_BMOD) || a.cs) {
      const double bmod = sp_bmod_from(t, rho, lRho, temp, lT, w);
      if ((out & Q_BMOD) && a.bmod) a.bmod[i] = bmod;
      if (a.cs) a.cs[i] = sqrt(bmod / rho);
    }
    if (lam) {
      lam[0] = lRho;
      lam[1] = lT;
    }
  }
}

} // namespace

cudaError_t launch_fill_mixed(const FillArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long want = (a.n + LOOKUP_BLOCK - 1) / LOOKUP_BLOCK;
  const long long cap = static_cast<long long>(sms) * 8;
  const int grid = static_cast<int>(want < cap ? want : cap);
  spiner_fill_mixed<<<grid, LOOKUP_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

} // namespace sgx
