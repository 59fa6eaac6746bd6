// Tabulated rho-T lookups with an FP32 bracket search and a lean FP64 root.
//
// FillEos of SpinerEOSDependsRhoT (eos/eos_spiner_rho_temp.hpp:1052-1101)
// inverts sie(lRho, lT) for lT by regula falsi over the bilinear table
// (lTFromlRhoSie_, :1192-1250): tens of FP64 iterations, each with a
// division. On GB300 the FP64 pipe, not HBM, bounds that loop. At fixed lRho
// the bilinear interpolant is piecewise linear in lT, so when sie increases
// along T (checked per table at load) its root is unique and lies in the one
// grid cell whose density-blended end values bracket the target. Per element:
//   1. lRho and the density weights in FP64 (computed once, reused below);
//   2. on-table classification in FP32 with a 1e-6 guard band (elements in
//      the band, off-table states, unbracketed targets and non-monotone
//      tables take the reference's FP64 iteration unchanged);
//   3. binary search for the bracketing cell over the FP32 corner-packed
//      copy of sie (8 probes for 256 nodes, one 16-byte load each);
//   4. the cell's linear interpolant solved for lT in FP64, with the
//      division and the square roots seeded in FP32 and finished by one FP64
//      Newton correction (relative error ~1e-14, well inside the reference's
//      own 1e-14 tolerance in lT);
//   5. P, bmod (and cv, cs) interpolated at the root with the cell weights
//      already in hand.
#include <cuda_runtime.h>

#include "sgx_dispatch.cuh"
#include "sgx_internal.h"

namespace sgx {

namespace {

constexpr int LOOKUP_BLOCK = 256;

// a / b: FP32 quotient seed plus one FP64 residual correction.
__device__ __forceinline__ double div_seeded(const double a, const double b) {
  const float bf = __double2float_rn(b);
  const float rf = __frcp_rn(bf);
  const double r = static_cast<double>(rf);
  const double q0 = static_cast<double>(__double2float_rn(a) * rf);
  const double res = fma(-b, q0, a);
  const double q = fma(res, r, q0);
  // outside FP32 range the seed is meaningless: divide exactly instead
  return (fabsf(bf) > 1e-30f && fabsf(bf) < 1e30f) ? q : a / b;
}

// sqrt(v) for v > 0: FP32 seed plus one FP64 Newton correction.
__device__ __forceinline__ double sqrt_seeded(const double v) {
  const float vf = __double2float_rn(v);
  const float sf = sqrtf(vf);
  const double s0 = static_cast<double>(sf);
  const double h = static_cast<double>(0.5f / sf);
  const double s = fma(fma(-s0, s0, v), h, s0);
  return (vf > 1e-30f && vf < 1e30f) ? s : sqrt(v);
}

// NQT pow10 (logs.hpp:202-214, 290-292) with the square root seeded in FP32.
__device__ __forceinline__ double pow10_nqt_fast(const double x) {
  using namespace nqt;
  constexpr int64_t a = 9007199254740992;
  constexpr int64_t c = 18014398509481984;
  const int64_t x_as_int = static_cast<int64_t>(x * (log10_over_log2 * scale_up));
  const int64_t frac_as_int = x_as_int & mantissa_mask;
  const double sq = sqrt_seeded(static_cast<double>(c - 3 * frac_as_int));
  const int64_t frac_sqrt = static_cast<int64_t>(67108864.0 * sq);
  return __longlong_as_double(x_as_int + a - frac_sqrt - frac_as_int + one_as_int);
}

struct Cell {
  int i;
  double a1;
};

// Steps 3-4 for one element; false = take the reference iteration.
__device__ __forceinline__ bool solve_cell(const SpinerTable &t, const int j, const double b0,
                                           const double b1, const double sie, Cell &out) {
  const int nc = t.nT - 1;
  const fq4 *row32 = t.sie4f + static_cast<long long>(j) * nc;
  const dq4 *row64 = t.sie4 + static_cast<long long>(j) * nc;
  const float b0f = static_cast<float>(b0), b1f = static_cast<float>(b1);
  const float ef = static_cast<float>(sie);
  int lo = 0, hi = nc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    const fq4 q = row32[mid];
    if (fmaf(b1f, q.z, b0f * q.x) <= ef)
      lo = mid;
    else
      hi = mid - 1;
  }
  int i = lo;
  double a1 = 0.0;
  for (int k = 0; k < 4; ++k) {
    const dq4 c = row64[i];
    const double r0 = fma(b1, c.z, b0 * c.x);
    const double r1 = fma(b1, c.w, b0 * c.y);
    a1 = div_seeded(sie - r0, r1 - r0);
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
  if (!(a1 >= 0.0 && a1 <= 1.0)) return false; // not bracketed by the row
  out.i = i;
  out.a1 = a1;
  return true;
}

__device__ __forceinline__ double blend(const dq4 &c, const double a0, const double a1,
                                        const double b0, const double b1) {
  return fma(b1, fma(a1, c.w, a0 * c.z), b0 * fma(a1, c.y, a0 * c.x));
}

__global__ void __launch_bounds__(LOOKUP_BLOCK) spiner_fill_mixed(const FillArgs a) {
  __shared__ SpinerTable st;
  if (threadIdx.x == 0) st = sp_table(a.eos);
  __syncthreads();
  const SpinerTable &t = st;
  const unsigned out = a.output;
  const bool cold_on_rho_grid = (t.gCold.min == t.gRho.min) && (t.gCold.dx == t.gRho.dx) &&
                                (t.gCold.n == t.gRho.n);
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < a.n;
       e += stride) {
    const double rho = a.rho[e];
    const double sie = a.sie[e];
    double *lam = a.lambda ? a.lambda + e * a.lambda_stride : nullptr;
    const double lRho = sp_lRho(t, rho);
    int j;
    double b0, b1;
    t.gRho.weights(lRho, j, b0, b1);
    bool fast = t.sie_monotone_T && cold_on_rho_grid && b0 >= 0.0 && b1 >= 0.0;
    if (fast) {
      const float b0f = static_cast<float>(b0), b1f = static_cast<float>(b1);
      const float ef = static_cast<float>(sie);
      const float sc = fmaf(b1f, t.sieCold32[j + 1], b0f * t.sieCold32[j]);
      const float sm = fmaf(b1f, t.sielTMax32[j + 1], b0f * t.sielTMax32[j]);
      fast = ef > sc + 1e-6f * fabsf(sc) && ef < sm - 1e-6f * fabsf(sm);
    }
    Cell c{0, 0.0};
    if (fast) fast = solve_cell(t, j, b0, b1, sie, c);
    if (fast) {
      const int nc = t.nT - 1;
      const double lT = fma(static_cast<double>(c.i) + c.a1, t.gT.dx, t.gT.min);
      const double temp = pow10_nqt_fast(lT) - t.lTOffset;
      const double a1 = c.a1, a0 = 1.0 - c.a1;
      const long long ci = static_cast<long long>(j) * nc + c.i;
      // getLocDependsRhoT_ (:1394-1404) on the root
      const bool on = lT > (1 + SP_SOFT_THRESH) * t.lTMin && lT < (1 - SP_SOFT_THRESH) * t.lTMax;
      if (on) {
        if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = temp;
        if ((out & Q_PRESSURE) && a.press) a.press[e] = blend(t.P4[ci], a0, a1, b0, b1);
        if ((out & Q_CV) && a.cv) {
          const double *d = t.f2[F_DEDT] + static_cast<long long>(j) * t.nT + c.i;
          const dq4 q{d[0], d[1], d[t.nT], d[t.nT + 1]};
          const double cv = blend(q, a0, a1, b0, b1);
          a.cv[e] = cv > lim<double>::eps ? cv : lim<double>::eps;
        }
        if ((out & Q_BMOD) || a.cs) {
          double bmod = blend(t.bmod4[ci], a0, a1, b0, b1);
          bmod = bmod > lim<double>::eps ? bmod : lim<double>::eps;
          if ((out & Q_BMOD) && a.bmod) a.bmod[e] = bmod;
          if (a.cs) a.cs[e] = sqrt_seeded(div_seeded(bmod, rho));
        }
        if (lam) {
          lam[0] = lRho;
          lam[1] = lT;
        }
        continue;
      }
    }
    // The reference's FP64 path (eos_spiner_rho_temp.hpp:1052-1101).
    TableStatus w;
    const double lT = sp_lT_from_lRho_sie(t, lRho, sie, w, lam);
    const double temp = sp_T(t, lT);
    w = sp_loc_rho_T(t, lRho, lT);
    if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = temp;
    if ((out & Q_PRESSURE) && a.press) a.press[e] = sp_P_from(t, rho, lRho, temp, lT, w);
    if ((out & Q_CV) && a.cv) a.cv[e] = sp_cv_from(t, lRho, lT, w);
    if ((out & Q_BMOD) || a.cs) {
      const double bmod = sp_bmod_from(t, rho, lRho, temp, lT, w);
      if ((out & Q_BMOD) && a.bmod) a.bmod[e] = bmod;
      if (a.cs) a.cs[e] = sqrt(bmod / rho);
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
