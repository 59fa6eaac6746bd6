// FillEos of SpinerEOSDependsRhoSie from (rho, sie) in float-float, for the
// FP32 pipe.
//
// The reference's FillEos (eos/eos_spiner_rho_sie.hpp:844-898) with T among
// the outputs takes lRho = to_log(rho), lE = to_log(sie) and interpolates
// T, P, 1 / dT/de and bMod bilinearly on the rho-sie grid: two NQT logs and
// four interpolations, no root find. In FP64 that is about forty operations
// on GB300's FP64 pipe (1/64 of the FP32 rate) per query, so the plain path
// runs at a few percent of the HBM bandwidth. Here FP64 keeps one addition
// per coordinate:
//   1. to_log(x, off) = log10_nqt(|max(x, -off) + off| + EPS): the sum in
//      FP64 as the reference rounds it, then the NQT log's integer core
//      (logs.hpp:188-200) on its bits -- the same integer v the reference
//      scales by scale_down log10(2) (lambda gets that value bit for bit);
//   2. the cell coordinate u = (lX - min) / dx straight from v in fixed
//      point (one 64 x 64 -> 128-bit product with the table's constant), its
//      index clamped to the grid and its weight unclamped (linear
//      extrapolation off the grid, as DataBox::interpToReal) -- about 2^-46
//      absolute, where a float-float lX would lose two to three digits to
//      the scaling by 1 / dx;
//   3. one 128-byte cell holding the four fields in difference form
//      (SieCellFF), each f = x + a dE + b dR + a b dRE evaluated in
//      float-float and converted to double by integer operations.
// The result differs from the FP64 path by the reference's own roundings of
// the coordinates (~1e-15 of the log) times the interpolant's slope, about
// 1e-13 relative wherever the cell's corners share a sign. Elements whose
// inputs lie outside the float range (or NaN), and tables with values
// outside it, take the reference's FP64 arithmetic.
#define SGX_BARE_MODELS
#include <cuda_runtime.h>

#include "sgx_dispatch.cuh"
#include "sgx_ff.cuh"
#include "sgx_ff_table.cuh"
#include "sgx_internal.h"

namespace sgx {

namespace {

constexpr int SIE_BLOCK = 256;


// Whether a double converts to float-float without leaving the float range.
__device__ __forceinline__ bool ff_in_range(const double x) { return d_zero_or_exp_in(x, -74, 120); }

// The NQT log's integer v of spiner_common::to_log (eos_spiner_common.hpp:
// 52-54): the argument |max(x, -off) + off| + EPS in FP64 as the reference
// rounds it.
__device__ __forceinline__ long long to_log_int(const double x, const double off,
                                                const bool has_off) {
  double y;
  if (has_off) {
    y = (x < -off ? -off : x) + off;
  } else { // std::max(x, -0.0) + 0.0: zero for every negative x
    unsigned lo, hi;
    d_words(x, lo, hi);
    y = (hi >> 31) != 0u ? 0.0 : x;
  }
  return lg_nqt_int(fabs(y) + lim<double>::eps);
}

// An int64 of magnitude below 2^62 as float-float (about 48 of its bits).
__device__ __forceinline__ ff ff_from_i64(const long long v) {
  const float hi = __ll2float_rn(v);
  return quick_two_sum(hi, __ll2float_rn(v - f2ll_bits(hi)));
}

// Cell index and weight on one axis from v: u 2^F = mulhi(v, M) - Off, the
// index floor(u) clamped to [0, n - 2], the weight u - index (unclamped) as
// float-float, exact for |weight| < 2^(47 - F) (two 24-bit halves).
__device__ __forceinline__ int cell_of(const long long v, const long long M, const long long off,
                                       const int F, const int n, ff &w) {
  const long long U = __mul64hi(v, M) - off;
  long long j = U >> F;
  j = j < 0 ? 0 : (j > n - 2 ? n - 2 : j);
  const long long frac = U - (j << F);
  const float scale = __int_as_float((127 - F) << 23); // 2^-F
  if (frac > -(1LL << 47) && frac < (1LL << 47)) {
    const int hi = static_cast<int>(frac >> 24), lo = static_cast<int>(frac & 0xffffff);
    w = quick_two_sum(__int2float_rn(hi) * (scale * 16777216.0f), __int2float_rn(lo) * scale);
  } else { // far off the grid
    const ff f = ff_from_i64(frac);
    w = ff_make(f.hi * scale, f.lo * scale);
  }
  return static_cast<int>(j);
}

// The reference's FP64 arithmetic for one element (inputs outside the float
// range), with the outputs of the float-float path.
__device__ __noinline__ void sie_fill_fp64(const SieTable &t, const FillArgs &a, const long long e,
                                           const double rho, const double sie) {
  const double lRho = ss_lRho(t, rho), lE = ss_lE(t, sie);
  const unsigned out = a.output;
  if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = se_interp(t, SE_T, lRho, lE);
  if ((out & Q_PRESSURE) && a.press) a.press[e] = se_interp(t, SE_P, lRho, lE);
  if ((out & Q_CV) && a.cv) a.cv[e] = 1. / se_interp(t, SE_DTDE, lRho, lE);
  if ((out & Q_BMOD) || a.cs) {
    const double bmod = se_interp(t, SE_BMOD, lRho, lE);
    if ((out & Q_BMOD) && a.bmod) a.bmod[e] = bmod;
    if (a.cs) a.cs[e] = sqrt(bmod / rho);
  }
  if (a.lambda) a.lambda[e * a.lambda_stride] = lRho;
}

// sqrt(bmod / rho) in FP64 for the rare states the float-float form does
// not take (out of line, off the hot loop).
__device__ __noinline__ double cs_fp64(const double bmod, const double rho) {
  return sqrt(bmod / rho);
}

template <int MINB>
__global__ void __launch_bounds__(SIE_BLOCK, MINB) sie_fill_fast(const FillArgs a) {
  __shared__ SieTable st;
  if (threadIdx.x == 0) st = ss_table(a.eos);
  __syncthreads();
  const SieTable &t = st;
  const unsigned out = a.output;
  const bool rho_off = t.lRhoOffset != 0.0, e_off = t.lEOffset != 0.0;
  const int ncE = t.nE - 1;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; e < a.n;
       e += stride) {
    const double rho = __ldg(a.rho + e);
    const double sie = __ldg(a.sie + e);
    if (!(ff_in_range(rho) && ff_in_range(sie))) {
      sie_fill_fp64(t, a, e, rho, sie);
      continue;
    }
    const long long vR = to_log_int(rho, t.lRhoOffset, rho_off);
    const long long vE = to_log_int(sie, t.lEOffset, e_off);
    ff B, A;
    const int j = cell_of(vR, t.fxM[0], t.fxOff[0], t.fxF[0], t.nRhoE, B);
    const int i = cell_of(vE, t.fxM[1], t.fxOff[1], t.fxF[1], t.nE, A);
    const SieCellFF *c = t.cellsE + static_cast<long long>(j) * ncE + i;
    const ff AB = ff_mul(A, B);
    if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = ff2d_add(ff_cell(load_rec(&c->T), A, B, AB));
    if ((out & Q_PRESSURE) && a.press) a.press[e] = ff2d_add(ff_cell(load_rec(&c->P), A, B, AB));
    if ((out & Q_CV) && a.cv) {
      const ff d = ff_cell(load_rec(&c->dTdE), A, B, AB);
      const ff dn = quick_two_sum(d.hi, d.lo);
      // 1 / dT/de: the reciprocal of a zero is the reference's signed infinity
      const unsigned long long inf =
          0x7ff0000000000000ULL |
          (static_cast<unsigned long long>(__float_as_uint(dn.hi) >> 31) << 63);
      a.cv[e] = dn.hi == 0.0f ? __longlong_as_double(static_cast<long long>(inf))
                              : ff2d_add(ff_div_fast(ff_make(1.0f), dn));
    }
    if ((out & Q_BMOD) || a.cs) {
      const ff bm = ff_cell(load_rec(&c->bMod), A, B, AB);
      const ff BM = quick_two_sum(bm.hi, bm.lo);
      if ((out & Q_BMOD) && a.bmod) a.bmod[e] = ff2d_add(BM);
      if (a.cs) {
        // sqrt(bmod / rho) by one rsqrt correction while b rho stays well
        // inside the float range (and positive); the FP64 form otherwise
        const ff R = d2ff(rho);
        const float pr = BM.hi * R.hi;
        if (BM.hi > 0.0f && R.hi > 0.0f && pr > 1e-30f && pr < 1e30f)
          a.cs[e] = ff2d_add(ff_sqrt_ratio(BM, R));
        else
          a.cs[e] = cs_fp64(ff2d(BM), rho);
      }
    }
    if (a.lambda) // log10(rho) as the reference rounds it
      a.lambda[e * a.lambda_stride] =
          __dmul_rn(nqt::log2_over_log10, __dmul_rn(static_cast<double>(vR), nqt::scale_down));
  }
}

} // namespace

cudaError_t launch_fill_sie_mixed(const FillArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // persistent grid: the blocks resident at once for the registers budgeted
  const int minb = tune_get(SGX_TUNE_LOOKUP_BLOCKS_PER_SM);
  int resident = 0;
  if (minb >= 6)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, sie_fill_fast<6>, SIE_BLOCK, 0);
  else if (minb == 5)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, sie_fill_fast<5>, SIE_BLOCK, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, sie_fill_fast<4>, SIE_BLOCK, 0);
  const int per_sm = resident > 0 ? resident : 1;
  const long long want = (a.n + SIE_BLOCK - 1) / SIE_BLOCK;
  const long long cap = static_cast<long long>(sms) * per_sm;
  const int grid = static_cast<int>(want < cap ? want : cap);
  if (minb >= 6)
    sie_fill_fast<6><<<grid, SIE_BLOCK, 0, stream>>>(a);
  else if (minb == 5)
    sie_fill_fast<5><<<grid, SIE_BLOCK, 0, stream>>>(a);
  else
    sie_fill_fast<4><<<grid, SIE_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

} // namespace sgx
