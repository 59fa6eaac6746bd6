// Tabulated rho-T lookups (FillEos from rho and sie) with float-float
// arithmetic, for the FP32 pipe.
//
// FillEos of SpinerEOSDependsRhoT (eos/eos_spiner_rho_temp.hpp:1052-1101)
// inverts sie(lRho, lT) for lT by regula falsi over the bilinear table
// (lTFromlRhoSie_, :1192-1250): tens of FP64 iterations per query. At fixed
// lRho the bilinear interpolant is piecewise linear in lT, so when sie
// increases along T (checked per table at load) its root is unique and lies
// in the one grid cell whose density-blended end values bracket the target.
// On GB300 the FP64 pipe issues 1/64 of the FP32 pipe's operations, so the
// fast path below keeps FP64 to about a dozen operations per query and does
// the rest in float-float (sgx_ff.cuh, ~48 bits) and integer arithmetic:
//   1. lRho: the NQT log (logs.hpp:188-200) in integers and two FP64
//      scalings, the density cell and its weight b in FP64, all rounded as
//      in the reference (the interpolant has a kink at each density node).
//   2. on-table classification in FP32 with a 1e-6 guard band; inside the
//      band the reference's FP64 test decides, and a state off the table's
//      bottom is answered from the cold curves right there (in FP64, with
//      the reference's roundings). Off-top states, non-monotone tables and
//      tables with values outside the float range take the reference's FP64
//      iteration unchanged;
//   3. the bracketing T cell from the per-row thermal-energy bin index (one
//      16-bit load per density row, then 0-2 probes of the FP32
//      corner-packed copy of sie), or by binary search over that copy for
//      tables without the index;
//   4. the cell's bilinear form in difference form, sie = s00 + a dT + b dR
//      + a b dRT (differences formed in FP64 at load), solved for a: the
//      numerator sie - s00 - b dR, which cancels where the cold energy
//      dominates, and the denominator by FP64 fma, the quotient in ff. A
//      target under (over) the whole row pair is one the reference's regula
//      falsi cannot bracket: its answer is then its guess, reproduced here;
//   5. T = 10^lT by the NQT pow (logs.hpp:202-214) in integers: its
//      argument lT log10(2)^-1 2^52 in fixed point from the cell position
//      (nqt_arg), its square root in float-float; P, bmod and cs from their
//      difference-form cells at (a, b), each rounded to double once by one
//      FP64 addition of its exactly widened parts (ff2d_add).
// Accuracy against the FP64 path: T within ~1e-13 relative plus the
// conditioning of the root itself (about eps * sie / (dsie/dlT) where the
// cold energy dominates); P, bmod and cs within 1e-10 relative, or, where P
// is a small difference of large table entries, within how far the FP64
// value itself moves when sie changes by 1e-14 relative.
//
// Two kernels: spiner_fill_fast runs the steps above and marks, one bit per
// element, what it leaves to spiner_fill_ref (sgx_fp64.cu, compiled without
// FMA contraction, so those elements are bit-identical to the plain path),
// which runs the reference's FP64 iteration on the marked elements only.
// Keeping that iteration out of the fast kernel keeps its registers within
// the 5-blocks-per-SM budget without spilling. Predicates on doubles are
// integer tests of the bit patterns (read through an opaque move, so that
// they are not turned into double compares), so the FP64 pipe sees the
// eight roundings that must be the reference's, one int64 conversion and
// the outputs' additions.
// a mixed-precision path: bare models only (see sgx_dispatch.cuh)
#define SGX_BARE_MODELS
#include <mutex>

#include <cuda_runtime.h>

#include "sgx_dispatch.cuh"
#include "sgx_ff.cuh"
#include "sgx_ff_table.cuh"
#include "sgx_internal.h"
#include "sgx_table.h"

namespace sgx {

namespace {

constexpr int LOOKUP_BLOCK = 256;

// Constants of one table, shared by a block.
struct FfConsts {
  float rho_min_f, rho_inv_f; // density grid in FP32, for the cell estimate
  ff t_min, t_dx;      // temperature grid: lT min and dlT (lambda cache)
  // The NQT pow's integer argument X = lT log10(2)^-1 2^52 at the cell
  // position i + a of the T grid (nqt_arg): the nodes in fixed point,
  // (pm + i pd) 2^-fx, and the cell width pd as float-float with the split
  // 2^sh of a pd into integers (|a pd| < 2^(sh + 22), sh >= 22)
  long long pm, pd;
  int fx, sh;
  float pdh, pdl;
  float split, split_inv, m2; // 2^sh, 2^-sh, 1.5 2^(sh + 1)
  long long x_lo, x_hi; // on-table X (getLocDependsRhoT_), a guard band inside
  bool x_ok;            // the grid's X fits these forms
  ff eps;
};

__device__ __forceinline__ ff ff_of_int(const int i) { return ff_make(static_cast<float>(i)); }

// X = lT log10(2)^-1 2^52 at the T-cell position i + a (a in [0, 1]): the
// node's value from the fixed-point constants, plus a pd as a float-float
// product rounded to an integer by two magic-number additions (the high
// part to multiples of 2^sh, the rest to multiples of 2^(sh - 22)). About
// 30 units of an integer of magnitude ~2^55 (a's own ~2^-45 included),
// where the float-float sum of the scaled lT it replaces carried ~100.
__device__ __forceinline__ long long nqt_arg(const FfConsts &c, const int i, const ff A) {
  constexpr float M1 = 12582912.0f; // 1.5 2^23: y + M1 rounds |y| < 2^22 to an integer
  const long long xb = (c.pm + static_cast<long long>(i) * c.pd) >> c.fx;
  const float ph = __fmul_rn(A.hi, c.pdh);
  const float pl = fmaf(A.lo, c.pdh, fmaf(A.hi, c.pdl, fmaf(A.hi, c.pdh, -ph)));
  const float y1 = fmaf(ph, c.split_inv, M1);
  const int xh = __float_as_int(y1) - __float_as_int(M1);
  // ph - xh 2^sh, exact (|.| <= 2^(sh - 1), on ph's grid)
  const float r = fmaf(-__fsub_rn(y1, M1), c.split, ph);
  // m2's binade has the grid 2^(sh - 22) and holds m2 + y for |y| < 2^sh
  const float y2 = __fadd_rn(__fadd_rn(r, pl), c.m2);
  const int xl = __float_as_int(y2) - __float_as_int(c.m2);
  return xb + (static_cast<long long>(xh) << c.sh) + (static_cast<long long>(xl) << (c.sh - 22));
}

// pow2_nqt's result (logs.hpp:202-214) from its integer argument X: the
// square root 2^26 sqrt(c - 3 frac) in float-float (one Newton step on the
// correctly rounded float root), its two parts truncated to integers by
// their bit fields (2^26 hi has 53 bits; |2^26 lo| < 2^29).
__device__ __forceinline__ double nqt_pow_int(const long long X) {
  using namespace nqt;
  constexpr long long ca = 1LL << 53, cc = 1LL << 54;
  const long long frac = X & mantissa_mask;
  const long long N = cc - 3 * frac; // in (2^52, 2^54]
  const ff NF = quick_two_sum(static_cast<float>(static_cast<int>(N >> 30)) * 1073741824.0f,
                              static_cast<float>(static_cast<int>(N & ((1LL << 30) - 1))));
  const ff SQ = ff_sqrt_fast(NF);
  const unsigned uh = __float_as_uint(SQ.hi), ul = __float_as_uint(SQ.lo);
  // 2^26 x = m 2^(e - 124) for a float x of biased exponent e, significand m
  const long long fhi = static_cast<long long>((uh & 0x7fffffu) | 0x800000u)
                        << (static_cast<int>(uh >> 23) - 124);
  const int sl = static_cast<int>((ul >> 23) & 0xffu) - 124;
  const unsigned ml = (ul & 0x7fffffu) | 0x800000u;
  int flo = sl >= 0 ? static_cast<int>(ml << sl) : static_cast<int>(ml >> (-sl < 31 ? -sl : 31));
  flo = (ul & 0x7fffffffu) == 0u ? 0 : flo;
  flo = (ul & 0x80000000u) ? -flo : flo;
  return __longlong_as_double(X + ca - (fhi + flo) - frac + one_as_int);
}

// T and the on-table test for the reference's guess lT (roots its regula
// falsi cannot bracket), in FP64 as the reference computes both.
__device__ __noinline__ bool guess_T(const SpinerTable &t, const double lT, double &temp) {
  if (sp_loc_rho_T(t, 0.0, lT) != TableStatus::OnTable) return false;
  temp = sp_T(t, lT);
  return true;
}

__device__ __forceinline__ SieRec load_sie(const SieRec *p) {
  SieRec r;
  asm("ld.global.nc.v4.f64 {%0,%1,%2,%3}, [%4];"
      : "=d"(r.x), "=d"(r.dT), "=d"(r.dR), "=d"(r.dRT)
      : "l"(p));
  return r;
}

// Integer tests of a double's bit pattern (no FP64 pipe).
__device__ __forceinline__ bool d_is_zero(const double x) { return d_zero_bits(x); }
// The unbiased binary exponent of x (normal x).
__device__ __forceinline__ int d_exp(const double x) {
  return static_cast<int>((__double_as_longlong(x) >> 52) & 0x7ff) - 1023;
}
// x > 0 and not NaN (for the callers' range checks that follow)
__device__ __forceinline__ bool d_positive(const double x) {
  unsigned lo, hi;
  d_words(x, lo, hi);
  return (hi >> 31) == 0u && (hi | lo) != 0u;
}
// x in [+0, 1] (non-negative doubles order as their bit patterns)
__device__ __forceinline__ bool d_in_unit(const double x) {
  unsigned lo, hi;
  d_words(x, lo, hi);
  return hi < 0x3FF00000u || (hi == 0x3FF00000u && lo == 0u);
}
// ff_from_double_ok
__device__ __forceinline__ bool ff_ok_bits(const double x) { return d_zero_or_exp_in(x, -74, 127); }

// One bulk copy (cp.async.bulk, the TMA engine) of `bytes` (a multiple of
// 16, both addresses 16-byte aligned) from global to shared memory, issued
// by thread 0 and completed on an mbarrier that every thread of the block
// waits on. The wait is bounded: if the copy has not landed after
// BULK_WAIT_LIMIT polls (it lands in about a microsecond), the block
// returns false and searches without the staged index, after a second
// bounded wait for the copy so that it never lands in a finished block.
constexpr int BULK_WAIT_LIMIT = 1 << 22;
__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ bool mbar_try_wait(const unsigned bar, const unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ bool bulk_stage(void *dst, const void *src, const unsigned bytes) {
  __shared__ __align__(8) unsigned long long mbar;
  const unsigned bar = smem_addr(&mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                 "[%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
  }
  bool done = false;
  for (int it = 0; it < BULK_WAIT_LIMIT && !done; ++it)
    done = mbar_try_wait(bar, 0);
  // the block agrees: staged only if every thread saw the copy land
  const bool all = __syncthreads_and(done) != 0;
  if (!all)
    for (int it = 0; it < BULK_WAIT_LIMIT && !done; ++it)
      done = mbar_try_wait(bar, 0);
  return all;
}

// A 1-D table at the density cell (j, b1) as interpToReal rounds it
// (w0 d[j] + w1 d[j+1], w0 = 1 - w1), without contraction.
__device__ __forceinline__ double interp_cell(const double *d, const int j, const double b1) {
  return __dadd_rn(__dmul_rn(__dsub_rn(1.0, b1), d[j]), __dmul_rn(b1, d[j + 1]));
}

// getLocDependsRhoSie_ (eos_spiner_rho_temp.hpp:1377-1392) at the density
// cell (j, b1), in FP64 with the reference's roundings: 0 on the table,
// 1 off its bottom (at or under the cold curve), 2 off its top.
__device__ __noinline__ int table_loc_fp64(const SpinerTable &t, const int j, const double b1,
                                           const double sie) {
  const double cold = interp_cell(t.f1[F_SIECOLD], j, b1);
  const double top = interp_cell(t.f1[F_SIELTMAX], j, b1);
  if (sie >= __dsub_rn(top, __dmul_rn(SP_SOFT_THRESH, fabs(top)))) return 2;
  if (sie <= __dadd_rn(cold, __dmul_rn(SP_SOFT_THRESH, fabs(cold)))) return 1;
  return 0;
}

// FillEos off the table's bottom (eos_spiner_rho_temp.hpp:1201-1207 and the
// cold-curve branches of PFromRholRhoTlT_, CvFromlRholT_ and
// bModFromRholRhoTlT_, :1320-1375): lT = lTMin and P, cv and bmod from the
// cold curves at the density cell, in FP64 with the reference's roundings.
__device__ __noinline__ void fill_off_bottom(const SpinerTable &t, const FillArgs &a,
                                             const long long e, const double rho,
                                             const double lRho, const int j, const double b1) {
  const unsigned out = a.output;
  if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = t.TatlTMin;
  if ((out & Q_PRESSURE) && a.press) a.press[e] = interp_cell(t.f1[F_PCOLD], j, b1);
  if ((out & Q_CV) && a.cv) {
    const double cv = interp_cell(t.f1[F_DEDTCOLD], j, b1);
    a.cv[e] = cv > lim<double>::eps ? cv : lim<double>::eps;
  }
  if ((out & Q_BMOD) || a.cs) {
    double bmod = interp_cell(t.f1[F_BMODCOLD], j, b1);
    bmod = bmod > lim<double>::eps ? bmod : lim<double>::eps;
    if ((out & Q_BMOD) && a.bmod) a.bmod[e] = bmod;
    if (a.cs) a.cs[e] = __dsqrt_rn(__ddiv_rn(bmod, rho));
  }
  if (a.lambda) {
    double *lam = a.lambda + e * a.lambda_stride;
    lam[0] = lRho;
    lam[1] = t.lTMin;
  }
}

// The reference's lT when its regula falsi cannot bracket sie inside
// [lTMin, lTMax] (on the table, but below the interpolant's value at lTMin
// or above it at lTMax, which a coarse table produces between density
// nodes): lTFromlRhoSie_ (:1222-1246) then returns its guess, the lambda
// cache when it lies in range or the middle of the range. Also the cell
// (i, a) of that lT, as Grid1D::weights rounds them.
__device__ __noinline__ double unbracketed_lT(const SpinerTable &t, const double *lam, int &i,
                                              double &a1) {
  double lT = __dmul_rn(0.5, __dadd_rn(t.lTMin, t.lTMax));
  if (lam != nullptr) {
    const double c = lam[1];
    if ((t.lTMin <= c) && (c <= t.lTMax)) lT = c;
  }
  const double u = __dmul_rn(__dsub_rn(lT, t.gT.min), t.gT.inv_dx);
  i = !(u >= 0.0) ? 0 : (u > static_cast<double>(t.gT.n - 2) ? t.gT.n - 2 : static_cast<int>(u));
  const double xl = __dadd_rn(t.gT.min, __dmul_rn(static_cast<double>(i), t.gT.dx));
  a1 = __dmul_rn(__dsub_rn(lT, xl), t.gT.inv_dx);
  return lT;
}

// Grid1D::index and ::weights in FP64 (the rare queries whose FP32 cell
// estimate lies within 1e-4 of a density node): the last cell takes
// everything above it (the weight check of the caller keeps only the table's
// own range). Out of line, keeping the rare path's FP64 code out of the hot
// loop. Returns whether lRho lies at or above the grid's start.
__device__ __noinline__ bool density_cell_fp64(const SpinerTable &t, const double lRho, int &j,
                                               double &b1) {
  const double u = __dmul_rn(__dsub_rn(lRho, t.gRho.min), t.gRho.inv_dx);
  const bool fast = u >= 0.0;
  j = !fast ? 0 : (u > static_cast<double>(t.nRho - 2) ? t.nRho - 2 : static_cast<int>(u));
  b1 = __dmul_rn(__dsub_rn(lRho, __ldg(t.rhoNodes + j)), t.gRho.inv_dx);
  return fast;
}

// cv on the table at the cell (j, i) and weights (a1, b1), in FP64 (out of
// line, off the hot loop of the FillEos forms that do not ask for cv).
__device__ __noinline__ double cv_fp64(const SpinerTable &t, const int j, const int i,
                                       const double b1, const double a1) {
  const double *d = t.f2[F_DEDT] + static_cast<long long>(j) * t.nT + i;
  const double cv = b1 * (a1 * d[t.nT + 1] + (1.0 - a1) * d[t.nT]) +
                    (1.0 - b1) * (a1 * d[1] + (1.0 - a1) * d[0]);
  return cv > lim<double>::eps ? cv : lim<double>::eps;
}

// MINB: resident blocks per SM the registers are budgeted for (4: 64
// registers, 5: 48, 6: 40).
template <int MINB>
__global__ void __launch_bounds__(LOOKUP_BLOCK, MINB)
    spiner_fill_fast(const FillArgs a, const int stage_coarse, unsigned *__restrict__ left) {
  __shared__ SpinerTable st;
  __shared__ FfConsts sc;
  extern __shared__ __align__(16) float2 s_coarse[]; // [nRho-1][SP_COARSE_ROW] when staged
  if (threadIdx.x == 0) {
    st = sp_table(a.eos);
    sc.rho_min_f = d2ff(st.gRho.min).hi;
    sc.rho_inv_f = d2ff(st.gRho.inv_dx).hi;
    sc.t_min = d2ff(st.gT.min);
    sc.t_dx = d2ff(st.gT.dx);
    // X = lT K; the nodes' X in fixed point with 2^fx their largest |X|
    // below 2^62, the cell width as float-float
    const double K = nqt::log10_over_log2 * nqt::scale_up;
    const double pmin = st.gT.min * K, pdx = st.gT.dx * K;
    const double mx = fabs(pmin) + (st.gT.n - 1) * fabs(pdx) + 1.0;
    sc.fx = 61 - ilogb(mx);
    sc.sh = ilogb(pdx) - 21;
    sc.sh = sc.sh < 22 ? 22 : sc.sh;
    sc.x_ok = sc.fx >= 0 && pdx > 0.0 && sc.sh <= 40 && ff_ok_bits(pdx);
    if (sc.x_ok) {
      sc.pm = llrint(ldexp(pmin, sc.fx));
      sc.pd = llrint(ldexp(pdx, sc.fx));
      const ff pd = d2ff(pdx);
      sc.pdh = pd.hi;
      sc.pdl = pd.lo;
      sc.split = ldexpf(1.0f, sc.sh);
      sc.split_inv = ldexpf(1.0f, -sc.sh);
      sc.m2 = ldexpf(1.5f, sc.sh + 1);
      // the reference's bounds, a band of 2^20 units (~3e-11 of lT) inside
      // them, far wider than X's error against the FP64 root, so that a
      // state the fast path answers is one the reference finds on the table
      constexpr long long band = 1LL << 20;
      sc.x_lo = llrint(floor((1 + SP_SOFT_THRESH) * st.lTMin * K)) + band;
      sc.x_hi = llrint(ceil((1 - SP_SOFT_THRESH) * st.lTMax * K)) - band;
    }
    sc.eps = d2ff(lim<double>::eps);
  }
  __syncthreads();
  // the coarse index, [nRho-1][SP_COARSE_ROW] float2, into shared memory:
  // stage_coarse 1 by vector loads, 2 by one bulk copy (TMA) completing on
  // an mbarrier; 0 leaves the whole search in global memory
  constexpr int CS = SP_COARSE_ROW;
  int staged = stage_coarse;
  if (stage_coarse == 1) {
    const int n4 = (st.nRho - 1) * CS / 2;
    const float4 *src = reinterpret_cast<const float4 *>(st.sieCoarse);
    float4 *dst = reinterpret_cast<float4 *>(s_coarse);
    for (int k = threadIdx.x; k < n4; k += blockDim.x)
      dst[k] = __ldg(src + k);
    __syncthreads();
  } else if (stage_coarse == 2) {
    const unsigned bytes = static_cast<unsigned>((st.nRho - 1) * CS * sizeof(float2));
    if (!bulk_stage(s_coarse, st.sieCoarse, bytes)) staged = 0;
  }
  const SpinerTable &t = st;
  const unsigned out = a.output;
  const int nc = t.nT - 1;
  const bool table_fast = t.ff_ok && sc.x_ok && t.sie_monotone_T && d_is_zero(t.lRhoOffset) &&
                          (t.gCold.min == t.gRho.min) && (t.gCold.dx == t.gRho.dx) &&
                          (t.gCold.n == t.gRho.n) && ff_ok_bits(t.gRho.min) &&
                          ff_ok_bits(t.gT.min);
  const bool t_offset = !d_is_zero(t.lTOffset);
  // getLocDependsRhoT_(lRho, lTMin) is OffBottom (lTMin > 0)
  const bool bottom_ok = t.lTMin <= (1 + SP_SOFT_THRESH) * t.lTMin;
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  // the next element's inputs are loaded while this one is computed
  long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  double rho_next = e < a.n ? __ldg(a.rho + e) : 0.0;
  double sie_next = e < a.n ? __ldg(a.sie + e) : 0.0;
  // Every warp covers 32 consecutive elements starting at a multiple of 32
  // (blocks and the stride are multiples of 256), so each iteration's
  // ballot is exactly one word of the left-over mask.
  for (; e < a.n; e += stride) {
    const double rho = rho_next;
    const double sie = sie_next;
    if (e + stride < a.n) {
      rho_next = __ldg(a.rho + e + stride);
      sie_next = __ldg(a.sie + e + stride);
    }
    bool fast = table_fast && d_positive(rho) && ff_ok_bits(rho) && ff_ok_bits(sie);
    bool done = false;
    double lt_guess = 0.0; // the reference's guess, when it is the answer
    int j = 0, i = 0;
    double lRho = 0.0, b1 = 0.0;
    ff B{0.f, 0.f}, A{0.f, 0.f};
    if (fast) {
      // 1. lRho = log10_nqt(rho + eps) (to_log with offset 0) in FP64 as
      //    the reference rounds it, its cell from an FP32 estimate, and the
      //    density weight in FP64 (its error is multiplied by the cell's
      //    density difference in the root below)
      using namespace nqt;
      // two roundings, as lg_nqt then log10 (scale_down is the reference's
      // 15-digit literal, not exactly 2^-52)
      lRho = __dmul_rn(log2_over_log10,
                       __dmul_rn(static_cast<double>(lg_nqt_int(rho + lim<double>::eps)), scale_down));
      // Grid1D::index and ::weights with the FP64 path's roundings: the
      // interpolant has a kink at every density node, so the cell must be the
      // reference's, and the root multiplies an error in b by dR / dT (up to
      // ~1e5 at low T)
      // Grid1D::index: an FP32 estimate decides unless it lies within 1e-4
      // of a node, where the FP64 index is taken
      const float uf = (d2ff(lRho).hi - sc.rho_min_f) * sc.rho_inv_f;
      const float jf = floorf(uf);
      bool exact = !(uf - jf > 1e-4f && uf - jf < 1.0f - 1e-4f) || !(jf >= 0.0f) ||
                   jf > static_cast<float>(t.nRho - 2);
      if (!exact) {
        j = static_cast<int>(jf);
        b1 = __dmul_rn(__dsub_rn(lRho, __ldg(t.rhoNodes + j)), t.gRho.inv_dx);
        // a wrong estimate shows as a weight outside [0, 1]
        exact = !d_in_unit(b1);
      }
      if (exact) fast = density_cell_fp64(t, lRho, j, b1);
      B = ff_ok_bits(b1) ? d2ff(b1) : ff_make(0.0f);
      fast = fast && B.hi >= 0.0f && B.hi <= 1.0f;
    }
    if (fast) {
      // 2. on-table, outside the guard band
      const float b1f = B.hi, b0f = 1.0f - B.hi;
      const float ef = d2ff(sie).hi;
      const float sc0 = fmaf(b1f, t.sieCold32[j + 1], b0f * t.sieCold32[j]);
      const float sm0 = fmaf(b1f, t.sielTMax32[j + 1], b0f * t.sielTMax32[j]);
      // inside the guard band FP64 decides, as the reference does; off the
      // bottom (where lT = lTMin is itself classified off the bottom) the
      // cold curves give the answer here
      if (!(ef > sc0 + 1e-6f * fabsf(sc0) && ef < sm0 - 1e-6f * fabsf(sm0))) {
        const int loc = table_loc_fp64(t, j, b1, sie);
        fast = loc == 0;
        if (loc == 1 && bottom_ok) {
          fill_off_bottom(t, a, e, rho, lRho, j, b1);
          done = true;
        }
      }
      if (fast) {
        // 3. bracketing cell in FP32: with the thermal bin index, between the
        //    two density rows' cells for the blended thermal target sie -
        //    sieCold (one or two cells apart); otherwise first among every
        //    coarse_stride-th node (shared memory), then within that stretch
        const fq4 *row32 = t.sie4f + static_cast<long long>(j) * nc;
        int lo = 0, hi = nc - 1;
        if (t.therm_idx) {
          const float ep = ef - sc0;
          int k = ep > 0.0f ? static_cast<int>(__float_as_uint(ep) >> t.therm_shift) - t.therm_base
                            : 0;
          k = k < 0 ? 0 : (k >= t.therm_bins ? t.therm_bins - 1 : k);
          const uint16_t *ti = t.therm_idx + static_cast<long long>(j) * t.therm_bins + k;
          const int c0 = __ldg(ti), c1 = __ldg(ti + t.therm_bins);
          lo = c0 < c1 ? c0 : c1;
          hi = (c0 < c1 ? c1 : c0) + 1;
          hi = hi < nc - 1 ? hi : nc - 1;
        } else if (staged) {
          const float2 *cr = s_coarse + j * CS;
          int kl = 0, kh = SP_COARSE - 1;
          while (kl < kh) {
            const int mid = (kl + kh + 1) >> 1;
            const float2 q = cr[mid];
            if (fmaf(b1f, q.y, b0f * q.x) <= ef)
              kl = mid;
            else
              kh = mid - 1;
          }
          lo = kl * t.coarse_stride;
          hi = min(lo + t.coarse_stride - 1, nc - 1);
        }
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          const fq4 q = row32[mid];
          if (fmaf(b1f, q.z, b0f * q.x) <= ef)
            lo = mid;
          else
            hi = mid - 1;
        }
        i = lo;
        // 4. a in the cell (neighbours when FP32 picked the wrong one)
        const SieRec *row = t.sieR + static_cast<long long>(j) * nc;
        bool ok = false;
        int edge = 0; // -1 / +1: sie below / above the whole row pair
        // (one probe almost always; not unrolled)
#pragma unroll 1
        for (int k = 0; k < 4; ++k) {
          const SieRec r = load_sie(row + i);
          // sie = x + a (dT + b dRT) + b dR: numerator and denominator in FP64
          const double num = fma(-b1, r.dR, sie - r.x);
          const double den = fma(b1, r.dRT, r.dT);
          // (ff_div_fast's reciprocal needs |den| < 2^126)
          if (!ff_ok_bits(num) || !ff_ok_bits(den) || d_is_zero(den) || d_exp(den) > 120) break;
          A = ff_div_fast(d2ff(num), d2ff(den));
          // a past the cell's upper node: a weight of 1 + 1e-9 has a float
          // leading part of exactly 1, so the test takes the low part too
          // (the lower cell's form extended past the node misses the root
          // in the next cell by up to ~1e-9 of a cell)
          const bool above = A.hi > 1.0f || (A.hi == 1.0f && A.lo > 0.0f);
          if (A.hi < 0.0f && i > 0) {
            --i;
            continue;
          }
          if (above && i < nc - 1) {
            ++i;
            continue;
          }
          ok = A.hi >= 0.0f && !above;
          if (!ok) edge = (i == 0 && A.hi < -1e-6f) ? -1 : (i == nc - 1 && A.hi > 1.000001f) ? 1 : 0;
          break;
        }
        fast = ok;
        if (!ok && edge != 0 && !t.reproducible) {
          // unbracketed: the reference's answer is its guess
          double a64;
          lt_guess = unbracketed_lT(t, a.lambda ? a.lambda + e * a.lambda_stride : nullptr, i, a64);
          A = d2ff(a64);
          fast = true;
        }
      }
    }
    if (fast) {
      // 5. T = 10^lT by the NQT pow in integers, its argument X = lT
      //    log10(2)^-1 2^52 from the cell position i + a; on the table in T
      //    too (getLocDependsRhoT_): a root within 1e-8 of either end takes
      //    the FP64 pass, whose off-table forms then apply
      const bool rooted = d_is_zero(lt_guess);
      double temp = 0.0;
      bool on;
      if (rooted) {
        const long long X = nqt_arg(sc, i, A);
        on = X > sc.x_lo && X < sc.x_hi;
        temp = nqt_pow_int(X);
        if (t_offset) temp -= t.lTOffset;
      } else {
        on = guess_T(t, lt_guess, temp);
      }
      if (on) {
        const long long ci = static_cast<long long>(j) * nc + i;
        const ff AB = ff_mul(A, B);
        if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = temp;
        if ((out & Q_PRESSURE) && a.press)
          a.press[e] = ff2d_add(ff_cell(load_rec(t.PR + ci), A, B, AB));
        if ((out & Q_BMOD) || a.cs) {
          const ff bm = ff_cell(load_rec(t.bmodR + ci), A, B, AB);
          ff BM = quick_two_sum(bm.hi, bm.lo);
          if (ff_lt(BM, sc.eps)) BM = sc.eps;
          if ((out & Q_BMOD) && a.bmod) a.bmod[e] = ff2d_add(BM);
          if (a.cs) {
            // sqrt(bmod / rho) by one rsqrt correction while b rho stays well
            // inside the float range, by the exact ff quotient otherwise
            const ff R = d2ff(rho);
            const float pr = BM.hi * R.hi;
            a.cs[e] = ff2d_add((pr > 1e-30f && pr < 1e30f) ? ff_sqrt_ratio(BM, R)
                                                            : ff_sqrt(ff_div(BM, R)));
          }
        }
        if ((out & Q_CV) && a.cv) a.cv[e] = cv_fp64(t, j, i, b1, ff2d(A));
        if (a.lambda) {
          double *lam = a.lambda + e * a.lambda_stride;
          lam[0] = lRho;
          lam[1] = rooted ? ff2d(ff_add(ff_mul(ff_add(ff_of_int(i), A), sc.t_dx), sc.t_min))
                          : lt_guess;
        }
        done = true;
      }
    }
    const unsigned mask = __ballot_sync(__activemask(), !done);
    if ((threadIdx.x & 31) == __ffs(__activemask()) - 1) left[e >> 5] = mask;
  }
}

} // namespace

// Sets aside L2 for persisting lines once per device (up to the device's
// maximum, at most the table's size); false where the device has none.
bool l2_persist_ready(const uint64_t table) {
  static std::mutex mu;
  static size_t set_aside[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  const size_t want = table_bytes(table);
  std::lock_guard<std::mutex> lk(mu);
  if (set_aside[dev] < want) {
    int maxp = 0, maxw = 0;
    cudaDeviceGetAttribute(&maxp, cudaDevAttrMaxPersistingL2CacheSize, dev);
    cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxAccessPolicyWindowSize, dev);
    if (maxp <= 0 || static_cast<size_t>(maxw) < want) return false;
    const size_t size = want < static_cast<size_t>(maxp) ? want : static_cast<size_t>(maxp);
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, size) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    set_aside[dev] = size;
  }
  return true;
}

cudaError_t launch_fill_mixed(const FillArgs &a, cudaStream_t stream) {
  if (a.n <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // the coarse index of the T search, staged per block when it fits
  const int nrho = table_nrho(a.eos.table);
  const size_t coarse =
      nrho > 1 ? static_cast<size_t>(nrho - 1) * SP_COARSE_ROW * sizeof(float2) : 0;
  // (the thermal bin index, where the table has one, replaces the staged
  // coarse index)
  const int stage = (coarse > 0 && coarse <= 40 * 1024 && !table_has_thermal_index(a.eos.table))
                        ? tune_get(SGX_TUNE_LOOKUP_STAGE)
                        : 0;
  // the left-over mask, one bit per element
  const size_t words = static_cast<size_t>((a.n + 31) >> 5);
  void *left = nullptr;
  cudaError_t e = scratch_alloc(&left, words * sizeof(unsigned), stream);
  if (e != cudaSuccess) return e;
  // persistent grid: the blocks resident at once (registers budgeted for
  // minb per SM, shared memory permitting), each staging the index once
  const int minb = tune_get(SGX_TUNE_LOOKUP_BLOCKS_PER_SM);
  const size_t smem = stage ? coarse : 0;
  int resident = 0;
  if (minb == 6)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, spiner_fill_fast<6>, LOOKUP_BLOCK,
                                                  smem);
  else if (minb == 5)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, spiner_fill_fast<5>, LOOKUP_BLOCK,
                                                  smem);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, spiner_fill_fast<4>, LOOKUP_BLOCK,
                                                  smem);
  const int per_sm = resident > 0 ? (resident < minb ? resident : minb) : 1;
  const long long want = (a.n + LOOKUP_BLOCK - 1) / LOOKUP_BLOCK;
  const long long cap = static_cast<long long>(sms) * per_sm;
  const int grid = static_cast<int>(want < cap ? want : cap);
  unsigned *lp = static_cast<unsigned *>(left);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(LOOKUP_BLOCK);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  // the table's lines persist in L2 across the streaming inputs and outputs
  cudaLaunchAttribute attr[1];
  if (tune_get(SGX_TUNE_L2_PERSIST) && l2_persist_ready(a.eos.table)) {
    attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
    attr[0].val.accessPolicyWindow.base_ptr = reinterpret_cast<void *>(a.eos.table);
    attr[0].val.accessPolicyWindow.num_bytes = table_bytes(a.eos.table);
    attr[0].val.accessPolicyWindow.hitRatio = 1.0f;
    attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  if (minb == 6)
    e = cudaLaunchKernelEx(&cfg, spiner_fill_fast<6>, a, stage, lp);
  else if (minb == 5)
    e = cudaLaunchKernelEx(&cfg, spiner_fill_fast<5>, a, stage, lp);
  else
    e = cudaLaunchKernelEx(&cfg, spiner_fill_fast<4>, a, stage, lp);
  if (e == cudaSuccess) e = launch_fill_ref(a, static_cast<const unsigned *>(left), stream);
  const cudaError_t f = scratch_free(left, stream);
  return e != cudaSuccess ? e : f;
}

} // namespace sgx
