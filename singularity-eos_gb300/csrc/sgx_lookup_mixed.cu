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
// fast path below keeps FP64 to about fifteen operations per query and does
// the rest in float-float (sgx_ff.cuh, ~48 bits) and integer arithmetic:
//   1. lRho: the NQT log (logs.hpp:188-200) in integers and two FP64
//      scalings, the density cell and its weight b in FP64, all rounded as
//      in the reference (the interpolant has a kink at each density node).
//   2. on-table classification in FP32 with a 1e-6 guard band (elements in
//      the band, off-table states, unbracketed targets, non-monotone tables
//      and tables with values outside the float range take the reference's
//      FP64 iteration unchanged);
//   3. binary search for the bracketing T cell over the FP32 corner-packed
//      copy of sie (8 probes for 256 nodes, one 16-byte load each);
//   4. the cell's bilinear form in difference form, sie = s00 + a dT + b dR
//      + a b dRT (differences formed in FP64 at load), solved for a: the
//      numerator sie - s00 - b dR, which cancels where the cold energy
//      dominates, and the denominator by FP64 fma, the quotient in ff;
//   5. T = 10^lT by the NQT pow (logs.hpp:202-214) in integers, with its
//      square root in float-float; P, bmod and cs from their difference-form
//      cells at (a, b), each rounded to double once.
// Accuracy against the FP64 path: T within ~1e-13 relative plus the
// conditioning of the root itself (about eps * sie / (dsie/dlT) where the
// cold energy dominates), P, bmod and cs within 1e-10 of the larger of the
// value and 1e-6 of the batch's largest magnitude.
#include <cuda_runtime.h>

#include "sgx_dispatch.cuh"
#include "sgx_ff.cuh"
#include "sgx_internal.h"
#include "sgx_table.h"

namespace sgx {

namespace {

constexpr int LOOKUP_BLOCK = 256;

// Constants of one table, in float-float, shared by a block.
struct FfConsts {
  float rho_min_f, rho_inv_f; // density grid in FP32, for the cell estimate
  ff t_min, t_dx;      // temperature grid: lT min and dlT
  ff p2_scale;         // log10(2)^-1 * 2^52: lT -> NQT pow integer
  ff lt_lo, lt_hi;     // on-table lT bounds (getLocDependsRhoT_)
  ff eps;
};

__device__ __forceinline__ ff ff_of_int(const int i) { return ff_make(static_cast<float>(i)); }

// The record's field f = x + a dT + b dR + a b dRT at (a, b); AB = a b.
__device__ __forceinline__ ff ff_cell(const FfRec &r, const ff A, const ff B, const ff AB) {
  const ff x = ff_make(r.x[0], r.x[1]);
  const ff t = ff_mul(A, ff_make(r.dT[0], r.dT[1]));
  const ff d = ff_mul(B, ff_make(r.dR[0], r.dR[1]));
  const ff c = ff_mul(AB, ff_make(r.dRT[0], r.dRT[1]));
  return ff_add(x, ff_add(t, ff_add(d, c)));
}

__device__ __forceinline__ FfRec load_rec(const FfRec *p) {
  const float4 u = __ldg(reinterpret_cast<const float4 *>(p));
  const float4 v = __ldg(reinterpret_cast<const float4 *>(p) + 1);
  FfRec r;
  r.x[0] = u.x, r.x[1] = u.y, r.dT[0] = u.z, r.dT[1] = u.w;
  r.dR[0] = v.x, r.dR[1] = v.y, r.dRT[0] = v.z, r.dRT[1] = v.w;
  return r;
}
__device__ __forceinline__ SieRec load_sie(const SieRec *p) {
  const double2 u = __ldg(reinterpret_cast<const double2 *>(p));
  const double2 v = __ldg(reinterpret_cast<const double2 *>(p) + 1);
  return {u.x, u.y, v.x, v.y};
}

__global__ void __launch_bounds__(LOOKUP_BLOCK, 4) spiner_fill_mixed(const FillArgs a,
                                                                     const int stage_coarse) {
  __shared__ SpinerTable st;
  __shared__ FfConsts sc;
  extern __shared__ float2 s_coarse[]; // [nRho-1][SP_COARSE] when staged
  if (threadIdx.x == 0) {
    st = sp_table(a.eos);
    sc.rho_min_f = d2ff(st.gRho.min).hi;
    sc.rho_inv_f = d2ff(st.gRho.inv_dx).hi;
    sc.t_min = d2ff(st.gT.min);
    sc.t_dx = d2ff(st.gT.dx);
    sc.p2_scale = d2ff(nqt::log10_over_log2 * nqt::scale_up);
    sc.lt_lo = d2ff((1 + SP_SOFT_THRESH) * st.lTMin);
    sc.lt_hi = d2ff((1 - SP_SOFT_THRESH) * st.lTMax);
    sc.eps = d2ff(lim<double>::eps);
  }
  __syncthreads();
  // shared rows padded to SP_COARSE + 1 entries: lanes probing the same
  // entry of different rows then fall in different banks
  constexpr int CS = SP_COARSE + 1;
  if (stage_coarse) {
    const int nco = (st.nRho - 1) * SP_COARSE;
    for (int k = threadIdx.x; k < nco; k += blockDim.x)
      s_coarse[(k / SP_COARSE) * CS + k % SP_COARSE] = __ldg(st.sieCoarse + k);
    __syncthreads();
  }
  const SpinerTable &t = st;
  const unsigned out = a.output;
  const int nc = t.nT - 1;
  const bool table_fast = t.ff_ok && t.sie_monotone_T && t.lRhoOffset == 0.0 &&
                          (t.gCold.min == t.gRho.min) && (t.gCold.dx == t.gRho.dx) &&
                          (t.gCold.n == t.gRho.n) &&
                          ff_from_double_ok(t.gRho.min) && ff_from_double_ok(t.gT.min);
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  // the next element's inputs are loaded while this one is computed
  long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  double rho_next = e < a.n ? __ldg(a.rho + e) : 0.0;
  double sie_next = e < a.n ? __ldg(a.sie + e) : 0.0;
  for (; e < a.n; e += stride) {
    const double rho = rho_next;
    const double sie = sie_next;
    if (e + stride < a.n) {
      rho_next = __ldg(a.rho + e + stride);
      sie_next = __ldg(a.sie + e + stride);
    }
    double *lam = a.lambda ? a.lambda + e * a.lambda_stride : nullptr;
    bool fast = table_fast && rho > 0.0 && ff_from_double_ok(rho);
    int j = 0, i = 0;
    double lRho = 0.0, b1 = 0.0;
    ff B{0.f, 0.f}, A{0.f, 0.f};
    if (fast) {
      // 1. lRho = log10_nqt(rho + eps) (to_log with offset 0) in FP64 as
      //    the reference rounds it, its cell from an FP32 estimate, and the
      //    density weight in FP64 (its error is multiplied by the cell's
      //    density difference in the root below)
      using namespace nqt;
      const long long x_as_int = __double_as_longlong(rho + lim<double>::eps) - one_as_int;
      const long long frac = x_as_int & mantissa_mask;
      const long long fh = frac >> 26, fl = frac & low_mask;
      const long long fsq = fh * fh + ((fh * fl) >> 25);
      // two roundings, as lg_nqt then log10 (scale_down is the reference's
      // 15-digit literal, not exactly 2^-52)
      lRho = __dmul_rn(log2_over_log10,
                       __dmul_rn(static_cast<double>(x_as_int + ((frac - fsq) / 3)), scale_down));
      // Grid1D::index and ::weights with the FP64 path's roundings: the
      // interpolant has a kink at every density node, so the cell must be the
      // reference's, and the root multiplies an error in b by dR / dT (up to
      // ~1e5 at low T)
      // Grid1D::index: an FP32 estimate decides unless it lies within 1e-4
      // of a node, where the FP64 index is taken
      const float uf = (d2ff(lRho).hi - sc.rho_min_f) * sc.rho_inv_f;
      const float jf = floorf(uf);
      if (uf - jf > 1e-4f && uf - jf < 1.0f - 1e-4f) {
        j = static_cast<int>(jf);
        fast = jf >= 0.0f && jf <= static_cast<float>(t.nRho - 2);
      } else {
        const double u = __dmul_rn(__dsub_rn(lRho, t.gRho.min), t.gRho.inv_dx);
        fast = u >= 0.0 && u <= static_cast<double>(t.nRho - 2);
        j = fast ? static_cast<int>(u) : 0;
      }
      b1 = __dmul_rn(__dsub_rn(lRho, __ldg(t.rhoNodes + j)), t.gRho.inv_dx);
      B = ff_from_double_ok(b1) ? d2ff(b1) : ff_make(0.0f);
      fast = fast && B.hi >= 0.0f && B.hi <= 1.0f;
    }
    if (fast) {
      // 2. on-table, outside the guard band
      const float b1f = B.hi, b0f = 1.0f - B.hi;
      const float ef = static_cast<float>(sie);
      const float sc0 = fmaf(b1f, t.sieCold32[j + 1], b0f * t.sieCold32[j]);
      const float sm0 = fmaf(b1f, t.sielTMax32[j + 1], b0f * t.sielTMax32[j]);
      fast = ef > sc0 + 1e-6f * fabsf(sc0) && ef < sm0 - 1e-6f * fabsf(sm0);
      if (fast) {
        // 3. bracketing cell in FP32: first among every coarse_stride-th
        //    node (shared memory), then within that stretch
        const fq4 *row32 = t.sie4f + static_cast<long long>(j) * nc;
        int lo = 0, hi = nc - 1;
        if (stage_coarse) {
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
        for (int k = 0; k < 4; ++k) {
          const SieRec r = load_sie(row + i);
          // sie = x + a (dT + b dRT) + b dR: numerator and denominator in FP64
          const double num = fma(-b1, r.dR, sie - r.x);
          const double den = fma(b1, r.dRT, r.dT);
          if (!ff_from_double_ok(num) || !ff_from_double_ok(den) || den == 0.0) break;
          A = ff_div(d2ff(num), d2ff(den));
          if (A.hi < 0.0f && i > 0) {
            --i;
            continue;
          }
          if (A.hi > 1.0f && i < nc - 1) {
            ++i;
            continue;
          }
          ok = A.hi >= 0.0f && A.hi <= 1.0f;
          break;
        }
        fast = ok;
      }
    }
    if (fast) {
      // 5. lT, then T = 10^lT by the NQT pow in integers
      using namespace nqt;
      const ff LT = ff_add(ff_mul(ff_add(ff_of_int(i), A), sc.t_dx), sc.t_min);
      const ff P52 = ff_mul(LT, sc.p2_scale);
      if (fabsf(P52.hi) >= 1.1e12f && ff_gt(LT, sc.lt_lo) && ff_lt(LT, sc.lt_hi)) {
        constexpr long long ca = 9007199254740992LL, cc = 18014398509481984LL;
        const long long x_as_int = f2ll_bits(P52.hi) + f2ll_bits(P52.lo);
        const long long frac = x_as_int & mantissa_mask;
        const long long N = cc - 3 * frac; // in [2^52, 2^54]
        const ff NF = quick_two_sum(static_cast<float>(static_cast<int>(N >> 30)) * 1073741824.0f,
                                    static_cast<float>(static_cast<int>(N & ((1LL << 30) - 1))));
        const ff SQ = ff_sqrt(NF);
        const long long fsqrt = f2ll_bits(SQ.hi * 67108864.0f) + f2ll_bits(SQ.lo * 67108864.0f);
        double temp = __longlong_as_double(x_as_int + ca - fsqrt - frac + one_as_int);
        if (t.lTOffset != 0.0) temp -= t.lTOffset;
        const long long ci = static_cast<long long>(j) * nc + i;
        const ff AB = ff_mul(A, B);
        if ((out & Q_TEMPERATURE) && a.temp) a.temp[e] = temp;
        if ((out & Q_PRESSURE) && a.press) a.press[e] = ff2d(ff_cell(load_rec(t.PR + ci), A, B, AB));
        if ((out & Q_BMOD) || a.cs) {
          ff BM = ff_cell(load_rec(t.bmodR + ci), A, B, AB);
          if (ff_lt(BM, sc.eps)) BM = sc.eps;
          if ((out & Q_BMOD) && a.bmod) a.bmod[e] = ff2d(BM);
          if (a.cs) a.cs[e] = ff2d(ff_sqrt(ff_div(BM, d2ff(rho))));
        }
        if ((out & Q_CV) && a.cv) {
          const double a1 = ff2d(A);
          const double *d = t.f2[F_DEDT] + static_cast<long long>(j) * t.nT + i;
          const double cv = b1 * (a1 * d[t.nT + 1] + (1.0 - a1) * d[t.nT]) +
                            (1.0 - b1) * (a1 * d[1] + (1.0 - a1) * d[0]);
          a.cv[e] = cv > lim<double>::eps ? cv : lim<double>::eps;
        }
        if (lam) {
          lam[0] = lRho;
          lam[1] = ff2d(LT);
        }
        continue;
      }
    }
    // The reference's FP64 path (eos_spiner_rho_temp.hpp:1052-1101).
    lRho = sp_lRho(t, rho);
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
  // the coarse index of the T search, staged per block when it fits
  const int nrho = table_nrho(a.eos.table);
  const size_t coarse =
      nrho > 1 ? static_cast<size_t>(nrho - 1) * (SP_COARSE + 1) * sizeof(float2) : 0;
  const int stage = (coarse > 0 && coarse <= 40 * 1024) ? 1 : 0;
  // persistent grid: the blocks resident at once, each staging the index once
  const long long want = (a.n + LOOKUP_BLOCK - 1) / LOOKUP_BLOCK;
  const long long cap = static_cast<long long>(sms) * 4;
  const int grid = static_cast<int>(want < cap ? want : cap);
  spiner_fill_mixed<<<grid, LOOKUP_BLOCK, stage ? coarse : 0, stream>>>(a, stage);
  return cudaGetLastError();
}

} // namespace sgx
