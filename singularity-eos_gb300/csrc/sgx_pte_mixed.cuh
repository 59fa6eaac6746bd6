// Mixed-precision PTE (PTESolverRhoT), one thread per cell, N materials.
//
// The reduced PTE system of the reference (closure/mixed_cell_models.hpp:
// 884-1193) in T and the N-1 free volume fractions, solved in two phases:
//
//   1. FP32 phase: the reference's damped Newton iteration (:2188-2291) run
//      entirely in float to 1e-4 relative residuals. The Jacobian uses the
//      closed-form derivatives of the analytic models (finite differences in
//      FP32 cannot resolve a thermal energy that is small against a cold one);
//      tabulated models keep finite differences, with a step of 2.5e-4 (the
//      FP32 optimum) instead of 3e-6. On GB300 the FP32 pipe is ~64x the FP64
//      pipe, which bounds the plain path.
//   2. FP64 refinement: from the FP32 equilibrium (T, alpha_m), residual-
//      correction steps x <- x + J32^-1 r64(x), where only the residual r64
//      -- the energy closure sum(u_m) = u_tot and the pressure equalities --
//      and the constraint sum(alpha_m) = 1 are evaluated in FP64 (from the
//      cell's exact FP64 inputs, with rhobar and uscale as InitBase computes
//      them); the Jacobian J32 and the solve stay in FP32. The iteration
//      contracts by ~|I - J32^-1 J| ~ 1e-4 per step, so two or three steps
//      reach 1e-12 relative residuals.
//   3. A cell whose refinement does not converge is appended to a retry queue
//      and left untouched; a second kernel drains the compacted queue with the
//      FP64 reference iteration (then refines it the same way), so the few hard
//      cells -- some need hundreds of iterations -- no longer hold up the
//      warps of the easy ones.
#pragma once

#include <cuda_runtime.h>

#include "sgx_internal.h"
#include "sgx_pte_kernel.cuh"

namespace sgx {

constexpr int PTE_MIXED_BLOCK = 128;
constexpr int SGX_REFINE_STEPS = 6;
constexpr double SGX_REFINE_TOL = 1e-12;

// FP32-phase controls: the reference's, with tolerances FP32 can reach
// (10^-tol_exp, the "sufficient" ones ten times looser).
SGX_HDI MixP<float> fp32_params(const sgx_mix_params &q, const int iters_per_mat = 8,
                                const int tol_exp = 4) {
  MixP<float> m(q);
  const float tol = tol_exp >= 6 ? 1e-6f : (tol_exp == 5 ? 1e-5f : (tol_exp <= 3 ? 1e-3f : 1e-4f));
  m.derivative_eps = 2.5e-4f;
  m.tol_p = tol;
  m.tol_e = tol;
  m.abs_p = tol;
  m.tol_p_suff = 10.0f * tol;
  m.tol_e_suff = 10.0f * tol;
  m.abs_p_suff = 10.0f * tol;
  m.max_iter_per_mat = iters_per_mat;
  m.small_step_thresh = 1e-7f;
  return m;
}

// FP64 residual of the reduced system at (T, alpha) with the materials'
// state (InitBase/TestUpdate/Residual, :627-662, 1010-1019, 1155-1187).
template <int N> struct Refine {
  const sgx_eos *eos[N];
  double *lam[N];
  double rhobar[N], alpha[N], rho[N], sie[N], u[N], press[N], res[N];
  double T, Tnorm, uscale, utotal_scale;
  // 1 / uscale: the scaled energies and pressures are products, one FP64
  // division per cell instead of two per material and step (a relative
  // change of at most an ulp or two, far inside the 1e-12 tolerance)
  double inv_uscale;
  int ms;

  SGX_HDI bool eval() {
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (!(alpha[m] > 0.0)) return false;
      rho[m] = ratio(rhobar[m], alpha[m]);
      const sgx_eos &e = *eos[m];
      const double e_m = ev_sie_from_rho_T<double>(e, rho[m], Tnorm * T, lam[m]);
      sie[m] = e_m;
      u[m] = rhobar[m] * e_m * inv_uscale;
      const double P = (preferred_input(e) & Q_SIE)
                           ? ev_P_from_rho_sie<double>(e, rho[m], e_m, lam[m])
                           : ev_P_from_rho_T<double>(e, rho[m], Tnorm * T, lam[m]);
      press[m] = P * inv_uscale;
    }
    res[0] = utotal_scale - sum_neumaier(u, N);
    int r = 1;
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (m == ms) continue;
      res[r++] = press[ms] - press[m];
    }
    return true;
  }
  // CheckPTE (:1021-1040) under the refinement tolerance, on the squared
  // pressure residual (no square root: both sides are non-negative).
  SGX_HDI bool converged() const {
    double mean_p = 0;
#pragma unroll
    for (int m = 0; m < N; ++m)
      mean_p += alpha[m] * press[m];
    double ep2 = 0;
#pragma unroll
    for (int r = 1; r < N; ++r)
      ep2 += res[r] * res[r];
    const double lim_p = SGX_REFINE_TOL * sabs(mean_p);
    constexpr double lim_abs = 0.1 * SGX_REFINE_TOL;
    return (ep2 < lim_p * lim_p || ep2 < lim_abs * lim_abs) && sabs(res[0]) < SGX_REFINE_TOL;
  }
};

// Step 2: returns whether the FP64 residual reached the refinement tolerance.
template <int N>
SGX_HDI bool refine_cell(PteRhoT<float, N> &f, Refine<N> &R, int &steps) {
  steps = 0;
  if (!R.eval()) return false;
  for (int k = 0; k < SGX_REFINE_STEPS; ++k) {
    if (R.converged()) return true;
    // FP32 Jacobian at the current state (same reduced system, same ms)
    f.ms = R.ms;
    f.Tequil = static_cast<float>(R.T);
#pragma unroll
    for (int m = 0; m < N; ++m) {
      f.vfrac[m] = static_cast<float>(R.alpha[m]);
      f.rho[m] = static_cast<float>(R.rho[m]);
      f.u[m] = static_cast<float>(R.u[m]);
      f.press[m] = static_cast<float>(R.press[m]);
    }
    f.jacobian();
#pragma unroll
    for (int r = 0; r < N; ++r)
      f.residual[r] = static_cast<float>(R.res[r]);
    if (!f.solve()) return false;
    const float scale = smin(1.0f, f.scale_dx());
    if (!(scale > 0.0f)) return false;
    // FP64 update; the excluded material closes sum(alpha) = 1 exactly
    R.T += static_cast<double>(f.dx[0]);
    int idx = 1;
#pragma unroll
    for (int m = 0; m < N; ++m) {
      if (m == R.ms) continue;
      R.alpha[m] += static_cast<double>(f.dx[idx++]);
    }
    R.alpha[R.ms] = 1 - sum_neumaier(R.alpha, N, 0, R.ms);
    ++steps;
    if (!(R.T > 0.0) || !R.eval()) return false;
    // A correction at roundoff level means the state is the FP64 fixed point:
    // where a pressure is a small difference of large terms (a stiffened gas
    // near P = 0) the residual itself cannot fall below its rounding noise.
    float dmax = sabs(f.dx[0]) / static_cast<float>(R.T);
#pragma unroll
    for (int r = 1; r < N; ++r)
      dmax = smax(dmax, sabs(f.dx[r]));
    if (dmax < 1e-13f) return true;
  }
  return R.converged();
}

// Writes one cell's equilibrium state, lambda cache and status.
template <int N>
__device__ __forceinline__ void pte_store(const PteArgs &a, const long long i,
                                          const int (&slot)[MAX_NMAT], const double *rho,
                                          const double *vf, const double *sie, const double *T,
                                          const double *P, const double (&cache)[N][3],
                                          const PteStatusLocal &st, const int flags) {
  const long long nc = a.ncell;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const long long k = static_cast<long long>(slot[q]) * nc + i;
    a.rho[k] = rho[q];
    a.vfrac[k] = vf[q];
    a.sie[k] = sie[q];
    a.temp[k] = T[q];
    a.press[k] = P[q];
    if (a.lambda) {
#pragma unroll
      for (int l = 0; l < 3; ++l)
        a.lambda[(static_cast<long long>(slot[q]) * 3 + l) * nc + i] = cache[q][l];
    }
  }
  if (a.status) {
    sgx_pte_status o;
    o.residual = st.residual;
    o.niter = st.niter;
    o.converged = st.converged ? 1 : 0;
    o.slow_convergence_detected = st.slow ? 1 : 0;
    o.max_line_niter = static_cast<uint8_t>(st.max_line_niter);
    o.small_step_iters = static_cast<uint8_t>((st.small_step_iters & 0x3F) | flags);
    a.status[i] = o;
  }
}

// Pass 1: every cell with N materials, FP32 solve + FP64 refinement.
template <int N>
__global__ void __launch_bounds__(PTE_MIXED_BLOCK) pte_mixed_kernel(const PteArgs a) {
  if (pte_block_idle<N>(a)) return;
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  long long i;
  if (!pte_bin_cell<N>(a, static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x, i))
    return;
  int slot[MAX_NMAT], eidx[MAX_NMAT];
  if (pte_gather(a, i, slot, eidx) != N) return;
  const long long nc = a.ncell;
  double cache[N][3];
  // ---- FP32 phase ----
  const MixP<float> mp32 = fp32_params(a.params, a.fp32_iters, a.fp32_tol_exp);
  PteRhoT<float, N> f;
  f.P = &mp32;
  f.vfrac_total = static_cast<float>(a.vfrac_tot[i]);
  f.sie_total = static_cast<float>(a.sie_tot[i]);
  f.Tnorm = 0.0f;
  f.err_flags = 0;
  f.use_analytic = true;
  Refine<N> R;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const long long k = static_cast<long long>(slot[q]) * nc + i;
#pragma unroll
    for (int l = 0; l < 3; ++l)
      cache[q][l] = a.lambda ? a.lambda[(static_cast<long long>(slot[q]) * 3 + l) * nc + i] : 0.0;
    f.eos[q] = R.eos[q] = &s_eos[eidx[q]];
    f.lam[q] = R.lam[q] = cache[q];
    const double r_in = a.rho[k], v_in = a.vfrac[k];
    R.rhobar[q] = r_in * v_in;
    f.rho[q] = static_cast<float>(r_in);
    f.vfrac[q] = static_cast<float>(v_in);
    f.sie[q] = static_cast<float>(a.sie[k]);
    f.temp[q] = static_cast<float>(a.temp[k]);
    f.press[q] = static_cast<float>(a.press[k]);
  }
  const PteStatusLocal st32 = pte_solve<PteRhoT<float, N>, float>(f);
  // ---- FP64 refinement from the FP32 equilibrium ----
  // InitBase's scalings from the exact FP64 inputs (:388-399, 632-635)
  const double rho_total = sum_neumaier(R.rhobar, N);
  const double utotal = rho_total * a.sie_tot[i];
  R.uscale = smax(sabs(utotal), 1.0e-14);
  R.utotal_scale = ratio(utotal, R.uscale);
  R.inv_uscale = 1.0 / R.uscale;
  bool done = false;
  int steps = 0;
  if (f.Tnorm > 0.0f && f.Tequil > 0.0f && f.Tequil < 1e30f) {
    R.Tnorm = static_cast<double>(f.Tnorm);
    R.T = static_cast<double>(f.Tequil);
    R.ms = f.ms;
#pragma unroll
    for (int q = 0; q < N; ++q)
      R.alpha[q] = static_cast<double>(f.vfrac[q]);
    R.alpha[R.ms] = 1 - sum_neumaier(R.alpha, N, 0, R.ms);
    done = refine_cell<N>(f, R, steps);
  }
  if (!done) {
    // each material count queues into its own segment of retry_idx, so
    // that its pass 2 can run while pass 1 of the next count does
    const unsigned pos = atomicAdd(&a.bins[2 * PTE_BINS + N], 1u);
    a.retry_idx[pte_bin_offset<N>(a) + pos] = static_cast<int>(i);
    return;
  }
  PteStatusLocal st;
  st.converged = true;
  st.niter = st32.niter + steps;
  double r2 = 0;
#pragma unroll
  for (int r = 0; r < N; ++r)
    r2 += R.res[r] * R.res[r];
  st.residual = 0.5 * r2;
  double out_T[N], out_P[N];
#pragma unroll
  for (int q = 0; q < N; ++q) {
    out_T[q] = R.T * R.Tnorm;
    out_P[q] = R.press[q] * R.uscale;
  }
  pte_store<N>(a, i, slot, R.rho, R.alpha, R.sie, out_T, out_P, cache, st, 0);
}

// Pass 2: the queued cells with N materials (their own segment of the
// queue), FP64 reference iteration (:2188-2291) from the original inputs,
// then the same FP64 refinement.
template <int N>
__global__ void __launch_bounds__(PTE_MIXED_BLOCK) pte_retry_kernel(const PteArgs a) {
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  const unsigned count = a.bins[2 * PTE_BINS + N];
  const unsigned off = pte_bin_offset<N>(a);
  const long long nc = a.ncell;
  // The reference's iteration, capped at a.retry_iters per material:
  // cells that converge do so within ~50 iterations, while a cell that does
  // not may run to the reference's 128 per material at FP64 latency, and
  // the slowest such cell sets the kernel's length. A capped cell is
  // reported unconverged, as the reference reports it.
  MixP<double> mp(a.params);
  if (mp.max_iter_per_mat > a.retry_iters) mp.max_iter_per_mat = a.retry_iters;
  const MixP<float> mp32 = fp32_params(a.params);
  for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += gridDim.x * blockDim.x) {
    const long long i = a.retry_idx[off + t];
    int slot[MAX_NMAT], eidx[MAX_NMAT];
    if (pte_gather(a, i, slot, eidx) != N) continue;
    double cache[N][3];
    PteRhoT<double, N> s;
    s.P = &mp;
    s.vfrac_total = a.vfrac_tot[i];
    s.sie_total = a.sie_tot[i];
    s.Tnorm = 0.0;
    s.err_flags = 0;
#pragma unroll
    for (int q = 0; q < N; ++q) {
      const long long k = static_cast<long long>(slot[q]) * nc + i;
#pragma unroll
      for (int l = 0; l < 3; ++l)
        cache[q][l] = a.lambda ? a.lambda[(static_cast<long long>(slot[q]) * 3 + l) * nc + i] : 0.0;
      s.eos[q] = &s_eos[eidx[q]];
      s.lam[q] = cache[q];
      s.rho[q] = a.rho[k];
      s.vfrac[q] = a.vfrac[k];
      s.sie[q] = a.sie[k];
      s.temp[q] = a.temp[k];
      s.press[q] = a.press[k];
    }
    PteStatusLocal st = pte_solve<PteRhoT<double, N>, double>(s);
    double out_rho[N], out_vf[N], out_sie[N], out_T[N], out_P[N];
#pragma unroll
    for (int q = 0; q < N; ++q) {
      out_rho[q] = s.rho[q];
      out_vf[q] = s.vfrac[q];
      out_sie[q] = s.sie[q];
      out_T[q] = s.temp[q];
      out_P[q] = s.press[q];
    }
    if (st.converged) {
      // refine the FP64 solution to the same tolerance as pass 1
      PteRhoT<float, N> f;
      f.P = &mp32;
      f.use_analytic = true;
      f.vfrac_total = static_cast<float>(s.vfrac_total);
      f.Tnorm = static_cast<float>(s.Tnorm);
      f.uscale = static_cast<float>(s.uscale);
      Refine<N> R;
#pragma unroll
      for (int q = 0; q < N; ++q) {
        f.eos[q] = R.eos[q] = s.eos[q];
        f.lam[q] = R.lam[q] = cache[q];
        f.rhobar[q] = static_cast<float>(s.rhobar[q]);
        R.rhobar[q] = s.rhobar[q];
        R.alpha[q] = s.vfrac[q];
      }
      R.uscale = s.uscale;
      R.utotal_scale = s.utotal_scale;
      R.inv_uscale = 1.0 / s.uscale;
      R.Tnorm = s.Tnorm;
      R.T = s.temp[0] / s.Tnorm;
      R.ms = s.ms;
      int steps = 0;
      if (refine_cell<N>(f, R, steps)) {
        st.niter += steps;
#pragma unroll
        for (int q = 0; q < N; ++q) {
          out_rho[q] = R.rho[q];
          out_vf[q] = R.alpha[q];
          out_sie[q] = R.sie[q];
          out_T[q] = R.T * R.Tnorm;
          out_P[q] = R.press[q] * R.uscale;
        }
      } else {
        // The refinement's plain Newton steps can fail from a state the
        // reference accepts far from equilibrium: its default tolerances
        // are 1e-6, and a cell of pressure-preferring gases with zero
        // pressure guesses passes its check at iteration 0 with P = 0. The
        // FP64 damped Newton continues from there under tight controls; if
        // it does not converge either, the reference's answer stands.
        MixP<double> tight = mp;
        tight.tol_p = tight.tol_e = 1e-13;
        tight.abs_p = 0.0;
        tight.tol_p_suff = tight.tol_e_suff = 1e-12;
        tight.abs_p_suff = 0.0;
        int taken = 0;
        if (pte_polish<N>(s, tight, taken)) {
          s.finalize();
          st.niter += taken;
#pragma unroll
          for (int q = 0; q < N; ++q) {
            out_rho[q] = s.rho[q];
            out_vf[q] = s.vfrac[q];
            out_sie[q] = s.sie[q];
            out_T[q] = s.temp[q];
            out_P[q] = s.press[q];
          }
        }
      }
    }
    pte_store<N>(a, i, slot, out_rho, out_vf, out_sie, out_T, out_P, cache, st, 0x40);
  }
}

template <int N> cudaError_t launch_pte_mixed_n(const PteArgs &a, cudaStream_t stream) {
  // smaller blocks free their SM slot sooner when their lanes' iteration
  // counts differ (SGX_TUNE_PTE_MIXED_BLOCK: 32, 64 or 128 threads)
  const int k = tune_get(SGX_TUNE_PTE_MIXED_BLOCK);
  const int bs = k >= 128 ? 128 : (k >= 64 ? 64 : 32);
  const long long blocks = (a.ncell + bs - 1) / bs;
  pte_mixed_kernel<N><<<static_cast<unsigned>(blocks), bs, 0, stream>>>(a);
  return cudaGetLastError();
}
template <int N> cudaError_t launch_pte_retry_n(const PteArgs &a, cudaStream_t stream) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // sized for the worst case but never more than a few waves; threads past
  // the queue length exit at once
  long long blocks = (a.ncell + PTE_MIXED_BLOCK - 1) / PTE_MIXED_BLOCK;
  if (blocks > 4LL * sms) blocks = 4LL * sms;
  pte_retry_kernel<N><<<static_cast<unsigned>(blocks), PTE_MIXED_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

} // namespace sgx
