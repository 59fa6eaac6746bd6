// Mixed-precision PTE (PTESolverRhoT), one thread per cell, N materials.
//
//   1. FP32 phase: the reference's damped-Newton iteration
//      (closure/mixed_cell_models.hpp:884-1193, 2188-2291) run entirely in
//      float, to FP32-reachable tolerances (1e-4 relative). On GB300 the FP32
//      pipe is ~64x the FP64 pipe, which bounds the plain path.
//   2. FP64 polish: from the FP32 equilibrium (T, alpha_m) the state is
//      rebuilt in FP64 from the cell's exact FP64 inputs (rhobar and uscale as
//      InitBase computes them, every material's energy and pressure
//      evaluated) and the same damped Newton loop continues in FP64 under
//      tight controls (1e-12 relative residuals) -- typically two steps. The
//      FP64 closure constraints (sum alpha = 1, sum u = u_tot) hold exactly by
//      construction, as in TestUpdate.
//   3. A cell whose FP32 phase fails, or whose polish does not converge, is
//      re-solved by the FP64 reference iteration in the same thread and then
//      polished the same way.
#pragma once

#include <cuda_runtime.h>

#include "sgx_internal.h"
#include "sgx_pte_kernel.cuh"

namespace sgx {

constexpr int PTE_MIXED_BLOCK = 128;

// FP32-phase controls: the reference's, with tolerances FP32 can reach.
__device__ __forceinline__ MixP<float> fp32_params(const sgx_mix_params &q) {
  MixP<float> m(q);
  m.tol_p = 1e-4f;
  m.tol_e = 1e-4f;
  m.abs_p = 1e-4f;
  m.tol_p_suff = 1e-3f;
  m.tol_e_suff = 1e-3f;
  m.abs_p_suff = 1e-3f;
  m.max_iter_per_mat = 32;
  m.small_step_thresh = 1e-7f;
  return m;
}

// FP64 polish controls: residuals to 1e-12 relative, at most 4 Newton
// iterations per material.
__device__ __forceinline__ MixP<double> polish_params(const sgx_mix_params &q) {
  MixP<double> m(q);
  m.tol_p = 1e-12;
  m.tol_e = 1e-12;
  m.abs_p = 1e-13;
  m.tol_p_suff = 1e-10;
  m.tol_e_suff = 1e-10;
  m.abs_p_suff = 1e-11;
  m.max_iter_per_mat = 4;
  return m;
}

template <int N> __global__ void __launch_bounds__(PTE_MIXED_BLOCK) pte_mixed_kernel(const PteArgs a) {
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.ncell) return;
  int slot[MAX_NMAT], eidx[MAX_NMAT];
  if (pte_gather(a, i, slot, eidx) != N) return;
  const long long nc = a.ncell;
  double rho_in[N], vf_in[N], sie_in[N], t_in[N], p_in[N];
  double cache[N][3];
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const long long k = static_cast<long long>(slot[q]) * nc + i;
    rho_in[q] = a.rho[k];
    vf_in[q] = a.vfrac[k];
    sie_in[q] = a.sie[k];
    t_in[q] = a.temp[k];
    p_in[q] = a.press[k];
#pragma unroll
    for (int l = 0; l < 3; ++l)
      cache[q][l] = a.lambda ? a.lambda[(static_cast<long long>(slot[q]) * 3 + l) * nc + i] : 0.0;
  }
  // ---- FP32 phase ----
  const MixP<float> mp32 = fp32_params(a.params);
  PteRhoT<float, N> f;
  f.P = &mp32;
  f.vfrac_total = static_cast<float>(a.vfrac_tot[i]);
  f.sie_total = static_cast<float>(a.sie_tot[i]);
  f.Tnorm = 0.0f;
  f.err_flags = 0;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    f.eos[q] = &s_eos[eidx[q]];
    f.lam[q] = cache[q];
    f.rho[q] = static_cast<float>(rho_in[q]);
    f.vfrac[q] = static_cast<float>(vf_in[q]);
    f.sie[q] = static_cast<float>(sie_in[q]);
    f.temp[q] = static_cast<float>(t_in[q]);
    f.press[q] = static_cast<float>(p_in[q]);
  }
  const PteStatusLocal st32 = pte_solve<PteRhoT<float, N>, float>(f);
  // ---- FP64 polish from the FP32 equilibrium ----
  const MixP<double> mp(a.params);
  const MixP<double> tight = polish_params(a.params);
  PteRhoT<double, N> s;
  s.P = &mp;
  s.vfrac_total = a.vfrac_tot[i];
  s.sie_total = a.sie_tot[i];
  s.err_flags = 0;
#pragma unroll
  for (int q = 0; q < N; ++q) {
    s.eos[q] = &s_eos[eidx[q]];
    s.lam[q] = cache[q];
    s.rho[q] = rho_in[q];
    s.vfrac[q] = vf_in[q];
  }
  bool done = false;
  int polish_steps = 0;
  // the polish also rescues most cells whose FP32 phase stalled short of the
  // FP32 tolerances; a non-finite FP32 state goes straight to the re-solve
  if (f.Tnorm > 0.0f && f.Tequil > 0.0f && f.Tequil < 1e30f) {
    // InitBase's FP64 scalings from the exact inputs (:627-662)
    s.init_rhobar();
    const double utotal = s.rho_total * s.sie_total;
    s.uscale = smax(sabs(utotal), 1.0e-14);
    s.utotal_scale = ratio(utotal, s.uscale);
    s.Tnorm = static_cast<double>(f.Tnorm);
    s.Tequil = static_cast<double>(f.Tequil);
    s.ms = f.ms;
#pragma unroll
    for (int q = 0; q < N; ++q)
      s.vfrac[q] = static_cast<double>(f.vfrac[q]);
    done = pte_polish<N>(s, tight, polish_steps);
    if (done) s.finalize();
  }
  PteStatusLocal st;
  if (done) {
    st.converged = true;
    st.niter = st32.niter + polish_steps;
    st.residual = s.residual_norm();
  } else {
    // the FP64 reference iteration from the original inputs
#pragma unroll
    for (int q = 0; q < N; ++q) {
      s.rho[q] = rho_in[q];
      s.vfrac[q] = vf_in[q];
      s.sie[q] = sie_in[q];
      s.temp[q] = t_in[q];
      s.press[q] = p_in[q];
    }
    s.Tnorm = 0.0;
    st = pte_solve<PteRhoT<double, N>, double>(s);
    if (st.converged) {
      // Polish the FP64 solution too, so every converged cell carries the
      // same accuracy: back to the solver's scaled variables, then Newton.
      double keep[5][N];
#pragma unroll
      for (int q = 0; q < N; ++q) {
        keep[0][q] = s.rho[q];
        keep[1][q] = s.vfrac[q];
        keep[2][q] = s.sie[q];
        keep[3][q] = s.temp[q];
        keep[4][q] = s.press[q];
      }
      s.Tequil = s.temp[0] / s.Tnorm;
      int extra = 0;
      if (pte_polish<N>(s, tight, extra)) {
        s.finalize();
        st.niter += extra;
        st.residual = s.residual_norm();
      } else {
#pragma unroll
        for (int q = 0; q < N; ++q) {
          s.rho[q] = keep[0][q];
          s.vfrac[q] = keep[1][q];
          s.sie[q] = keep[2][q];
          s.temp[q] = keep[3][q];
          s.press[q] = keep[4][q];
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < N; ++q) {
    const long long k = static_cast<long long>(slot[q]) * nc + i;
    a.rho[k] = s.rho[q];
    a.vfrac[k] = s.vfrac[q];
    a.sie[k] = s.sie[q];
    a.temp[k] = s.temp[q];
    a.press[k] = s.press[q];
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
    o.small_step_iters = static_cast<uint8_t>((st.small_step_iters & 0x3F) | (done ? 0 : 0x40) |
                                              (s.err_flags ? 0x80 : 0));
    a.status[i] = o;
  }
}

template <int N> cudaError_t launch_pte_mixed_n(const PteArgs &a, cudaStream_t stream) {
  const long long blocks = (a.ncell + PTE_MIXED_BLOCK - 1) / PTE_MIXED_BLOCK;
  pte_mixed_kernel<N><<<static_cast<unsigned>(blocks), PTE_MIXED_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

} // namespace sgx
