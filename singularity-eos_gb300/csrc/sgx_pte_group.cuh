// Warp-cooperative pass 1 of the mixed-precision PTE (PTESolverRhoT): a
// group of G lanes (G a power of two, G >= N) per cell, one material per
// lane, for cells with several materials.
//
// The thread-per-cell pass 1 (sgx_pte_mixed.cuh) unrolls every material's
// EOS evaluation and a dense N x N solve into one thread: at N = 5 its code
// outgrows the instruction cache, its warps wait on their slowest lane, and
// 128 registers hold occupancy to 16 warps per SM. Here each lane evaluates
// only its own material, and the cell-wide quantities -- sums over
// materials, the excluded material's pressure, maxima and minima -- come from
// butterfly shuffles inside the group (every lane ends with the same bits,
// so the group takes its branches together).
//
// The Newton step of the reduced system (mixed_cell_models.hpp:1042-1105:
// unknowns T and the N-1 volume fractions other than the excluded ms;
// residuals the energy closure and P_ms - P_m) is the same step the
// reference's dense solve returns, taken in closed form. With a common
// linearised pressure offset Pi (relative to P_ms) and D_m = P_m - P_ms,
// every material satisfies
//   d alpha_m = (Pi - D_m - dP_m/dT dT) / (dP_m/d alpha_m),
// the volume fractions keep their sum (sum_m d alpha_m = 0) and the energy
// closure is linear in (dT, Pi): a 2 x 2 system in six sums over materials.
// Everything is relative to P_ms, so the step stays accurate when the
// residuals are tiny against the pressures, which the FP64 refinement needs.
//
// The rest follows the thread-per-cell pass 1 step for step: the reference's
// initial guess (GetTguess, SetVfracFromT), damped Newton with the
// parabolic line search and ScaleDx's limits (:2188-2291, :1107-1187) in
// FP32 to 1e-4, then FP64 residual correction with the FP32 step to 1e-12.
// ScaleDx's sequential minimum is order-independent, so its per-material
// limits reduce as a group minimum. Cells it cannot finish go to the same
// retry queue as before, for the FP64 reference iteration of pass 2.
#pragma once

#include <cooperative_groups.h>

#include "sgx_pte_mixed.cuh"

namespace sgx {
SGX_DISPATCH_BEGIN

namespace cg = cooperative_groups;

// Butterfly reductions over a group of G lanes: all lanes get the same
// result (IEEE addition, minimum and maximum are commutative).
template <int G> struct Lanes {
  cg::thread_block_tile<G> t;
  int l; // lane in the group = material slot
  template <typename X> __device__ __forceinline__ X sum(X x) const {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
      x += t.shfl_xor(x, o);
    return x;
  }
  template <typename X> __device__ __forceinline__ X max(X x) const {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
      x = smax(x, t.shfl_xor(x, o));
    return x;
  }
  template <typename X> __device__ __forceinline__ X min(X x) const {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1)
      x = smin(x, t.shfl_xor(x, o));
    return x;
  }
  template <typename X> __device__ __forceinline__ X from(X x, int src) const {
    return t.shfl(x, src);
  }
  __device__ __forceinline__ bool any(bool p) const { return t.any(p); }
  // The first lane whose x is the largest strictly above 0 (the reference's
  // loop `if (x > xmax) { xmax = x; ms = m; }` from xmax = 0, ms = 0); NaN
  // and inactive lanes never win.
  __device__ __forceinline__ int argmax_first(float x, bool act) const {
    float v = (act && x > 0.0f) ? x : 0.0f;
    int k = (act && x > 0.0f) ? l : G;
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      const float v2 = t.shfl_xor(v, o);
      const int k2 = t.shfl_xor(k, o);
      if (v2 > v || (v2 == v && k2 < k)) {
        v = v2;
        k = k2;
      }
    }
    return k >= G ? 0 : k;
  }
};

// One lane's material in the FP32 phase: the reference's per-material
// arrays (PTESolverBase, PTESolverRhoT members), one element each.
struct GroupMat {
  const sgx_eos *eos;
  double *lam;
  unsigned pref;
  float rho, vf, sie, press, u, rhobar, vtemp;
  float dpdv, dedv, dpdT, dedT, dxm;
  __device__ float e_of(float r, float t) const {
    return ev_sie_from_rho_T<float>(*eos, r, t, lam);
  }
  __device__ float p_pref(float r, float t, float e) const {
    if (pref & Q_SIE) return ev_P_from_rho_sie<float>(*eos, r, e, lam);
    return ev_P_from_rho_T<float>(*eos, r, t, lam);
  }
};

// The FP32 solver state of one cell, replicated on the group's lanes.
template <int N, int G> struct GroupRhoT {
  Lanes<G> g;
  bool act; // this lane holds a material
  GroupMat m;
  const MixP<float> *P;
  float vfrac_total, sie_total, rho_total, uscale, utotal_scale, Tnorm;
  float Tequil, Ttemp, res0, res, dx0;
  int ms;
  __device__ explicit GroupRhoT(const Lanes<G> &lanes) : g(lanes) {}

  __device__ float residual_norm() const { return 0.5f * (res0 * res0 + g.sum(res * res)); }
  __device__ void residual_eval() {
    res0 = utotal_scale - g.sum(act ? m.u : 0.0f);
    const float pms = g.from(m.press, ms);
    res = (act && g.l != ms) ? pms - m.press : 0.0f;
  }
  // GetSieCvFromTAndPreferred (:599-620) for this lane's material
  __device__ void sie_cv_pref(float r, const float Pin, const float Tk, float &s, float &cv) const {
    const sgx_eos &e = *m.eos;
    if (m.pref & Q_PRESSURE) {
      // a closed-form model with a usable pressure needs no FP64 (its
      // maximum pressure is 1e100, beyond any float)
      if (!mix_bad_f(Pin) && ev_rho_sie_from_PT_f(e, smax(float(ev_min_pressure(e)), Pin), Tk, r,
                                                  s)) {
        cv = ev_cv_from_rho_sie<float>(e, r, s, m.lam);
        return;
      }
      int err = 0;
      const float Pmin = float(ev_min_pressure(e));
      const float Pmax = float(ev_max_pressure_at_T(e, double(Tk), &err));
      const float Pguess = bad_value(double(Pin)) ? 0.5f * (Pmin + Pmax) : smax(Pmin, smin(Pmax, Pin));
      double rr = double(r), ss = 0;
      ev_rho_sie_from_PT(e, double(Pguess), double(Tk), rr, ss, m.lam, &err);
      r = float(rr);
      s = float(ss);
      cv = ev_cv_from_rho_sie<float>(e, r, s, m.lam);
    } else {
      s = ev_sie_from_rho_T<float>(e, r, Tk, m.lam);
      cv = ev_cv_from_rho_T<float>(e, r, Tk, m.lam);
    }
  }
  __device__ float vfrac_max(const float Tk) const {
    const float rho_min = ev_rho_pmin_t<float>(*m.eos, Tk);
    return smin(0.9f * ratio(m.rhobar, rho_min), 1.0f);
  }
  __device__ void normalize_vfrac() {
    const float s = g.sum(act ? m.vf : 0.0f);
    if (act) m.vf *= ratio(vfrac_total, s);
  }
  // SetVfracFromT (:423-498); true = FAIL
  __device__ bool set_vfrac_from_T(const float Tk) {
    const float min_dv = 1e-12f;
    const float vmax = act ? vfrac_max(Tk) : 0.0f;
    if (act && m.vf <= 0.0f) m.vf = vmax;
    if (g.sum(vmax) < vfrac_total) return true;
    normalize_vfrac();
    for (int it = 0; it < N; ++it) {
      float dv = 0.0f;
      if (act) {
        const float vnew = smin(vmax, m.vf);
        dv = m.vf - vnew;
        m.vf -= dv;
      }
      const float remaining = g.sum(dv);
      const int n_uncapped = N - g.sum((act && dv > min_dv) ? 1 : 0);
      if (sabs(remaining) < min_dv) break;
      if (act && (vmax - m.vf) > min_dv) m.vf += remaining / float(n_uncapped);
    }
    normalize_vfrac();
    return false;
  }
  // GetTguess (:500-581)
  __device__ float get_tguess(const float temp_in, const float press_in) {
    float Tguess = g.max(act ? smax(P->default_tguess, temp_in) : P->default_tguess);
    auto newton_step = [&](float Tk) {
      float s = 0.0f, cv = 0.0f;
      if (act) sie_cv_pref(smin(m.rho, float(ev_max_density(*m.eos))), press_in, Tk, s, cv);
      const float usum = g.sum(m.rhobar * s);
      const float dudt = g.sum(m.rhobar * cv);
      return Tk - ratio((usum - utotal_scale * uscale), dudt);
    };
    const float min_T = g.max(act ? float(ev_min_temperature(*m.eos)) : -3.4e38f);
    for (int i = 0; i < 3; i++) {
      if (P->iterate_t_guess)
        Tguess = smin(P->temperature_limit, smax(Tguess, newton_step(Tguess)));
      Tguess = smax(min_T, Tguess);
      if (set_vfrac_from_T(Tguess)) {
        Tguess *= 10.0f;
        continue;
      }
      if (act) m.rho = ratio(m.rhobar, m.vf);
      const bool bad = g.any(act && m.rho < ev_rho_pmin_t<float>(*m.eos, Tguess));
      if (!bad) break;
      Tguess *= 10.0f;
    }
    return Tguess;
  }
  // InitBase (:627-662) and PTESolverRhoT::Init (:947-984)
  __device__ float init(const float temp_in, const float press_in) {
    m.rhobar = act ? m.rho * m.vf : 0.0f;
    rho_total = g.sum(m.rhobar);
    const float utotal = rho_total * sie_total;
    uscale = smax(sabs(utotal), 1.0e-14f);
    utotal_scale = ratio(utotal, uscale);
    const float Tguess = get_tguess(temp_in, press_in);
    Tnorm = Tguess;
    if (act) {
      m.sie = m.e_of(m.rho, Tguess);
      if ((m.pref & Q_PRESSURE) && !bad_value(double(press_in)))
        m.press = ratio(press_in, uscale);
      else
        m.press = ratio(m.p_pref(m.rho, Tguess, m.sie), uscale);
      m.u = m.sie * ratio(m.rhobar, uscale);
    } else {
      m.press = m.u = 0.0f;
    }
    ms = P->exclude_idx >= 0 ? P->exclude_idx : g.argmax_first(ratio(m.rhobar, rho_total), act);
    residual_eval();
    Tequil = 1.0f;
    return residual_norm();
  }
  __device__ void fixup() {
    if (P->exclude_idx < 0) {
      ms = g.argmax_first(m.vf, act);
      residual_eval();
    }
  }
  // CheckPTE (:1021-1040)
  __device__ void check(bool &conv, bool &acceptable) const {
    const float mean_p = g.sum(act ? m.vf * m.press : 0.0f);
    const float error_p = ssqrt(g.sum(res * res));
    const float error_u = sabs(res0);
    conv = (error_p < P->tol_p * sabs(mean_p) || error_p < P->abs_p) && (error_u < P->tol_e);
    acceptable = (error_p < P->tol_p_suff * sabs(mean_p) || error_p < P->abs_p_suff) &&
                 (error_u < P->tol_e_suff);
  }
  // This lane's Jacobian entries (:1042-1105): closed form for the analytic
  // models, the reference's finite differences otherwise.
  __device__ void jacobian_lane() {
    if (!act) {
      m.dpdv = -1.0f;
      m.dedv = m.dpdT = m.dedT = 0.0f;
      return;
    }
    float de_drho, de_dT, dP_drho, dP_dT;
    if (eos_derivs<float>(*m.eos, m.rho, Tnorm * Tequil, de_drho, de_dT, dP_drho, dP_dT)) {
      const float drho_dalpha = -m.rho / m.vf;
      m.dpdv = smin(dP_drho * drho_dalpha / uscale, -sabs(P->max_dpdv));
      m.dedv = m.rhobar * de_drho * drho_dalpha / uscale;
      m.dpdT = dP_dT * Tnorm / uscale;
      m.dedT = m.rhobar * de_dT * Tnorm / uscale;
      return;
    }
    const float dv = (m.vf < 0.5f ? 1.0f : -1.0f) * m.vf * P->derivative_eps;
    const float vf_pert = m.vf + dv;
    const float rho_pert = ratio(m.rhobar, vf_pert);
    float e_pert = m.e_of(rho_pert, Tnorm * Tequil);
    float p_pert = ratio(m.p_pref(rho_pert, Tnorm * Tequil, e_pert), uscale);
    m.dpdv = smin(ratio((p_pert - m.press), dv), -sabs(P->max_dpdv));
    m.dedv = ratio(m.rhobar * ratio(e_pert, uscale) - m.u, dv);
    const float dT = Tequil * P->derivative_eps;
    e_pert = m.e_of(m.rho, Tnorm * (Tequil + dT));
    p_pert = ratio(m.p_pref(m.rho, Tnorm * (Tequil + dT), e_pert), uscale);
    m.dpdT = ratio((p_pert - m.press), dT);
    m.dedT = ratio(m.rhobar * ratio(e_pert, uscale) - m.u, dT);
  }
  // The Newton step for residuals (r0, D_m = P_m - P_ms) in closed form;
  // false when it is not finite (solve_Ax_b's failure).
  __device__ bool solve(const float r0, const float D) {
    const float inv = act ? 1.0f / m.dpdv : 0.0f;
    const float Dm = act ? D : 0.0f;
    const float S1 = g.sum(inv);
    const float S2 = g.sum(Dm * inv);
    const float S3 = g.sum(m.dpdT * inv);
    const float S4 = g.sum(m.dedv * m.dpdT * inv);
    const float S5 = g.sum(m.dedv * inv);
    const float S6 = g.sum(m.dedv * Dm * inv);
    const float dedT = g.sum(m.dedT);
    const float q = 1.0f / S1;
    const float dT = (r0 + S6 - S5 * S2 * q) / (dedT - S4 + S5 * S3 * q);
    const float Pi = (S2 + dT * S3) * q;
    dx0 = dT;
    m.dxm = (act && g.l != ms) ? (Pi - Dm - m.dpdT * dT) * inv : 0.0f;
    return !g.any(!mix_isfinite(dT) || !mix_isfinite(m.dxm));
  }
  // ScaleDx (:1107-1151); the sequential minimum as a group minimum
  __device__ float scale_dx() {
    const float dalphaskip = -g.sum(m.dxm);
    const float mydx = (g.l == ms) ? dalphaskip : m.dxm;
    float c = 1.0f;
    if (act && mydx < -P->vfrac_safety_fac * m.vf)
      c = sabs(P->vfrac_safety_fac * ratio(m.vf, mydx));
    float scale = smin(1.0f, g.min(c));
    const float Tnew = Tequil + scale * dx0;
    c = 1.0f;
    if (act) {
      const float rho_min = smax(ev_rho_pmin_t<float>(*m.eos, Tnorm * Tequil),
                                 ev_rho_pmin_t<float>(*m.eos, Tnorm * Tnew));
      const float alpha_max = smin(1.0f, ratio(m.rhobar, rho_min));
      if (!(alpha_max < m.vf) && scale * mydx > 0.5f * (alpha_max - m.vf))
        c = ratio(0.5f * (alpha_max - m.vf), mydx);
    }
    scale = smin(scale, g.min(c));
    if (scale * dx0 < -0.95f * Tequil) scale = smin(scale, ratio(-0.95f * Tequil, dx0));
    dx0 *= scale;
    m.dxm *= scale;
    return scale;
  }
  // TestUpdate (:1155-1187)
  __device__ float test_update(const float scale, const bool cache_state = false) {
    if (cache_state) {
      Ttemp = Tequil;
      m.vtemp = m.vf;
    }
    Tequil = Ttemp + scale * dx0;
    if (act && g.l != ms) m.vf = m.vtemp + scale * m.dxm;
    const float others = g.sum((act && g.l != ms) ? m.vf : 0.0f);
    if (g.l == ms) m.vf = 1.0f - others;
    if (act) {
      m.rho = ratio(m.rhobar, m.vf);
      m.u = m.rhobar * m.e_of(m.rho, Tnorm * Tequil);
      m.sie = ratio(m.u, m.rhobar);
      m.u = ratio(m.u, uscale);
      m.press = ratio(m.p_pref(m.rho, Tnorm * Tequil, m.sie), uscale);
    }
    residual_eval();
    return residual_norm();
  }
  // PTESolver (:2188-2291)
  __device__ PteStatusLocal iterate(float err) {
    PteStatusLocal st;
    bool converged = false, close_enough = false;
    const int pte_max_iter = N * P->max_iter_per_mat;
    int niter, max_line_niter = 0, small_step_iters = 0;
    for (niter = 0; niter < pte_max_iter; ++niter) {
      check(converged, close_enough);
      if (converged) break;
      jacobian_lane();
      if (!solve(res0, -res)) {
        converged = false;
        break;
      }
      float scale = smin(1.0f, scale_dx());
      if (sabs(scale) < P->small_step_thresh) small_step_iters++;
      if (small_step_iters >= P->small_step_tries) {
        converged = false;
        break;
      }
      const float gradfdx = -2.0f * scale * err;
      scale = 1.0f;
      const float err_old = err;
      err = test_update(scale, true);
      if (err > err_old + P->ls_alpha * gradfdx) {
        scale = 0.5f;
        const float err_mid = test_update(scale);
        if (err_mid < err && err_mid < err_old)
          scale = 0.75f + 0.5f * ratio(err_mid - err, err - 2.0f * err_mid + err_old);
        for (int line_iter = 0; line_iter < P->ls_max_iter; line_iter++) {
          err = test_update(scale);
          if (err < err_old + P->ls_alpha * scale * gradfdx) break;
          scale *= P->ls_fac;
          max_line_niter = max_line_niter > line_iter ? max_line_niter : line_iter;
        }
      }
      fixup();
      if (((err > P->slow_thresh * err_old) || niter == pte_max_iter - 1) && close_enough) {
        converged = true;
        st.slow = true;
        break;
      }
    }
    st.residual = double(err);
    st.niter = niter;
    st.converged = converged;
    st.max_line_niter = max_line_niter;
    st.small_step_iters = small_step_iters;
    return st;
  }
};

// FP64 residual correction of one cell from the FP32 equilibrium (the
// group form of Refine / refine_cell in sgx_pte_mixed.cuh).
template <int N, int G> struct GroupRefine {
  const Lanes<G> &g;
  bool act;
  double rhobar, alpha, rho, sie, u, press, res, res0;
  double T, Tnorm, uscale, utotal_scale, inv_uscale; // (see Refine)
  int ms;
  __device__ GroupRefine(const Lanes<G> &lanes) : g(lanes) {}

  __device__ bool eval(const GroupMat &m) {
    if (g.any(act && !(alpha > 0.0))) return false;
    double usum_part = 0.0;
    if (act) {
      rho = ratio(rhobar, alpha);
      const double e_m = ev_sie_from_rho_T<double>(*m.eos, rho, Tnorm * T, m.lam);
      sie = e_m;
      u = rhobar * e_m * inv_uscale;
      const double P = (m.pref & Q_SIE) ? ev_P_from_rho_sie<double>(*m.eos, rho, e_m, m.lam)
                                        : ev_P_from_rho_T<double>(*m.eos, rho, Tnorm * T, m.lam);
      press = P * inv_uscale;
      usum_part = u;
    } else {
      press = 0.0;
    }
    res0 = utotal_scale - g.sum(usum_part);
    const double pms = g.from(press, ms);
    res = (act && g.l != ms) ? pms - press : 0.0;
    return true;
  }
  __device__ bool converged() const {
    const double mean_p = g.sum(act ? alpha * press : 0.0);
    const double ep2 = g.sum(res * res);
    const double lim_p = SGX_REFINE_TOL * sabs(mean_p);
    constexpr double lim_abs = 0.1 * SGX_REFINE_TOL;
    return (ep2 < lim_p * lim_p || ep2 < lim_abs * lim_abs) && sabs(res0) < SGX_REFINE_TOL;
  }
  // Up to SGX_REFINE_STEPS corrections x <- x + J32^-1 r64(x); true when
  // the FP64 residual meets the refinement tolerance.
  __device__ bool run(GroupRhoT<N, G> &f, int &steps) {
    steps = 0;
    if (!eval(f.m)) return false;
    for (int k = 0; k < SGX_REFINE_STEPS; ++k) {
      if (converged()) return true;
      f.ms = ms;
      f.Tequil = static_cast<float>(T);
      if (act) {
        f.m.vf = static_cast<float>(alpha);
        f.m.rho = static_cast<float>(rho);
        f.m.u = static_cast<float>(u);
        f.m.press = static_cast<float>(press);
      }
      f.jacobian_lane();
      if (!f.solve(static_cast<float>(res0), static_cast<float>(-res))) return false;
      const float scale = smin(1.0f, f.scale_dx());
      if (!(scale > 0.0f)) return false;
      T += static_cast<double>(f.dx0);
      if (act && g.l != ms) alpha += static_cast<double>(f.m.dxm);
      const double others = g.sum((act && g.l != ms) ? alpha : 0.0);
      if (g.l == ms) alpha = 1.0 - others;
      ++steps;
      if (!(T > 0.0) || !eval(f.m)) return false;
      // a correction at roundoff level: the FP64 fixed point (see refine_cell)
      const float dmax = smax(sabs(f.dx0) / static_cast<float>(T), g.max(sabs(f.m.dxm)));
      if (dmax < 1e-13f) return true;
    }
    return converged();
  }
};

template <int N, int G>
__global__ void __launch_bounds__(PTE_MIXED_BLOCK) pte_group_kernel(const PteArgs a) {
  constexpr int CELLS = PTE_MIXED_BLOCK / G;
  if (a.perm && static_cast<long long>(blockIdx.x) * CELLS >= a.bins[N]) return;
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  Lanes<G> g{cg::tiled_partition<G>(cg::this_thread_block()), 0};
  g.l = static_cast<int>(g.t.thread_rank());
  long long i;
  if (!pte_bin_cell<N>(a, static_cast<long long>(blockIdx.x) * CELLS + threadIdx.x / G, i))
    return;
  int slot[MAX_NMAT], eidx[MAX_NMAT];
  if (pte_gather(a, i, slot, eidx) != N) return;
  const bool act = g.l < N;
  int my_slot = slot[0], my_e = eidx[0];
#pragma unroll
  for (int q = 1; q < N; ++q)
    if (q == g.l) {
      my_slot = slot[q];
      my_e = eidx[q];
    }
  const long long nc = a.ncell;
  const long long k = static_cast<long long>(my_slot) * nc + i;
  double cache[3];
#pragma unroll
  for (int l = 0; l < 3; ++l)
    cache[l] = (a.lambda && act) ? a.lambda[(static_cast<long long>(my_slot) * 3 + l) * nc + i] : 0.0;
  const double rho_in = act ? a.rho[k] : 0.0, vf_in = act ? a.vfrac[k] : 0.0;
  const float temp_in = act ? static_cast<float>(a.temp[k]) : 0.0f;
  const float press_in = act ? static_cast<float>(a.press[k]) : 0.0f;
  // ---- FP32 phase ----
  const MixP<float> mp32 = fp32_params(a.params, a.fp32_iters, a.fp32_tol_exp);
  GroupRhoT<N, G> f(g);
  f.act = act;
  f.P = &mp32;
  f.m.eos = &s_eos[my_e];
  f.m.lam = cache;
  f.m.pref = preferred_input(s_eos[my_e]);
  f.m.rho = static_cast<float>(rho_in);
  f.m.vf = static_cast<float>(vf_in);
  f.m.sie = act ? static_cast<float>(a.sie[k]) : 0.0f;
  f.m.dxm = 0.0f;
  f.vfrac_total = static_cast<float>(a.vfrac_tot[i]);
  f.sie_total = static_cast<float>(a.sie_tot[i]);
  f.res = 0.0f;
  const float err0 = f.init(temp_in, press_in);
  const PteStatusLocal st32 = f.iterate(err0);
  f.fixup();
  // ---- FP64 refinement from the FP32 equilibrium ----
  GroupRefine<N, G> R(g);
  R.act = act;
  R.rhobar = rho_in * vf_in;
  const double rho_total = g.sum(R.rhobar);
  const double utotal = rho_total * a.sie_tot[i];
  R.uscale = smax(sabs(utotal), 1.0e-14);
  R.utotal_scale = ratio(utotal, R.uscale);
  R.inv_uscale = 1.0 / R.uscale;
  R.res = 0.0;
  bool done = false;
  int steps = 0;
  if (f.Tnorm > 0.0f && f.Tequil > 0.0f && f.Tequil < 1e30f) {
    R.Tnorm = static_cast<double>(f.Tnorm);
    R.T = static_cast<double>(f.Tequil);
    R.ms = f.ms;
    R.alpha = act ? static_cast<double>(f.m.vf) : 0.0;
    const double others = g.sum(g.l != R.ms ? R.alpha : 0.0);
    if (g.l == R.ms) R.alpha = 1.0 - others;
    done = R.run(f, steps);
  }
  if (!done) {
    if (g.l == 0) {
      const unsigned pos = atomicAdd(&a.bins[2 * PTE_BINS + N], 1u);
      a.retry_idx[pte_bin_offset<N>(a) + pos] = static_cast<int>(i);
    }
    return;
  }
  const double r2 = R.res0 * R.res0 + g.sum(R.res * R.res);
  if (act) {
    a.rho[k] = R.rho;
    a.vfrac[k] = R.alpha;
    a.sie[k] = R.sie;
    a.temp[k] = R.T * R.Tnorm;
    a.press[k] = R.press * R.uscale;
    if (a.lambda) {
#pragma unroll
      for (int l = 0; l < 3; ++l)
        a.lambda[(static_cast<long long>(my_slot) * 3 + l) * nc + i] = cache[l];
    }
  }
  if (g.l == 0 && a.status) {
    sgx_pte_status o;
    o.residual = 0.5 * r2;
    o.niter = st32.niter + steps;
    o.converged = 1;
    o.slow_convergence_detected = 0;
    o.max_line_niter = 0;
    o.small_step_iters = 0;
    a.status[i] = o;
  }
}

} // inline namespace

// Lanes per cell for N materials: the next power of two.
template <int N> constexpr int pte_group_size() { return N <= 2 ? 2 : (N <= 4 ? 4 : 8); }

template <int N> cudaError_t launch_pte_group_n(const PteArgs &a, cudaStream_t stream) {
  constexpr int G = pte_group_size<N>();
  constexpr int CELLS = PTE_MIXED_BLOCK / G;
  const long long blocks = (a.ncell + CELLS - 1) / CELLS;
  pte_group_kernel<N, G><<<static_cast<unsigned>(blocks), PTE_MIXED_BLOCK, 0, stream>>>(a);
  return cudaGetLastError();
}

} // namespace sgx
