// Per-cell pressure-temperature-equilibrium solvers, one GPU thread per cell,
// state in registers/local memory.
//
// Restates, step for step and in the same floating-point operation order,
// singularity-eos's closure/mixed_cell_models.hpp:
//   PTESolverBase        :329-786  (InitBase, GetTguess, SetVfracFromT, ...)
//   PTESolverRhoT        :873-1193 (reduced system in T and n-1 volume fractions)
//   PTESolverPT          :1198-1446 (2x2 system in T and P)
//   solve_Ax_b_wscr      :176-278  (Jacobi scaling, Cramer for 2x2, QR beyond)
//   PTESolver            :2188-2291 (damped Newton with backtracking)
// The compile-time material count N lets every per-material array live in
// registers; ms (the excluded material) stays a runtime value.
//
// The arithmetic type T is double for the plain path (bit-identical to the
// reference built without FP contraction) and float for the iteration phase
// of the mixed-precision path, which is then refined in double.
#pragma once

#include "sgx_dispatch.cuh"

namespace sgx {
SGX_DISPATCH_BEGIN

struct PteStatusLocal {
  double residual = 0;
  int niter = 0;
  bool converged = false;
  bool slow = false;
  int max_line_niter = 0;
  int small_step_iters = 0;
};

// Column-pivoted Householder QR solve of the n x n row-major system
// A x = b (A, b overwritten; x written). Same loops and order as the oracle's
// Eigen-lite (Businger-Golub; Golub & Van Loan Alg. 5.4.1, Eigen's
// Householder convention); a zero pivot gives a zero component.
template <typename T, int N>
SGX_HD void colpiv_qr_solve(T (&R)[N * N], T (&b)[N], T (&x)[N]) {
  constexpr int n = N;
  int perm[N];
#pragma unroll
  for (int j = 0; j < n; ++j)
    perm[j] = j;
#pragma unroll
  for (int k = 0; k < n; ++k) {
    int p = k;
    T cmax = T(-1.0);
#pragma unroll
    for (int j = k; j < n; ++j) {
      T c = T(0.0);
#pragma unroll
      for (int i = k; i < n; ++i)
        c += R[i * n + j] * R[i * n + j];
      if (c > cmax) {
        cmax = c;
        p = j;
      }
    }
    if (p != k) {
#pragma unroll
      for (int j = k + 1; j < n; ++j) {
        if (j == p) {
#pragma unroll
          for (int i = 0; i < n; ++i) {
            const T t = R[i * n + k];
            R[i * n + k] = R[i * n + j];
            R[i * n + j] = t;
          }
          const int t = perm[k];
          perm[k] = perm[j];
          perm[j] = t;
        }
      }
    }
    T sigma = T(0.0);
#pragma unroll
    for (int i = k + 1; i < n; ++i)
      sigma += R[i * n + k] * R[i * n + k];
    if (sigma == T(0.0)) continue;
    const T x0 = R[k * n + k];
#if defined(__CUDA_ARCH__)
    const T mu = sqrt(x0 * x0 + sigma);
#else
    const T mu = __builtin_sqrt(x0 * x0 + sigma);
#endif
    const T beta = (x0 >= T(0.0)) ? -mu : mu;
    const T v0 = x0 - beta;
    const T tau = (beta - x0) / beta;
#pragma unroll
    for (int i = k + 1; i < n; ++i)
      R[i * n + k] = R[i * n + k] / v0;
    R[k * n + k] = beta;
#pragma unroll
    for (int j = k + 1; j < n; ++j) {
      T s = R[k * n + j];
#pragma unroll
      for (int i = k + 1; i < n; ++i)
        s += R[i * n + k] * R[i * n + j];
      s = s * tau;
      R[k * n + j] -= s;
#pragma unroll
      for (int i = k + 1; i < n; ++i)
        R[i * n + j] -= s * R[i * n + k];
    }
    T s = b[k];
#pragma unroll
    for (int i = k + 1; i < n; ++i)
      s += R[i * n + k] * b[i];
    s = s * tau;
    b[k] -= s;
#pragma unroll
    for (int i = k + 1; i < n; ++i)
      b[i] -= s * R[i * n + k];
  }
  T z[N];
#pragma unroll
  for (int i = n - 1; i >= 0; --i) {
    T s = b[i];
#pragma unroll
    for (int j = i + 1; j < n; ++j)
      s -= R[i * n + j] * z[j];
    z[i] = (R[i * n + i] == T(0.0)) ? T(0.0) : s / R[i * n + i];
  }
#pragma unroll
  for (int i = 0; i < n; ++i) {
#pragma unroll
    for (int j = 0; j < n; ++j)
      if (perm[i] == j) x[j] = z[i];
  }
}

// mix_impl::isfinite (mixed_cell_models.hpp:155-157)
template <typename T> SGX_HD bool mix_isfinite(const T a) {
  return (a == a) && ((a == T(0)) || (a != 2 * a));
}

// solve_Ax_b_wscr (mixed_cell_models.hpp:176-278); b holds x on return.
template <typename T, int N> SGX_HD bool solve_Ax_b(T (&a)[N * N], T (&b)[N]) {
  constexpr int n = N;
#pragma unroll
  for (int row = 0; row < n; ++row) {
    T maxabs = T(0);
#pragma unroll
    for (int column = 0; column < n; ++column)
      maxabs = smax(sabs(a[row * n + column]), maxabs);
    if (maxabs == T(0)) return false;
#pragma unroll
    for (int column = 0; column < n; ++column)
      a[row * n + column] /= maxabs;
    b[row] /= maxabs;
  }
  if constexpr (N == 1) {
    b[0] = ratio(b[0], a[0]);
  } else if constexpr (N == 2) {
    const T det = a[0] * a[3] - a[1] * a[2];
    const T x0 = ratio(a[3] * b[0] - a[1] * b[1], det);
    const T x1 = ratio(a[0] * b[1] - a[2] * b[0], det);
    b[0] = x0;
    b[1] = x1;
  } else {
    T x[N];
    colpiv_qr_solve<T, N>(a, b, x);
#pragma unroll
    for (int i = 0; i < n; ++i)
      b[i] = x[i];
  }
  bool ok = true;
#pragma unroll
  for (int i = 0; i < n; ++i)
    if (!mix_isfinite(b[i])) ok = false;
  return ok;
}

// Parameters used inside the iteration, converted to the arithmetic type.
template <typename T> struct MixP {
  bool iterate_t_guess;
  T derivative_eps, tol_p, tol_e, tol_v, abs_p, slow_thresh;
  T tol_p_suff, tol_e_suff, tol_v_suff, abs_p_suff;
  T tol_t, abs_t, tol_t_suff, abs_t_suff, min_dtde;
  int max_iter_per_mat;
  T ls_alpha;
  int ls_max_iter;
  T ls_fac, vfrac_safety_fac, temperature_limit, default_tguess;
  int small_step_tries;
  T small_step_thresh, max_dpdv;
  int exclude_idx;
  SGX_HD MixP() {}
  SGX_HD explicit MixP(const sgx_mix_params &q) {
    iterate_t_guess = q.iterate_t_guess != 0;
    derivative_eps = T(q.derivative_eps);
    tol_p = T(q.pte_rel_tolerance_p);
    tol_e = T(q.pte_rel_tolerance_e);
    tol_v = T(q.pte_rel_tolerance_v);
    abs_p = T(q.pte_abs_tolerance_p);
    slow_thresh = T(q.pte_slow_convergence_thresh);
    tol_p_suff = T(q.pte_rel_tolerance_p_sufficient);
    tol_e_suff = T(q.pte_rel_tolerance_e_sufficient);
    tol_v_suff = T(q.pte_rel_tolerance_v_sufficient);
    abs_p_suff = T(q.pte_abs_tolerance_p_sufficient);
    tol_t = T(q.pte_rel_tolerance_t);
    abs_t = T(q.pte_abs_tolerance_t);
    tol_t_suff = T(q.pte_rel_tolerance_t_sufficient);
    abs_t_suff = T(q.pte_abs_tolerance_t_sufficient);
    min_dtde = T(q.min_dtde);
    max_iter_per_mat = int(q.pte_max_iter_per_mat);
    ls_alpha = T(q.line_search_alpha);
    ls_max_iter = int(q.line_search_max_iter);
    ls_fac = T(q.line_search_fac);
    vfrac_safety_fac = T(q.vfrac_safety_fac);
    temperature_limit = T(q.temperature_limit);
    default_tguess = T(q.default_tguess);
    small_step_tries = int(q.pte_small_step_tries);
    small_step_thresh = T(q.pte_small_step_thresh);
    max_dpdv = T(q.pte_max_dpdv);
    exclude_idx = int(q.pte_reduced_system_exclude_idx);
  }
};

// ===========================================================================
// Shared base: PTESolverBase (mixed_cell_models.hpp:329-786)
// ===========================================================================
template <typename T, int N, int NEQ> struct PteBase {
  static constexpr int n = N;
  const sgx_eos *eos[N];
  double *lam[N]; // per-material lambda cache (3 doubles) or nullptr
  const MixP<T> *P;
  T rho[N], vfrac[N], sie[N], temp[N], press[N];
  T u[N], rhobar[N];
  T jac[NEQ * NEQ], dx[NEQ], residual[NEQ];
  T vfrac_total, sie_total, rho_total, uscale, utotal_scale, Tnorm;
  int niter;
  int err_flags; // non-zero when a reference abort path was taken

  // The constructor arguments: the cell's specific internal energy (or
  // the fixed T or P of PTESolverFixedT / FixedP, which override this) and
  // the temperature normalisation passed in (0: none).
  SGX_HD void configure(const T target) {
    sie_total = target;
    Tnorm = T(0.0);
  }
  SGX_HD T e_of(int m, T r, T t) const { return ev_sie_from_rho_T<T>(*eos[m], r, t, lam[m]); }
  SGX_HD T p_of(int m, T r, T t) const { return ev_P_from_rho_T<T>(*eos[m], r, t, lam[m]); }
  SGX_HD T t_of(int m, T r, T e) const { return ev_T_from_rho_sie<T>(*eos[m], r, e, lam[m]); }
  // GetPressureFromPreferred with do_e_lookup = false (:583-597)
  SGX_HD T p_pref(int m, T r, T t, T e) const {
    if (preferred_input(*eos[m]) & Q_SIE) return ev_P_from_rho_sie<T>(*eos[m], r, e, lam[m]);
    return ev_P_from_rho_T<T>(*eos[m], r, t, lam[m]);
  }
  // GetPressureFromPreferred with do_e_lookup = true
  SGX_HD T p_pref_lookup(int m, T r, T t) const {
    if (preferred_input(*eos[m]) & Q_SIE)
      return ev_P_from_rho_sie<T>(*eos[m], r, e_of(m, r, t), lam[m]);
    return ev_P_from_rho_T<T>(*eos[m], r, t, lam[m]);
  }
  SGX_HD void fixup() {}
  // PTESolverBase::Finalize (:351-357)
  SGX_HD void finalize() {
#pragma unroll
    for (int m = 0; m < n; m++) {
      temp[m] *= Tnorm;
      u[m] *= uscale;
      press[m] *= uscale;
    }
  }

  SGX_HD void init_rhobar() {
#pragma unroll
    for (int m = 0; m < n; ++m)
      rhobar[m] = rho[m] * vfrac[m];
    rho_total = sum_neumaier(rhobar, n);
  }
  SGX_HD void normalize_vfrac() {
    const T vfrac_sum = sum_neumaier(vfrac, n);
#pragma unroll
    for (int m = 0; m < n; ++m)
      vfrac[m] *= ratio(vfrac_total, vfrac_sum);
  }
  SGX_HD T vfrac_max(int m, T Tk) const {
    const T rho_min = ev_rho_pmin_t<T>(*eos[m], Tk);
    return smin(T(0.9) * ratio(rhobar[m], rho_min), T(1.0));
  }
  // SetVfracFromT (:423-498); true = FAIL
  SGX_HD bool set_vfrac_from_T(const T Tk) {
    const T min_dv = T(1e-12);
    T vfrac_max_sum = 0;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      const T vmax = vfrac_max(m, Tk);
      if (vfrac[m] <= T(0)) vfrac[m] = vmax;
      vfrac_max_sum += vmax;
    }
    if (vfrac_max_sum < vfrac_total) return true;
    normalize_vfrac();
    for (int it = 0; it < n; ++it) {
      T remaining = 0;
      unsigned n_uncapped = n;
#pragma unroll
      for (int m = 0; m < n; ++m) {
        const T vnew = smin(vfrac_max(m, Tk), vfrac[m]);
        const T dv = vfrac[m] - vnew;
        vfrac[m] -= dv;
        remaining += dv;
        n_uncapped -= (dv > min_dv);
      }
      if (sabs(remaining) < min_dv) break;
#pragma unroll
      for (int m = 0; m < n; ++m) {
        const bool uncapped = ((vfrac_max(m, Tk) - vfrac[m]) > min_dv);
        if (uncapped) vfrac[m] += remaining / T(n_uncapped);
      }
    }
    normalize_vfrac();
    return false;
  }
  // GetSieCvFromTAndPreferred (:599-620)
  SGX_HD void sie_cv_pref(int m, T r, const T Pin, const T Tk, T &s, T &cv) const {
    const sgx_eos &e = *eos[m];
    if (preferred_input(e) & Q_PRESSURE) {
      if constexpr (sizeof(T) == sizeof(float)) {
        // the FP32 phase: a closed-form model with a usable pressure needs
        // no FP64 (its maximum pressure is 1e100, beyond any float)
        T rf, sf;
        if (!mix_bad_f(Pin) && ev_rho_sie_from_PT_f(e, smax(T(ev_min_pressure(e)), Pin), Tk, rf,
                                                    sf)) {
          s = sf;
          cv = ev_cv_from_rho_sie<T>(e, rf, sf, lam[m]);
          return;
        }
      }
      int err = 0;
      const T Pmin = T(ev_min_pressure(e));
      const T Pmax = T(ev_max_pressure_at_T(e, double(Tk), &err));
      T Pguess;
      if (bad_value(double(Pin)))
        Pguess = T(0.5) * (Pmin + Pmax);
      else
        Pguess = smax(Pmin, smin(Pmax, Pin));
      double rr = double(r), ss = 0;
      ev_rho_sie_from_PT(e, double(Pguess), double(Tk), rr, ss, lam[m], &err);
      r = T(rr);
      s = T(ss);
      cv = ev_cv_from_rho_sie<T>(e, r, s, lam[m]);
    } else {
      s = ev_sie_from_rho_T<T>(e, r, Tk, lam[m]);
      cv = ev_cv_from_rho_T<T>(e, r, Tk, lam[m]);
    }
  }
  // GetTguess (:500-581)
  SGX_HD T get_tguess() {
    T Tguess;
    if (Tnorm > T(0.0)) {
      Tguess = Tnorm;
    } else {
      Tguess = P->default_tguess;
#pragma unroll
      for (int m = 0; m < n; ++m)
        Tguess = smax(Tguess, temp[m]);
    }
    auto newton_step = [&](T Tk) {
      T dudt = 0, usum = 0;
#pragma unroll
      for (int m = 0; m < n; ++m) {
        const T rho_max = T(ev_max_density(*eos[m]));
        T s, cv;
        sie_cv_pref(m, smin(rho[m], rho_max), press[m], Tk, s, cv);
        usum += rhobar[m] * s;
        dudt += rhobar[m] * cv;
      }
      return Tk - ratio((usum - utotal_scale * uscale), dudt);
    };
    const T Tfactor = T(10.0);
    bool bad = false;
    for (int i = 0; i < 3; i++) {
      if (P->iterate_t_guess)
        Tguess = smin(P->temperature_limit, smax(Tguess, newton_step(Tguess)));
#pragma unroll
      for (int m = 0; m < n; ++m)
        Tguess = smax(T(ev_min_temperature(*eos[m])), Tguess);
      bad = set_vfrac_from_T(Tguess);
      if (bad) {
        Tguess *= Tfactor;
        continue;
      }
#pragma unroll
      for (int m = 0; m < n; ++m)
        rho[m] = ratio(rhobar[m], vfrac[m]);
      bad = false;
      for (int m = 0; m < n; ++m) {
        const T rho_min = T(ev_rho_pmin(*eos[m], double(Tguess)));
        if (rho[m] < rho_min) {
          bad = true;
          Tguess *= Tfactor;
          break;
        }
      }
      if (!bad) break;
    }
    return Tguess;
  }
  // InitBase (:627-662)
  SGX_HD void init_base() {
    init_rhobar();
    const T utotal = rho_total * sie_total;
    uscale = smax(sabs(utotal), T(1.0e-14));
    utotal_scale = ratio(utotal, uscale);
    const T Tguess = get_tguess();
    Tnorm = Tguess;
#pragma unroll
    for (int m = 0; m < n; m++) {
      temp[m] = T(1.0);
      sie[m] = e_of(m, rho[m], Tguess);
      if ((preferred_input(*eos[m]) & Q_PRESSURE) && !bad_value(double(press[m])))
        press[m] = ratio(press[m], uscale);
      else
        press[m] = ratio(p_pref(m, rho[m], Tguess, sie[m]), uscale);
    }
#pragma unroll
    for (int m = 0; m < n; ++m)
      u[m] = sie[m] * ratio(rhobar[m], uscale);
  }
  SGX_HD T residual_norm() const { return T(0.5) * sum_neumaier_sq(residual, NEQ); }
  SGX_HD bool solve() {
#pragma unroll
    for (int m = 0; m < NEQ; m++)
      dx[m] = residual[m];
    return solve_Ax_b<T, NEQ>(jac, dx);
  }
};

// ===========================================================================
// PTESolverRhoT (:884-1193)
// ===========================================================================
template <typename T, int N> struct PteRhoT : PteBase<T, N, N> {
  using B = PteBase<T, N, N>;
  using B::dx;
  using B::eos;
  using B::jac;
  using B::P;
  using B::press;
  using B::residual;
  using B::rho;
  using B::rhobar;
  using B::sie;
  using B::temp;
  using B::Tnorm;
  using B::u;
  using B::uscale;
  using B::utotal_scale;
  using B::vfrac;
  static constexpr int n = N;
  T dpdv[N], dedv[N], dpdT[N], vtemp[N];
  T Tequil, Ttemp;
  int ms;
  // Mixed-precision solver only: closed-form derivatives for the analytic
  // models instead of the reference's finite differences.
  bool use_analytic = false;

  SGX_HD void residual_eval() {
    const T esum = sum_neumaier(u, n);
    residual[0] = utotal_scale - esum;
    int ires = 1;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      if (m == ms) continue;
      residual[ires++] = press[ms] - press[m];
    }
  }
  SGX_HD T init() {
    B::init_base();
    if (P->exclude_idx >= 0) {
      ms = P->exclude_idx;
    } else {
      ms = 0;
      T xmax = 0;
#pragma unroll
      for (int m = 0; m < n; ++m) {
        const T x = ratio(rhobar[m], B::rho_total);
        if (x > xmax) {
          xmax = x;
          ms = m;
        }
      }
    }
    residual_eval();
    Tequil = temp[0];
    return B::residual_norm();
  }
  SGX_HD void fixup() {
    if (P->exclude_idx < 0) {
      T alphamax = 0;
      ms = 0;
#pragma unroll
      for (int m = 0; m < n; ++m) {
        if (vfrac[m] > alphamax) {
          alphamax = vfrac[m];
          ms = m;
        }
      }
      residual_eval();
    }
  }
  // CheckPTE (:1021-1040): {converged, acceptable}
  SGX_HD void check(bool &conv, bool &acceptable) const {
    T mean_p = 0;
#pragma unroll
    for (int m = 0; m < n; ++m)
      mean_p += vfrac[m] * press[m];
#if defined(__CUDA_ARCH__)
    const T error_p = sqrt(sum_neumaier_sq(residual, n - 1, 1));
#else
    const T error_p = __builtin_sqrt(sum_neumaier_sq(residual, n - 1, 1));
#endif
    const T error_u = sabs(residual[0]);
    const bool converged_p = (error_p < P->tol_p * sabs(mean_p) || error_p < P->abs_p);
    const bool converged_u = (error_u < P->tol_e);
    const bool acceptable_p =
        (error_p < P->tol_p_suff * sabs(mean_p) || error_p < P->abs_p_suff);
    const bool acceptable_u = (error_u < P->tol_e_suff);
    conv = converged_p && converged_u;
    acceptable = acceptable_p && acceptable_u;
  }
  // Closed-form counterpart of the finite-difference columns below (same
  // scaled quantities: d(P_m/uscale)/d alpha_m, d u_m / d alpha_m,
  // d(P_m/uscale)/dT and d u_m / dT with T scaled by Tnorm). False if a
  // material is tabulated.
  SGX_HD bool derivs_analytic(T &dedT_sum) {
    dedT_sum = 0;
#pragma unroll
    for (int m = 0; m < n; m++) {
      T de_drho, de_dT, dP_drho, dP_dT;
      if (!eos_derivs<T>(*eos[m], rho[m], Tnorm * Tequil, de_drho, de_dT, dP_drho, dP_dT))
        return false;
      const T drho_dalpha = -rho[m] / vfrac[m];
      dpdv[m] = smin(dP_drho * drho_dalpha / uscale, -sabs(P->max_dpdv));
      dedv[m] = rhobar[m] * de_drho * drho_dalpha / uscale;
      dpdT[m] = dP_dT * Tnorm / uscale;
      dedT_sum += rhobar[m] * de_dT * Tnorm / uscale;
    }
    return true;
  }
  SGX_HD void jacobian() {
    T dedT_sum = 0.0;
    if (!(use_analytic && derivs_analytic(dedT_sum))) {
    dedT_sum = 0.0;
#pragma unroll
    for (int m = 0; m < n; m++) {
      const T dv = (vfrac[m] < T(0.5) ? T(1.0) : T(-1.0)) * vfrac[m] * P->derivative_eps;
      const T vf_pert = vfrac[m] + dv;
      const T rho_pert = ratio(rhobar[m], vf_pert);
      T e_pert = B::e_of(m, rho_pert, Tnorm * Tequil);
      T p_pert = ratio(B::p_pref(m, rho_pert, Tnorm * Tequil, e_pert), uscale);
      dpdv[m] = smin(ratio((p_pert - press[m]), dv), -sabs(P->max_dpdv));
      dedv[m] = ratio(rhobar[m] * ratio(e_pert, uscale) - u[m], dv);
      const T dT = Tequil * P->derivative_eps;
      e_pert = B::e_of(m, rho[m], Tnorm * (Tequil + dT));
      p_pert = ratio(B::p_pref(m, rho[m], Tnorm * (Tequil + dT), e_pert), uscale);
      dpdT[m] = ratio((p_pert - press[m]), dT);
      dedT_sum += ratio(rhobar[m] * ratio(e_pert, uscale) - u[m], dT);
    }
    }
#pragma unroll
    for (int i = 0; i < n * n; ++i)
      jac[i] = 0.0;
    jac[0] = dedT_sum;
    int col = 1;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      if (m == ms) continue;
      jac[col++] = dedv[m] - dedv[ms];
    }
    int row = 1;
#pragma unroll
    for (int m = 0; m < n; m++) {
      if (m == ms) continue;
      jac[row * n + 0] = dpdT[m] - dpdT[ms];
      int c = 1;
#pragma unroll
      for (int mm = 0; mm < n; ++mm) {
        if (mm == ms) continue;
        jac[row * n + c] = (mm == m) ? dpdv[m] + dpdv[ms] : dpdv[ms];
        c++;
      }
      row++;
    }
  }
  SGX_HD T scale_dx() {
    T scale = 1.0;
    const T dalphaskip = -sum_neumaier(dx, n - 1, 1);
    int idx = 1;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      const T mydx = (m == ms) ? dalphaskip : dx[idx++];
      if (scale * mydx < -P->vfrac_safety_fac * vfrac[m])
        scale = smin(scale, sabs(P->vfrac_safety_fac * ratio(vfrac[m], mydx)));
    }
    const T Tnew = Tequil + scale * dx[0];
    idx = 1;
#pragma unroll
    for (int m = 0; m < n; m++) {
      const T rho_min = smax(ev_rho_pmin_t<T>(*eos[m], Tnorm * Tequil),
                             ev_rho_pmin_t<T>(*eos[m], Tnorm * Tnew));
      const T alpha_max = smin(T(1.0), ratio(rhobar[m], rho_min));
      if (alpha_max < vfrac[m]) continue;
      const T mydx = (m == ms) ? dalphaskip : dx[idx++];
      if (scale * mydx > T(0.5) * (alpha_max - vfrac[m]))
        scale = smin(ratio(T(0.5) * (alpha_max - vfrac[m]), mydx), scale);
    }
    if (scale * dx[0] < T(-0.95) * Tequil) scale = smin(scale, ratio(T(-0.95) * Tequil, dx[0]));
#pragma unroll
    for (int i = 0; i < n; ++i)
      dx[i] *= scale;
    return scale;
  }
  SGX_HD T test_update(const T scale, const bool cache_state = false) {
    if (cache_state) {
      Ttemp = Tequil;
#pragma unroll
      for (int m = 0; m < n; ++m)
        vtemp[m] = vfrac[m];
    }
    Tequil = Ttemp + scale * dx[0];
    int idx = 1;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      if (ms == m) continue;
      vfrac[m] = vtemp[m] + scale * dx[idx++];
    }
    vfrac[ms] = sum_neumaier(vfrac, n, 0, ms);
    vfrac[ms] = 1 - vfrac[ms];
#pragma unroll
    for (int m = 0; m < n; ++m) {
      rho[m] = ratio(rhobar[m], vfrac[m]);
      u[m] = rhobar[m] * B::e_of(m, rho[m], Tnorm * Tequil);
      sie[m] = ratio(u[m], rhobar[m]);
      u[m] = ratio(u[m], uscale);
      temp[m] = Tequil;
      press[m] = ratio(B::p_pref(m, rho[m], Tnorm * Tequil, sie[m]), uscale);
    }
    residual_eval();
    return B::residual_norm();
  }
  // PTESolverBase::Finalize (:351-357)
  SGX_HD void finalize() {
#pragma unroll
    for (int m = 0; m < n; m++) {
      temp[m] *= Tnorm;
      u[m] *= uscale;
      press[m] *= uscale;
    }
  }
};

// ===========================================================================
// PTESolverPT (:1207-1446)
// ===========================================================================
template <typename T, int N> struct PtePT : PteBase<T, N, 2> {
  using B = PteBase<T, N, 2>;
  using B::dx;
  using B::eos;
  using B::jac;
  using B::lam;
  using B::P;
  using B::press;
  using B::residual;
  using B::rho;
  using B::rhobar;
  using B::sie;
  using B::temp;
  using B::Tnorm;
  using B::u;
  using B::uscale;
  using B::utotal_scale;
  using B::vfrac;
  using B::vfrac_total;
  static constexpr int n = N;
  T Pequil, Tequil, Ptemp, Ttemp;
  int ms = 0;

  SGX_HD void rho_sie_PT(int m, T Pk, T Tk, T &r, T &s) {
    double rr = double(r), ss = double(s);
    ev_rho_sie_from_PT(*eos[m], double(Pk), double(Tk), rr, ss, lam[m], &this->err_flags);
    r = T(rr);
    s = T(ss);
  }
  SGX_HD void residual_eval() {
    const T vsum = sum_neumaier(vfrac, n);
    const T esum = sum_neumaier(u, n);
    residual[0] = vfrac_total - vsum;
    residual[1] = utotal_scale - esum;
  }
  SGX_HD T init() {
    B::init_base();
    residual_eval();
    Pequil = 0;
#pragma unroll
    for (int m = 0; m < n; ++m)
      Pequil += sabs(press[m]) * vfrac[m];
    const T vsum = sum_neumaier(vfrac, n);
    Pequil /= vsum;
    Tequil = 1;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      rho_sie_PT(m, Pequil * uscale, Tequil * Tnorm, rho[m], sie[m]);
      vfrac[m] = ratio(rhobar[m], rho[m]);
      u[m] = ratio(sie[m] * rhobar[m], uscale);
      temp[m] = Tequil;
    }
    residual_eval();
    return B::residual_norm();
  }
  SGX_HD void fixup() {}
  SGX_HD void finalize() {
#pragma unroll
    for (int m = 0; m < n; m++) {
      press[m] = Pequil * uscale;
      temp[m] = Tequil * Tnorm;
      u[m] *= uscale;
    }
  }
  SGX_HD void check(bool &conv, bool &acceptable) const {
    const T error_v = sabs(residual[0]);
    const T error_u = sabs(residual[1]);
    const bool converged_u = error_u < P->tol_e;
    const bool converged_v = error_v < P->tol_v;
    const bool acceptable_u = error_u < P->tol_e_suff;
    const bool acceptable_v = error_v < P->tol_v_suff;
    conv = converged_v && converged_u;
    acceptable = acceptable_u && acceptable_v;
  }
  SGX_HD void jacobian() {
    T dudT_P_sum = 0.0, dudP_T_sum = 0.0, rbor2_dr_dT_P_sum = 0.0, rbor2_dr_dP_T_sum = 0.0;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      T r_pert = rho[m];
      T e_pert = sie[m];
      const T dp = -Pequil * P->derivative_eps;
      rho_sie_PT(m, uscale * (Pequil + dp), Tnorm * Tequil, r_pert, e_pert);
      const T drdp = ratio(r_pert - rho[m], dp);
      const T dudp = ratio(ratio(rhobar[m] * e_pert, uscale) - u[m], dp);
      rbor2_dr_dP_T_sum += ratio(rhobar[m], rho[m] * rho[m]) * drdp;
      dudP_T_sum += dudp;
      const T dT = Tequil * P->derivative_eps;
      rho_sie_PT(m, uscale * Pequil, Tnorm * (Tequil + dT), r_pert, e_pert);
      const T drdT = ratio(r_pert - rho[m], dT);
      const T dudT = ratio(ratio(rhobar[m] * e_pert, uscale) - u[m], dT);
      rbor2_dr_dT_P_sum += ratio(rhobar[m], rho[m] * rho[m]) * drdT;
      dudT_P_sum += dudT;
    }
    jac[0] = -rbor2_dr_dT_P_sum;
    jac[1] = -rbor2_dr_dP_T_sum;
    jac[2] = dudT_P_sum;
    jac[3] = dudP_T_sum;
  }
  SGX_HD T scale_dx() {
    T scale = 1.0;
    if (scale * dx[0] < T(-0.95) * Tequil) scale = ratio(T(-0.95) * Tequil, dx[0]);
    auto bounded = [&](T Pbound, T delta) { return ratio(ratio(Pbound, uscale) - Pequil, delta); };
#pragma unroll
    for (int m = 0; m < n; ++m) {
      const T Pmin = T(ev_min_pressure(*eos[m]));
      scale = smin(sabs(scale), sabs(T(0.95) * bounded(Pmin, dx[1])));
    }
#pragma unroll
    for (int m = 0; m < n; ++m) {
      const T Ttest = (Tequil + scale * dx[0]) * Tnorm;
      const T Pmax = T(ev_max_pressure_at_T(*eos[m], double(Ttest), &this->err_flags));
      scale = smin(sabs(scale), sabs(T(0.95) * bounded(Pmax, dx[0])));
    }
    dx[0] *= scale;
    dx[1] *= scale;
    return scale;
  }
  SGX_HD T test_update(const T scale, const bool cache_state = false) {
    if (cache_state) {
      Ttemp = Tequil;
      Ptemp = Pequil;
    }
    Tequil = Ttemp + scale * dx[0];
    Pequil = Ptemp + scale * dx[1];
#pragma unroll
    for (int m = 0; m < n; ++m) {
      rho_sie_PT(m, Pequil * uscale, Tequil * Tnorm, rho[m], sie[m]);
      vfrac[m] = ratio(rhobar[m], rho[m]);
      u[m] = ratio(sie[m] * rhobar[m], uscale);
      temp[m] = Tequil;
      press[m] = Pequil;
    }
    residual_eval();
    return B::residual_norm();
  }
};

// ===========================================================================
// PTESolverFixedT (:1451-1637): volume fractions at a given temperature
// ===========================================================================
// Unknowns: the n volume fractions. Residuals: the volume sum and the n-1
// pressure differences P_m - P_{m+1}. The temperature is the constructor's
// T_true (the per-cell target); temp[] is passed through (x Tnorm = 1).
template <typename T, int N> struct PteFixedT : PteBase<T, N, N> {
  using B = PteBase<T, N, N>;
  using B::dx;
  using B::jac;
  using B::P;
  using B::press;
  using B::residual;
  using B::rho;
  using B::rhobar;
  using B::sie;
  using B::Tnorm;
  using B::u;
  using B::uscale;
  using B::vfrac;
  using B::vfrac_total;
  static constexpr int n = N;
  T dpdv[N], vtemp[N];
  T Tequil, Ttemp;

  // ctor (:1497-1508): base(sie_tot = 1, Tnorm = T_true), then Tnorm = 1
  SGX_HD void configure(const T T_true) {
    this->sie_total = T(1.0);
    Tequil = T_true;
    Ttemp = T_true;
    Tnorm = T(1.0);
  }
  SGX_HD void residual_eval() {
    const T vsum = sum_neumaier(vfrac, n);
    residual[0] = vfrac_total - vsum;
#pragma unroll
    for (int m = 0; m < n - 1; ++m)
      residual[1 + m] = press[m] - press[m + 1];
  }
  // Init (:1520-1548)
  SGX_HD T init() {
    Tnorm = T(1.0);
    B::init_rhobar();
    B::set_vfrac_from_T(Tequil);
    uscale = T(0.0);
#pragma unroll
    for (int m = 0; m < n; m++) {
      rho[m] = ratio(rhobar[m], vfrac[m]);
      sie[m] = B::e_of(m, rho[m], Tequil);
      uscale += sabs(sie[m]) * rho[m];
      press[m] = B::p_of(m, rho[m], Tequil);
    }
    uscale = smax(uscale, T(1.0e-14));
#pragma unroll
    for (int m = 0; m < n; ++m) {
      press[m] = ratio(press[m], uscale);
      u[m] = sie[m] * ratio(rhobar[m], uscale);
    }
    residual_eval();
    return B::residual_norm();
  }
  // CheckPTE (:1560-1578)
  SGX_HD void check(bool &conv, bool &acceptable) const {
    T mean_p = vfrac[0] * press[0];
    T error_p = 0;
#pragma unroll
    for (int m = 1; m < n; ++m) {
      mean_p += vfrac[m] * press[m];
      error_p += residual[m] * residual[m];
    }
    error_p = ssqrt(error_p);
    const T error_v = sabs(residual[0]);
    const bool converged_p = (error_p < P->tol_p * sabs(mean_p) || error_p < P->abs_p);
    const bool converged_v = error_v < P->tol_v;
    const bool acceptable_p =
        (error_p < P->tol_p_suff * sabs(mean_p) || error_p < P->abs_p_suff);
    const bool acceptable_v = error_v < P->tol_v_suff;
    conv = converged_p && converged_v;
    acceptable = acceptable_p && acceptable_v;
  }
  // Jacobian (:1580-1606)
  SGX_HD void jacobian() {
#pragma unroll
    for (int m = 0; m < n; m++) {
      const T dv = (vfrac[m] < T(0.5) ? T(1.0) : T(-1.0)) * vfrac[m] * P->derivative_eps;
      const T vf_pert = vfrac[m] + dv;
      const T rho_pert = ratio(rhobar[m], vf_pert);
      const T p_pert = ratio(B::p_of(m, rho_pert, Tequil), uscale);
      dpdv[m] = smin(ratio((p_pert - press[m]), dv), -sabs(P->max_dpdv));
    }
#pragma unroll
    for (int i = 0; i < n * n; ++i)
      jac[i] = T(0.0);
#pragma unroll
    for (int m = 0; m < n; ++m)
      jac[m] = T(1.0);
#pragma unroll
    for (int m = 0; m < n - 1; m++) {
      jac[(m + 1) * n + m] = -dpdv[m];
      jac[(m + 1) * n + m + 1] = dpdv[m + 1];
    }
  }
  // ScaleDx (:1608-1633)
  SGX_HD T scale_dx() {
    T scale = 1.0;
#pragma unroll
    for (int m = 0; m < n; ++m)
      if (scale * dx[m] < -P->vfrac_safety_fac * vfrac[m])
        scale = ratio(-P->vfrac_safety_fac * vfrac[m], dx[m]);
#pragma unroll
    for (int m = 0; m < n; m++) {
      const T rho_min = T(ev_rho_pmin(*this->eos[m], double(Tequil)));
      const T alpha_max = ratio(rhobar[m], rho_min);
      if (alpha_max < vfrac[m]) continue;
      if (scale * dx[m] > T(0.5) * (alpha_max - vfrac[m]))
        scale = ratio(T(0.5) * (alpha_max - vfrac[m]), dx[m]);
    }
#pragma unroll
    for (int i = 0; i < n; ++i)
      dx[i] *= scale;
    return scale;
  }
  // TestUpdate (:1637-1660)
  SGX_HD T test_update(const T scale, const bool cache_state = false) {
    if (cache_state) {
#pragma unroll
      for (int m = 0; m < n; ++m)
        vtemp[m] = vfrac[m];
    }
#pragma unroll
    for (int m = 0; m < n; ++m) {
      vfrac[m] = vtemp[m] + scale * dx[m];
      rho[m] = ratio(rhobar[m], vfrac[m]);
      u[m] = rhobar[m] * B::e_of(m, rho[m], Tequil);
      sie[m] = ratio(u[m], rhobar[m]);
      u[m] = ratio(u[m], uscale);
      press[m] = ratio(B::p_of(m, rho[m], Tequil), uscale);
    }
    residual_eval();
    return B::residual_norm();
  }
};

// ===========================================================================
// PTESolverFixedP (:1665-1919): volume fractions and temperature at a given
// pressure
// ===========================================================================
// Unknowns: the n volume fractions and T. Residuals: P - P_m for every
// material and the volume sum. The pressure is the constructor's P (the
// per-cell target).
template <typename T, int N> struct PteFixedP : PteBase<T, N, N + 1> {
  using B = PteBase<T, N, N + 1>;
  using B::dx;
  using B::jac;
  using B::P;
  using B::press;
  using B::residual;
  using B::rho;
  using B::rhobar;
  using B::sie;
  using B::temp;
  using B::Tnorm;
  using B::u;
  using B::uscale;
  using B::vfrac;
  using B::vfrac_total;
  static constexpr int n = N;
  static constexpr int neq = N + 1;
  T dpdv[N], dpdT[N], vtemp[N];
  T Tequil, Ttemp, Pequil;

  // ctor (:1722-1734): base(sie_tot = 1, Tnorm = 0). The reference's
  // GetTguess reads uscale and utotal_scale before this solver sets them
  // (its Newton step on the energy sum, :522-535); they are zero here,
  // which is what the reference computes when that memory is zero.
  SGX_HD void configure(const T Ptarget) {
    this->sie_total = T(1.0);
    Tnorm = T(0.0);
    Pequil = Ptarget;
    uscale = T(0.0);
    this->utotal_scale = T(0.0);
  }
  SGX_HD void residual_eval() {
    const T vsum = sum_neumaier(vfrac, n);
#pragma unroll
    for (int m = 0; m < n; ++m)
      residual[m] = ratio(Pequil, uscale) - press[m];
    residual[n] = vfrac_total - vsum;
  }
  // Init (:1746-1779)
  SGX_HD T init() {
    B::init_rhobar();
    const T Tguess = B::get_tguess();
    Tnorm = Tguess;
    uscale = smax(sabs(Pequil), T(1.0e-14));
#pragma unroll
    for (int m = 0; m < n; m++) {
      temp[m] = T(1.0);
      sie[m] = B::e_of(m, rho[m], Tguess);
    }
#pragma unroll
    for (int m = 0; m < n; ++m) {
      u[m] = ratio(sie[m] * rhobar[m], uscale);
      press[m] = ratio(B::p_of(m, rho[m], Tguess), uscale);
    }
    residual_eval();
    Tequil = temp[0];
    Ttemp = Tequil;
    return B::residual_norm();
  }
  // CheckPTE (:1790-1808)
  SGX_HD void check(bool &conv, bool &acceptable) const {
    T error_p = 0;
#pragma unroll
    for (int m = 0; m < n; ++m)
      error_p += residual[m] * residual[m];
    error_p = ssqrt(error_p);
    error_p *= uscale;
    const T error_v = sabs(residual[neq - 1]);
    const bool converged_p = (error_p < P->tol_p || error_p < P->abs_p);
    const bool converged_v = error_v < P->tol_v;
    const bool acceptable_p = (error_p < P->tol_p_suff || error_p < P->abs_p_suff);
    const bool acceptable_v = error_v < P->tol_v_suff;
    conv = converged_p && converged_v;
    acceptable = acceptable_p && acceptable_v;
  }
  // Jacobian (:1810-1852)
  SGX_HD void jacobian() {
#pragma unroll
    for (int m = 0; m < n; m++) {
      const T dv = (vfrac[m] < T(0.5) ? T(1.0) : T(-1.0)) * vfrac[m] * P->derivative_eps;
      const T vf_pert = vfrac[m] + dv;
      const T rho_pert = ratio(rhobar[m], vf_pert);
      T p_pert = ratio(B::p_pref_lookup(m, rho_pert, Tnorm * Tequil), uscale);
      dpdv[m] = smin(ratio((p_pert - press[m]), dv), -sabs(P->max_dpdv));
      const T dT = Tequil * P->derivative_eps;
      p_pert = ratio(B::p_pref_lookup(m, rho[m], Tnorm * (Tequil + dT)), uscale);
      dpdT[m] = ratio((p_pert - press[m]), dT);
    }
#pragma unroll
    for (int i = 0; i < neq * neq; ++i)
      jac[i] = T(0.0);
#pragma unroll
    for (int m = 0; m < n; m++) {
      jac[m * neq + m] = dpdv[m];
      jac[m * neq + n] = dpdT[m];
    }
#pragma unroll
    for (int m = 0; m < neq - 1; ++m)
      jac[(neq - 1) * neq + m] = T(1.0);
  }
  // ScaleDx (:1854-1885)
  SGX_HD T scale_dx() {
    T scale = 1.0;
#pragma unroll
    for (int m = 0; m < n; ++m)
      if (scale * dx[m] < -P->vfrac_safety_fac * vfrac[m])
        scale = -P->vfrac_safety_fac * ratio(vfrac[m], dx[m]);
    const T Tnew = Tequil + scale * dx[n];
#pragma unroll
    for (int m = 0; m < n; m++) {
      const T rho_min = T(smax(ev_rho_pmin(*this->eos[m], double(Tnorm * Tequil)),
                               ev_rho_pmin(*this->eos[m], double(Tnorm * Tnew))));
      const T alpha_max = ratio(rhobar[m], rho_min);
      if (alpha_max < vfrac[m]) continue;
      if (scale * dx[m] > T(0.5) * (alpha_max - vfrac[m]))
        scale = T(0.5) * ratio(alpha_max - vfrac[m], dx[m]);
    }
    if (scale * dx[n] < T(-0.95) * Tequil) scale = T(-0.95) * ratio(Tequil, dx[n]);
#pragma unroll
    for (int i = 0; i < neq; ++i)
      dx[i] *= scale;
    return scale;
  }
  // TestUpdate (:1889-1913)
  SGX_HD T test_update(const T scale, const bool cache_state = false) {
    if (cache_state) {
      Ttemp = Tequil;
#pragma unroll
      for (int m = 0; m < n; ++m)
        vtemp[m] = vfrac[m];
    }
    Tequil = Ttemp + scale * dx[n];
#pragma unroll
    for (int m = 0; m < n; ++m) {
      vfrac[m] = vtemp[m] + scale * dx[m];
      rho[m] = ratio(rhobar[m], vfrac[m]);
      u[m] = rhobar[m] * B::e_of(m, rho[m], Tnorm * Tequil);
      press[m] = ratio(B::p_of(m, rho[m], Tnorm * Tequil), uscale);
      sie[m] = ratio(u[m], rhobar[m]);
      u[m] = ratio(u[m], uscale);
      temp[m] = Tequil;
    }
    residual_eval();
    return B::residual_norm();
  }
};

// ===========================================================================
// PTESolverRhoU (:1921-2183): full system in volume fractions and energies
// ===========================================================================
// Unknowns: the n volume fractions and the n scaled energy densities u_m.
// Residuals: volume sum, energy sum, n-1 pressure differences and n-1
// temperature differences; each material's T comes from T(rho, sie).
template <typename T, int N> struct PteRhoU : PteBase<T, N, 2 * N> {
  using B = PteBase<T, N, 2 * N>;
  using B::dx;
  using B::jac;
  using B::P;
  using B::press;
  using B::residual;
  using B::rho;
  using B::rho_total;
  using B::rhobar;
  using B::sie;
  using B::temp;
  using B::Tnorm;
  using B::u;
  using B::uscale;
  using B::utotal_scale;
  using B::vfrac;
  using B::vfrac_total;
  static constexpr int n = N;
  static constexpr int neq = 2 * N;
  T dpdv[N], dtdv[N], dpde[N], dtde[N], vtemp[N], utemp[N];

  // Out-of-range writes are dropped: for n = 1 the reference's fixed
  // Jacobian positions (:2094-2101) fall past the 2 x 2 matrix (into the
  // next scratch array, which Solve overwrites).
  SGX_HD void jset(const int idx, const T v) {
    if (idx < neq * neq) jac[idx] = v;
  }
  SGX_HD void residual_eval() {
    const T vsum = sum_neumaier(vfrac, n);
    const T esum = sum_neumaier(u, n);
    residual[0] = vfrac_total - vsum;
    residual[1] = utotal_scale - esum;
#pragma unroll
    for (int m = 0; m < n - 1; ++m)
      residual[2 + m] = press[m + 1] - press[m];
#pragma unroll
    for (int m = n + 1; m < neq; m++)
      residual[m] = temp[m - n] - temp[m - n - 1];
  }
  // PTESolverBase::GetIdealPTE + TryIdealPTE (:676-763): replace the
  // initial state by the ideal-gas PTE estimate when its residual is lower.
  SGX_HD void try_ideal_pte() {
    T rhoBsum = 0.0, Asum = 0.0;
#pragma unroll
    for (int m = 0; m < n; m++) {
      Asum += vfrac[m] * ratio(press[m], temp[m]);
      rhoBsum += rho[m] * vfrac[m] * ratio(sie[m], temp[m]);
    }
    Asum *= uscale / Tnorm;
    rhoBsum /= Tnorm;
    const T Tideal = uscale / rhoBsum / Tnorm;
    const T Pideal = ratio(Tnorm * Tideal * Asum, uscale * vfrac_total);
    T etemp[N], ptemp[N], vkeep[N], rtemp[N], res[neq];
#pragma unroll
    for (int m = 0; m < n; ++m) {
      etemp[m] = u[m];
      ptemp[m] = press[m];
      vkeep[m] = vfrac[m];
      rtemp[m] = rho[m];
    }
    T res_norm_old = 0.0;
#pragma unroll
    for (int m = 0; m < neq; ++m) {
      res[m] = residual[m];
      res_norm_old += res[m] * res[m];
    }
    const T alpha = ratio(Pideal, Tideal);
    for (int m = 0; m < n; ++m) {
      vfrac[m] *= ratio(press[m], (temp[m] * alpha));
      if (Tnorm * Tideal < T(0) ||
          ratio(rhobar[m], vfrac[m]) < T(ev_rho_pmin(*this->eos[m], double(Tnorm * Tideal)))) {
        for (int q = 0; q <= m; q++)
          vfrac[q] = vkeep[q];
        return;
      }
    }
#pragma unroll
    for (int m = 0; m < n; ++m) {
      rho[m] = ratio(rhobar[m], vfrac[m]);
      const T sie_m = B::e_of(m, rho[m], Tnorm * Tideal);
      u[m] = rhobar[m] * ratio(sie_m, uscale);
      press[m] = ratio(B::p_pref(m, rho[m], Tnorm * Tideal, sie_m), uscale);
    }
    residual_eval();
    T res_norm_new = 0.0;
#pragma unroll
    for (int m = 0; m < neq; m++)
      res_norm_new += residual[m] * residual[m];
    if (res_norm_new > res_norm_old) {
#pragma unroll
      for (int m = 0; m < n; ++m) {
        vfrac[m] = vkeep[m];
        rho[m] = rtemp[m];
        u[m] = etemp[m];
        press[m] = ptemp[m];
      }
#pragma unroll
      for (int m = 0; m < neq; ++m)
        residual[m] = res[m];
    } else {
#pragma unroll
      for (int m = 0; m < n; ++m) {
        temp[m] = Tideal;
        sie[m] = uscale * ratio(u[m], rhobar[m]);
      }
    }
  }
  // Init (:2000-2006)
  SGX_HD T init() {
    B::init_base();
    residual_eval();
    try_ideal_pte();
    return B::residual_norm();
  }
  // CheckPTE (:2022-2050)
  SGX_HD void check(bool &conv, bool &acceptable) const {
    T mean_p = vfrac[0] * press[0];
    T mean_t = rhobar[0] * temp[0];
    T error_p = 0.0, error_t = 0.0;
#pragma unroll
    for (int m = 1; m < n; ++m) {
      mean_p += vfrac[m] * press[m];
      mean_t += rhobar[m] * temp[m];
      error_p += residual[m + 1] * residual[m + 1];
      error_t += residual[m + n] * residual[m + n];
    }
    mean_t = ratio(mean_t, rho_total);
    error_p = ssqrt(error_p);
    error_t = ssqrt(error_t);
    const bool converged_p = (error_p < P->tol_p * sabs(mean_p) || error_p < P->abs_p);
    const bool converged_t = (error_t < P->tol_t * mean_t || error_t < P->abs_t);
    const bool acceptable_p =
        (error_p < P->tol_p_suff * sabs(mean_p) || error_p < P->abs_p_suff);
    const bool acceptable_t = (error_t < P->tol_t_suff * mean_t || error_t < P->abs_t_suff);
    conv = converged_p && converged_t;
    acceptable = acceptable_p && acceptable_t;
  }
  // Jacobian (:2052-2116)
  SGX_HD void jacobian() {
#pragma unroll
    for (int m = 0; m < n; m++) {
      const T dv = (vfrac[m] < T(0.5) ? T(1.0) : T(-1.0)) * vfrac[m] * P->derivative_eps;
      const T vf_pert = vfrac[m] + dv;
      const T rho_pert = ratio(rhobar[m], vf_pert);
      T t_pert = ratio(B::t_of(m, rho_pert, sie[m]), Tnorm);
      T p_pert = ratio(B::p_pref(m, rho_pert, Tnorm * t_pert, sie[m]), uscale);
      dpdv[m] = smin(ratio(p_pert - press[m], dv), -sabs(P->max_dpdv));
      dtdv[m] = ratio(t_pert - temp[m], dv);
      const T de = sabs(u[m]) * P->derivative_eps;
      const T e_pert = ratio(u[m] + de, rhobar[m]);
      t_pert = ratio(B::t_of(m, rho[m], uscale * e_pert), Tnorm);
      p_pert = ratio(B::p_pref(m, rho[m], Tnorm * t_pert, uscale * e_pert), uscale);
      dpde[m] = ratio(p_pert - press[m], de);
      dtde[m] = ratio(t_pert - temp[m], de);
      if (sabs(dtde[m]) < P->min_dtde) dtde[m] = P->derivative_eps;
    }
#pragma unroll
    for (int i = 0; i < neq * neq; ++i)
      jac[i] = T(0.0);
    constexpr int w = 2 * N; // row length
#pragma unroll
    for (int m = 0; m < n; ++m) {
      jset(m, T(1.0));
      jset(w + n + m, T(1.0));
    }
    jset(2 * w, dpdv[0]);
    jset(n * w + n - 1, -dpdv[n - 1]);
    jset((n + 1) * w, dtdv[0]);
    jset((2 * n - 1) * w + n - 1, -dtdv[n - 1]);
    jset(2 * w + n, dpde[0]);
    jset(n * w + 2 * n - 1, -dpde[n - 1]);
    jset((n + 1) * w + n, dtde[0]);
    jset((2 * n - 1) * w + 2 * n - 1, -dtde[n - 1]);
#pragma unroll
    for (int m = 1; m < n - 1; ++m) {
      jset((1 + m) * w + m, -dpdv[m]);
      jset((2 + m) * w + m, dpdv[m]);
      jset((n + m) * w + m, -dtdv[m]);
      jset((n + m + 1) * w + m, dtdv[m]);
      jset((1 + m) * w + n + m, -dpde[m]);
      jset((2 + m) * w + n + m, dpde[m]);
      jset((n + m) * w + n + m, -dtde[m]);
      jset((n + m + 1) * w + n + m, dtde[m]);
    }
  }
  // ScaleDx (:2118-2151)
  SGX_HD T scale_dx() {
    T scale = 1.0;
#pragma unroll
    for (int m = 0; m < n; ++m) {
      if (scale * dx[m] < T(-0.1) * vfrac[m]) scale = T(-0.1) * ratio(vfrac[m], dx[m]);
      const T dt = (dtdv[m] * dx[m] + dtde[m] * dx[m + n]);
      if (scale * dt < T(-0.1) * temp[m]) scale = T(-0.1) * ratio(temp[m], dt);
      const T tt = temp[m] + scale * dt;
      const T rho_min = T(smax(ev_rho_pmin(*this->eos[m], double(Tnorm * temp[m])),
                               ev_rho_pmin(*this->eos[m], double(Tnorm * tt))));
      const T alpha_max = ratio(rhobar[m], rho_min);
      if (alpha_max < vfrac[m]) continue;
      if (scale * dx[m] > T(0.5) * (alpha_max - vfrac[m]))
        scale = T(0.5) * ratio(alpha_max - vfrac[m], dx[m]);
    }
#pragma unroll
    for (int i = 0; i < neq; ++i)
      dx[i] *= scale;
    return scale;
  }
  // TestUpdate (:2155-2178)
  SGX_HD T test_update(const T scale, const bool cache_state = false) {
    if (cache_state) {
#pragma unroll
      for (int m = 0; m < n; ++m) {
        vtemp[m] = vfrac[m];
        utemp[m] = u[m];
      }
    }
#pragma unroll
    for (int m = 0; m < n; ++m) {
      vfrac[m] = vtemp[m] + scale * dx[m];
      rho[m] = ratio(rhobar[m], vfrac[m]);
      u[m] = utemp[m] + scale * dx[n + m];
      sie[m] = uscale * ratio(u[m], rhobar[m]);
      temp[m] = ratio(B::t_of(m, rho[m], sie[m]), Tnorm);
      press[m] = ratio(B::p_pref(m, rho[m], Tnorm * temp[m], sie[m]), uscale);
    }
    residual_eval();
    return B::residual_norm();
  }
};

// ===========================================================================
// PTESolver driver (:2188-2291)
// ===========================================================================
// The damped-Newton loop of PTESolver (:2202-2285) from an initialised state
// whose residual norm is `err`; fixup/finalize are left to the caller.
template <typename S, typename T> SGX_HD PteStatusLocal pte_iterate(S &s, T err) {
  PteStatusLocal st;
  const MixP<T> &params = *s.P;
  bool converged = false, close_enough = false;
  const int pte_max_iter = S::n * params.max_iter_per_mat;
  int niter;
  int max_line_niter = 0, small_step_iters = 0;
  for (niter = 0; niter < pte_max_iter; ++niter) {
    bool c, ce;
    s.check(c, ce);
    converged = c;
    close_enough = ce;
    if (converged) break;
    s.jacobian();
    if (!s.solve()) {
      converged = false;
      break;
    }
    T scale = smin(T(1.0), s.scale_dx());
    if (sabs(scale) < params.small_step_thresh) small_step_iters++;
    if (small_step_iters >= params.small_step_tries) {
      converged = false;
      break;
    }
    const T gradfdx = T(-2.0) * scale * err;
    scale = 1.0;
    const T err_old = err;
    err = s.test_update(scale, true);
    if (err > err_old + params.ls_alpha * gradfdx) {
      scale = 0.5;
      const T err_mid = s.test_update(scale);
      if (err_mid < err && err_mid < err_old)
        scale = T(0.75) + T(0.5) * ratio(err_mid - err, err - T(2.0) * err_mid + err_old);
      for (int line_iter = 0; line_iter < params.ls_max_iter; line_iter++) {
        err = s.test_update(scale);
        if (err < err_old + params.ls_alpha * scale * gradfdx) break;
        scale *= params.ls_fac;
        max_line_niter = max_line_niter > line_iter ? max_line_niter : line_iter;
      }
    }
    s.fixup();
    if (((err > params.slow_thresh * err_old) || niter == pte_max_iter - 1) && close_enough) {
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

// PTESolver (:2188-2291)
template <typename S, typename T> SGX_HD PteStatusLocal pte_solve(S &s) {
  const T err = s.init();
  PteStatusLocal st = pte_iterate<S, T>(s, err);
  s.fixup();
  s.finalize();
  return st;
}

// FP64 continuation of the mixed-precision path: rebuilds the FP64 state at
// the solver's current (Tequil, vfrac) -- every material's energy and
// pressure evaluated -- and runs the same damped Newton loop under the
// (tight) controls `tight`. Returns whether it converged; `taken` receives
// the Newton iterations used. The caller finalizes.
template <int N>
SGX_HDI bool pte_polish(PteRhoT<double, N> &s, const MixP<double> &tight, int &taken) {
#pragma unroll
  for (int q = 0; q < N; ++q)
    s.dx[q] = 0.0;
  const double err = s.test_update(0.0, true);
  const MixP<double> *keep = s.P;
  s.P = &tight;
  const PteStatusLocal st = pte_iterate<PteRhoT<double, N>, double>(s, err);
  s.P = keep;
  s.fixup();
  taken = st.niter;
  return st.converged && (st.residual == st.residual);
}

} // inline namespace
} // namespace sgx
