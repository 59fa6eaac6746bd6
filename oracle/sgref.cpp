// sgref: a C entry layer over the UNMODIFIED singularity-eos hot-path
// headers, compiled against this folder's shims (ports-of-call-lite,
// spiner-lite, hdf5-lite, Eigen-lite) into oracle/_ref/libsgref.so.
//
// TEST INFRASTRUCTURE ONLY: the oracle. Only tests/ (to make and check the
// golden fixtures) and bench.py's CPU baseline may load it; the product
// never does. It is built in the development container only, where the
// reference sources are present (oracle/build_ref.sh).
//
// Each entry point calls the reference's own API the way its callers do:
//   - PTE: PTESolverRhoT / PTESolverPT / PTESolverRhoU / PTESolverFixedT /
//     PTESolverFixedP + PTESolver(), as get_sg_eos_rho_e.cpp:30-88,
//     get_sg_eos_rho_t.cpp, get_sg_eos_rho_p.cpp and test_pte.cpp:200-245
//     drive them;
//   - vector lookups: the Variant vector overloads (eos_base.hpp:169-230,
//     eos_variant.hpp:56-143) with a 2-D lambda indexer shaped like
//     lambdaIndexer2D (singularity_eos.cpp:39-49);
//   - FillEos vector (eos_base.hpp:503-531).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include <singularity-eos/closure/mixed_cell_models.hpp>
#include <singularity-eos/eos/eos.hpp>
#include <singularity-eos/eos/singularity_eos_init_utils.hpp>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace singularity;

extern "C" {

// EOS description passed across the oracle's C boundary.
struct sgref_eos {
  int32_t type; // 1 IdealGas, 2 StiffGas, 3 NobleAbel, 4 Gruneisen,
                // 5 SpinerEOSDependsRhoT, 6 Helmholtz,
                // 7 SpinerEOSDependsRhoSie
  int32_t flags;
  int32_t matid;
  int32_t pad;
  double p[16];
  const char *path;
  // modifiers: bit 0 ShiftedEOS(shift), bit 1 ScaledEOS(scale), bit 2
  // BilinearRampEOS(ramp[0..3] = r0, a, b, c), nested ramp(scaled(shifted))
  int32_t mods;
  int32_t pad2;
  double shift, scale;
  double ramp[4];
};

// Field-for-field copy of singularity::MixParams (mixed_cell_models.hpp:43-78).
struct sgref_mix_params {
  int32_t verbose;
  int32_t iterate_t_guess;
  double derivative_eps;
  double pte_rel_tolerance_p, pte_rel_tolerance_t, pte_rel_tolerance_e;
  double pte_rel_tolerance_v, pte_abs_tolerance_p, pte_abs_tolerance_t;
  double pte_slow_convergence_thresh;
  double pte_rel_tolerance_p_sufficient, pte_rel_tolerance_t_sufficient;
  double pte_rel_tolerance_e_sufficient, pte_rel_tolerance_v_sufficient;
  double pte_abs_tolerance_p_sufficient, pte_abs_tolerance_t_sufficient;
  int64_t pte_max_iter_per_mat;
  double line_search_alpha;
  int64_t line_search_max_iter;
  double line_search_fac;
  double vfrac_safety_fac;
  double temperature_limit;
  double default_tguess;
  double min_dtde;
  int64_t pte_small_step_tries;
  double pte_small_step_thresh;
  double pte_max_dpdv;
  int64_t pte_reduced_system_exclude_idx;
};

} // extern "C"

namespace {

EOS make_model(const sgref_eos &d) {
  switch (d.type) {
  // flags bit 1: the constructor with a reference state (IdealGas entropy
  // reference in p[2..3]; StiffGas / NobleAbel qp, T0, P0 in p[4..6])
  case 1:
    if (d.flags & 2) return IdealGas(d.p[0], d.p[1], d.p[2], d.p[3]);
    return IdealGas(d.p[0], d.p[1]);
  case 2:
    if (d.flags & 2) return StiffGas(d.p[0], d.p[1], d.p[2], d.p[3], d.p[4], d.p[5], d.p[6]);
    return StiffGas(d.p[0], d.p[1], d.p[2], d.p[3]);
  case 3:
    if (d.flags & 2) return NobleAbel(d.p[0], d.p[1], d.p[2], d.p[3], d.p[4], d.p[5], d.p[6]);
    return NobleAbel(d.p[0], d.p[1], d.p[2], d.p[3]);
  case 4:
    return Gruneisen(d.p[0], d.p[1], d.p[2], d.p[3], d.p[4], d.p[5], d.p[6], d.p[7],
                     d.p[8], d.p[9]);
  case 5:
    return SpinerEOSDependsRhoT(std::string(d.path), d.matid, (d.flags & 1) != 0);
  case 6:
    return Helmholtz(std::string(d.path), (d.flags & 1) != 0, (d.flags & 2) != 0,
                     (d.flags & 4) != 0, (d.flags & 8) != 0, (d.flags & 16) != 0, false,
                     (d.flags & 32) == 0);
  case 7:
    return SpinerEOSDependsRhoSie(std::string(d.path), d.matid, (d.flags & 1) != 0);
  }
  PORTABLE_ALWAYS_THROW_OR_ABORT("sgref: unknown EOS type");
  return IdealGas(0.4, 1.0);
}

// The model wrapped by the Variant's own Modify (eos_variant.hpp:213-223).
EOS make_eos(const sgref_eos &d) {
  EOS eos = make_model(d);
  if (d.mods & 1) eos = eos.Modify<ShiftedEOS>(d.shift);
  if (d.mods & 2) eos = eos.Modify<ScaledEOS>(d.scale);
  if (d.mods & 4) eos = eos.Modify<BilinearRampEOS>(d.ramp[0], d.ramp[1], d.ramp[2], d.ramp[3]);
  return eos;
}

MixParams to_mix(const sgref_mix_params *q) {
  MixParams m;
  if (q == nullptr) return m;
  m.verbose = q->verbose != 0;
  m.iterate_t_guess = q->iterate_t_guess != 0;
  m.derivative_eps = q->derivative_eps;
  m.pte_rel_tolerance_p = q->pte_rel_tolerance_p;
  m.pte_rel_tolerance_t = q->pte_rel_tolerance_t;
  m.pte_rel_tolerance_e = q->pte_rel_tolerance_e;
  m.pte_rel_tolerance_v = q->pte_rel_tolerance_v;
  m.pte_abs_tolerance_p = q->pte_abs_tolerance_p;
  m.pte_abs_tolerance_t = q->pte_abs_tolerance_t;
  m.pte_slow_convergence_thresh = q->pte_slow_convergence_thresh;
  m.pte_rel_tolerance_p_sufficient = q->pte_rel_tolerance_p_sufficient;
  m.pte_rel_tolerance_t_sufficient = q->pte_rel_tolerance_t_sufficient;
  m.pte_rel_tolerance_e_sufficient = q->pte_rel_tolerance_e_sufficient;
  m.pte_rel_tolerance_v_sufficient = q->pte_rel_tolerance_v_sufficient;
  m.pte_abs_tolerance_p_sufficient = q->pte_abs_tolerance_p_sufficient;
  m.pte_abs_tolerance_t_sufficient = q->pte_abs_tolerance_t_sufficient;
  m.pte_max_iter_per_mat = static_cast<std::size_t>(q->pte_max_iter_per_mat);
  m.line_search_alpha = q->line_search_alpha;
  m.line_search_max_iter = static_cast<std::size_t>(q->line_search_max_iter);
  m.line_search_fac = q->line_search_fac;
  m.vfrac_safety_fac = q->vfrac_safety_fac;
  m.temperature_limit = q->temperature_limit;
  m.default_tguess = q->default_tguess;
  m.min_dtde = q->min_dtde;
  m.pte_small_step_tries = static_cast<std::size_t>(q->pte_small_step_tries);
  m.pte_small_step_thresh = q->pte_small_step_thresh;
  m.pte_max_dpdv = q->pte_max_dpdv;
  m.pte_reduced_system_exclude_idx = q->pte_reduced_system_exclude_idx;
  return m;
}

// Indexes the per-cell list of EOS objects (as EOSAccessor_ does in
// get_sg_eos_functors.hpp, via an index array).
struct CellEOS {
  const EOS *all;
  const int *idx;
  const EOS &operator[](const int m) const { return all[idx[m]]; }
};

// lambdaIndexer2D shape (singularity_eos.cpp:39-49).
struct Lambda2D {
  int n;
  double *data;
  double *operator[](int i) const { return data + static_cast<std::size_t>(n) * i; }
};

std::vector<EOS> make_all(const sgref_eos *descs, int neos) {
  std::vector<EOS> v;
  v.reserve(neos);
  for (int k = 0; k < neos; ++k)
    v.push_back(make_eos(descs[k]));
  return v;
}

// Builds a solver in zero-filled storage. PTESolverFixedP reads its
// uscale and utotal_scale members in GetTguess before it sets them
// (mixed_cell_models.hpp:522-535 via :1754); zeroed storage (with
// -fno-lifetime-dse, so the fill is kept) makes that read well defined.
template <class M> struct Zeroed {
  alignas(M) unsigned char buf[sizeof(M)];
  M *m = nullptr;
  template <class... A> explicit Zeroed(A &&...a) {
    std::memset(buf, 0, sizeof(buf));
    m = new (buf) M(std::forward<A>(a)...);
  }
  ~Zeroed() { m->~M(); }
};

// The solvers' constructors differ in their scalar arguments: RhoT, PT and
// RhoU take (sie_tot, ..., Tnorm, params), FixedT (T_true, ..., params) and
// FixedP (P, ..., params). `target` is that scalar.
template <template <class, class, class> class Solver> constexpr bool takes_tnorm() {
  return true;
}
template <> constexpr bool takes_tnorm<PTESolverFixedT>() { return false; }
template <> constexpr bool takes_tnorm<PTESolverFixedP>() { return false; }

template <template <class, class, class> class Solver>
void pte_run(int nmat_max, int ncell, const sgref_eos *descs, int neos,
             const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
             double *rho, double *vfrac, double *sie, double *temp, double *press,
             double *lambda, const sgref_mix_params *params, int32_t *converged,
             int32_t *niter, double *residual, int nthreads) {
  const MixParams mp = to_mix(params);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    // One copy of the EOS objects per thread (Spiner's root counters are
    // mutable members, eos_spiner_rho_temp.hpp:260).
    std::vector<EOS> eos = make_all(descs, neos);
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64)
#endif
    for (int i = 0; i < ncell; ++i) {
      int idx[16];
      double r[16], v[16], e[16], t[16], p[16];
      double cache[16 * MAX_NUM_LAMBDAS];
      int n = 0;
      for (int m = 0; m < nmat_max; ++m) {
        const std::size_t k = static_cast<std::size_t>(m) * ncell + i;
        const int ie = eos_idx ? eos_idx[k] : m;
        if (ie < 0) continue;
        idx[n] = ie;
        r[n] = rho[k];
        v[n] = vfrac[k];
        e[n] = sie[k];
        t[n] = temp[k];
        p[n] = press[k];
        for (std::size_t l = 0; l < MAX_NUM_LAMBDAS; ++l)
          cache[n * MAX_NUM_LAMBDAS + l] =
              lambda ? lambda[(static_cast<std::size_t>(m) * MAX_NUM_LAMBDAS + l) * ncell + i]
                     : 0.0;
        ++n;
      }
      CellEOS ceos{eos.data(), idx};
      std::vector<double> scratch(Solver<CellEOS, double *, mix_impl::CacheAccessor>::
                                      RequiredScratch(n) +
                                  8);
      mix_impl::CacheAccessor cacc(cache);
      double *pr = r, *pv = v, *pe = e, *pt = t, *pp = p;
      using M = Solver<CellEOS, double *, mix_impl::CacheAccessor>;
      double *ps = scratch.data();
      std::unique_ptr<Zeroed<M>> z;
      if constexpr (takes_tnorm<Solver>())
        z.reset(new Zeroed<M>(n, ceos, vfrac_tot[i], sie_tot[i], pr, pv, pe, pt, pp, cacc, ps,
                              0.0, mp));
      else
        z.reset(
            new Zeroed<M>(n, ceos, vfrac_tot[i], sie_tot[i], pr, pv, pe, pt, pp, cacc, ps, mp));
      M &method = *z->m;
      SolverStatus st = PTESolver(method);
      int q = 0;
      for (int m = 0; m < nmat_max; ++m) {
        const std::size_t k = static_cast<std::size_t>(m) * ncell + i;
        const int ie = eos_idx ? eos_idx[k] : m;
        if (ie < 0) continue;
        rho[k] = r[q];
        vfrac[k] = v[q];
        sie[k] = e[q];
        temp[k] = t[q];
        press[k] = p[q];
        if (lambda)
          for (std::size_t l = 0; l < MAX_NUM_LAMBDAS; ++l)
            lambda[(static_cast<std::size_t>(m) * MAX_NUM_LAMBDAS + l) * ncell + i] =
                cache[q * MAX_NUM_LAMBDAS + l];
        ++q;
      }
      converged[i] = st.converged ? 1 : 0;
      niter[i] = static_cast<int32_t>(method.Niter());
      residual[i] = st.residual;
    }
  }
}

} // namespace

extern "C" {

void sgref_mix_params_default(sgref_mix_params *q) {
  const MixParams m;
  q->verbose = m.verbose;
  q->iterate_t_guess = m.iterate_t_guess;
  q->derivative_eps = m.derivative_eps;
  q->pte_rel_tolerance_p = m.pte_rel_tolerance_p;
  q->pte_rel_tolerance_t = m.pte_rel_tolerance_t;
  q->pte_rel_tolerance_e = m.pte_rel_tolerance_e;
  q->pte_rel_tolerance_v = m.pte_rel_tolerance_v;
  q->pte_abs_tolerance_p = m.pte_abs_tolerance_p;
  q->pte_abs_tolerance_t = m.pte_abs_tolerance_t;
  q->pte_slow_convergence_thresh = m.pte_slow_convergence_thresh;
  q->pte_rel_tolerance_p_sufficient = m.pte_rel_tolerance_p_sufficient;
  q->pte_rel_tolerance_t_sufficient = m.pte_rel_tolerance_t_sufficient;
  q->pte_rel_tolerance_e_sufficient = m.pte_rel_tolerance_e_sufficient;
  q->pte_rel_tolerance_v_sufficient = m.pte_rel_tolerance_v_sufficient;
  q->pte_abs_tolerance_p_sufficient = m.pte_abs_tolerance_p_sufficient;
  q->pte_abs_tolerance_t_sufficient = m.pte_abs_tolerance_t_sufficient;
  q->pte_max_iter_per_mat = static_cast<int64_t>(m.pte_max_iter_per_mat);
  q->line_search_alpha = m.line_search_alpha;
  q->line_search_max_iter = static_cast<int64_t>(m.line_search_max_iter);
  q->line_search_fac = m.line_search_fac;
  q->vfrac_safety_fac = m.vfrac_safety_fac;
  q->temperature_limit = m.temperature_limit;
  q->default_tguess = m.default_tguess;
  q->min_dtde = m.min_dtde;
  q->pte_small_step_tries = static_cast<int64_t>(m.pte_small_step_tries);
  q->pte_small_step_thresh = m.pte_small_step_thresh;
  q->pte_max_dpdv = m.pte_max_dpdv;
  q->pte_reduced_system_exclude_idx = m.pte_reduced_system_exclude_idx;
}

// solver: 0 = PTESolverRhoT, 1 = PTESolverPT, 2 = PTESolverRhoU,
// 3 = PTESolverFixedT, 4 = PTESolverFixedP; sie_tot holds each cell's scalar
// constructor argument (sie_tot, or T_true for FixedT, P for FixedP).
// Arrays are [nmat_max][ncell] (cell index fastest, the LayoutLeft of
// get_sg_eos.hpp:30-31); eos_idx of -1 marks an absent material. lambda
// (nullable) is [nmat_max][3][ncell].
int sgref_pte(int solver, int nmat_max, int ncell, const sgref_eos *descs, int neos,
              const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
              double *rho, double *vfrac, double *sie, double *temp, double *press,
              double *lambda, const sgref_mix_params *params, int32_t *converged,
              int32_t *niter, double *residual, int nthreads) {
  try {
#define SGREF_PTE_RUN(S)                                                                   \
  pte_run<S>(nmat_max, ncell, descs, neos, eos_idx, vfrac_tot, sie_tot, rho, vfrac, sie,    \
             temp, press, lambda, params, converged, niter, residual, nthreads)
    switch (solver) {
    case 0: SGREF_PTE_RUN(PTESolverRhoT); break;
    case 1: SGREF_PTE_RUN(PTESolverPT); break;
    case 2: SGREF_PTE_RUN(PTESolverRhoU); break;
    case 3: SGREF_PTE_RUN(PTESolverFixedT); break;
    case 4: SGREF_PTE_RUN(PTESolverFixedP); break;
    default: return 1;
    }
#undef SGREF_PTE_RUN
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_pte: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// Vector lookup through the Variant's vector overloads.
// fn: 0 T(rho,e) 1 e(rho,T) 2 P(rho,T) 3 P(rho,e) 4 Cv(rho,T) 5 Cv(rho,e)
//     6 B(rho,T) 7 B(rho,e) 8 G(rho,T) 9 G(rho,e) 10 emin(rho)
//     11 S(rho,T) 12 S(rho,e) 13 e(rho,P)
// lambda (nullable) is row-per-element with lambda_stride doubles.
int sgref_eos_vec(const sgref_eos *desc, int fn, int n, const double *in1,
                  const double *in2, double *out, double *lambda, int lambda_stride) {
  try {
    EOS eos = make_eos(*desc);
    auto run = [&](auto &&lam) {
      switch (fn) {
      case 0:
        eos.TemperatureFromDensityInternalEnergy(in1, in2, out, n, lam);
        break;
      case 1:
        eos.InternalEnergyFromDensityTemperature(in1, in2, out, n, lam);
        break;
      case 2:
        eos.PressureFromDensityTemperature(in1, in2, out, n, lam);
        break;
      case 3:
        eos.PressureFromDensityInternalEnergy(in1, in2, out, n, lam);
        break;
      case 4:
        eos.SpecificHeatFromDensityTemperature(in1, in2, out, n, lam);
        break;
      case 5:
        eos.SpecificHeatFromDensityInternalEnergy(in1, in2, out, n, lam);
        break;
      case 6:
        eos.BulkModulusFromDensityTemperature(in1, in2, out, n, lam);
        break;
      case 7:
        eos.BulkModulusFromDensityInternalEnergy(in1, in2, out, n, lam);
        break;
      case 8:
        eos.GruneisenParamFromDensityTemperature(in1, in2, out, n, lam);
        break;
      case 9:
        eos.GruneisenParamFromDensityInternalEnergy(in1, in2, out, n, lam);
        break;
      case 10:
        eos.MinInternalEnergyFromDensity(in1, out, n, lam);
        break;
      case 11:
        eos.EntropyFromDensityTemperature(in1, in2, out, n, lam);
        break;
      case 12:
        eos.EntropyFromDensityInternalEnergy(in1, in2, out, n, lam);
        break;
      case 13:
        eos.InternalEnergyFromDensityPressure(in1, in2, out, n, lam);
        break;
      default:
        PORTABLE_ALWAYS_THROW_OR_ABORT("sgref_eos_vec: unknown function");
      }
    };
    if (lambda)
      run(Lambda2D{lambda_stride, lambda});
    else
      run(NullIndexer());
    eos.Finalize();
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_eos_vec: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// Vector FillEos (eos_base.hpp:503-531); output is a thermalqs bit set.
int sgref_fill_eos(const sgref_eos *desc, int n, double *rho, double *temp, double *sie,
                   double *press, double *cv, double *bmod, unsigned long output,
                   double *lambda, int lambda_stride) {
  try {
    EOS eos = make_eos(*desc);
    if (lambda)
      eos.FillEos(rho, temp, sie, press, cv, bmod, n, output,
                  Lambda2D{lambda_stride, lambda});
    else
      eos.FillEos(rho, temp, sie, press, cv, bmod, n, output, NullIndexer());
    eos.Finalize();
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_fill_eos: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// Scalar DensityEnergyFromPressureTemperature over an array (PT-space
// inversion used by PTESolverPT).
int sgref_rho_sie_from_pt(const sgref_eos *desc, int n, const double *P, const double *T,
                          double *rho, double *sie) {
  try {
    EOS eos = make_eos(*desc);
    for (int i = 0; i < n; ++i) {
      Real r = rho[i], e = sie[i];
      eos.DensityEnergyFromPressureTemperature(P[i], T[i], static_cast<Real *>(nullptr), r,
                                               e);
      rho[i] = r;
      sie[i] = e;
    }
    eos.Finalize();
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_rho_sie_from_pt: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// PTDerivativesFromPreferred through the Variant (eos_variant.hpp:386-398)
// at n states; out = [dedP_T | drdP_T | dedT_P | drdT_P], n each.
// lambda (nullable) is row-per-element with lambda_stride doubles. A null
// lambda leaves SpinerEOSDependsRhoT::lRhoFromPlT_ reading an uninitialised
// cache (eos_spiner_rho_temp.hpp:1147-1151), so fixtures pass rows of NaN.
int sgref_pt_derivs(const sgref_eos *desc, int n, const double *rho, const double *sie,
                    const double *P, const double *T, double *out, double *lambda,
                    int lambda_stride) {
  try {
    EOS eos = make_eos(*desc);
    for (int i = 0; i < n; ++i) {
      Real a, b, c, d;
      Real *lam = lambda ? lambda + static_cast<std::size_t>(lambda_stride) * i : nullptr;
      eos.PTDerivativesFromPreferred(rho[i], sie[i], P[i], T[i], lam, a, b, c, d);
      out[i] = a;
      out[n + i] = b;
      out[2 * n + i] = c;
      out[3 * n + i] = d;
    }
    eos.Finalize();
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_pt_derivs: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// pAlpha2BilinearRampParams (ramps_eos.hpp:43-77) of the EOS desc describes
// (its shift and scale; a ramp in desc is ignored). out = r0, a, b, c.
int sgref_p_alpha(const sgref_eos *desc, double alpha0, double Pe, double Pc, double *out) {
  try {
    sgref_eos d = *desc;
    d.mods &= 3;
    EOS eos = make_eos(d);
    Real r0, a, b, c;
    pAlpha2BilinearRampParams(eos, alpha0, Pe, Pc, r0, a, b, c);
    out[0] = r0;
    out[1] = a;
    out[2] = b;
    out[3] = c;
    eos.Finalize();
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_p_alpha: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// The modifier step of init_sg_IdealGas and its siblings
// (singularity_eos.cpp:67-79), with the reference's own SGAPPLYMODSIMPLE /
// SGAPPLYMOD macros (singularity_eos_init_utils.hpp), for the bare model of
// desc: vals[2..5] are rewritten by the p-alpha conversion when enabled[3]
// is 1, exactly as there.
int sgref_init_mods(const sgref_eos *desc, const int *enabled, double *vals) {
  auto run = [&](auto &&mk) {
    EOS eosi = SGAPPLYMODSIMPLE(mk());
    if (enabled[3] == 1) {
      singularity::pAlpha2BilinearRampParams(eosi, vals[2], vals[3], vals[4], vals[2],
                                             vals[3], vals[4], vals[5]);
    }
    EOS eos_ = SGAPPLYMOD(mk());
    eos_.Finalize();
    eosi.Finalize();
  };
  try {
    const sgref_eos &d = *desc;
    switch (d.type) {
    case 1:
      run([&] { return IdealGas(d.p[0], d.p[1]); });
      break;
    case 2:
      run([&] { return StiffGas(d.p[0], d.p[1], d.p[2], d.p[3]); });
      break;
    case 3:
      run([&] { return NobleAbel(d.p[0], d.p[1], d.p[2], d.p[3]); });
      break;
    case 4:
      run([&] {
        return Gruneisen(d.p[0], d.p[1], d.p[2], d.p[3], d.p[4], d.p[5], d.p[6], d.p[7],
                         d.p[8], d.p[9]);
      });
      break;
    case 5:
      run([&] {
        return SpinerEOSDependsRhoT(std::string(d.path), d.matid, (d.flags & 1) != 0);
      });
      break;
    default:
      return 1;
    }
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_init_mods: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// Bounds introspection used by the PTE solvers.
// what: 0 MinimumDensity 1 MinimumTemperature 2 MaximumDensity
//       3 MinimumPressure 4 MaximumPressureAtTemperature(x) 5 RhoPmin(x)
int sgref_eos_bounds(const sgref_eos *desc, int what, int n, const double *x, double *out) {
  try {
    EOS eos = make_eos(*desc);
    for (int i = 0; i < n; ++i) {
      switch (what) {
      case 0:
        out[i] = eos.MinimumDensity();
        break;
      case 1:
        out[i] = eos.MinimumTemperature();
        break;
      case 2:
        out[i] = eos.MaximumDensity();
        break;
      case 3:
        out[i] = eos.MinimumPressure();
        break;
      case 4:
        out[i] = eos.MaximumPressureAtTemperature(x[i]);
        break;
      case 5:
        out[i] = eos.RhoPmin(x[i]);
        break;
      }
    }
    eos.Finalize();
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_eos_bounds: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// Copies out every DataBox of a loaded SpinerEOSDependsRhoT through its
// public DumpDynamicMemory (eos_spiner_rho_temp.hpp:513-526): the boxes in
// DBLIST order (P_, sie_, bMod_, dPdRho_, dPdE_, dTdRho_, dTdE_, dEdRho_,
// dEdT_, mF_, PMax_, sielTMax_, dEdTMax_, gm1Max_, lTColdCrit_, PCold_,
// sieCold_, bModCold_, dPdRhoCold_, dPdECold_, dTdRhoCold_, dTdECold_,
// dEdTCold_, rho_at_pmin_), concatenated. scal receives rhoMin, rhoMax, TMin,
// TMax, MinimumPressure, lRhoOffset, lTOffset. Returns the double count.
long sgref_spiner_dump(const char *path, int matid, double *out, long cap, double *scal) {
  try {
    SpinerEOSDependsRhoT eos(std::string(path), matid);
    const long n = static_cast<long>(eos.DynamicMemorySizeInBytes() / sizeof(double));
    if (out && cap >= n) eos.DumpDynamicMemory(reinterpret_cast<char *>(out));
    if (scal) {
      scal[0] = eos.rhoMin();
      scal[1] = eos.rhoMax();
      scal[2] = eos.TMin();
      scal[3] = eos.TMax();
      scal[4] = eos.MinimumPressure();
      scal[5] = eos.lRhoOffset();
      scal[6] = eos.lTOffset();
    }
    eos.Finalize();
    return n;
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_spiner_dump: %s\n", ex.what());
    return -1;
  }
}

// The same for SpinerEOSDependsRhoSie (DBLIST at eos_spiner_rho_sie.hpp:
// 329-336: sie_, T_, rho_at_pmin_, the seven rho-T then the seven rho-sie
// tables, mF_, PlRhoMax_, dPdRhoMax_, PCold_, sieCold_, bModCold_,
// dPdRhoCold_). scal receives rhoMin, rhoMax, TMin, TMax, sieMin, sieMax,
// MinimumPressure, the three offsets, then ValuesAtReferenceState's eight
// values (rho, T, sie, P, cv, bmod, dpde, dvdt).
long sgref_spiner_sie_dump(const char *path, int matid, double *out, long cap, double *scal) {
  try {
    SpinerEOSDependsRhoSie eos(std::string(path), matid);
    const long n = static_cast<long>(eos.DynamicMemorySizeInBytes() / sizeof(double));
    if (out && cap >= n) eos.DumpDynamicMemory(reinterpret_cast<char *>(out));
    if (scal) {
      scal[0] = eos.rhoMin();
      scal[1] = eos.rhoMax();
      scal[2] = eos.TMin();
      scal[3] = eos.TMax();
      scal[4] = eos.sieMin();
      scal[5] = eos.sieMax();
      scal[6] = eos.MinimumPressure();
      scal[7] = eos.lRhoOffset();
      scal[8] = eos.lTOffset();
      scal[9] = eos.lEOffset();
      Real *lam = nullptr;
      eos.ValuesAtReferenceState(scal[10], scal[11], scal[12], scal[13], scal[14], scal[15],
                                 scal[16], scal[17], lam);
    }
    eos.Finalize();
    return n;
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_spiner_sie_dump: %s\n", ex.what());
    return -1;
  }
}

// The Helmholtz table as the reference holds it after loading
// (HelmElectrons::DumpDynamicMemory: node values, then the 21 fields in
// DBLIST order, eos_helmholtz.hpp:281-292).
long sgref_helm_dump(const char *path, double *out, long cap) {
  try {
    Helmholtz eos{std::string(path)};
    const long n = static_cast<long>(eos.DynamicMemorySizeInBytes() / sizeof(double));
    if (out && cap >= n) eos.DumpDynamicMemory(reinterpret_cast<char *>(out));
    eos.Finalize();
    return n;
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_helm_dump: %s\n", ex.what());
    return -1;
  }
}

// T(rho, sie) of the Helmholtz EOS as lTFromRhoSie_ (eos_helmholtz.hpp:867-960)
// intends it, without the final read of the lT cache over the root: the
// reference's own RootFinding1D::newton_raphson and regula_falsi over the
// reference's public e(rho, T) and cv(rho, T), from the analytic guess
// (lTAnalytic_, :728-731), for the default options. The lambda cache is
// absent here, so the reference's defect does not arise.
int sgref_helm_T_from_rho_sie(const char *path, int n, const double *rho, const double *sie,
                              const double *abar, const double *zbar, double *T) {
  try {
    const Helmholtz eos{std::string(path)};
    for (int i = 0; i < n; ++i) {
      const Real r = rho[i], e = sie[i];
      auto eval = [&](const Real t, Real &ee, Real &cv) {
        Real lam[3] = {abar[i], zbar[i], 0.0};
        ee = eos.InternalEnergyFromDensityTemperature(r, t, lam);
        cv = eos.SpecificHeatFromDensityTemperature(r, t, lam);
      };
      const Real abari = robust::ratio(1.0, abar[i]);
      const Real ni = abari * r * HelmIon::NA;
      const Real ne = zbar[i] * ni;
      Real lTguess = std::log10((2.0 / 3.0) * robust::ratio(e * r, ni + ne) * HelmIon::KBi);
      if (!((3.0 <= lTguess) && (lTguess <= 13.0))) lTguess = 8;
      const Real Tguess = math_utils::pow10(lTguess);
      const Real Ta = math_utils::pow10(3.0), Tb = math_utils::pow10(13.0);
      Real Tr = 0;
      auto status = RootFinding1D::newton_raphson(
          [&](Real t) {
            Real ee, cv;
            eval(t, ee, cv);
            return std::make_tuple(ee, cv);
          },
          e, Tguess, Ta, Tb, 1e-10, Tr, nullptr, false, false);
      if (status != RootFinding1D::Status::SUCCESS) {
        status = RootFinding1D::regula_falsi(
            [&](Real t) {
              Real ee, cv;
              eval(t, ee, cv);
              return ee;
            },
            e, Tguess, Ta, Tb, 1e-14, 1e-14, Tr, nullptr, false);
        if (status != RootFinding1D::Status::SUCCESS)
          Tr = math_utils::pow10(
              std::log10((2.0 / 3.0) * robust::ratio(e * r, ni + ne) * HelmIon::KBi));
      }
      Real lT = std::log10(Tr);
      if (lT < 3.0) lT = 3.0;
      if (lT > 13.0) lT = 13.0;
      T[i] = math_utils::pow10(lT);
    }
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_helm_T_from_rho_sie: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// get_sg_eos (get_sg_eos.cpp:35-280) in all its input modes. The reference
// compiles get_sg_eos only under Kokkos (get_sg_eos.cpp:75), so this
// restates its per-cell drivers around the reference's own solver, root
// finder and EOS calls, serially:
//   input_int 0, 1  (rho, sie)  get_sg_eos_rho_e.cpp:30-88, PTESolverRhoT
//   input_int -3    (rho, T)    get_sg_eos_rho_t.cpp:21-110, PTESolverFixedT
//   input_int -2    (rho, P)    get_sg_eos_rho_p.cpp:21-118, PTESolverFixedP
//   input_int -1    (P, T)      get_sg_eos_p_t.cpp:23-102, no solve
// with init_functor (get_sg_eos_functors.hpp:28-118) and final_functor
// (:185-300). The lambda cache sits inside the solver scratch at the
// reference's offsets. Arrays are host, LayoutLeft: per-material (i, m) at
// i + m * cell_dim.
int sgref_get_sg_eos(int nmat, int ncell, int cell_dim, int input_int, const int *eos_offsets,
                     const sgref_eos *descs, int neos, const int *offsets, double *press,
                     double *pmax, double *vol, double *spvol, double *sie, double *temp,
                     double *bmod, double *dpde, double *cv, double *frac_mass,
                     double *frac_vol, double *frac_ie, double *frac_bmod, double *frac_dpde,
                     double *frac_cv, double mass_frac_cutoff, int32_t *converged) {
  if (input_int < -3 || input_int > 1) return 1;
  try {
    std::vector<EOS> eos = make_all(descs, neos);
    constexpr double ev2k = 1.160451930280894026e4;
    auto FM = [&](int i, int m) -> double & { return frac_mass[i + m * cell_dim]; };
    std::vector<int> idxs(nmat), mats(nmat);
    std::vector<double> vfrac_pte(nmat), sie_pte(nmat), temp_pte(nmat), press_pte(nmat),
        rho_pte(nmat);
    // scratch per cell: the largest solver's need plus the lambda cache
    const std::size_t nscr =
        std::max({static_cast<std::size_t>(PTESolverRhoTRequiredScratch(nmat)),
                  static_cast<std::size_t>(PTESolverFixedTRequiredScratch(nmat)),
                  static_cast<std::size_t>(PTESolverFixedPRequiredScratch(nmat))}) +
        nmat * MAX_NUM_LAMBDAS + 8;
    for (int iloop = 0; iloop < ncell; ++iloop) {
      const int i = offsets[iloop] - 1;
      double mass_sum = 0.0, vfrac_sum = 0.0;
      int npte = 0;
      std::vector<double> scratch(nscr, 0.0);
      bool pte_converged = true;
      double t_mult = 0.0, s_mult = 0.0, p_mult = 0.0; // final_functor's
      if (input_int == -1) {
        // (P, T): every material at the cell's P and T (get_sg_eos_p_t.cpp:40-86)
        mix_impl::CacheAccessor cache(scratch.data());
        for (int m = 0; m < nmat; ++m) {
          mass_sum += FM(i, m);
          idxs[m] = eos_offsets[m] - 1;
          mats[m] = m;
          temp_pte[m] = temp[i] * ev2k;
          press_pte[m] = press[i];
        }
        for (int m = 0; m < nmat; ++m)
          FM(i, m) /= mass_sum;
        double vfrac_tot = 0.0, sie_tot = 0.0;
        for (int m = 0; m < nmat; ++m) {
          eos[idxs[m]].DensityEnergyFromPressureTemperature(press_pte[m], temp_pte[m], cache[m],
                                                            rho_pte[m], sie_pte[m]);
          vfrac_pte[m] = FM(i, m) / rho_pte[m] * mass_sum;
          vfrac_tot += vfrac_pte[m];
          sie_tot += sie_pte[m] * FM(i, m);
        }
        sie[i] = sie_tot;
        vol[i] = vfrac_tot;
        spvol[i] = vol[i] / mass_sum;
        for (int m = 0; m < nmat; ++m)
          vfrac_pte[m] /= vfrac_tot;
        npte = nmat;
        if (converged) converged[iloop] = 1;
        // final_functor below with t_mult = s_mult = p_mult = 0
      }
      {
        // init_functor (get_sg_eos_functors.hpp:60-118)
        double it = 0.0, is = 0.0, ip = 0.0;
        if (input_int >= 0) is = 1.0;      // (rho, sie): t 0, s 1, p 0
        else if (input_int == -3) it = 1.0; // (rho, T):   t 1, s 0, p 0
        else if (input_int == -2) ip = 1.0; // (rho, P):   t 0, s 0, p 1
        if (input_int != -1) {
          for (int m = 0; m < nmat; ++m) {
            mass_sum += FM(i, m);
            idxs[m] = eos_offsets[m] - 1;
            frac_vol[i + m * cell_dim] = FM(i, m);
            frac_ie[i + m * cell_dim] = sie[i] * FM(i, m) * is;
          }
          for (int m = 0; m < nmat; ++m)
            FM(i, m) /= mass_sum;
          for (int m = 0; m < nmat; ++m) {
            if (FM(i, m) > mass_frac_cutoff) {
              idxs[npte] = eos_offsets[m] - 1;
              mats[npte] = m;
              npte += 1;
            }
            vfrac_pte[m] = 0.0;
            sie_pte[m] = 0.0;
            temp_pte[m] = 0.0;
            press_pte[m] = 0.0;
          }
          for (int mp = 0; mp < npte; ++mp) {
            const int m = mats[mp];
            vfrac_pte[mp] = FM(i, m);
            vfrac_sum += vfrac_pte[mp];
            rho_pte[mp] = FM(i, m) / spvol[i] / vfrac_pte[mp];
            temp_pte[mp] = temp[i] * ev2k * it;
            press_pte[mp] = press[i] * ip;
            sie_pte[mp] = sie[i] * FM(i, m) * is;
          }
        }
      }
      {
        // the solve (or pure-cell lookups) of each mode
        int neq = 0;
        if (input_int >= 0) neq = npte + 1;       // get_sg_eos_rho_e.cpp:50
        else if (input_int == -3) neq = npte;     // get_sg_eos_rho_t.cpp:53
        else if (input_int == -2) neq = npte + 1; // get_sg_eos_rho_p.cpp:50
        mix_impl::CacheAccessor cache(input_int == -1
                                          ? scratch.data()
                                          : scratch.data() + neq * (neq + 4) + 2 * npte);
        CellEOS ceos{eos.data(), idxs.data()};
        double *pr = rho_pte.data(), *pv = vfrac_pte.data(), *ps = sie_pte.data(),
               *pt = temp_pte.data(), *pp = press_pte.data();
        if (input_int >= 0) {
          if (npte > 1) {
            PTESolverRhoT<CellEOS, double *, mix_impl::CacheAccessor> method(
                npte, ceos, vfrac_sum, sie[i], pr, pv, ps, pt, pp, cache, scratch.data());
            pte_converged = PTESolver(method).converged;
          } else {
            const EOS &e0 = eos[idxs[0]];
            temp_pte[0] =
                e0.TemperatureFromDensityInternalEnergy(rho_pte[0], sie_pte[0], cache[0]);
            press_pte[0] = e0.PressureFromDensityTemperature(rho_pte[0], temp_pte[0], cache[0]);
          }
          t_mult = 1.0, s_mult = 0.0, p_mult = 1.0;
        } else if (input_int == -3) {
          double sie_tot_true = 0.0;
          if (npte > 1) {
            Zeroed<PTESolverFixedT<CellEOS, double *, mix_impl::CacheAccessor>> z(
                npte, ceos, vfrac_sum, temp_pte[0], pr, pv, ps, pt, pp, cache, scratch.data());
            pte_converged = PTESolver(*z.m).converged;
            for (int mp = 0; mp < npte; ++mp)
              sie_tot_true += sie_pte[mp] * FM(i, mats[mp]);
          } else {
            const EOS &e0 = eos[idxs[0]];
            sie_pte[0] = e0.InternalEnergyFromDensityTemperature(rho_pte[0], temp_pte[0], cache[0]);
            sie_tot_true = sie_pte[0];
            press_pte[0] = e0.PressureFromDensityTemperature(rho_pte[0], temp_pte[0], cache[0]);
          }
          sie[i] = sie_tot_true;
          t_mult = 0.0, s_mult = 0.0, p_mult = 1.0;
        } else if (input_int == -2) {
          double sie_tot_true = 0.0;
          if (npte > 1) {
            Zeroed<PTESolverFixedP<CellEOS, double *, mix_impl::CacheAccessor>> z(
                npte, ceos, vfrac_sum, press_pte[0], pr, pv, ps, pt, pp, cache, scratch.data());
            pte_converged = PTESolver(*z.m).converged;
            for (int mp = 0; mp < npte; ++mp)
              sie_tot_true += sie_pte[mp] * FM(i, mats[mp]);
          } else {
            const EOS &e0 = eos[idxs[0]];
            auto p_from_t = [&](const Real &t_i) {
              return e0.PressureFromDensityTemperature(rho_pte[0], t_i, cache[0]);
            };
            Real r_rho{}, r_temp{}, r_sie{}, r_press{}, r_cv{}, r_bmod{}, r_dpde{}, r_dvdt{};
            e0.ValuesAtReferenceState(r_rho, r_temp, r_sie, r_press, r_cv, r_bmod, r_dpde,
                                      r_dvdt);
            // the reference leaves temp_i uninitialised when every root
            // finder gives up without writing it; 0 here
            Real temp_i = 0.0;
            RootFinding1D::findRoot(p_from_t, press[i], r_temp, 1.e-10 * r_temp,
                                    1.e10 * r_temp, 1.e-12, 1.e-12, temp_i);
            sie_pte[0] = e0.InternalEnergyFromDensityTemperature(rho_pte[0], temp_i, cache[0]);
            sie_tot_true = sie_pte[0];
            temp_pte[0] = temp_i;
          }
          sie[i] = sie_tot_true;
          t_mult = 1.0, s_mult = 0.0, p_mult = 0.0;
        }
        if (converged && input_int != -1) converged[iloop] = pte_converged ? 1 : 0;
        // final_functor (get_sg_eos_functors.hpp:185-300)
        const bool do_t = t_mult == 1.0, do_s = s_mult == 1.0, do_p = p_mult == 1.0;
        if (do_t) temp[i] = 0.0;
        if (do_p) press[i] = 0.0;
        if (do_s) sie[i] = 0.0;
        bmod[i] = 0.0;
        cv[i] = 0.0;
        dpde[i] = 0.0;
        for (int mp = 0; mp < npte; ++mp) {
          const int m = mats[mp];
          press[i] += press_pte[mp] * vfrac_pte[mp] * p_mult;
          temp[i] += temp_pte[mp] * vfrac_pte[mp] * t_mult;
          const double ie_m = sie_pte[mp] * FM(i, m) * mass_sum;
          sie[i] += ie_m * s_mult;
          frac_ie[i + m * cell_dim] = ie_m;
          frac_vol[i + m * cell_dim] = vfrac_pte[mp] * vol[i];
          const EOS &em = eos[idxs[mp]];
          const double bmod_m =
              em.BulkModulusFromDensityTemperature(rho_pte[mp], temp_pte[mp], cache[mp]);
          bmod[i] += bmod_m * vfrac_pte[mp];
          const double cv_m = ev2k * em.SpecificHeatFromDensityTemperature(
                                         rho_pte[mp], temp_pte[mp], cache[mp]);
          cv[i] += cv_m * FM(i, m);
          const double dpde_m =
              em.GruneisenParamFromDensityTemperature(rho_pte[mp], temp_pte[mp], cache[mp]);
          dpde[i] += dpde_m * vfrac_pte[mp];
          if (frac_bmod) frac_bmod[i + m * cell_dim] = bmod_m;
          if (frac_cv) frac_cv[i + m * cell_dim] = cv_m;
          if (frac_dpde) frac_dpde[i + m * cell_dim] = dpde_m;
        }
        if (do_t) temp[i] /= ev2k;
        if (do_s) sie[i] /= mass_sum;
        for (int m = 0; m < nmat; ++m)
          FM(i, m) *= mass_sum;
        pmax[i] = press[i] > pmax[i] ? press[i] : pmax[i];
      }
    }
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_get_sg_eos: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// The (rho, sie) entry kept under its own name.
int sgref_get_sg_eos_rho_e(int nmat, int ncell, int cell_dim, const int *eos_offsets,
                           const sgref_eos *descs, int neos, const int *offsets, double *press,
                           double *pmax, double *vol, double *spvol, double *sie, double *temp,
                           double *bmod, double *dpde, double *cv, double *frac_mass,
                           double *frac_vol, double *frac_ie, double *frac_bmod,
                           double *frac_dpde, double *frac_cv, double mass_frac_cutoff,
                           int32_t *converged) {
  return sgref_get_sg_eos(nmat, ncell, cell_dim, 1, eos_offsets, descs, neos, offsets, press,
                          pmax, vol, spvol, sie, temp, bmod, dpde, cv, frac_mass, frac_vol,
                          frac_ie, frac_bmod, frac_dpde, frac_cv, mass_frac_cutoff, converged);
}

// ApproxTemperatureFromRhoMatU (mixed_cell_models.hpp:790-847) per cell over
// [nmat_max][ncell] arrays (eos_idx -1 = absent; lambda nullable
// [nmat_max][3][ncell]; Tguess nullable).
int sgref_approx_temperature(int nmat_max, int ncell, const sgref_eos *descs, int neos,
                             const int32_t *eos_idx, const double *u_tot, const double *rho,
                             const double *vfrac, const double *Tguess, double *lambda,
                             double *temp_out) {
  try {
    std::vector<EOS> eos = make_all(descs, neos);
    for (int i = 0; i < ncell; ++i) {
      int idx[16], slot[16], n = 0;
      double r[16], v[16], cache[16 * MAX_NUM_LAMBDAS];
      for (int m = 0; m < nmat_max; ++m) {
        const std::size_t k = static_cast<std::size_t>(m) * ncell + i;
        const int ie = eos_idx ? eos_idx[k] : m;
        if (ie < 0) continue;
        idx[n] = ie;
        slot[n] = m;
        r[n] = rho[k];
        v[n] = vfrac[k];
        for (std::size_t l = 0; l < MAX_NUM_LAMBDAS; ++l)
          cache[n * MAX_NUM_LAMBDAS + l] =
              lambda ? lambda[(static_cast<std::size_t>(m) * MAX_NUM_LAMBDAS + l) * ncell + i]
                     : 0.0;
        ++n;
      }
      CellEOS ceos{eos.data(), idx};
      mix_impl::CacheAccessor cacc(cache);
      double *pr = r, *pv = v;
      temp_out[i] = ApproxTemperatureFromRhoMatU(n, ceos, u_tot[i], pr, pv,
                                                 Tguess ? Tguess[i] : 0.0, cacc);
      if (lambda)
        for (int q = 0; q < n; ++q)
          for (std::size_t l = 0; l < MAX_NUM_LAMBDAS; ++l)
            lambda[(static_cast<std::size_t>(slot[q]) * MAX_NUM_LAMBDAS + l) * ncell + i] =
                cache[q * MAX_NUM_LAMBDAS + l];
    }
  } catch (const std::exception &ex) {
    std::fprintf(stderr, "sgref_approx_temperature: %s\n", ex.what());
    return 1;
  }
  return 0;
}

// MixUtils::EnforceMassVolumesSum (which = 0; uses tot) and EnforceEnergiesSum
// (which = 1; uses tot_rho, tot) (mixed_cell_models.hpp:93-150) per cell
// over the present slots.
int sgref_enforce_sums(int which, int nmat_max, int ncell, const int32_t *eos_idx,
                       const double *tot, const double *tot_rho, double *rho, double *vfrac,
                       double *sie) {
  for (int i = 0; i < ncell; ++i) {
    int slot[16], n = 0;
    double r[16], v[16], e[16];
    for (int m = 0; m < nmat_max; ++m) {
      const std::size_t k = static_cast<std::size_t>(m) * ncell + i;
      if (eos_idx && eos_idx[k] < 0) continue;
      slot[n] = m;
      r[n] = rho[k];
      v[n] = vfrac[k];
      e[n] = sie ? sie[k] : 0.0;
      ++n;
    }
    if (n == 0) continue;
    double *pr = r, *pv = v, *pe = e;
    if (which == 0)
      MixUtils::EnforceMassVolumesSum(n, tot[i], pr, pv);
    else
      MixUtils::EnforceEnergiesSum(n, tot_rho[i], tot[i], pr, pv, pe);
    for (int q = 0; q < n; ++q) {
      const std::size_t k = static_cast<std::size_t>(slot[q]) * ncell + i;
      rho[k] = r[q];
      vfrac[k] = v[q];
      if (sie) sie[k] = e[q];
    }
  }
  return 0;
}

// FastMath NQT transforms (logs.hpp:188-214, 282-292), element-wise.
void sgref_nqt(int which, int n, const double *x, double *y) {
  for (int i = 0; i < n; ++i)
    y[i] = which == 0 ? FastMath::log10(x[i]) : FastMath::pow10(x[i]);
}

} // extern "C"
