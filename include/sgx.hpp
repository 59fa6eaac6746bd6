/*
 * sgx.hpp -- the C++ layer of the GB300 closure library, in the reference's
 * own terms, for C++ callers (the C ABI of sgx.h stays the boundary for C
 * and Fortran).
 *
 * Two parts, both header-only above libsgx.so:
 *
 *  1. Vector EOS calls on an EOS value with any indexers: the overloads that
 *     SG_EOS_VEC_2IN_1OUT generates and Variant forwards
 *     (singularity-eos/eos/eos_base.hpp:169-230, eos_variant.hpp:56-143,
 *     543-708), and FillEos (eos_base.hpp:503-531). An indexer is anything
 *     with operator[](int) that a kernel can use: a device pointer, or a
 *     small trivially copyable object holding device pointers (strided or
 *     gathered views). The lambda argument is either a per-element row
 *     (lambdas[i] is a Real*, indexed by number as the models number their
 *     cache) or a type-indexed row (lambdas[i] is a VariadicIndexer or
 *     another type with is_type_indexable), read and written through
 *     IndexerUtils::SafeGet / SafeSet (base/indexable_types.hpp:184-335).
 *     Raw double pointers without a lambda go straight to the library's
 *     precompiled kernel (sgx_eos_eval); any other indexer runs a kernel
 *     instantiated here over the same device model code.
 *
 *  2. The per-cell PTE solver objects for callers that write their own
 *     kernels: PTESolverRhoT, PTESolverPT, PTESolver(System&), MixParams,
 *     SolverStatus and the RequiredScratch functions
 *     (closure/mixed_cell_models.hpp:43-87, 873-935, 1198-1253, 2188-2291),
 *     usable on the device and, for the analytic models, on the host. The
 *     solver holds references to the caller's indexers, as the reference's
 *     does, and writes the equilibrium state back through them. Its state
 *     lives in registers; the scratch pointer is accepted for the
 *     reference's signature and not used, and RequiredScratch returns the
 *     reference's counts so that callers size their buffers unchanged.
 *
 * Device code needs nvcc and the library's device headers on the include
 * path (singularity-eos_gb300/csrc).
 */
#ifndef SGX_HPP_
#define SGX_HPP_

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <type_traits>
#include <utility>

#include "sgx.h"

#ifdef __CUDACC__
#include "sgx_pte.cuh"
#define SGX_API_HD __host__ __device__
#else
#define SGX_API_HD
#endif

namespace sgx {

using Real = double;

// ---------------------------------------------------------------------------
// Indexers (base/indexable_types.hpp)
// ---------------------------------------------------------------------------
namespace IndexableTypes {
struct LogDensity {};
struct LogTemperature {};
struct MeanAtomicMass {};
struct MeanAtomicNumber {};
struct MeanIonizationState {};
struct ElectronFraction {};
} // namespace IndexableTypes

namespace detail {
template <typename T, typename... Ts> struct index_of;
template <typename T, typename... Ts> struct index_of<T, T, Ts...> {
  static constexpr std::size_t value = 0;
};
template <typename T, typename U, typename... Ts> struct index_of<T, U, Ts...> {
  static constexpr std::size_t value = 1 + index_of<T, Ts...>::value;
};
template <typename T, typename... Ts> struct contains : std::false_type {};
template <typename T, typename... Ts>
struct contains<T, T, Ts...> : std::true_type {};
template <typename T, typename U, typename... Ts>
struct contains<T, U, Ts...> : contains<T, Ts...> {};

template <typename I, typename = void> struct type_indexable : std::false_type {};
template <typename I>
struct type_indexable<I, std::void_t<decltype(std::decay_t<I>::is_type_indexable)>>
    : std::bool_constant<std::decay_t<I>::is_type_indexable> {};
template <typename I, typename T, typename = void> struct has_type_index : std::false_type {};
template <typename I, typename T>
struct has_type_index<I, T, std::void_t<decltype(std::declval<I &>()[T{}])>> : std::true_type {};
} // namespace detail

namespace IndexerUtils {
// A fixed set of named slots, indexable by slot type or by number.
template <typename... Ts> class VariadicIndexer {
 public:
  static constexpr bool is_type_indexable = true;
  SGX_API_HD VariadicIndexer() : data_{} {}
  template <typename T, typename = std::enable_if_t<detail::contains<T, Ts...>::value>>
  SGX_API_HD Real &operator[](const T &) {
    return data_[detail::index_of<T, Ts...>::value];
  }
  template <typename T, typename = std::enable_if_t<detail::contains<T, Ts...>::value>>
  SGX_API_HD const Real &operator[](const T &) const {
    return data_[detail::index_of<T, Ts...>::value];
  }
  SGX_API_HD Real &operator[](const std::size_t i) { return data_[i]; }
  SGX_API_HD const Real &operator[](const std::size_t i) const { return data_[i]; }
  static constexpr std::size_t size() { return sizeof...(Ts); }

 private:
  Real data_[sizeof...(Ts)];
};

// SafeGet / SafeSet: by slot type when the indexer is type-indexable (false
// when it has no such slot), else by number at idx; false for a null row.
template <typename T, typename Indexer>
SGX_API_HD bool SafeGet(const Indexer &lam, const std::size_t idx, Real &out) {
  if constexpr (std::is_pointer_v<Indexer>) {
    if (lam == nullptr) return false;
    out = lam[idx];
    return true;
  } else if constexpr (detail::type_indexable<Indexer>::value) {
    if constexpr (detail::has_type_index<const Indexer, T>::value) {
      out = lam[T{}];
      return true;
    } else {
      return false;
    }
  } else {
    out = lam[idx];
    return true;
  }
}
template <typename T, typename Indexer>
SGX_API_HD bool SafeSet(Indexer &lam, const std::size_t idx, const Real in) {
  if constexpr (std::is_pointer_v<Indexer>) {
    if (lam == nullptr) return false;
    lam[idx] = in;
    return true;
  } else if constexpr (detail::type_indexable<Indexer>::value) {
    if constexpr (detail::has_type_index<Indexer, T>::value) {
      lam[T{}] = in;
      return true;
    } else {
      return false;
    }
  } else {
    lam[idx] = in;
    return true;
  }
}
template <typename T, typename Indexer>
SGX_API_HD Real SafeMustGet(const Indexer &lam, const std::size_t idx) {
  Real v = 0;
  SafeGet<T>(lam, idx, v);
  return v;
}
} // namespace IndexerUtils

// No lambda (eos_variant.hpp:47-52): every row is null.
struct NullIndexer {
  SGX_API_HD Real *operator[](const int) const { return nullptr; }
};

// ---------------------------------------------------------------------------
// EOS values
// ---------------------------------------------------------------------------

// The lambda slots each model numbers (its Lambda enum): the tabulated
// models cache log10 rho and log10 T (eos_spiner_rho_temp.hpp:79-81;
// SpinerEOSDependsRhoSie log10 rho only, eos_spiner_rho_sie.hpp:85-87).
namespace detail {
struct LambdaRow {
  Real v[3];
  template <typename Row> SGX_API_HD void load(const Row &row) {
    v[0] = v[1] = v[2] = 0.0;
    IndexerUtils::SafeGet<IndexableTypes::LogDensity>(row, 0, v[0]);
    IndexerUtils::SafeGet<IndexableTypes::LogTemperature>(row, 1, v[1]);
  }
  template <typename Row> SGX_API_HD void store(Row &row) const {
    IndexerUtils::SafeSet<IndexableTypes::LogDensity>(row, 0, v[0]);
    IndexerUtils::SafeSet<IndexableTypes::LogTemperature>(row, 1, v[1]);
  }
};
} // namespace detail

class EOS {
 public:
  sgx_eos e;
  EOS() : e{} {}
  explicit EOS(const sgx_eos &x) : e(x) {}
  SGX_API_HD operator const sgx_eos &() const { return e; }

  // Constructors of the reference's models (the C ABI's, sgx.h); a failure
  // throws std::runtime_error with sgx_last_error().
  static EOS IdealGas(Real gm1, Real Cv) {
    EOS x;
    check(sgx_eos_ideal_gas(&x.e, gm1, Cv));
    return x;
  }
  static EOS StiffGas(Real gm1, Real Cv, Real Pinf, Real qq) {
    EOS x;
    check(sgx_eos_stiff_gas(&x.e, gm1, Cv, Pinf, qq));
    return x;
  }
  static EOS NobleAbel(Real gm1, Real Cv, Real bb, Real qq) {
    EOS x;
    check(sgx_eos_noble_abel(&x.e, gm1, Cv, bb, qq));
    return x;
  }
  static EOS Gruneisen(Real C0, Real s1, Real s2, Real s3, Real G0, Real b, Real rho0, Real T0,
                       Real P0, Real Cv, Real rho_max = 0.0) {
    EOS x;
    check(sgx_eos_gruneisen(&x.e, C0, s1, s2, s3, G0, b, rho0, T0, P0, Cv, rho_max));
    return x;
  }
  static EOS SpinerEOSDependsRhoT(const char *path, int matid, bool reproducible = false) {
    EOS x;
    check(sgx_eos_spiner_rhot(&x.e, path, matid, reproducible ? 1 : 0));
    return x;
  }
  static EOS SpinerEOSDependsRhoSie(const char *path, int matid, bool reproducible = false) {
    EOS x;
    check(sgx_eos_spiner_rhosie(&x.e, path, matid, reproducible ? 1 : 0));
    return x;
  }
  // Frees a tabulated model's device table (Finalize, eos_variant.hpp:865-867).
  void Finalize() { sgx_eos_finalize(&e); }

#ifdef __CUDACC__
  // ---- scalar members, host or device (the analytic models on the host) ----
  SGX_API_HD Real TemperatureFromDensityInternalEnergy(Real rho, Real sie,
                                                       Real *lambda = nullptr) const {
    return ev_T_from_rho_sie<Real>(e, rho, sie, lambda);
  }
  SGX_API_HD Real InternalEnergyFromDensityTemperature(Real rho, Real T,
                                                       Real *lambda = nullptr) const {
    return ev_sie_from_rho_T<Real>(e, rho, T, lambda);
  }
  SGX_API_HD Real PressureFromDensityTemperature(Real rho, Real T, Real *lambda = nullptr) const {
    return ev_P_from_rho_T<Real>(e, rho, T, lambda);
  }
  SGX_API_HD Real PressureFromDensityInternalEnergy(Real rho, Real sie,
                                                    Real *lambda = nullptr) const {
    return ev_P_from_rho_sie<Real>(e, rho, sie, lambda);
  }
  SGX_API_HD Real SpecificHeatFromDensityTemperature(Real rho, Real T,
                                                     Real *lambda = nullptr) const {
    return ev_cv_from_rho_T<Real>(e, rho, T, lambda);
  }
  SGX_API_HD Real SpecificHeatFromDensityInternalEnergy(Real rho, Real sie,
                                                        Real *lambda = nullptr) const {
    return ev_cv_from_rho_sie<Real>(e, rho, sie, lambda);
  }
  SGX_API_HD Real BulkModulusFromDensityTemperature(Real rho, Real T,
                                                    Real *lambda = nullptr) const {
    return ev_B_from_rho_T<Real>(e, rho, T, lambda);
  }
  SGX_API_HD Real BulkModulusFromDensityInternalEnergy(Real rho, Real sie,
                                                       Real *lambda = nullptr) const {
    return ev_B_from_rho_sie<Real>(e, rho, sie, lambda);
  }
  SGX_API_HD Real GruneisenParamFromDensityTemperature(Real rho, Real T,
                                                       Real *lambda = nullptr) const {
    return ev_gamma_from_rho_T<Real>(e, rho, T, lambda);
  }
  SGX_API_HD Real GruneisenParamFromDensityInternalEnergy(Real rho, Real sie,
                                                          Real *lambda = nullptr) const {
    return ev_gamma_from_rho_sie<Real>(e, rho, sie, lambda);
  }
  SGX_API_HD Real MinInternalEnergyFromDensity(Real rho, Real * = nullptr) const {
    return ev_min_sie<Real>(e, rho);
  }
  SGX_API_HD void FillEos(Real &rho, Real &temp, Real &sie, Real &press, Real &cv, Real &bmod,
                          const unsigned long output, Real *lambda = nullptr) const {
    int err = 0;
    ev_fill(e, rho, temp, sie, press, cv, bmod, static_cast<unsigned>(output), lambda, &err);
  }

  // ---- vector members (eos_base.hpp:169-230, 503-531) ----
  // Each takes (in1, in2, out, [Real *scratch], num, [lambdas]) and runs on
  // the legacy default stream, or on `stream` with the trailing overload;
  // the scratch array is ignored, as the reference's base overloads ignore
  // it for these models.
#define SGX_VEC(NAME, FN)                                                                      \
  template <typename In1, typename In2, typename Out, typename Lam = NullIndexer>               \
  void NAME(In1 &&in1, In2 &&in2, Out &&out, const int num, Lam &&lambdas = Lam(),            \
            sgx_stream_t stream = nullptr) const {                                             \
    vec<FN>(in1, in2, out, num, lambdas, stream);                                              \
  }                                                                                            \
  template <typename In1, typename In2, typename Out, typename Lam = NullIndexer>               \
  void NAME(In1 &&in1, In2 &&in2, Out &&out, Real *, const int num, Lam &&lambdas = Lam(),    \
            sgx_stream_t stream = nullptr) const {                                             \
    vec<FN>(in1, in2, out, num, lambdas, stream);                                              \
  }
  SGX_VEC(TemperatureFromDensityInternalEnergy, SGX_FN_T_FROM_RHO_SIE)
  SGX_VEC(InternalEnergyFromDensityTemperature, SGX_FN_SIE_FROM_RHO_T)
  SGX_VEC(PressureFromDensityTemperature, SGX_FN_P_FROM_RHO_T)
  SGX_VEC(PressureFromDensityInternalEnergy, SGX_FN_P_FROM_RHO_SIE)
  SGX_VEC(SpecificHeatFromDensityTemperature, SGX_FN_CV_FROM_RHO_T)
  SGX_VEC(SpecificHeatFromDensityInternalEnergy, SGX_FN_CV_FROM_RHO_SIE)
  SGX_VEC(BulkModulusFromDensityTemperature, SGX_FN_B_FROM_RHO_T)
  SGX_VEC(BulkModulusFromDensityInternalEnergy, SGX_FN_B_FROM_RHO_SIE)
  SGX_VEC(GruneisenParamFromDensityTemperature, SGX_FN_G_FROM_RHO_T)
  SGX_VEC(GruneisenParamFromDensityInternalEnergy, SGX_FN_G_FROM_RHO_SIE)
#undef SGX_VEC

  // FillEos over arrays: output is the thermalqs bits to compute.
  template <typename RI, typename TI, typename SI, typename PI, typename CI, typename BI,
            typename Lam = NullIndexer>
  void FillEos(RI &&rhos, TI &&temps, SI &&sies, PI &&pressures, CI &&cvs, BI &&bmods,
               const int num, const unsigned long output, Lam &&lambdas = Lam(),
               sgx_stream_t stream = nullptr) const;
#endif // __CUDACC__

 private:
  static void check(int rc) {
    if (rc != SGX_OK) throw_error();
  }
  [[noreturn]] static void throw_error() { throw std::runtime_error(sgx_last_error()); }
#ifdef __CUDACC__
  template <int FN, typename In1, typename In2, typename Out, typename Lam>
  void vec(In1 &in1, In2 &in2, Out &out, int num, Lam &lambdas, sgx_stream_t stream) const;
#endif
};

// ---------------------------------------------------------------------------
// PTE (closure/mixed_cell_models.hpp)
// ---------------------------------------------------------------------------

// MixParams (:43-78) with the reference's defaults.
struct MixParams : sgx_mix_params {
  SGX_API_HD MixParams() {
    verbose = 0;
    iterate_t_guess = 1;
    derivative_eps = 3.0e-6;
    pte_rel_tolerance_p = 1.0e-6;
    pte_rel_tolerance_t = 1.0e-4;
    pte_rel_tolerance_e = 1.0e-6;
    pte_rel_tolerance_v = 1.0e-6;
    pte_abs_tolerance_p = 1.0e-6;
    pte_abs_tolerance_t = 1.0e-4;
    pte_slow_convergence_thresh = 0.99;
    pte_rel_tolerance_p_sufficient = 1.e2 * pte_rel_tolerance_p;
    pte_rel_tolerance_t_sufficient = 10 * pte_rel_tolerance_t;
    pte_rel_tolerance_e_sufficient = 1.e2 * pte_rel_tolerance_e;
    pte_rel_tolerance_v_sufficient = 1.e2 * pte_rel_tolerance_v;
    pte_abs_tolerance_p_sufficient = 1.e2 * pte_abs_tolerance_p;
    pte_abs_tolerance_t_sufficient = 10 * pte_abs_tolerance_t;
    pte_max_iter_per_mat = 128;
    line_search_alpha = 1.e-2;
    line_search_max_iter = 6;
    line_search_fac = 0.5;
    vfrac_safety_fac = 0.95;
    temperature_limit = 1.0e15;
    default_tguess = 300.;
    min_dtde = 1.0e-16;
    pte_small_step_tries = 2;
    pte_small_step_thresh = 1e-16;
    pte_max_dpdv = -1e-8;
    pte_reduced_system_exclude_idx = -1;
  }
};

// SolverStatus (:80-87).
struct SolverStatus {
  bool converged = false;
  bool slow_convergence_detected = false;
  std::size_t max_niter = 0;
  std::size_t max_line_niter = 0;
  std::size_t small_step_iters = 0;
  Real residual = 0;
};

// The reference's scratch counts (:873-881, :1198-1206).
constexpr inline int PTESolverRhoTRequiredScratch(const std::size_t nmat) {
  return static_cast<int>(nmat * nmat + 4 * nmat + 6 * nmat);
}
constexpr inline std::size_t PTESolverRhoTRequiredScratchInBytes(const std::size_t nmat) {
  return PTESolverRhoTRequiredScratch(nmat) * sizeof(Real);
}
constexpr inline int PTESolverPTRequiredScratch(const std::size_t nmat) {
  return static_cast<int>(2 * 2 + 4 * 2 + 2 * nmat);
}
constexpr inline std::size_t PTESolverPTRequiredScratchInBytes(const std::size_t nmat) {
  return PTESolverPTRequiredScratch(nmat) * sizeof(Real);
}

#ifdef __CUDACC__
namespace detail {
// One cell's solve through the register-resident solver of the library's
// kernels, for a count of materials fixed at compile time: the state is
// read from the caller's indexers, solved, and written back.
template <template <typename, int> class Solver, int N, typename EI, typename RI, typename LI>
SGX_API_HD SolverStatus pte_cell(const EI &eos, const Real vfrac_tot, const Real sie_tot,
                                 RI &rho, RI &vfrac, RI &sie, RI &temp, RI &press, LI &lambda,
                                 const Real Tnorm, const sgx_mix_params &params) {
  const MixP<double> mp(params);
  sgx_eos e[N];
  double cache[N][3];
  Solver<double, N> s;
  s.P = &mp;
  s.vfrac_total = vfrac_tot;
  s.configure(sie_tot);
  s.Tnorm = Tnorm;
  s.err_flags = 0;
  for (int m = 0; m < N; ++m) {
    e[m] = static_cast<const sgx_eos &>(eos[m]);
    s.eos[m] = &e[m];
    s.rho[m] = rho[m];
    s.vfrac[m] = vfrac[m];
    s.sie[m] = sie[m];
    s.temp[m] = temp[m];
    s.press[m] = press[m];
    Real *row = lambda[m];
    for (int l = 0; l < 3; ++l)
      cache[m][l] = row ? row[l] : 0.0;
    s.lam[m] = cache[m];
  }
  const PteStatusLocal st = pte_solve<Solver<double, N>, double>(s);
  for (int m = 0; m < N; ++m) {
    rho[m] = s.rho[m];
    vfrac[m] = s.vfrac[m];
    sie[m] = s.sie[m];
    temp[m] = s.temp[m];
    press[m] = s.press[m];
    Real *row = lambda[m];
    if (row)
      for (int l = 0; l < 3; ++l)
        row[l] = cache[m][l];
  }
  SolverStatus out;
  out.converged = st.converged;
  out.slow_convergence_detected = st.slow;
  out.max_niter = static_cast<std::size_t>(st.niter);
  out.max_line_niter = static_cast<std::size_t>(st.max_line_niter);
  out.small_step_iters = static_cast<std::size_t>(st.small_step_iters);
  out.residual = st.residual;
  return out;
}

// SGX_HPP_MAX_NMAT (1..6, default 6) bounds the material counts compiled
// into a caller's kernel; each count is its own register-resident solver.
#ifndef SGX_HPP_MAX_NMAT
#define SGX_HPP_MAX_NMAT 6
#endif
template <template <typename, int> class Solver, int N, typename EI, typename RI, typename LI>
SGX_API_HD SolverStatus pte_dispatch_n(const std::size_t nmat, const EI &eos, Real vt, Real st,
                                       RI &rho, RI &vfrac, RI &sie, RI &temp, RI &press,
                                       LI &lam, Real Tnorm, const sgx_mix_params &p) {
  if (nmat == N)
    return pte_cell<Solver, N>(eos, vt, st, rho, vfrac, sie, temp, press, lam, Tnorm, p);
  if constexpr (N < SGX_HPP_MAX_NMAT)
    return pte_dispatch_n<Solver, N + 1>(nmat, eos, vt, st, rho, vfrac, sie, temp, press, lam,
                                         Tnorm, p);
  return SolverStatus{}; // more materials than the register solver holds: not converged
}
template <template <typename, int> class Solver, typename EI, typename RI, typename LI>
SGX_API_HD SolverStatus pte_dispatch(const std::size_t nmat, const EI &eos, Real vt, Real st,
                                     RI &rho, RI &vfrac, RI &sie, RI &temp, RI &press, LI &lam,
                                     Real Tnorm, const sgx_mix_params &p) {
  return pte_dispatch_n<Solver, 1>(nmat, eos, vt, st, rho, vfrac, sie, temp, press, lam, Tnorm,
                                   p);
}
} // namespace detail

// PTESolverRhoT (:884-1193) / PTESolverPT (:1207-1446) for one cell: nmat
// (1..SGX_HPP_MAX_NMAT) materials, eos[m] an EOS (or sgx_eos), rho/vfrac/sie/temp/press
// indexed by material and updated in place by PTESolver, lambda[m] a Real*
// row of the material's cache (or NullIndexer).
template <typename EOSIndexer, typename RealIndexer, typename LambdaIndexer>
class PTESolverRhoT {
 public:
  template <typename EOS_t, typename Real_t, typename Lambda_t>
  SGX_API_HD PTESolverRhoT(const std::size_t nmat, EOS_t &&eos, const Real vfrac_tot,
                           const Real sie_tot, Real_t &&rho, Real_t &&vfrac, Real_t &&sie,
                           Real_t &&temp, Real_t &&press, Lambda_t &&lambda, Real * /*scratch*/,
                           const Real Tnorm = 0.0, const MixParams &params = MixParams())
      : nmat_(nmat), eos_(eos), vfrac_tot_(vfrac_tot), sie_tot_(sie_tot), rho_(rho),
        vfrac_(vfrac), sie_(sie), temp_(temp), press_(press), lambda_(lambda), Tnorm_(Tnorm),
        params_(params) {}
  static constexpr int RequiredScratch(const std::size_t nmat) {
    return PTESolverRhoTRequiredScratch(nmat);
  }
  static constexpr std::size_t RequiredScratchInBytes(const std::size_t nmat) {
    return PTESolverRhoTRequiredScratchInBytes(nmat);
  }
  SGX_API_HD const MixParams &GetParams() const { return params_; }
  SGX_API_HD SolverStatus Solve() {
    return detail::pte_dispatch<PteRhoT>(nmat_, eos_, vfrac_tot_, sie_tot_, rho_, vfrac_, sie_,
                                         temp_, press_, lambda_, Tnorm_, params_);
  }

 private:
  std::size_t nmat_;
  const EOSIndexer &eos_;
  Real vfrac_tot_, sie_tot_;
  RealIndexer &rho_, &vfrac_, &sie_, &temp_, &press_;
  LambdaIndexer &lambda_;
  Real Tnorm_;
  MixParams params_;
};

template <typename EOSIndexer, typename RealIndexer, typename LambdaIndexer>
class PTESolverPT {
 public:
  template <typename EOS_t, typename Real_t, typename Lambda_t>
  SGX_API_HD PTESolverPT(const std::size_t nmat, EOS_t &&eos, const Real vfrac_tot,
                         const Real sie_tot, Real_t &&rho, Real_t &&vfrac, Real_t &&sie,
                         Real_t &&temp, Real_t &&press, Lambda_t &&lambda, Real * /*scratch*/,
                         const Real Tnorm = 0.0, const MixParams &params = MixParams())
      : nmat_(nmat), eos_(eos), vfrac_tot_(vfrac_tot), sie_tot_(sie_tot), rho_(rho),
        vfrac_(vfrac), sie_(sie), temp_(temp), press_(press), lambda_(lambda), Tnorm_(Tnorm),
        params_(params) {}
  static constexpr int RequiredScratch(const std::size_t nmat) {
    return PTESolverPTRequiredScratch(nmat);
  }
  static constexpr std::size_t RequiredScratchInBytes(const std::size_t nmat) {
    return PTESolverPTRequiredScratchInBytes(nmat);
  }
  SGX_API_HD const MixParams &GetParams() const { return params_; }
  SGX_API_HD SolverStatus Solve() {
    return detail::pte_dispatch<PtePT>(nmat_, eos_, vfrac_tot_, sie_tot_, rho_, vfrac_, sie_,
                                       temp_, press_, lambda_, Tnorm_, params_);
  }

 private:
  std::size_t nmat_;
  const EOSIndexer &eos_;
  Real vfrac_tot_, sie_tot_;
  RealIndexer &rho_, &vfrac_, &sie_, &temp_, &press_;
  LambdaIndexer &lambda_;
  Real Tnorm_;
  MixParams params_;
};

// Class template argument deduction, as the reference's templated
// constructors provide it (with and without the optional Tnorm, params).
#define SGX_PTE_GUIDES(S)                                                                      \
  template <typename E, typename R, typename L>                                                \
  S(std::size_t, E &&, Real, Real, R &&, R &&, R &&, R &&, R &&, L &&, Real *)                 \
      ->S<std::remove_reference_t<E>, std::remove_reference_t<R>, std::remove_reference_t<L>>; \
  template <typename E, typename R, typename L>                                                \
  S(std::size_t, E &&, Real, Real, R &&, R &&, R &&, R &&, R &&, L &&, Real *, Real)           \
      ->S<std::remove_reference_t<E>, std::remove_reference_t<R>, std::remove_reference_t<L>>; \
  template <typename E, typename R, typename L>                                                \
  S(std::size_t, E &&, Real, Real, R &&, R &&, R &&, R &&, R &&, L &&, Real *, Real,           \
    const MixParams &)                                                                         \
      ->S<std::remove_reference_t<E>, std::remove_reference_t<R>, std::remove_reference_t<L>>;
SGX_PTE_GUIDES(PTESolverRhoT)
SGX_PTE_GUIDES(PTESolverPT)
#undef SGX_PTE_GUIDES

// PTESolver (:2188-2291): runs the damped Newton iteration of the system.
template <class System> SGX_API_HD SolverStatus PTESolver(System &s) { return s.Solve(); }

// ---------------------------------------------------------------------------
// Vector members: kernels over the caller's indexers
// ---------------------------------------------------------------------------
namespace detail {
template <int FN>
__device__ __forceinline__ Real eval_fn(const sgx_eos &e, Real a, Real b, Real *lam) {
  switch (FN) {
  case SGX_FN_T_FROM_RHO_SIE: return ev_T_from_rho_sie<Real>(e, a, b, lam);
  case SGX_FN_SIE_FROM_RHO_T: return ev_sie_from_rho_T<Real>(e, a, b, lam);
  case SGX_FN_P_FROM_RHO_T: return ev_P_from_rho_T<Real>(e, a, b, lam);
  case SGX_FN_P_FROM_RHO_SIE: return ev_P_from_rho_sie<Real>(e, a, b, lam);
  case SGX_FN_CV_FROM_RHO_T: return ev_cv_from_rho_T<Real>(e, a, b, lam);
  case SGX_FN_CV_FROM_RHO_SIE: return ev_cv_from_rho_sie<Real>(e, a, b, lam);
  case SGX_FN_B_FROM_RHO_T: return ev_B_from_rho_T<Real>(e, a, b, lam);
  case SGX_FN_B_FROM_RHO_SIE: return ev_B_from_rho_sie<Real>(e, a, b, lam);
  case SGX_FN_G_FROM_RHO_T: return ev_gamma_from_rho_T<Real>(e, a, b, lam);
  default: return ev_gamma_from_rho_sie<Real>(e, a, b, lam);
  }
}
template <typename Lam> __device__ __forceinline__ constexpr bool lam_is_null() {
  return std::is_same_v<std::decay_t<Lam>, NullIndexer>;
}
// lambdas[i] as the model's numbered row: a Real* row is passed as it is; a
// type-indexed row goes through a local copy in the model's slot order.
template <int FN, typename In1, typename In2, typename Out, typename Lam>
__global__ void vec_kernel(const sgx_eos e, In1 in1, In2 in2, Out out, const int num,
                           Lam lambdas) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) {
    if constexpr (lam_is_null<Lam>()) {
      out[i] = eval_fn<FN>(e, in1[i], in2[i], nullptr);
    } else if constexpr (std::is_pointer_v<std::decay_t<decltype(lambdas[i])>>) {
      out[i] = eval_fn<FN>(e, in1[i], in2[i], lambdas[i]);
    } else {
      auto &&row = lambdas[i];
      LambdaRow r;
      r.load(row);
      out[i] = eval_fn<FN>(e, in1[i], in2[i], r.v);
      r.store(row);
    }
  }
}
template <typename RI, typename TI, typename SI, typename PI, typename CI, typename BI,
          typename Lam>
__global__ void fill_kernel(const sgx_eos e, RI rhos, TI temps, SI sies, PI pressures, CI cvs,
                            BI bmods, const int num, const unsigned output, Lam lambdas) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) {
    Real rho = rhos[i], temp = temps[i], sie = sies[i], press = pressures[i], cv = cvs[i],
         bmod = bmods[i];
    int err = 0;
    if constexpr (lam_is_null<Lam>()) {
      ev_fill(e, rho, temp, sie, press, cv, bmod, output, nullptr, &err);
    } else if constexpr (std::is_pointer_v<std::decay_t<decltype(lambdas[i])>>) {
      ev_fill(e, rho, temp, sie, press, cv, bmod, output, lambdas[i], &err);
    } else {
      auto &&row = lambdas[i];
      LambdaRow r;
      r.load(row);
      ev_fill(e, rho, temp, sie, press, cv, bmod, output, r.v, &err);
      r.store(row);
    }
    rhos[i] = rho;
    temps[i] = temp;
    sies[i] = sie;
    pressures[i] = press;
    cvs[i] = cv;
    bmods[i] = bmod;
  }
}
constexpr int VEC_BLOCK = 256;
inline int vec_grid(const int num) {
  const int g = (num + VEC_BLOCK - 1) / VEC_BLOCK;
  return g < 152 * 16 ? (g > 0 ? g : 1) : 152 * 16;
}
template <typename X> constexpr bool is_real_ptr() {
  using D = std::decay_t<X>;
  return std::is_same_v<D, Real *> || std::is_same_v<D, const Real *>;
}
} // namespace detail

template <int FN, typename In1, typename In2, typename Out, typename Lam>
void EOS::vec(In1 &in1, In2 &in2, Out &out, const int num, Lam &lambdas,
              sgx_stream_t stream) const {
  if (num <= 0) return;
  using L = std::decay_t<Lam>;
  if constexpr (detail::is_real_ptr<In1>() && detail::is_real_ptr<In2>() &&
                detail::is_real_ptr<Out>() && std::is_same_v<L, NullIndexer>) {
    // plain arrays without a cache: the library's precompiled kernel
    check(sgx_eos_eval(&e, FN, num, in1, in2, out, nullptr, 0, stream));
  } else {
    detail::vec_kernel<FN><<<detail::vec_grid(num), detail::VEC_BLOCK, 0,
                             reinterpret_cast<cudaStream_t>(stream)>>>(
        e, std::decay_t<In1>(in1), std::decay_t<In2>(in2), std::decay_t<Out>(out), num, L(lambdas));
    if (cudaGetLastError() != cudaSuccess) throw_error();
  }
}

template <typename RI, typename TI, typename SI, typename PI, typename CI, typename BI,
          typename Lam>
void EOS::FillEos(RI &&rhos, TI &&temps, SI &&sies, PI &&pressures, CI &&cvs, BI &&bmods,
                  const int num, const unsigned long output, Lam &&lambdas,
                  sgx_stream_t stream) const {
  if (num <= 0) return;
  using L = std::decay_t<Lam>;
  detail::fill_kernel<<<detail::vec_grid(num), detail::VEC_BLOCK, 0,
                        reinterpret_cast<cudaStream_t>(stream)>>>(
      e, std::decay_t<RI>(rhos), std::decay_t<TI>(temps), std::decay_t<SI>(sies),
      std::decay_t<PI>(pressures), std::decay_t<CI>(cvs), std::decay_t<BI>(bmods), num,
      static_cast<unsigned>(output), L(lambdas));
  if (cudaGetLastError() != cudaSuccess) throw_error();
}
#endif // __CUDACC__

} // namespace sgx

#endif // SGX_HPP_
