// The C ABI (include/sgx.h): argument checks, error reporting, EOS
// construction, table residency, and the launches of the kernels in
// sgx_fp64.cu / sgx_mixed.cu.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sgx_eos.cuh"
#include "sgx_internal.h"
#include "sgx_table.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char *what) {
  return fail(SGX_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool valid_type(int t) { return t >= SGX_IDEAL_GAS && t <= SGX_SPINER_RHOSIE; }
// Models the PTE kernels dispatch on (Helmholtz is a lookup-only model here).
bool pte_type(int t) { return sgx::pte_model(t); }
// Entries a lambda row must hold: SpinerEOSDependsRhoSie caches log10(rho)
// only (nlambda() == 1); the other tabulated models read and write two
// (Helmholtz checks its three itself).
int min_lambda_stride(int t) { return t == SGX_SPINER_RHOSIE ? 1 : 2; }
// Modifier bits must be known ones; Helmholtz carries none; the
// mixed-precision paths take bare models only.
int check_mods(const sgx_eos &e, const bool mixed, const char *who) {
  if (e.mods & ~static_cast<uint32_t>(SGX_MOD_SHIFTED | SGX_MOD_SCALED | SGX_MOD_RAMP))
    return fail(SGX_ERR_INVALID, std::string(who) + ": unknown modifier bits");
  if (e.mods && e.type == SGX_HELMHOLTZ)
    return fail(SGX_ERR_UNSUPPORTED, std::string(who) + ": Helmholtz takes no modifiers");
  if (e.mods && mixed)
    return fail(SGX_ERR_UNSUPPORTED,
                std::string(who) + ": the mixed-precision path takes unmodified EOS only");
  return SGX_OK;
}

} // namespace

namespace sgx {
int set_error(int code, const std::string &msg) { return fail(code, msg); }
int check_eos_mods(const sgx_eos &e, const bool mixed, const char *who) {
  return check_mods(e, mixed, who);
}
} // namespace sgx

extern "C" {

const char *sgx_version(void) { return "sgx 0.1 (sm_103a)"; }
const char *sgx_last_error(void) { return g_last_error.c_str(); }

int sgx_mix_params_default(sgx_mix_params *p) {
  if (!p) return fail(SGX_ERR_INVALID, "sgx_mix_params_default: null");
  // MixParams defaults (closure/mixed_cell_models.hpp:43-78)
  std::memset(p, 0, sizeof(*p));
  p->verbose = 0;
  p->iterate_t_guess = 1;
  p->derivative_eps = 3.0e-6;
  p->pte_rel_tolerance_p = 1.0e-6;
  p->pte_rel_tolerance_t = 1.0e-4;
  p->pte_rel_tolerance_e = 1.0e-6;
  p->pte_rel_tolerance_v = 1.0e-6;
  p->pte_abs_tolerance_p = 1.0e-6;
  p->pte_abs_tolerance_t = 1.0e-4;
  p->pte_slow_convergence_thresh = 0.99;
  p->pte_rel_tolerance_p_sufficient = 1.e2 * p->pte_rel_tolerance_p;
  p->pte_rel_tolerance_t_sufficient = 10 * p->pte_rel_tolerance_t;
  p->pte_rel_tolerance_e_sufficient = 1.e2 * p->pte_rel_tolerance_e;
  p->pte_rel_tolerance_v_sufficient = 1.e2 * p->pte_rel_tolerance_v;
  p->pte_abs_tolerance_p_sufficient = 1.e2 * p->pte_abs_tolerance_p;
  p->pte_abs_tolerance_t_sufficient = 10 * p->pte_abs_tolerance_t;
  p->pte_max_iter_per_mat = 128;
  p->line_search_alpha = 1.e-2;
  p->line_search_max_iter = 6;
  p->line_search_fac = 0.5;
  p->vfrac_safety_fac = 0.95;
  p->temperature_limit = 1.0e15;
  p->default_tguess = 300.;
  p->min_dtde = 1.0e-16;
  p->pte_small_step_tries = 2;
  p->pte_small_step_thresh = 1e-16;
  p->pte_max_dpdv = -1e-8;
  p->pte_reduced_system_exclude_idx = -1;
  return SGX_OK;
}

// PTESolverRhoTRequiredScratch / PTESolverPTRequiredScratch
// (mixed_cell_models.hpp:873-881, 1198-1206). The GPU solver keeps this
// state in registers; the numbers are reported for API compatibility.
int sgx_pte_rhot_required_scratch(int nmat) { return nmat * nmat + 4 * nmat + 6 * nmat; }
int sgx_pte_pt_required_scratch(int nmat) { return 2 * 2 + 4 * 2 + 2 * nmat; }
int sgx_pte_fixed_t_required_scratch(int nmat) {
  return nmat * nmat + 4 * nmat + 2 * nmat + 2 * nmat;
}
int sgx_pte_fixed_p_required_scratch(int nmat) {
  return (nmat + 1) * (nmat + 1) + 4 * (nmat + 1) + 2 * nmat + 3 * nmat;
}
int sgx_pte_rhou_required_scratch(int nmat) {
  return 4 * nmat * nmat + 4 * 2 * nmat + 8 * nmat;
}

size_t sgx_pte_required_scratch_bytes(int solver, int nmat) {
  int n = 0;
  switch (solver) {
  case SGX_PTE_RHOT: n = sgx_pte_rhot_required_scratch(nmat); break;
  case SGX_PTE_PT: n = sgx_pte_pt_required_scratch(nmat); break;
  case SGX_PTE_RHOU: n = sgx_pte_rhou_required_scratch(nmat); break;
  case SGX_PTE_FIXED_T: n = sgx_pte_fixed_t_required_scratch(nmat); break;
  case SGX_PTE_FIXED_P: n = sgx_pte_fixed_p_required_scratch(nmat); break;
  default: return 0;
  }
  return static_cast<size_t>(n) * sizeof(double);
}

int sgx_eos_ideal_gas_entropy(sgx_eos *out, double gm1, double Cv, double EntropyT0,
                              double EntropyRho0) {
  if (!out) return fail(SGX_ERR_INVALID, "sgx_eos_ideal_gas: null");
  // IdealGas::CheckParams (eos_ideal.hpp:65-76)
  if (!(Cv >= 0) || !(gm1 >= 0)) return fail(SGX_ERR_INVALID, "IdealGas: Cv and gm1 must be >= 0");
  if (!(EntropyT0 >= 0))
    return fail(SGX_ERR_INVALID, "Entropy reference temperature must be positive");
  if (!(EntropyRho0 >= 0))
    return fail(SGX_ERR_INVALID, "Entropy reference density must be positive");
  std::memset(out, 0, sizeof(*out));
  out->type = SGX_IDEAL_GAS;
  out->p[0] = gm1;
  out->p[1] = Cv;
  out->p[sgx::pi::ST0] = EntropyT0;
  out->p[sgx::pi::SRho0] = EntropyRho0;
  return SGX_OK;
}

int sgx_eos_ideal_gas(sgx_eos *out, double gm1, double Cv) {
  // IdealGas(gm1, Cv) (eos_ideal.hpp:41-47): the entropy reference is the
  // STP state, T0 and rho0 = P0 / (gm1 Cv T0)
  const double T0 = sgx::ROOM_TEMPERATURE, P0 = sgx::ATMOSPHERIC_PRESSURE;
  return sgx_eos_ideal_gas_entropy(out, gm1, Cv, T0, P0 / (gm1 * Cv * T0));
}

int sgx_eos_stiff_gas_ref(sgx_eos *out, double gm1, double Cv, double Pinf, double qq,
                          double qp, double T0, double P0) {
  if (!out) return fail(SGX_ERR_INVALID, "sgx_eos_stiff_gas: null");
  if (!(Cv >= 0) || !(gm1 >= 0)) return fail(SGX_ERR_INVALID, "StiffGas: Cv and gm1 must be >= 0");
  std::memset(out, 0, sizeof(*out));
  out->type = SGX_STIFF_GAS;
  out->p[0] = gm1;
  out->p[1] = Cv;
  out->p[2] = Pinf;
  out->p[3] = qq;
  out->p[sgx::pi::qp] = qp;
  out->p[sgx::pi::rT0] = T0;
  out->p[sgx::pi::rP0] = P0;
  return SGX_OK;
}

int sgx_eos_stiff_gas(sgx_eos *out, double gm1, double Cv, double Pinf, double qq) {
  // StiffGas(gm1, Cv, Pinf, qq) (eos_stiff.hpp:40-50): qp 0, STP
  return sgx_eos_stiff_gas_ref(out, gm1, Cv, Pinf, qq, 0.0, sgx::ROOM_TEMPERATURE,
                               sgx::ATMOSPHERIC_PRESSURE);
}

int sgx_eos_noble_abel_ref(sgx_eos *out, double gm1, double Cv, double bb, double qq,
                           double qp, double T0, double P0) {
  if (!out) return fail(SGX_ERR_INVALID, "sgx_eos_noble_abel: null");
  if (!(Cv > 0) || !(gm1 >= 0) || !(bb >= 0))
    return fail(SGX_ERR_INVALID, "NobleAbel: Cv > 0, gm1 >= 0 and b >= 0 required");
  std::memset(out, 0, sizeof(*out));
  out->type = SGX_NOBLE_ABEL;
  out->p[0] = gm1;
  out->p[1] = Cv;
  out->p[2] = bb;
  out->p[3] = qq;
  out->p[sgx::pi::qp] = qp;
  out->p[sgx::pi::rT0] = T0;
  out->p[sgx::pi::rP0] = P0;
  return SGX_OK;
}

int sgx_eos_noble_abel(sgx_eos *out, double gm1, double Cv, double bb, double qq) {
  // NobleAbel(gm1, Cv, bb, qq) (eos_noble_abel.hpp:40-50): qp 0, STP
  return sgx_eos_noble_abel_ref(out, gm1, Cv, bb, qq, 0.0, sgx::ROOM_TEMPERATURE,
                                sgx::ATMOSPHERIC_PRESSURE);
}

int sgx_eos_gruneisen(sgx_eos *out, double C0, double s1, double s2, double s3, double G0,
                      double b, double rho0, double T0, double P0, double Cv, double rho_max) {
  if (!out) return fail(SGX_ERR_INVALID, "sgx_eos_gruneisen: null");
  if (!(rho_max > 0)) {
    int err = 0;
    rho_max = 0.99 * sgx::gruneisen_compute_rho_max(s1, s2, s3, rho0, &err);
    if (err) return fail(SGX_ERR_INVALID, "Gruneisen: cubic root find for rho_max failed");
  }
  std::memset(out, 0, sizeof(*out));
  out->type = SGX_GRUNEISEN;
  const double v[11] = {C0, s1, s2, s3, G0, b, rho0, T0, P0, Cv, rho_max};
  for (int k = 0; k < 11; ++k)
    out->p[k] = v[k];
  return SGX_OK;
}

int sgx_eos_spiner_rhot(sgx_eos *out, const char *path, int matid, int reproducible) {
  if (!out || !path) return fail(SGX_ERR_INVALID, "sgx_eos_spiner_rhot: null");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    return fail(SGX_ERR_NO_DEVICE, "sgx_eos_spiner_rhot: no CUDA device");
  std::string msg;
  uint64_t handle = 0;
  const int rc = sgx::table_load_spiner(path, matid, reproducible != 0, &handle, msg);
  if (rc != SGX_OK) return fail(rc, msg);
  std::memset(out, 0, sizeof(*out));
  out->type = SGX_SPINER_RHOT;
  out->flags = reproducible ? 1 : 0;
  out->table = handle;
  return SGX_OK;
}

int sgx_eos_spiner_rhosie(sgx_eos *out, const char *path, int matid, int reproducible) {
  if (!out || !path) return fail(SGX_ERR_INVALID, "sgx_eos_spiner_rhosie: null");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    return fail(SGX_ERR_NO_DEVICE, "sgx_eos_spiner_rhosie: no CUDA device");
  std::string msg;
  uint64_t handle = 0;
  const int rc = sgx::table_load_spiner_sie(path, matid, reproducible != 0, &handle, msg);
  if (rc != SGX_OK) return fail(rc, msg);
  std::memset(out, 0, sizeof(*out));
  out->type = SGX_SPINER_RHOSIE;
  out->flags = reproducible ? 1 : 0;
  out->table = handle;
  return SGX_OK;
}

int sgx_eos_helmholtz(sgx_eos *out, const char *path, int options) {
  if (!out || !path) return fail(SGX_ERR_INVALID, "sgx_eos_helmholtz: null");
  if (options & ~127) return fail(SGX_ERR_INVALID, "sgx_eos_helmholtz: unknown option bits");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    return fail(SGX_ERR_NO_DEVICE, "sgx_eos_helmholtz: no CUDA device");
  std::string msg;
  uint64_t handle = 0;
  const int rc = sgx::table_load_helm(path, &handle, msg);
  if (rc != SGX_OK) return fail(rc, msg);
  std::memset(out, 0, sizeof(*out));
  out->type = SGX_HELMHOLTZ;
  out->flags = options;
  out->table = handle;
  return SGX_OK;
}

long sgx_eos_helmholtz_dump(const sgx_eos *eos, double *out, long cap) {
  if (!eos || eos->type != SGX_HELMHOLTZ || !eos->table) {
    fail(SGX_ERR_INVALID, "sgx_eos_helmholtz_dump: not a Helmholtz EOS");
    return -1;
  }
  return sgx::table_dump(eos->table, out, cap);
}

int sgx_eos_finalize(sgx_eos *eos) {
  if (!eos) return fail(SGX_ERR_INVALID, "sgx_eos_finalize: null");
  if (eos->table) {
    std::string msg;
    const int rc = sgx::table_free(eos->table, msg);
    eos->table = 0;
    if (rc != SGX_OK) return fail(rc, msg);
  }
  return SGX_OK;
}

size_t sgx_eos_table_bytes(const sgx_eos *eos) {
  return (eos && eos->table) ? sgx::table_bytes(eos->table) : 0;
}

int sgx_eos_bounds(const sgx_eos *eos, int what, int64_t n, const double *temp, double *out,
                   sgx_stream_t stream) {
  if (!eos || !valid_type(eos->type)) return fail(SGX_ERR_INVALID, "sgx_eos_bounds: bad eos");
  if (eos->type == SGX_HELMHOLTZ)
    return fail(SGX_ERR_UNSUPPORTED, "sgx_eos_bounds: not available for Helmholtz");
  if (what < SGX_BOUND_MIN_DENSITY || what > SGX_BOUND_RHO_PMIN)
    return fail(SGX_ERR_INVALID, "sgx_eos_bounds: bad bound");
  if (n < 0) return fail(SGX_ERR_INVALID, "sgx_eos_bounds: n < 0");
  if (n == 0) return SGX_OK;
  if (!out || (!temp && what >= SGX_BOUND_MAX_PRESSURE_AT_T))
    return fail(SGX_ERR_INVALID, "sgx_eos_bounds: null array");
  if (const int rc = check_mods(*eos, false, "sgx_eos_bounds")) return rc;
  const cudaError_t e =
      sgx::launch_bounds_fp64(*eos, what, n, temp, out, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "sgx_eos_bounds");
  return SGX_OK;
}

long sgx_eos_spiner_dump(const sgx_eos *eos, double *out, long cap) {
  if (!eos || (eos->type != SGX_SPINER_RHOT && eos->type != SGX_SPINER_RHOSIE) || !eos->table) {
    fail(SGX_ERR_INVALID, "sgx_eos_spiner_dump: not a tabulated EOS");
    return -1;
  }
  return sgx::table_dump(eos->table, out, cap);
}

int sgx_eos_eval(const sgx_eos *eos, int fn, int64_t n, const double *in1, const double *in2,
                 double *out, double *lambda, int lambda_stride, sgx_stream_t stream) {
  if (!eos || !valid_type(eos->type)) return fail(SGX_ERR_INVALID, "sgx_eos_eval: bad eos");
  if (fn < SGX_FN_T_FROM_RHO_SIE || fn > SGX_FN_SIE_FROM_RHO_P)
    return fail(SGX_ERR_INVALID, "sgx_eos_eval: bad fn");
  if ((fn == SGX_FN_S_FROM_RHO_T || fn == SGX_FN_S_FROM_RHO_SIE) &&
      eos->type != SGX_IDEAL_GAS && eos->type != SGX_STIFF_GAS && eos->type != SGX_NOBLE_ABEL)
    return fail(SGX_ERR_UNSUPPORTED, "sgx_eos_eval: Entropy is not enabled for this EOS");
  if (fn > SGX_FN_MIN_SIE_FROM_RHO && eos->type == SGX_HELMHOLTZ)
    return fail(SGX_ERR_UNSUPPORTED, "sgx_eos_eval: Helmholtz takes functions 0..9 here");
  if (n < 0) return fail(SGX_ERR_INVALID, "sgx_eos_eval: n < 0");
  if (n == 0) return SGX_OK;
  if (!in1 || !out || (!in2 && fn != SGX_FN_MIN_SIE_FROM_RHO))
    return fail(SGX_ERR_INVALID, "sgx_eos_eval: null array");
  if (lambda && lambda_stride < min_lambda_stride(eos->type))
    return fail(SGX_ERR_INVALID, "sgx_eos_eval: lambda_stride below the model's lambda length");
  if (const int rc = check_mods(*eos, false, "sgx_eos_eval")) return rc;
  if (eos->type == SGX_HELMHOLTZ) {
    // Abar and Zbar come in through lambda (SafeMustGet in the reference)
    if (!lambda || lambda_stride < 3)
      return fail(SGX_ERR_INVALID, "sgx_eos_eval: Helmholtz needs lambda rows [Abar, Zbar, lT]");
    if (fn == SGX_FN_MIN_SIE_FROM_RHO)
      return fail(SGX_ERR_UNSUPPORTED,
                  "sgx_eos_eval: MinInternalEnergyFromDensity needs a temperature of 0, "
                  "outside the Helmholtz table");
  }
  sgx::EvalArgs a;
  a.eos = *eos;
  a.fn = fn;
  a.n = n;
  a.in1 = in1;
  a.in2 = in2;
  a.out = out;
  a.lambda = lambda;
  a.lambda_stride = lambda_stride;
  const cudaError_t e = eos->type == SGX_HELMHOLTZ
                            ? sgx::launch_helm_eval(a, reinterpret_cast<cudaStream_t>(stream))
                            : sgx::launch_eval_fp64(a, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "sgx_eos_eval");
  return SGX_OK;
}

int sgx_eos_pt_derivatives(const sgx_eos *eos, int64_t n, const double *rho, const double *sie,
                           const double *press, const double *temp, double *dedP_T,
                           double *drdP_T, double *dedT_P, double *drdT_P, double *lambda,
                           int lambda_stride, sgx_stream_t stream) {
  static const char *who = "sgx_eos_pt_derivatives";
  if (!eos || !valid_type(eos->type)) return fail(SGX_ERR_INVALID, std::string(who) + ": bad eos");
  if (eos->type == SGX_HELMHOLTZ)
    return fail(SGX_ERR_UNSUPPORTED,
                std::string(who) + ": Helmholtz has no DensityEnergyFromPressureTemperature here");
  if (const int rc = check_mods(*eos, false, who)) return rc;
  if (n < 0) return fail(SGX_ERR_INVALID, std::string(who) + ": n < 0");
  if (n == 0) return SGX_OK;
  if (!rho || !sie || !press || !temp || !dedP_T || !drdP_T || !dedT_P || !drdT_P)
    return fail(SGX_ERR_INVALID, std::string(who) + ": null array");
  if (lambda && lambda_stride < min_lambda_stride(eos->type))
    return fail(SGX_ERR_INVALID, std::string(who) + ": lambda_stride below the model's lambda length");
  sgx::PtDerivArgs a;
  a.eos = *eos;
  a.n = n;
  a.rho = rho;
  a.sie = sie;
  a.press = press;
  a.temp = temp;
  a.d[0] = dedP_T;
  a.d[1] = drdP_T;
  a.d[2] = dedT_P;
  a.d[3] = drdT_P;
  a.lambda = lambda;
  a.lambda_stride = lambda_stride;
  const cudaError_t e = sgx::launch_pt_derivs(a, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, who);
  return SGX_OK;
}

int sgx_eos_fill_ex(const sgx_eos *eos, int64_t n, double *rho, double *temp, double *sie,
                    double *press, double *cv, double *bmod, double *cs, uint32_t output,
                    double *lambda, int lambda_stride, int precision, sgx_stream_t stream) {
  if (!eos || !valid_type(eos->type)) return fail(SGX_ERR_INVALID, "sgx_eos_fill: bad eos");
  if (n < 0) return fail(SGX_ERR_INVALID, "sgx_eos_fill: n < 0");
  if (n == 0) return SGX_OK;
  if (!rho) return fail(SGX_ERR_INVALID, "sgx_eos_fill: rho is required");
  if (lambda && lambda_stride < min_lambda_stride(eos->type))
    return fail(SGX_ERR_INVALID, "sgx_eos_fill: lambda_stride below the model's lambda length");
  if (precision != SGX_PREC_FP64 && precision != SGX_PREC_MIXED)
    return fail(SGX_ERR_INVALID, "sgx_eos_fill: bad precision");
  if (const int rc = check_mods(*eos, precision == SGX_PREC_MIXED, "sgx_eos_fill")) return rc;
  if (eos->type == SGX_HELMHOLTZ) {
    // Helmholtz::FillEos (eos_helmholtz.hpp:818-865)
    if (!lambda || lambda_stride < 3)
      return fail(SGX_ERR_INVALID, "sgx_eos_fill: Helmholtz needs lambda rows [Abar, Zbar, lT]");
    if (output & SGX_Q_DENSITY)
      return fail(SGX_ERR_INVALID, "sgx_eos_fill: Density output not supported by this EOS");
    if ((output & SGX_Q_TEMPERATURE) && (output & SGX_Q_SIE))
      return fail(SGX_ERR_INVALID, "sgx_eos_fill: Either specific internal energy or "
                                   "temperature must be provided.");
    if ((output & SGX_Q_TEMPERATURE) ? !sie : !temp)
      return fail(SGX_ERR_INVALID, "sgx_eos_fill: the input (sie or temp) array is null");
  }
  sgx::FillArgs a;
  a.eos = *eos;
  a.n = n;
  a.rho = rho;
  a.temp = temp;
  a.sie = sie;
  a.press = press;
  a.cv = cv;
  a.bmod = bmod;
  a.cs = cs;
  a.lambda = lambda;
  a.lambda_stride = lambda_stride;
  a.output = output;
  a.err = nullptr;
  cudaError_t e;
  if (eos->type == SGX_HELMHOLTZ) {
    // mixed: the T(rho, sie) inversion's Newton iteration starts with an
    // FP32 phase; evaluations and outputs stay FP64
    e = sgx::launch_helm_fill(a, reinterpret_cast<cudaStream_t>(stream),
                              precision == SGX_PREC_MIXED);
  } else if (precision == SGX_PREC_MIXED) {
    // The mixed path covers the hot call: a tabulated model with (rho, sie)
    // in and any of T, P, cv, bmod out.
    const uint32_t allowed = SGX_Q_TEMPERATURE | SGX_Q_PRESSURE | SGX_Q_SPECIFIC_HEAT |
                             SGX_Q_BULK_MODULUS;
    if ((eos->type != SGX_SPINER_RHOT && eos->type != SGX_SPINER_RHOSIE) ||
        (output & ~allowed) || !(output & SGX_Q_TEMPERATURE) || !sie)
      return fail(SGX_ERR_UNSUPPORTED,
                  "sgx_eos_fill: mixed precision needs a tabulated EOS, (rho, sie) "
                  "inputs and T among the outputs");
    const cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (eos->type == SGX_SPINER_RHOT)
      e = sgx::launch_fill_mixed(a, s);
    else if (sgx::table_has_sie_cells(eos->table))
      e = sgx::launch_fill_sie_mixed(a, s);
    else // a table with values outside the float range: the FP64 path
      e = sgx::launch_fill_fp64(a, s);
  } else {
    e = sgx::launch_fill_fp64(a, reinterpret_cast<cudaStream_t>(stream));
  }
  if (e != cudaSuccess) return cuda_fail(e, "sgx_eos_fill");
  return SGX_OK;
}

// FillEos over host arrays, streamed through the device in chunks: on each
// of three streams in turn, the chunk's inputs go up, sgx_eos_fill_ex runs on
// them and its outputs come back, so the copies of one chunk overlap the
// kernel of the next and the copies of the one after. Inputs are the
// non-null arrays whose bit is not in output (rho always; lambda both ways);
// outputs are the arrays whose bit is in output, cs and lambda.
int sgx_eos_fill_host(const sgx_eos *eos, int64_t n, double *rho, double *temp, double *sie,
                      double *press, double *cv, double *bmod, double *cs, uint32_t output,
                      double *lambda, int lambda_stride, int precision) {
  if (!eos || !valid_type(eos->type)) return fail(SGX_ERR_INVALID, "sgx_eos_fill_host: bad eos");
  if (n < 0) return fail(SGX_ERR_INVALID, "sgx_eos_fill_host: n < 0");
  if (n == 0) return SGX_OK;
  if (!rho) return fail(SGX_ERR_INVALID, "sgx_eos_fill_host: rho is required");
  if (lambda && lambda_stride < min_lambda_stride(eos->type))
    return fail(SGX_ERR_INVALID, "sgx_eos_fill_host: lambda_stride below the model's lambda length");
  struct Arr {
    double *h;
    int width;
    bool in, out;
  };
  Arr arr[8] = {{rho, 1, !(output & SGX_Q_DENSITY), (output & SGX_Q_DENSITY) != 0},
                {temp, 1, !(output & SGX_Q_TEMPERATURE), (output & SGX_Q_TEMPERATURE) != 0},
                {sie, 1, !(output & SGX_Q_SIE), (output & SGX_Q_SIE) != 0},
                {press, 1, !(output & SGX_Q_PRESSURE), (output & SGX_Q_PRESSURE) != 0},
                {cv, 1, !(output & SGX_Q_SPECIFIC_HEAT), (output & SGX_Q_SPECIFIC_HEAT) != 0},
                {bmod, 1, !(output & SGX_Q_BULK_MODULUS), (output & SGX_Q_BULK_MODULUS) != 0},
                {cs, 1, false, true},
                {lambda, lambda_stride, true, true}};
  // a modified EOS may write any quantity (see fill_kernel): every array goes
  // both ways
  if (eos->mods)
    for (int k = 0; k < 6; ++k)
      arr[k].in = arr[k].out = true;
  // On a coherent CPU-GPU system (the GPU walks the host's page tables, as on
  // Grace over NVLink-C2C) a kernel reads and writes page-locked host memory
  // at link bandwidth: run the fill in place on the mapped host arrays, the
  // transfers overlapping the arithmetic inside the kernel.
  {
    int dev = 0, coherent = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    double *mapped[8] = {};
    bool all_mapped = coherent != 0 && !sgx::tune_get(SGX_TUNE_HOST_FILL_STAGED);
    for (int k = 0; k < 8 && all_mapped; ++k) {
      if (!arr[k].h) continue;
      cudaPointerAttributes at;
      if (cudaPointerGetAttributes(&at, arr[k].h) != cudaSuccess ||
          at.type != cudaMemoryTypeHost || !at.devicePointer) {
        cudaGetLastError(); // clear a lookup failure on unregistered memory
        all_mapped = false;
        break;
      }
      mapped[k] = static_cast<double *>(at.devicePointer);
    }
    if (all_mapped) {
      cudaStream_t s0 = nullptr;
      cudaError_t e0 = cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking);
      if (e0 != cudaSuccess) return cuda_fail(e0, "sgx_eos_fill_host");
      const int r0 = sgx_eos_fill_ex(eos, n, mapped[0], mapped[1], mapped[2], mapped[3],
                                     mapped[4], mapped[5], mapped[6], output, mapped[7],
                                     lambda_stride, precision, reinterpret_cast<sgx_stream_t>(s0));
      e0 = cudaStreamSynchronize(s0);
      cudaStreamDestroy(s0);
      if (r0 != SGX_OK) return r0;
      if (e0 != cudaSuccess) return cuda_fail(e0, "sgx_eos_fill_host");
      return SGX_OK;
    }
  }
  constexpr int S = 3;
  const int64_t chunk = n < (int64_t(1) << 21) ? n : (int64_t(1) << 21);
  cudaStream_t st[S] = {};
  double *dev[S][8] = {};
  int rc = SGX_OK;
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < S && e == cudaSuccess; ++s) {
    e = cudaStreamCreateWithFlags(&st[s], cudaStreamNonBlocking);
    for (int k = 0; k < 8 && e == cudaSuccess; ++k)
      if (arr[k].h)
        e = sgx::scratch_alloc(reinterpret_cast<void **>(&dev[s][k]),
                               static_cast<size_t>(chunk) * arr[k].width * sizeof(double), st[s]);
  }
  for (int64_t off = 0, c = 0; off < n && e == cudaSuccess && rc == SGX_OK; off += chunk, ++c) {
    const int s = static_cast<int>(c % S);
    const int64_t len = (n - off) < chunk ? (n - off) : chunk;
    for (int k = 0; k < 8 && e == cudaSuccess; ++k)
      if (arr[k].h && arr[k].in)
        e = cudaMemcpyAsync(dev[s][k], arr[k].h + off * arr[k].width,
                            static_cast<size_t>(len) * arr[k].width * sizeof(double),
                            cudaMemcpyHostToDevice, st[s]);
    if (e != cudaSuccess) break;
    rc = sgx_eos_fill_ex(eos, len, dev[s][0], dev[s][1], dev[s][2], dev[s][3], dev[s][4],
                         dev[s][5], dev[s][6], output, dev[s][7], lambda_stride, precision,
                         reinterpret_cast<sgx_stream_t>(st[s]));
    if (rc != SGX_OK) break;
    for (int k = 0; k < 8 && e == cudaSuccess; ++k)
      if (arr[k].h && arr[k].out)
        e = cudaMemcpyAsync(arr[k].h + off * arr[k].width, dev[s][k],
                            static_cast<size_t>(len) * arr[k].width * sizeof(double),
                            cudaMemcpyDeviceToHost, st[s]);
  }
  for (int s = 0; s < S; ++s) {
    if (!st[s]) continue;
    for (int k = 0; k < 8; ++k)
      if (dev[s][k]) sgx::scratch_free(dev[s][k], st[s]);
    const cudaError_t f = cudaStreamSynchronize(st[s]);
    if (e == cudaSuccess) e = f;
    cudaStreamDestroy(st[s]);
  }
  if (rc != SGX_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "sgx_eos_fill_host");
  return SGX_OK;
}

int sgx_eos_fill(const sgx_eos *eos, int64_t n, double *rho, double *temp, double *sie,
                 double *press, double *cv, double *bmod, uint32_t output, double *lambda,
                 int lambda_stride, sgx_stream_t stream) {
  return sgx_eos_fill_ex(eos, n, rho, temp, sie, press, cv, bmod, nullptr, output, lambda,
                         lambda_stride, SGX_PREC_FP64, stream);
}

} // extern "C"

namespace sgx {
// The argument checks of sgx_pte_solve and its PteArgs; empty is set when
// ncell is 0 (nothing to launch).
int pte_prepare(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
                double *rho, double *vfrac, double *sie, double *temp, double *press,
                double *lambda, const sgx_mix_params *params, sgx_pte_status *status,
                int precision, PteArgs &a, bool &empty) {
  empty = false;
  if (solver < SGX_PTE_RHOT || solver > SGX_PTE_FIXED_P)
    return fail(SGX_ERR_INVALID, "sgx_pte_solve: bad solver");
  if (precision != SGX_PREC_FP64 && precision != SGX_PREC_MIXED)
    return fail(SGX_ERR_INVALID, "sgx_pte_solve: bad precision");
  if (precision == SGX_PREC_MIXED && solver != SGX_PTE_RHOT)
    return fail(SGX_ERR_UNSUPPORTED, "sgx_pte_solve: SGX_PREC_MIXED is for SGX_PTE_RHOT only");
  if (nmat < 1 || nmat > sgx::PTE_MAX_N)
    return fail(SGX_ERR_UNSUPPORTED, "sgx_pte_solve: nmat must be in 1..6");
  if (neos < 1 || neos > sgx::MAX_EOS || !eos_list)
    return fail(SGX_ERR_INVALID, "sgx_pte_solve: neos must be in 1..16");
  if (!eos_idx && neos < nmat)
    return fail(SGX_ERR_INVALID, "sgx_pte_solve: eos_idx NULL needs neos >= nmat");
  if (ncell < 0) return fail(SGX_ERR_INVALID, "sgx_pte_solve: ncell < 0");
  if (ncell == 0) {
    empty = true;
    return SGX_OK;
  }
  if (!vfrac_tot || !sie_tot || !rho || !vfrac || !sie || !temp || !press)
    return fail(SGX_ERR_INVALID, "sgx_pte_solve: null array");
  for (int k = 0; k < neos; ++k)
    if (!valid_type(eos_list[k].type)) return fail(SGX_ERR_INVALID, "sgx_pte_solve: bad eos");
    else if (!pte_type(eos_list[k].type))
      return fail(SGX_ERR_UNSUPPORTED, "sgx_pte_solve: Helmholtz is not available in PTE");
    else if (const int rc = check_mods(eos_list[k], precision == SGX_PREC_MIXED, "sgx_pte_solve"))
      return rc;
  std::memset(&a, 0, sizeof(a));
  a.solver = solver;
  a.nmat = nmat;
  a.ncell = ncell;
  a.neos = neos;
  for (int k = 0; k < neos; ++k)
    a.eos[k] = eos_list[k];
  a.eos_idx = eos_idx;
  a.vfrac_tot = vfrac_tot;
  a.sie_tot = sie_tot;
  a.rho = rho;
  a.vfrac = vfrac;
  a.sie = sie;
  a.temp = temp;
  a.press = press;
  a.lambda = lambda;
  a.status = status;
  if (params)
    a.params = *params;
  else
    sgx_mix_params_default(&a.params);
  return SGX_OK;
}
} // namespace sgx

extern "C" {

int sgx_pte_solve(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                  const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
                  double *rho, double *vfrac, double *sie, double *temp, double *press,
                  double *lambda, const sgx_mix_params *params, sgx_pte_status *status,
                  int precision, sgx_stream_t stream) {
  sgx::PteArgs a;
  bool empty = false;
  if (const int rc = sgx::pte_prepare(solver, nmat, ncell, eos_list, neos, eos_idx, vfrac_tot,
                                      sie_tot, rho, vfrac, sie, temp, press, lambda, params,
                                      status, precision, a, empty))
    return rc;
  if (empty) return SGX_OK;
  cudaError_t e;
  if (precision == SGX_PREC_MIXED)
    e = sgx::launch_pte_mixed(a, reinterpret_cast<cudaStream_t>(stream));
  else
    e = sgx::launch_pte_fp64(a, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "sgx_pte_solve");
  return SGX_OK;
}

// The mixed RhoT solve with static scratch (sgx_noalloc.cu); argument checks
// as sgx_pte_solve's, plus the scratch capacity, all before any CUDA call.
int sgx_pte_solve_noalloc(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list,
                          int neos, const int32_t *eos_idx, const double *vfrac_tot,
                          const double *sie_tot, double *rho, double *vfrac, double *sie,
                          double *temp, double *press, double *lambda,
                          const sgx_mix_params *params, sgx_pte_status *status,
                          sgx_stream_t stream) {
  static const char *who = "sgx_pte_solve_noalloc";
  if (solver != SGX_PTE_RHOT && solver != SGX_PTE_PT)
    return fail(SGX_ERR_INVALID, std::string(who) + ": bad solver");
  if (solver != SGX_PTE_RHOT)
    return fail(SGX_ERR_UNSUPPORTED, std::string(who) + ": only SGX_PTE_RHOT");
  if (nmat < 1 || nmat > sgx::PTE_MAX_N)
    return fail(SGX_ERR_UNSUPPORTED, std::string(who) + ": nmat must be in 1..6");
  if (neos < 1 || neos > sgx::MAX_EOS || !eos_list)
    return fail(SGX_ERR_INVALID, std::string(who) + ": neos must be in 1..16");
  if (!eos_idx && neos < nmat)
    return fail(SGX_ERR_INVALID, std::string(who) + ": eos_idx NULL needs neos >= nmat");
  if (ncell < 0) return fail(SGX_ERR_INVALID, std::string(who) + ": ncell < 0");
  if (ncell > SGX_PTE_NOALLOC_MAX_CELLS)
    return fail(SGX_ERR_INVALID,
                std::string(who) + ": ncell = " + std::to_string(ncell) +
                    " exceeds the static scratch capacity of SGX_PTE_NOALLOC_MAX_CELLS = " +
                    std::to_string(SGX_PTE_NOALLOC_MAX_CELLS) +
                    " cells; split the batch or call sgx_pte_solve");
  if (ncell == 0) return SGX_OK;
  if (!vfrac_tot || !sie_tot || !rho || !vfrac || !sie || !temp || !press)
    return fail(SGX_ERR_INVALID, std::string(who) + ": null array");
  for (int k = 0; k < neos; ++k)
    if (!valid_type(eos_list[k].type))
      return fail(SGX_ERR_INVALID, std::string(who) + ": bad eos");
    else if (!pte_type(eos_list[k].type))
      return fail(SGX_ERR_UNSUPPORTED, std::string(who) + ": Helmholtz is not available in PTE");
    else if (const int rc = check_mods(eos_list[k], true, who))
      return rc;
  sgx::PteArgs a;
  std::memset(&a, 0, sizeof(a));
  a.solver = solver;
  a.nmat = nmat;
  a.ncell = ncell;
  a.neos = neos;
  for (int k = 0; k < neos; ++k)
    a.eos[k] = eos_list[k];
  a.eos_idx = eos_idx;
  a.vfrac_tot = vfrac_tot;
  a.sie_tot = sie_tot;
  a.rho = rho;
  a.vfrac = vfrac;
  a.sie = sie;
  a.temp = temp;
  a.press = press;
  a.lambda = lambda;
  a.status = status;
  if (params)
    a.params = *params;
  else
    sgx_mix_params_default(&a.params);
  const cudaError_t e = sgx::launch_pte_mixed_noalloc(a, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, who);
  return SGX_OK;
}

} // extern "C"
