// The EOS modifiers of sgx.h: ShiftedEOS, ScaledEOS and BilinearRampEOS
// (eos/modifiers/) set on an sgx_eos value, pAlpha2BilinearRampParams
// (eos/modifiers/ramps_eos.hpp:43-77) and the modifier step of the
// reference's init_sg_* functions (eos/singularity_eos.cpp:67-79).
//
// The wrapped evaluations themselves live in sgx_dispatch.cuh, which every
// kernel calls. pAlpha2BilinearRampParams runs its reference-state read and
// its two root finds on the device, through that same code, so tabulated
// models work as analytic ones do; only the exp/log of the bracket are taken
// on the host, with the C library the reference calls. This unit is compiled
// without contraction, like the other FP64 units.
#include <cmath>
#include <cfloat>
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "sgx_internal.h"
#include "sgx_dispatch.cuh"

namespace sgx {
namespace {

struct RampOut {
  double rho0, T0, P0, bmod0; // reference state
  double rmid, r1;             // the two roots
  int status[2];
};

__global__ void reference_state_kernel(const sgx_eos e, RampOut *out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  ev_reference_state(e, out->rho0, out->T0, out->P0, out->bmod0);
}

// The root finds of pAlpha2BilinearRampParams (ramps_eos.hpp:57-66):
// P(alpha0 x, T0) = Pe from the guess rho0 on [r0, rho_ub], then
// P(x, T0) = Pc from the guess rmid on the same bracket, both to 1e-12.
// The reference leaves rmid and r1 uninitialised before findRoot; a root
// find that writes nothing leaves 0 here.
__global__ void p_alpha_roots_kernel(const sgx_eos e, const double alpha0, const double Pe,
                                     const double Pc, const double r0, const double rho_ub,
                                     RampOut *out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const double rho0 = out->rho0, T0 = out->T0;
  auto rmid_func = [&](const double x) {
    return ev_P_from_rho_T<double>(e, alpha0 * x, T0, nullptr);
  };
  double rmid = 0.0;
  out->status[0] =
      static_cast<int>(find_root(rmid_func, Pe, rho0, r0, rho_ub, 1.e-12, 1.e-12, rmid));
  auto r1_func = [&](const double x) { return ev_P_from_rho_T<double>(e, x, T0, nullptr); };
  double r1 = 0.0;
  out->status[1] =
      static_cast<int>(find_root(r1_func, Pc, rmid, r0, rho_ub, 1.e-12, 1.e-12, r1));
  out->rmid = rmid;
  out->r1 = r1;
}

int check_target(const sgx_eos *eos, const char *who) {
  if (!eos) return set_error(SGX_ERR_INVALID, std::string(who) + ": null");
  if (eos->type < SGX_IDEAL_GAS || eos->type > SGX_HELMHOLTZ)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": bad eos");
  if (eos->type == SGX_HELMHOLTZ)
    return set_error(SGX_ERR_UNSUPPORTED, std::string(who) + ": Helmholtz takes no modifiers");
  return check_eos_mods(*eos, false, who);
}

int cuda_error(const cudaError_t e, const char *who) {
  return set_error(SGX_ERR_CUDA, std::string(who) + ": " + cudaGetErrorString(e));
}

} // namespace
} // namespace sgx

extern "C" {

int sgx_eos_modify_shifted(sgx_eos *eos, double shift) {
  static const char *who = "sgx_eos_modify_shifted";
  if (const int rc = sgx::check_target(eos, who)) return rc;
  if (eos->mods)
    return sgx::set_error(SGX_ERR_UNSUPPORTED,
                          std::string(who) + ": ShiftedEOS wraps a bare model only");
  // ShiftedEOS::CheckParams (shifted_eos.hpp:58-61)
  if (std::isnan(shift)) return sgx::set_error(SGX_ERR_INVALID, "Shift must be a number");
  eos->mods |= SGX_MOD_SHIFTED;
  eos->shift = shift;
  return SGX_OK;
}

int sgx_eos_modify_scaled(sgx_eos *eos, double scale) {
  static const char *who = "sgx_eos_modify_scaled";
  if (const int rc = sgx::check_target(eos, who)) return rc;
  if (eos->mods & ~static_cast<uint32_t>(SGX_MOD_SHIFTED))
    return sgx::set_error(SGX_ERR_UNSUPPORTED,
                          std::string(who) + ": ScaledEOS wraps a bare or shifted model only");
  // ScaledEOS(t, scale): inv_scale_(1. / scale), then CheckParams
  // (scaled_eos.hpp:53-66)
  const double inv_scale = 1. / scale;
  if (!(std::abs(scale) > 0)) return sgx::set_error(SGX_ERR_INVALID, "Scale must not be zero.");
  if (!(std::abs(inv_scale) > 0))
    return sgx::set_error(SGX_ERR_INVALID, "Inverse scale must not be zero.");
  if (std::isnan(scale)) return sgx::set_error(SGX_ERR_INVALID, "Scale must be well defined.");
  if (std::isnan(inv_scale))
    return sgx::set_error(SGX_ERR_INVALID, "Inverse scale must be well defined.");
  eos->mods |= SGX_MOD_SCALED;
  eos->scale = scale;
  eos->inv_scale = inv_scale;
  return SGX_OK;
}

int sgx_eos_modify_bilinear_ramp(sgx_eos *eos, double r0, double a, double b, double c) {
  static const char *who = "sgx_eos_modify_bilinear_ramp";
  if (const int rc = sgx::check_target(eos, who)) return rc;
  if (eos->mods & SGX_MOD_RAMP)
    return sgx::set_error(SGX_ERR_UNSUPPORTED, std::string(who) + ": already ramped");
  // BilinearRampEOS(t, r0, a, b, c) and CheckParams (ramps_eos.hpp:86-104)
  const double rmid = r0 * (a - b * c) / (a - b);
  const double Pmid = a * (rmid / r0 - 1.0);
  if (!(r0 > 0.0)) return sgx::set_error(SGX_ERR_INVALID, "Reference density > 0");
  if (!(a > 0.0)) return sgx::set_error(SGX_ERR_INVALID, "Ramp a coefficient > 0");
  if (!(b >= 0)) return sgx::set_error(SGX_ERR_INVALID, "Non-negative ramp b coefficient");
  if (!(a != b))
    return sgx::set_error(SGX_ERR_INVALID, "Ramp a and b coefficients may not be the same");
  if (std::isnan(rmid)) return sgx::set_error(SGX_ERR_INVALID, "Mid density must be well defined");
  if (std::isnan(Pmid))
    return sgx::set_error(SGX_ERR_INVALID, "Mid pressure must be well defined");
  eos->mods |= SGX_MOD_RAMP;
  eos->ramp[0] = r0;
  eos->ramp[1] = a;
  eos->ramp[2] = b;
  eos->ramp[3] = c;
  eos->ramp[4] = rmid;
  eos->ramp[5] = Pmid;
  return SGX_OK;
}

int sgx_eos_p_alpha_ramp_params(const sgx_eos *eos, double alpha0, double Pe, double Pc,
                                double *r0, double *a, double *b, double *c) {
  static const char *who = "sgx_eos_p_alpha_ramp_params";
  if (const int rc = sgx::check_target(eos, who)) return rc;
  if (!r0 || !a || !b || !c) return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": null");
  // the reference asserts alpha0 > 1 (ramps_eos.hpp:50)
  if (!(alpha0 > 1.0)) return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": alpha0 <= 1");
  sgx::RampOut *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(sgx::RampOut));
  if (e != cudaSuccess) return sgx::cuda_error(e, who);
  sgx::RampOut h;
  std::memset(&h, 0, sizeof(h));
  e = cudaMemcpy(d, &h, sizeof(h), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    sgx::reference_state_kernel<<<1, 1>>>(*eos, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  double rr0 = 0.0;
  if (e == cudaSuccess) {
    // the bracket (ramps_eos.hpp:51-56)
    rr0 = sgx::ratio(h.rho0, alpha0);
    const double max_exp_arg = std::log(DBL_MAX * 0.99);
    const double arg = sgx::ratio((2.0 * Pc - h.P0), h.bmod0);
    const double exp_arg = (arg < max_exp_arg) ? arg : max_exp_arg; // std::min
    const double rho_ub = h.rho0 * std::exp(exp_arg);
    sgx::p_alpha_roots_kernel<<<1, 1>>>(*eos, alpha0, Pe, Pc, rr0, rho_ub, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return sgx::cuda_error(e, who);
  // ramps_eos.hpp:72-75
  const double rmid = h.rmid, r1 = h.r1;
  const double aa = sgx::ratio(rr0 * Pe, rmid - rr0);
  const double bb = sgx::ratio(rr0 * (Pc - Pe), r1 - rmid);
  const double cc = sgx::ratio(Pc * rmid - Pe * r1, rr0 * (Pc - Pe));
  *r0 = rr0;
  *a = aa;
  *b = bb;
  *c = cc;
  return SGX_OK;
}

int sgx_eos_apply_modifiers(sgx_eos *eos, const int enabled[4], double vals[6]) {
  static const char *who = "sgx_eos_apply_modifiers";
  if (!eos || !enabled || !vals) return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": null");
  const bool scaled = enabled[0] == 1, shifted = enabled[1] == 1;
  const bool ramped = enabled[2] == 1 || enabled[3] == 1;
  if (!scaled && !shifted && !ramped) return SGX_OK; // applyShiftAndScale returns eos as is
  if (const int rc = sgx::check_target(eos, who)) return rc;
  if (eos->mods)
    return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": the EOS is already modified");
  // SGAPPLYMODSIMPLE (singularity_eos_init_utils.hpp): ShiftedEOS inside
  // ScaledEOS; then, for enabled[3], the p-alpha ramp of that EOS with its
  // parameters written over vals[2..5] (singularity_eos.cpp:71-74); then
  // SGAPPLYMOD wraps the ramp around it.
  sgx_eos e = *eos;
  int rc = SGX_OK;
  if (shifted && (rc = sgx_eos_modify_shifted(&e, vals[1]))) return rc;
  if (scaled && (rc = sgx_eos_modify_scaled(&e, vals[0]))) return rc;
  if (enabled[3] == 1) {
    const double alpha0 = vals[2], Pe = vals[3], Pc = vals[4];
    double r0, a, b, c;
    if ((rc = sgx_eos_p_alpha_ramp_params(&e, alpha0, Pe, Pc, &r0, &a, &b, &c))) return rc;
    vals[2] = r0;
    vals[3] = a;
    vals[4] = b;
    vals[5] = c;
  }
  if (ramped && (rc = sgx_eos_modify_bilinear_ramp(&e, vals[2], vals[3], vals[4], vals[5])))
    return rc;
  *eos = e;
  return SGX_OK;
}

} // extern "C"
