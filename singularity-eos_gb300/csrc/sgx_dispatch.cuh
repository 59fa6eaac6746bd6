// Model dispatch: one switch over the packed sgx_eos code, standing in for
// the reference Variant's visit (eos/eos_variant.hpp:152-868). Analytic
// models come from sgx_eos.cuh, the tabulated rho-T model from
// sgx_spiner.cuh, the tabulated model on rho-T and rho-sie grids from
// sgx_spiner_sie.cuh. `lam` is the per-element lambda row (nullable); only
// the tabulated models read or write it.
//
// Two levels: md_* evaluates the bare model; ev_* (what every kernel calls)
// adds the modifiers of sgx_eos.mods around it, nested as the reference's
// variant nests them, BilinearRamp(Scaled(Shifted(model))). A bare model
// (mods == 0) takes one predictable branch to md_*.
#pragma once

#include "sgx_eos.cuh"
#include "sgx_spiner.cuh"
#include "sgx_spiner_sie.cuh"

// The translation units of the mixed-precision paths, which take bare models
// only (the C API rejects a modified EOS there), define SGX_BARE_MODELS
// before including this header: the modifier arithmetic compiles out of
// their kernels. Their copy of the dispatch sits in its own inline namespace,
// so the two variants of these inline functions never share a symbol.
#ifdef SGX_BARE_MODELS
#define SGX_MODS(e) 0u
#define SGX_DISPATCH_BEGIN inline namespace bare_models {
#else
#define SGX_MODS(e) ((e).mods)
#define SGX_DISPATCH_BEGIN inline namespace all_models {
#endif

namespace sgx {
SGX_DISPATCH_BEGIN

SGX_HD const SpinerTable &sp_table(const sgx_eos &e) {
  return *reinterpret_cast<const SpinerTable *>(static_cast<uintptr_t>(e.table));
}
SGX_HD bool is_spiner(const sgx_eos &e) { return e.type == SGX_SPINER_RHOT; }
SGX_HD const SieTable &ss_table(const sgx_eos &e) {
  return *reinterpret_cast<const SieTable *>(static_cast<uintptr_t>(e.table));
}
SGX_HD bool is_spiner_sie(const sgx_eos &e) { return e.type == SGX_SPINER_RHOSIE; }

template <typename T>
SGX_HD T md_T_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_T_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  if (is_spiner_sie(e)) return T(ss_T_from_rho_sie(ss_table(e), double(rho), double(sie), lam));
  return eos_T_from_rho_sie<T>(e, rho, sie);
}
template <typename T>
SGX_HD T md_sie_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_sie_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  if (is_spiner_sie(e)) return T(ss_sie_from_rho_T(ss_table(e), double(rho), double(temp), lam));
  return eos_sie_from_rho_T<T>(e, rho, temp);
}
template <typename T>
SGX_HD T md_P_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_P_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  if (is_spiner_sie(e)) return T(ss_P_from_rho_T(ss_table(e), double(rho), double(temp), lam));
  return eos_P_from_rho_T<T>(e, rho, temp);
}
template <typename T>
SGX_HD T md_P_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_P_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  if (is_spiner_sie(e)) return T(ss_P_from_rho_sie(ss_table(e), double(rho), double(sie), lam));
  return eos_P_from_rho_sie<T>(e, rho, sie);
}
template <typename T>
SGX_HD T md_cv_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_cv_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  if (is_spiner_sie(e)) return T(ss_cv_from_rho_T(ss_table(e), double(rho), double(temp), lam));
  return eos_cv<T>(e);
}
template <typename T>
SGX_HD T md_cv_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_cv_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  if (is_spiner_sie(e)) return T(ss_cv_from_rho_sie(ss_table(e), double(rho), double(sie), lam));
  return eos_cv<T>(e);
}
template <typename T>
SGX_HD T md_B_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_bmod_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  if (is_spiner_sie(e)) return T(ss_bmod_from_rho_T(ss_table(e), double(rho), double(temp), lam));
  return eos_B_from_rho_T<T>(e, rho, temp);
}
template <typename T>
SGX_HD T md_B_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_bmod_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  if (is_spiner_sie(e)) return T(ss_bmod_from_rho_sie(ss_table(e), double(rho), double(sie), lam));
  return eos_B_from_rho_sie<T>(e, rho, sie);
}
template <typename T>
SGX_HD T md_gamma_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_gamma_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  if (is_spiner_sie(e)) return T(ss_gamma_from_rho_T(ss_table(e), double(rho), double(temp), lam));
  return eos_gamma<T>(e, rho);
}
template <typename T>
SGX_HD T md_gamma_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_gamma_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  if (is_spiner_sie(e)) return T(ss_gamma_from_rho_sie(ss_table(e), double(rho), double(sie), lam));
  return eos_gamma<T>(e, rho);
}
template <typename T> SGX_HD T md_min_sie(const sgx_eos &e, T rho) {
  if (is_spiner(e)) return T(sp_min_sie(sp_table(e), double(rho)));
  if (is_spiner_sie(e)) return T(ss_min_sie(ss_table(e), double(rho)));
  return eos_min_sie<T>(e, rho);
}

// Bounds (eos_base.hpp:594-613; SpinerEOSDependsRhoT :241-246, :1117-1123)
SGX_HD double md_min_temperature(const sgx_eos &e) {
  if (is_spiner(e)) return sp_T(sp_table(e), sp_table(e).lTMin);
  if (is_spiner_sie(e)) return from_log(ss_table(e).gT.min, ss_table(e).lTOffset);
  return eos_min_temperature(e);
}
SGX_HD double md_max_density(const sgx_eos &e) {
  if (is_spiner(e)) return sp_table(e).rhoMax;
  if (is_spiner_sie(e)) return ss_table(e).rhoMax;
  return eos_max_density(e);
}
SGX_HD double md_min_density(const sgx_eos &e) {
  if (is_spiner(e)) return sp_rho(sp_table(e), sp_table(e).lRhoMin);
  if (is_spiner_sie(e)) return from_log(ss_table(e).lRhoMin, ss_table(e).lRhoOffset);
  return 0;
}
// The temperature ValuesAtReferenceState reports (eos_ideal.hpp:178-190,
// eos_stiff.hpp:153-164, eos_noble_abel.hpp:167-178: room temperature;
// eos_gruneisen.hpp:554-567: T0; eos_spiner_rho_temp.hpp:1104-1115: TNormal_).
SGX_HD double md_reference_T(const sgx_eos &e) {
  if (is_spiner(e)) return sp_table(e).TNormal;
  if (is_spiner_sie(e)) return ss_table(e).TNormal;
  if (e.type == SGX_GRUNEISEN) return e.p[7];
  if (e.type == SGX_STIFF_GAS || e.type == SGX_NOBLE_ABEL) return e.p[pi::rT0];
  return ROOM_TEMPERATURE;
}
// Density, temperature, pressure and bulk modulus of ValuesAtReferenceState,
// per model: eos_ideal.hpp:41-45 + :178-190 (STP: 1e6, room temperature),
// eos_stiff.hpp:40-48 + :153-164, eos_noble_abel.hpp:40-48 + :167-178,
// eos_gruneisen.hpp:554-567 (rho0, T0, and P, bmod at sie = 0),
// eos_spiner_rho_temp.hpp:1104-1115 (the load-time normal state).
SGX_HDI void md_reference_state(const sgx_eos &e, double &rho, double &temp, double &press,
                                double &bmod) {
  const double gm1 = e.p[pi::gm1], Cv = e.p[pi::Cv];
  const double T0 = ROOM_TEMPERATURE, P0 = ATMOSPHERIC_PRESSURE;
  switch (e.type) {
  case SGX_IDEAL_GAS:
    rho = P0 / (gm1 * Cv * T0);
    temp = T0;
    press = P0;
    bmod = (gm1 + 1) * gm1 * rho * Cv * T0;
    return;
  case SGX_STIFF_GAS: {
    const double Pinf = e.p[pi::Pinf], sT0 = e.p[pi::rT0], sP0 = e.p[pi::rP0];
    rho = ratio(sP0 + Pinf, gm1 * Cv * sT0);
    temp = sT0;
    press = sP0;
    bmod = gm1 * (gm1 + 1.0) * ratio(sP0 + Pinf, gm1 * Cv * sT0) * Cv * sT0;
    return;
  }
  case SGX_NOBLE_ABEL: {
    const double bb = e.p[pi::bb], nT0 = e.p[pi::rT0], nP0 = e.p[pi::rP0];
    rho = ratio(nP0, gm1 * Cv * nT0 + bb * nP0);
    temp = nT0;
    press = nP0;
    bmod = ratio(rho * Cv * nT0 * gm1 * (gm1 + 1.0), (1.0 - bb * rho) * (1.0 - bb * rho));
    return;
  }
  case SGX_GRUNEISEN:
    rho = e.p[pi::rho0];
    temp = e.p[pi::T0];
    press = eos_P_from_rho_sie<double>(e, rho, 0.0);
    bmod = eos_B_from_rho_sie<double>(e, rho, 0.0);
    return;
  case SGX_SPINER_RHOT: {
    const SpinerTable &t = sp_table(e);
    rho = t.rhoNormal;
    temp = t.TNormal;
    press = t.PNormal;
    bmod = t.bModNormal;
    return;
  }
  case SGX_SPINER_RHOSIE: {
    const SieTable &t = ss_table(e);
    rho = t.rhoNormal;
    temp = t.TNormal;
    press = t.PNormal;
    bmod = t.bModNormal;
    return;
  }
  }
  rho = temp = press = bmod = 0.0;
}
SGX_HD double md_rho_pmin(const sgx_eos &e, const double T) {
  if (is_spiner(e)) return sp_rho_pmin(sp_table(e), T);
  if (is_spiner_sie(e)) return ss_rho_pmin(ss_table(e), T);
  return eos_rho_pmin(e, T);
}
SGX_HD double md_min_pressure(const sgx_eos &e) {
  if (is_spiner(e)) return sp_table(e).PMin;
  if (is_spiner_sie(e)) return ss_table(e).PMin;
  return eos_min_pressure(e);
}
SGX_HDI double md_max_pressure_at_T(const sgx_eos &e, const double T, int *err) {
  if (is_spiner(e) || is_spiner_sie(e)) return 1e100;
  return eos_max_pressure_at_T(e, T, err);
}
SGX_HDI void md_rho_sie_from_PT(const sgx_eos &e, const double P, const double T, double &rho,
                                double &sie, double *lam, int *err) {
  if (is_spiner(e)) {
    sp_rho_sie_from_PT(sp_table(e), P, T, rho, sie, lam);
    return;
  }
  if (is_spiner_sie(e)) {
    ss_rho_sie_from_PT(ss_table(e), P, T, rho, sie, lam);
    return;
  }
  eos_rho_sie_from_PT(e, P, T, rho, sie, err);
}

// FillEos per model. The reference's UNDEFINED_ERROR / EOS_ERROR aborts
// (base/eos_error.hpp:19-20) become *err = 1 and the element is left as is.
//   IdealGas  eos_ideal.hpp:236-262     StiffGas  eos_stiff.hpp:203-229
//   NobleAbel eos_noble_abel.hpp:216-242  Gruneisen eos_gruneisen.hpp:527-546
//   SpinerEOSDependsRhoT eos_spiner_rho_temp.hpp:1052-1101
//   SpinerEOSDependsRhoSie eos_spiner_rho_sie.hpp:844-898
SGX_HDI void md_fill(const sgx_eos &e, double &rho, double &temp, double &sie, double &press,
                     double &cv, double &bmod, const unsigned output, double *lam, int *err) {
  const double gm1 = e.p[pi::gm1];
  switch (e.type) {
  case SGX_IDEAL_GAS:
  case SGX_STIFF_GAS:
  case SGX_NOBLE_ABEL: {
    if ((output & Q_DENSITY) && (output & Q_SIE)) {
      if ((output & Q_PRESSURE) || (output & Q_TEMPERATURE)) {
        *err = 1;
        return;
      }
      eos_rho_sie_from_PT(e, press, temp, rho, sie, err);
    }
    if ((output & Q_PRESSURE) && (output & Q_SIE)) {
      if ((output & Q_DENSITY) || (output & Q_TEMPERATURE)) {
        *err = 1;
        return;
      }
      sie = eos_sie_from_rho_T<double>(e, rho, temp);
    }
    if ((output & Q_TEMPERATURE) && (output & Q_SIE)) {
      if (e.type == SGX_IDEAL_GAS)
        sie = press / (gm1 * rho);
      else if (e.type == SGX_STIFF_GAS)
        sie = ratio(press + (gm1 + 1.0) * e.p[pi::Pinf], gm1 * rho) + e.p[pi::qq];
      else
        sie = press * (1.0 - e.p[pi::bb] * rho) / gm1 + e.p[pi::qq];
    }
    if (output & Q_PRESSURE) press = eos_P_from_rho_sie<double>(e, rho, sie);
    if (output & Q_TEMPERATURE) temp = eos_T_from_rho_sie<double>(e, rho, sie);
    if (output & Q_BMOD) bmod = eos_B_from_rho_sie<double>(e, rho, sie);
    if (output & Q_CV) cv = eos_cv<double>(e);
    return;
  }
  case SGX_GRUNEISEN: {
    const unsigned input = ~output;
    if ((Q_TEMPERATURE & input) && (Q_PRESSURE & input)) {
      eos_rho_sie_from_PT(e, press, temp, rho, sie, err);
    } else if ((Q_DENSITY & output) || (Q_SIE & output)) {
      *err = 1;
      return;
    }
    const double r = smin(rho, e.p[pi::rho_max]);
    if (output & Q_PRESSURE) press = gru_P_rho_e(e, r, sie);
    if (output & Q_TEMPERATURE) temp = eos_T_from_rho_sie<double>(e, r, sie);
    if (output & Q_BMOD) bmod = gru_B_rho_e(e, r, sie);
    if (output & Q_CV) cv = e.p[pi::gCv];
    return;
  }
  case SGX_SPINER_RHOT: {
    const SpinerTable &t = sp_table(e);
    const unsigned input = ~output;
    double lRho, lT;
    TableStatus w;
    if (output == 0) {
      *err = 1;
      return;
    }
    if (output & Q_DENSITY) {
      if ((input & Q_PRESSURE) && (input & Q_TEMPERATURE)) {
        lT = sp_lT(t, temp);
        lRho = sp_lRho_from_P_lT(t, press, lT, w, lam);
        rho = sp_rho(t, lRho);
      } else {
        *err = 1;
        return;
      }
    } else {
      lRho = sp_lRho(t, rho);
    }
    if (output & Q_TEMPERATURE) {
      if ((input & Q_DENSITY) && (input & Q_SIE)) {
        lT = sp_lT_from_lRho_sie(t, lRho, sie, w, lam);
      } else {
        // lTFromlRhoP_ is not on the hot path; report it as unsupported.
        *err = 1;
        return;
      }
      temp = sp_T(t, lT);
    } else {
      lT = sp_lT(t, temp);
    }
    w = sp_loc_rho_T(t, lRho, lT);
    if (output & Q_SIE) sie = sp_sie_from(t, lRho, temp, lT, w);
    if (output & Q_PRESSURE) press = sp_P_from(t, rho, lRho, temp, lT, w);
    if (output & Q_CV) cv = sp_cv_from(t, lRho, lT, w);
    if (output & Q_BMOD) bmod = sp_bmod_from(t, rho, lRho, temp, lT, w);
    if (lam != nullptr) {
      lam[0] = lRho;
      lam[1] = lT;
    }
    return;
  }
  case SGX_SPINER_RHOSIE: {
    // SpinerEOSDependsRhoSie::FillEos (eos_spiner_rho_sie.hpp:844-898):
    // outputs other than rho need T or sie among the outputs, which picks
    // the grid they come from
    const SieTable &t = ss_table(e);
    if (output == 0 || ((output & Q_TEMPERATURE) && (output & Q_SIE))) {
      *err = 1;
      return;
    }
    double lRho;
    if (output & Q_DENSITY) {
      if ((output & Q_PRESSURE) || (output & Q_TEMPERATURE)) {
        *err = 1;
        return;
      }
      lRho = ss_lRho_from_P_lT(t, press, ss_lT(t, temp), lam);
      rho = from_log(lRho, t.lRhoOffset);
    } else {
      lRho = ss_lRho(t, rho);
      if (lam != nullptr) lam[0] = lRho;
    }
    if (output & Q_TEMPERATURE) {
      const double lE = ss_lE(t, sie);
      temp = se_interp(t, SE_T, lRho, lE);
      if (output & Q_PRESSURE) press = se_interp(t, SE_P, lRho, lE);
      if (output & Q_CV) cv = 1. / se_interp(t, SE_DTDE, lRho, lE);
      if (output & Q_BMOD) bmod = se_interp(t, SE_BMOD, lRho, lE);
    }
    if (output & Q_SIE) {
      const double lT = ss_lT(t, temp);
      sie = st_interp(t, ST_SIE, lRho, lT);
      if (output & Q_PRESSURE) press = st_interp(t, ST_P, lRho, lT);
      if (output & Q_CV) cv = 1. / st_interp(t, ST_DTDE, lRho, lT);
      if (output & Q_BMOD) bmod = st_interp(t, ST_BMOD, lRho, lT);
    }
    return;
  }
  }
  *err = 1;
}

// ---------------------------------------------------------------------------
// Modifiers (eos/modifiers/). Each reads its parameters from the sgx_eos
// value; the arithmetic is the reference's, operation for operation.

// BilinearRampEOS::get_ramp_pressure / get_ramp_density / get_ramp_dpdrho
// (ramps_eos.hpp:113-133). ramp[] = r0, a, b, c, rmid, Pmid.
SGX_HD double ramp_pressure(const sgx_eos &e, const double rho) {
  const double r_r0 = ratio(rho, e.ramp[0]);
  return rho < e.ramp[0]   ? 0.0
         : rho < e.ramp[4] ? e.ramp[1] * (r_r0 - 1.0)
                           : e.ramp[2] * (r_r0 - e.ramp[3]);
}
SGX_HD double ramp_density(const sgx_eos &e, const double P) {
  return P < e.ramp[5] ? e.ramp[0] * (ratio(P, e.ramp[1]) + 1.0)
                       : e.ramp[0] * (ratio(P, e.ramp[2]) + e.ramp[3]);
}
SGX_HD double ramp_dpdrho(const sgx_eos &e, const double rho) {
  return rho < e.ramp[4] ? ratio(e.ramp[1], e.ramp[0]) : ratio(e.ramp[2], e.ramp[0]);
}

// Each ev_* below calls its md_* once, on the arguments the wrapped model
// sees, and applies the modifiers' output arithmetic around that call, so a
// kernel carries one copy of the model code whether or not an EOS is
// modified. For T = float (the mixed-precision paths, which take bare
// models only) the transforms are never active.
template <typename T> SGX_HD T mrho(const sgx_eos &e, const T rho) {
  return (SGX_MODS(e) & SGX_MOD_SCALED) ? T(e.scale) * rho : rho;
}
template <typename T> SGX_HD T msie(const sgx_eos &e, T sie) {
  if (SGX_MODS(e) & SGX_MOD_SCALED) sie = T(e.inv_scale) * sie;
  if (SGX_MODS(e) & SGX_MOD_SHIFTED) sie = sie - T(e.shift);
  return sie;
}
// BilinearRampEOS pressure (ramps_eos.hpp:149-154, 186-191): the ramp's
// pressure where the EOS lies below it.
template <typename T> SGX_HD T ramp_max(const sgx_eos &e, const T rho, const T p_eos) {
  if (!(SGX_MODS(e) & SGX_MOD_RAMP)) return p_eos;
  const T p_ramp = T(ramp_pressure(e, double(rho)));
  return p_eos < p_ramp ? p_ramp : p_eos;
}
// BilinearRampEOS bulk modulus (ramps_eos.hpp:170-181, 203-212): below the
// ramp, rho times the ramp's slope; the wrapped pressure decides.
SGX_HDN bool ramp_below_rho_sie(const sgx_eos &e, const double rho, const double r,
                                const double s, double *lam) {
  const double p_ramp = ramp_pressure(e, rho);
  const double p_eos = md_P_from_rho_sie<double>(e, r, s, lam);
  return p_eos < p_ramp;
}
SGX_HDN bool ramp_below_rho_T(const sgx_eos &e, const double rho, const double r,
                              const double temp, double *lam) {
  const double p_ramp = ramp_pressure(e, rho);
  const double p_eos = md_P_from_rho_T<double>(e, r, temp, lam);
  return p_eos < p_ramp;
}

// Functions of (rho, sie): ScaledEOS passes (scale_ rho, sie / scale_)
// (scaled_eos.hpp:68-133), ShiftedEOS sie - shift_ (shifted_eos.hpp:66-106).
template <typename T>
SGX_HD T ev_T_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  return md_T_from_rho_sie<T>(e, mrho(e, rho), msie(e, sie), lam);
}
template <typename T>
SGX_HD T ev_P_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  return ramp_max(e, rho, md_P_from_rho_sie<T>(e, mrho(e, rho), msie(e, sie), lam));
}
template <typename T>
SGX_HD T ev_cv_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  return md_cv_from_rho_sie<T>(e, mrho(e, rho), msie(e, sie), lam);
}
template <typename T>
SGX_HD T ev_B_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  const T r = mrho(e, rho), s = msie(e, sie);
  if ((SGX_MODS(e) & SGX_MOD_RAMP) && ramp_below_rho_sie(e, double(rho), double(r), double(s), lam))
    return rho * T(ramp_dpdrho(e, double(rho)));
  return md_B_from_rho_sie<T>(e, r, s, lam);
}
template <typename T>
SGX_HD T ev_gamma_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  return md_gamma_from_rho_sie<T>(e, mrho(e, rho), msie(e, sie), lam);
}
// Functions of (rho, T): ScaledEOS passes scale_ rho.
template <typename T>
SGX_HD T ev_P_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  return ramp_max(e, rho, md_P_from_rho_T<T>(e, mrho(e, rho), temp, lam));
}
template <typename T>
SGX_HD T ev_cv_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  return md_cv_from_rho_T<T>(e, mrho(e, rho), temp, lam);
}
template <typename T>
SGX_HD T ev_B_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  const T r = mrho(e, rho);
  if ((SGX_MODS(e) & SGX_MOD_RAMP) && ramp_below_rho_T(e, double(rho), double(r), double(temp), lam))
    return rho * T(ramp_dpdrho(e, double(rho)));
  return md_B_from_rho_T<T>(e, r, temp, lam);
}
template <typename T>
SGX_HD T ev_gamma_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  return md_gamma_from_rho_T<T>(e, mrho(e, rho), temp, lam);
}
// InternalEnergyFromDensityTemperature: ShiftedEOS adds shift_
// (shifted_eos.hpp:72-76); ScaledEOS multiplies by scale_ and passes rho
// unscaled (scaled_eos.hpp:77-81).
template <typename T>
SGX_HD T ev_sie_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  T energy = md_sie_from_rho_T<T>(e, rho, temp, lam);
  if (SGX_MODS(e) & SGX_MOD_SHIFTED) energy = energy + T(e.shift);
  if (SGX_MODS(e) & SGX_MOD_SCALED) energy = T(e.scale) * energy;
  return energy;
}
// MinInternalEnergyFromDensity: ScaledEOS passes scale_ rho and leaves the
// result unscaled (scaled_eos.hpp:84-88); ShiftedEOS adds shift_ (:83-86).
template <typename T> SGX_HD T ev_min_sie(const sgx_eos &e, T rho) {
  T m = md_min_sie<T>(e, mrho(e, rho));
  if (SGX_MODS(e) & SGX_MOD_SHIFTED) m = m + T(e.shift);
  return m;
}

// Bounds. ScaledEOS divides the density bounds by scale_
// (scaled_eos.hpp:254-275); ShiftedEOS and BilinearRampEOS forward them
// (SG_ADD_MODIFIER_INTROSPECTION_METHODS, eos_base.hpp:134-153;
// ramps_eos.hpp:248-265).
SGX_HD double ev_min_temperature(const sgx_eos &e) { return md_min_temperature(e); }
SGX_HD double ev_max_density(const sgx_eos &e) {
  return (SGX_MODS(e) & SGX_MOD_SCALED) ? e.inv_scale * md_max_density(e) : md_max_density(e);
}
SGX_HD double ev_min_density(const sgx_eos &e) {
  return (SGX_MODS(e) & SGX_MOD_SCALED) ? e.inv_scale * md_min_density(e) : md_min_density(e);
}
SGX_HD double ev_rho_pmin(const sgx_eos &e, const double T) {
  return (SGX_MODS(e) & SGX_MOD_SCALED) ? e.inv_scale * md_rho_pmin(e, T) : md_rho_pmin(e, T);
}
SGX_HD double ev_min_pressure(const sgx_eos &e) { return md_min_pressure(e); }
SGX_HDI double ev_max_pressure_at_T(const sgx_eos &e, const double T, int *err) {
  return md_max_pressure_at_T(e, T, err);
}
// RhoPmin in the caller's arithmetic type: the analytic models' 0 without
// leaving it (for T = double the same value as ev_rho_pmin), the tabulated
// and scaled ones through the FP64 form. Keeps float-double conversions,
// which issue on the FP64 pipe, out of the FP32 Newton iterations.
template <typename T> SGX_HD T ev_rho_pmin_t(const sgx_eos &e, const T temp) {
  if (is_spiner(e) || is_spiner_sie(e) || (SGX_MODS(e) & SGX_MOD_SCALED))
    return T(ev_rho_pmin(e, double(temp)));
  return T(0);
}
// DensityEnergyFromPressureTemperature of the bare closed-form models
// (eos_rho_sie_from_PT) in float, for the FP32 phase; false for the others,
// which take the FP64 form.
SGX_HD bool ev_rho_sie_from_PT_f(const sgx_eos &e, const float press, const float temp,
                                 float &rho, float &sie) {
  if (SGX_MODS(e)) return false;
  const float gm1 = float(e.p[pi::gm1]), Cv = float(e.p[pi::Cv]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    sie = mymax(0.0f, Cv * temp);
    rho = mymax(0.0f, press / (gm1 * sie));
    return true;
  case SGX_STIFF_GAS: {
    const float Pinf = float(e.p[pi::Pinf]), qq = float(e.p[pi::qq]);
    sie = smax(qq, ratio(press + (gm1 + 1.0f) * Pinf, press + Pinf) * Cv * temp + qq);
    rho = smax(lim<float>::small, ratio(press + Pinf, gm1 * Cv * temp));
    return true;
  }
  case SGX_NOBLE_ABEL: {
    const float qq = float(e.p[pi::qq]);
    sie = smax(qq, Cv * temp + qq);
    rho = smax(lim<float>::small, ratio(press, gm1 * Cv * temp + float(e.p[pi::bb]) * press));
    return true;
  }
  }
  return false;
}

// The temperature of ValuesAtReferenceState; no modifier changes it.
SGX_HD double ev_reference_T(const sgx_eos &e) { return md_reference_T(e); }
// ValuesAtReferenceState through the modifiers: ScaledEOS divides rho by
// scale_ (scaled_eos.hpp:183-190); P, T and bmod pass through
// (shifted_eos.hpp:406-412, ramps_eos.hpp:528-533).
SGX_HDI void ev_reference_state(const sgx_eos &e, double &rho, double &temp, double &press,
                                double &bmod) {
  md_reference_state(e, rho, temp, press, bmod);
  if (SGX_MODS(e) & SGX_MOD_SCALED) rho = rho * e.inv_scale;
}
// DensityEnergyFromPressureTemperature: ShiftedEOS adds shift_ to sie
// (shifted_eos.hpp:398-403), ScaledEOS then divides rho and multiplies sie
// by scale_ (scaled_eos.hpp:244-250); BilinearRampEOS forwards (:521-525).
SGX_HDI void ev_rho_sie_from_PT(const sgx_eos &e, const double P, const double T, double &rho,
                                double &sie, double *lam, int *err) {
  md_rho_sie_from_PT(e, P, T, rho, sie, lam, err);
  if (SGX_MODS(e) & SGX_MOD_SHIFTED) sie = sie + e.shift;
  if (SGX_MODS(e) & SGX_MOD_SCALED) {
    rho = rho * e.inv_scale;
    sie = sie * e.scale;
  }
}

// FillEos through the modifiers. ShiftedEOS and ScaledEOS switch on the
// model's PreferredInput and abort on any value but rho-T or rho-sie
// (shifted_eos.hpp:150-167, scaled_eos.hpp:160-181), which takes in
// IdealGas (it prefers all four); the abort becomes *err = 1 here.
SGX_HDI void fill_shifted(const sgx_eos &e, double &rho, double &temp, double &sie,
                          double &press, double &cv, double &bmod, const unsigned output,
                          double *lam, int *err) {
  if (!(SGX_MODS(e) & SGX_MOD_SHIFTED)) {
    md_fill(e, rho, temp, sie, press, cv, bmod, output, lam, err);
    return;
  }
  const unsigned pref = preferred_input(e);
  if (pref == (Q_DENSITY | Q_TEMPERATURE)) {
    md_fill(e, rho, temp, sie, press, cv, bmod, output, lam, err);
    sie = sie + e.shift;
  } else if (pref == (Q_DENSITY | Q_SIE)) {
    double senergy = sie - e.shift;
    md_fill(e, rho, temp, senergy, press, cv, bmod, output, lam, err);
  } else {
    *err = 1;
  }
}
SGX_HDI void fill_scaled(const sgx_eos &e, double &rho, double &temp, double &sie,
                         double &press, double &cv, double &bmod, const unsigned output,
                         double *lam, int *err) {
  if (!(SGX_MODS(e) & SGX_MOD_SCALED)) {
    fill_shifted(e, rho, temp, sie, press, cv, bmod, output, lam, err);
    return;
  }
  const unsigned pref = preferred_input(e);
  double srho = e.scale * rho;
  if (pref == (Q_DENSITY | Q_TEMPERATURE)) {
    fill_shifted(e, srho, temp, sie, press, cv, bmod, output, lam, err);
    sie = e.scale * sie;
  } else if (pref == (Q_DENSITY | Q_SIE)) {
    double senergy = e.inv_scale * sie;
    fill_shifted(e, srho, temp, senergy, press, cv, bmod, output, lam, err);
  } else {
    *err = 1;
  }
}
// BilinearRampEOS::FillEos (ramps_eos.hpp:221-243): the pressure comes from
// the ramped P(rho, sie) or P(rho, T), the wrapped EOS fills the rest, a
// density output is capped by the ramp's density at that pressure, and
// bmod is always recomputed from the ramped bulk modulus.
SGX_HDI void ev_fill(const sgx_eos &e, double &rho, double &temp, double &sie, double &press,
                     double &cv, double &bmod, const unsigned output, double *lam, int *err) {
  if (!(SGX_MODS(e) & SGX_MOD_RAMP)) {
    fill_scaled(e, rho, temp, sie, press, cv, bmod, output, lam, err);
    return;
  }
  const unsigned ramp_out = output & ~Q_PRESSURE;
  if (output & Q_PRESSURE) {
    if (!(output & Q_SIE))
      press = ev_P_from_rho_sie<double>(e, rho, sie, lam);
    else if (!(output & Q_TEMPERATURE))
      press = ev_P_from_rho_T<double>(e, rho, temp, lam);
  }
  fill_scaled(e, rho, temp, sie, press, cv, bmod, ramp_out, lam, err);
  double rho_ramp = rho;
  if (output & Q_DENSITY) rho_ramp = ramp_density(e, press);
  rho = rho_ramp < rho ? rho_ramp : rho;
  bmod = ev_B_from_rho_sie<double>(e, rho, sie, lam);
}

// ---------------------------------------------------------------------------
// Entropy (the SG_EOS_VEC_FOR(Entropy) vector members, eos_base.hpp:497).
// The analytic gases use their reference state, kept in p[] by the
// constructors (STP, 293 K and 1e6, and qp = 0 unless given):
//   IdealGas  eos_ideal.hpp:100-114 (EntropyT0, EntropyRho0)
//   StiffGas  eos_stiff.hpp:93-109
//   NobleAbel eos_noble_abel.hpp:100-119
// Gruneisen and the tabulated model have no entropy (EntropyIsNotEnabled,
// eos_base.hpp:588-600, which aborts); the C API rejects them.
SGX_HDI double md_entropy_rho_T(const sgx_eos &e, const double rho, const double T) {
  const double gm1 = e.p[pi::gm1], Cv = e.p[pi::Cv];
  const double T0 = e.p[pi::rT0], P0 = e.p[pi::rP0], qp = e.p[pi::qp];
  const double SMALL = lim<double>::small;
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return Cv * log(ratio(T, e.p[pi::ST0])) + gm1 * Cv * log(ratio(e.p[pi::SRho0], rho));
  case SGX_STIFF_GAS: {
    const double rho0 = ratio(P0 + e.p[pi::Pinf], gm1 * Cv * T0);
    return Cv * log(ratio(T, T0) + SMALL) + gm1 * Cv * log(ratio(rho0, rho) + SMALL) + qp;
  }
  case SGX_NOBLE_ABEL: {
    const double bb = e.p[pi::bb];
    const double vol0 = ratio(gm1 * Cv * T0 + bb * P0, P0);
    const double vol = ratio(1.0, rho);
    return Cv * log(ratio(T, T0) + SMALL) +
           gm1 * Cv * log(ratio(vol - bb, vol0 - bb) + SMALL) + qp;
  }
  }
  return NAN;
}
SGX_HDI double md_entropy_rho_sie(const sgx_eos &e, const double rho, const double sie) {
  const double gm1 = e.p[pi::gm1], Cv = e.p[pi::Cv];
  const double T0 = e.p[pi::rT0], P0 = e.p[pi::rP0], qp = e.p[pi::qp];
  const double SMALL = lim<double>::small;
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return md_entropy_rho_T(e, rho, eos_T_from_rho_sie<double>(e, rho, sie));
  case SGX_STIFF_GAS: {
    const double Pinf = e.p[pi::Pinf], qq = e.p[pi::qq];
    const double vol0 = ratio(gm1 * Cv * T0, P0 + Pinf);
    const double sie0 = ratio(P0 + (gm1 + 1.0) * Pinf, P0 + Pinf) * Cv * T0 + qq;
    const double vol = ratio(1.0, rho);
    return Cv * log(ratio((sie - qq - Pinf * vol), (sie0 - qq - Pinf * vol0)) + SMALL) +
           Cv * gm1 * log(ratio(vol, vol0) + SMALL) + qp;
  }
  case SGX_NOBLE_ABEL: {
    const double bb = e.p[pi::bb], qq = e.p[pi::qq];
    const double vol0 = ratio(gm1 * Cv * T0 + bb * P0, P0);
    const double sie0 = Cv * T0 + qq;
    const double vol = ratio(1.0, rho);
    return Cv * log(ratio(sie - qq, sie0 - qq) + SMALL) +
           gm1 * Cv * log(ratio(vol - bb, vol0 - bb) + SMALL) + qp;
  }
  }
  return NAN;
}
// Through the modifiers: ScaledEOS returns scale_ S(scale_ rho, sie / scale_)
// (scaled_eos.hpp:92-97, 121-125); ShiftedEOS passes sie - shift_ and T as
// is; BilinearRampEOS forwards.
SGX_HDI double ev_entropy_rho_T(const sgx_eos &e, const double rho, const double T) {
  const double S = md_entropy_rho_T(e, mrho(e, rho), T);
  return (SGX_MODS(e) & SGX_MOD_SCALED) ? e.scale * S : S;
}
SGX_HDI double ev_entropy_rho_sie(const sgx_eos &e, const double rho, const double sie) {
  const double S = md_entropy_rho_sie(e, mrho(e, rho), msie(e, sie));
  return (SGX_MODS(e) & SGX_MOD_SCALED) ? e.scale * S : S;
}

// ---------------------------------------------------------------------------
// InternalEnergyFromDensityPressure.

// EosBase::InternalEnergyFromDensityPressure with sie in and out
// (eos_base.hpp:685-707): regula falsi on P(rho, sie) between the energies
// at the minimum temperature and at 1e20, from the middle when sie lies in
// that range, else from sie. A root find that fails leaves what
// regula_falsi leaves (the reference only warns).
template <typename PF, typename EF>
SGX_HDI void iefdp_base(const PF &P_of, const EF &e_of, const double minT, const double rho,
                        const double P, double &sie) {
  auto f = [&](const double s) { return P_of(rho, s); };
  const double sie_min = e_of(rho, minT);
  const double sie_max = e_of(rho, 1e20);
  const double sie_guess =
      (((sie_min < sie) && (sie < sie_max)) ? 0.5 * (sie_min + sie_max) : sie);
  regula_falsi(f, P, sie_guess, sie_min, sie_max, lim<double>::eps, lim<double>::eps, sie);
}
// The bare models: IdealGas in closed form (eos_ideal.hpp:208-214), the
// others through the base class.
SGX_HDI void md_sie_from_rho_P(const sgx_eos &e, const double rho, const double P, double &sie,
                               double *lam) {
  if (e.type == SGX_IDEAL_GAS) {
    sie = P / (e.p[pi::gm1] * rho);
    return;
  }
  iefdp_base([&](const double r, const double s) { return md_P_from_rho_sie<double>(e, r, s, lam); },
             [&](const double r, const double t) { return md_sie_from_rho_T<double>(e, r, t, lam); },
             md_min_temperature(e), rho, P, sie);
}
// The sie-in-and-out member through the modifiers: BilinearRampEOS has none
// and takes the base class's over its own P and sie (ramped pressure);
// ScaledEOS passes scale_ rho (scaled_eos.hpp:141-146); ShiftedEOS shifts sie
// in and back (shifted_eos.hpp:132-139).
SGX_HDI void ev_sie_from_rho_P_inout(const sgx_eos &e, const double rho, const double P,
                                     double &sie, double *lam) {
  if (SGX_MODS(e) & SGX_MOD_RAMP) {
    iefdp_base([&](const double r, const double s) { return ev_P_from_rho_sie<double>(e, r, s, lam); },
               [&](const double r, const double t) { return ev_sie_from_rho_T<double>(e, r, t, lam); },
               ev_min_temperature(e), rho, P, sie);
    return;
  }
  if (SGX_MODS(e) & SGX_MOD_SHIFTED) sie -= e.shift;
  md_sie_from_rho_P(e, mrho(e, rho), P, sie, lam);
  if (SGX_MODS(e) & SGX_MOD_SHIFTED) sie += e.shift;
}
// The value-returning member the vector call loops over (eos_base.hpp:708-721):
// start from the middle of the energy range, then the member above.
SGX_HDI double ev_sie_from_rho_P(const sgx_eos &e, const double rho, const double P,
                                 double *lam) {
  const double sie_min = ev_sie_from_rho_T<double>(e, rho, ev_min_temperature(e), lam);
  const double sie_max = ev_sie_from_rho_T<double>(e, rho, 1e20, lam);
  double sie = 0.5 * (sie_min + sie_max);
  ev_sie_from_rho_P_inout(e, rho, P, sie, lam);
  return sie;
}

// ---------------------------------------------------------------------------
// PTDerivativesFromPreferred: (dsie/dP)_T, (drho/dP)_T, (dsie/dT)_P and
// (drho/dT)_P at a state (rho, sie, P, T).

// PTDerivativesByFiniteDifferences (eos_base.hpp:299-320): one-sided
// differences of DensityEnergyFromPressureTemperature with eps 3e-6 (the
// default of EosBase::PTDerivativesFromPreferred, :410-419). The perturbed
// state starts at 0 where the reference leaves it uninitialised.
template <typename DEFPT>
SGX_HDI void pt_derivs_fd(const DEFPT &defpt, const double rho, const double sie,
                          const double P, const double T, double &dedP_T, double &drdP_T,
                          double &dedT_P, double &drdT_P) {
  constexpr double derivative_eps = 3.0e-6;
  const double absP = smax(sabs(P), lim<double>::eps / derivative_eps);
  const double dP = -rsgn(P) * absP * derivative_eps; // might be negative
  const double absT = smax(sabs(T), lim<double>::eps / derivative_eps);
  const double dT = absT * derivative_eps;
  double r_pert = 0.0, e_pert = 0.0;
  defpt(P + dP, T, r_pert, e_pert);
  drdP_T = ratio(r_pert - rho, dP);
  dedP_T = ratio(e_pert - sie, dP);
  defpt(P, T + dT, r_pert, e_pert);
  drdT_P = ratio(r_pert - rho, dT);
  dedT_P = ratio(e_pert - sie, dT);
}

// The bare models: IdealGas in closed form (eos_ideal.hpp:152-168); the
// others take the base class's finite differences (the tabulated model's own
// version is commented out in eos_spiner_rho_temp.hpp:199-206, 1015-1048).
SGX_HDI void md_pt_derivs(const sgx_eos &e, const double rho, const double sie, const double P,
                          const double T, double *lam, double &dedP_T, double &drdP_T,
                          double &dedT_P, double &drdT_P, int *err) {
  if (e.type == SGX_IDEAL_GAS) {
    const double gm1 = e.p[pi::gm1], Cv = e.p[pi::Cv];
    dedP_T = 0;
    dedT_P = Cv;
    drdP_T = ratio(1.0, gm1 * sie);
    drdT_P = -ratio(P, gm1 * Cv * T * T);
    return;
  }
  auto defpt = [&](const double p, const double t, double &r, double &s) {
    md_rho_sie_from_PT(e, p, t, r, s, lam, err);
  };
  pt_derivs_fd(defpt, rho, sie, P, T, dedP_T, drdP_T, dedT_P, drdT_P);
}

// Through the modifiers: BilinearRampEOS keeps the base class's finite
// differences over its own DensityEnergyFromPressureTemperature, which
// forwards to the wrapped EOS (ramps_eos.hpp:220, 521-525); ScaledEOS
// evaluates at (scale rho, sie / scale) and rescales the four derivatives
// (scaled_eos.hpp:148-159); ShiftedEOS evaluates at sie - shift
// (shifted_eos.hpp:141-148).
SGX_HDI void ev_pt_derivs(const sgx_eos &e, const double rho, const double sie, const double P,
                          const double T, double *lam, double &dedP_T, double &drdP_T,
                          double &dedT_P, double &drdT_P, int *err) {
  if (SGX_MODS(e) & SGX_MOD_RAMP) {
    auto defpt = [&](const double p, const double t, double &r, double &s) {
      ev_rho_sie_from_PT(e, p, t, r, s, lam, err);
    };
    pt_derivs_fd(defpt, rho, sie, P, T, dedP_T, drdP_T, dedT_P, drdT_P);
    return;
  }
  double r = rho, s = sie;
  if (SGX_MODS(e) & SGX_MOD_SCALED) {
    r = e.scale * rho;
    s = e.inv_scale * sie;
  }
  if (SGX_MODS(e) & SGX_MOD_SHIFTED) s = s - e.shift;
  md_pt_derivs(e, r, s, P, T, lam, dedP_T, drdP_T, dedT_P, drdT_P, err);
  if (SGX_MODS(e) & SGX_MOD_SCALED) {
    dedP_T *= e.scale;
    drdP_T *= e.inv_scale;
    dedT_P *= e.scale;
    drdT_P *= e.inv_scale;
  }
}

// One vector-lookup element (EosBase vector members, eos_base.hpp:421-494).
SGX_HDI double ev_eval(const sgx_eos &e, const int fn, const double a, const double b,
                       double *lam) {
  switch (fn) {
  case SGX_FN_T_FROM_RHO_SIE:
    return ev_T_from_rho_sie<double>(e, a, b, lam);
  case SGX_FN_SIE_FROM_RHO_T:
    return ev_sie_from_rho_T<double>(e, a, b, lam);
  case SGX_FN_P_FROM_RHO_T:
    return ev_P_from_rho_T<double>(e, a, b, lam);
  case SGX_FN_P_FROM_RHO_SIE:
    return ev_P_from_rho_sie<double>(e, a, b, lam);
  case SGX_FN_CV_FROM_RHO_T:
    return ev_cv_from_rho_T<double>(e, a, b, lam);
  case SGX_FN_CV_FROM_RHO_SIE:
    return ev_cv_from_rho_sie<double>(e, a, b, lam);
  case SGX_FN_B_FROM_RHO_T:
    return ev_B_from_rho_T<double>(e, a, b, lam);
  case SGX_FN_B_FROM_RHO_SIE:
    return ev_B_from_rho_sie<double>(e, a, b, lam);
  case SGX_FN_G_FROM_RHO_T:
    return ev_gamma_from_rho_T<double>(e, a, b, lam);
  case SGX_FN_G_FROM_RHO_SIE:
    return ev_gamma_from_rho_sie<double>(e, a, b, lam);
  case SGX_FN_MIN_SIE_FROM_RHO:
    return ev_min_sie<double>(e, a);
  case SGX_FN_S_FROM_RHO_T:
    return ev_entropy_rho_T(e, a, b);
  case SGX_FN_S_FROM_RHO_SIE:
    return ev_entropy_rho_sie(e, a, b);
  case SGX_FN_SIE_FROM_RHO_P:
    return ev_sie_from_rho_P(e, a, b, lam);
  }
  return 0.0;
}

} // inline namespace
} // namespace sgx
