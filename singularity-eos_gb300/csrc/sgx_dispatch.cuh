// Model dispatch: one switch over the packed sgx_eos code, standing in for
// the reference Variant's visit (eos/eos_variant.hpp:152-868). Analytic
// models come from sgx_eos.cuh, the tabulated rho-T model from
// sgx_spiner.cuh. `lam` is the per-element lambda row (nullable); only the
// tabulated model reads or writes it.
#pragma once

#include "sgx_eos.cuh"
#include "sgx_spiner.cuh"

namespace sgx {

SGX_HD const SpinerTable &sp_table(const sgx_eos &e) {
  return *reinterpret_cast<const SpinerTable *>(static_cast<uintptr_t>(e.table));
}
SGX_HD bool is_spiner(const sgx_eos &e) { return e.type == SGX_SPINER_RHOT; }

template <typename T>
SGX_HD T ev_T_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_T_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  return eos_T_from_rho_sie<T>(e, rho, sie);
}
template <typename T>
SGX_HD T ev_sie_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_sie_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  return eos_sie_from_rho_T<T>(e, rho, temp);
}
template <typename T>
SGX_HD T ev_P_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_P_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  return eos_P_from_rho_T<T>(e, rho, temp);
}
template <typename T>
SGX_HD T ev_P_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_P_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  return eos_P_from_rho_sie<T>(e, rho, sie);
}
template <typename T>
SGX_HD T ev_cv_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_cv_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  return eos_cv<T>(e);
}
template <typename T>
SGX_HD T ev_cv_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_cv_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  return eos_cv<T>(e);
}
template <typename T>
SGX_HD T ev_B_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_bmod_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  return eos_B_from_rho_T<T>(e, rho, temp);
}
template <typename T>
SGX_HD T ev_B_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_bmod_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  return eos_B_from_rho_sie<T>(e, rho, sie);
}
template <typename T>
SGX_HD T ev_gamma_from_rho_T(const sgx_eos &e, T rho, T temp, double *lam) {
  if (is_spiner(e)) return T(sp_gamma_from_rho_T(sp_table(e), double(rho), double(temp), lam));
  return eos_gamma<T>(e, rho);
}
template <typename T>
SGX_HD T ev_gamma_from_rho_sie(const sgx_eos &e, T rho, T sie, double *lam) {
  if (is_spiner(e)) return T(sp_gamma_from_rho_sie(sp_table(e), double(rho), double(sie), lam));
  return eos_gamma<T>(e, rho);
}
template <typename T> SGX_HD T ev_min_sie(const sgx_eos &e, T rho) {
  if (is_spiner(e)) return T(sp_min_sie(sp_table(e), double(rho)));
  return eos_min_sie<T>(e, rho);
}

// Bounds (eos_base.hpp:594-613; SpinerEOSDependsRhoT :241-246, :1117-1123)
SGX_HD double ev_min_temperature(const sgx_eos &e) {
  if (is_spiner(e)) return sp_T(sp_table(e), sp_table(e).lTMin);
  return eos_min_temperature(e);
}
SGX_HD double ev_max_density(const sgx_eos &e) {
  if (is_spiner(e)) return sp_table(e).rhoMax;
  return eos_max_density(e);
}
SGX_HD double ev_min_density(const sgx_eos &e) {
  if (is_spiner(e)) return sp_rho(sp_table(e), sp_table(e).lRhoMin);
  return 0;
}
// The temperature ValuesAtReferenceState reports (eos_ideal.hpp:178-190,
// eos_stiff.hpp:153-164, eos_noble_abel.hpp:167-178: room temperature;
// eos_gruneisen.hpp:554-567: T0; eos_spiner_rho_temp.hpp:1104-1115: TNormal_).
SGX_HD double ev_reference_T(const sgx_eos &e) {
  if (is_spiner(e)) return sp_table(e).TNormal;
  if (e.type == SGX_GRUNEISEN) return e.p[7];
  return ROOM_TEMPERATURE;
}
SGX_HD double ev_rho_pmin(const sgx_eos &e, const double T) {
  if (is_spiner(e)) return sp_rho_pmin(sp_table(e), T);
  return eos_rho_pmin(e, T);
}
SGX_HD double ev_min_pressure(const sgx_eos &e) {
  if (is_spiner(e)) return sp_table(e).PMin;
  return eos_min_pressure(e);
}
SGX_HDI double ev_max_pressure_at_T(const sgx_eos &e, const double T, int *err) {
  if (is_spiner(e)) return 1e100;
  return eos_max_pressure_at_T(e, T, err);
}
SGX_HDI void ev_rho_sie_from_PT(const sgx_eos &e, const double P, const double T, double &rho,
                                double &sie, double *lam, int *err) {
  if (is_spiner(e)) {
    sp_rho_sie_from_PT(sp_table(e), P, T, rho, sie, lam);
    return;
  }
  eos_rho_sie_from_PT(e, P, T, rho, sie, err);
}

// FillEos per model. The reference's UNDEFINED_ERROR / EOS_ERROR aborts
// (base/eos_error.hpp:19-20) become *err = 1 and the element is left as is.
//   IdealGas  eos_ideal.hpp:236-262     StiffGas  eos_stiff.hpp:203-229
//   NobleAbel eos_noble_abel.hpp:216-242  Gruneisen eos_gruneisen.hpp:527-546
//   SpinerEOSDependsRhoT eos_spiner_rho_temp.hpp:1052-1101
SGX_HDI void ev_fill(const sgx_eos &e, double &rho, double &temp, double &sie, double &press,
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
  }
  *err = 1;
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
  }
  return 0.0;
}

} // namespace sgx
