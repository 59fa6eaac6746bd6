// Analytic EOS models evaluated on a packed sgx_eos value. One switch on the
// model code replaces the reference's PortsOfCall::visit over the Variant
// (eos/eos_variant.hpp:152-868); each branch restates the model's scalar
// member function with the reference's operation order, so the FP64 build
// (--fmad=false) is bit-identical to the reference compiled without FP
// contraction.
//
// Models: IdealGas (eos/eos_ideal.hpp:38-262), StiffGas (eos/eos_stiff.hpp:
// 36-229), NobleAbel (eos/eos_noble_abel.hpp:36-242), Gruneisen
// (eos/eos_gruneisen.hpp:36-567). Tabulated models live in sgx_spiner.cuh.
#pragma once

#include "../../include/sgx.h"
#include "sgx_math.cuh"

namespace sgx {

// thermalqs bits (base/constants.hpp:22-34)
constexpr unsigned Q_DENSITY = 1, Q_SIE = 2, Q_PRESSURE = 4, Q_TEMPERATURE = 8;
constexpr unsigned Q_CV = 16, Q_BMOD = 32;

// Model parameter slots inside sgx_eos::p.
namespace pi {
constexpr int gm1 = 0, Cv = 1, Pinf = 2, qq = 3, bb = 2;
// IdealGas entropy reference (EntropyT0, EntropyRho0; eos_ideal.hpp:49-56)
constexpr int ST0 = 2, SRho0 = 3;
// StiffGas / NobleAbel reference state (qp, T0, P0; eos_stiff.hpp:52-59,
// eos_noble_abel.hpp:52-60)
constexpr int qp = 4, rT0 = 5, rP0 = 6;
// Gruneisen
constexpr int C0 = 0, s1 = 1, s2 = 2, s3 = 3, G0 = 4, b = 5, rho0 = 6, T0 = 7, P0 = 8,
              gCv = 9, rho_max = 10;
} // namespace pi

// Reference state constants (base/constants.hpp:39-40).
constexpr double ROOM_TEMPERATURE = 293;
constexpr double ATMOSPHERIC_PRESSURE = 1e6;

// ---------------------------------------------------------------------------
// Gruneisen helpers (eos_gruneisen.hpp:191-195, 331-371), templated on the
// arithmetic type (double reproduces the reference; float serves the FP32
// iteration phase of the mixed-precision solver).
template <typename T> SGX_HD T gru_gamma(const sgx_eos &e, const T rho_in) {
  const double *p = e.p;
  const T rho = smin(rho_in, T(p[pi::rho_max]));
  const T rho0 = T(p[pi::rho0]), G0 = T(p[pi::G0]);
  return rho < rho0 ? G0 : G0 * rho0 / rho + T(p[pi::b]) * (1 - rho0 / rho);
}
template <typename T> SGX_HD T gru_P_rho_e(const sgx_eos &e, const T rho_in, const T sie) {
  const double *p = e.p;
  const T rho = smin(rho_in, T(p[pi::rho_max]));
  const T rho0 = T(p[pi::rho0]), C0 = T(p[pi::C0]), P0 = T(p[pi::P0]);
  T P_H, E_H;
  if (rho >= rho0) {
    const T eta = 1 - rho0 / rho;
    const T s = T(p[pi::s1]) * eta + T(p[pi::s2]) * (eta * eta) + T(p[pi::s3]) * (eta * (eta * eta));
    P_H = P0 + (C0 * C0) * rho0 * eta / ((1 - s) * (1 - s));
    E_H = (P_H + P0) * eta / rho0 / T(2.);
  } else {
    P_H = P0 + (C0 * C0) * (rho - rho0);
    E_H = T(0.);
  }
  return P_H + gru_gamma<T>(e, rho) * rho * (sie - E_H);
}
template <typename T> SGX_HD T gru_dPdrho_e(const sgx_eos &e, const T rho_in, const T sie) {
  const double *p = e.p;
  const T rho = smin(rho_in, T(p[pi::rho_max]));
  const T rho0 = T(p[pi::rho0]), C0 = T(p[pi::C0]), P0 = T(p[pi::P0]);
  if (rho < rho0) {
    return (C0 * C0) + gru_gamma<T>(e, rho) * sie;
  }
  const T s1 = T(p[pi::s1]), s2 = T(p[pi::s2]), s3 = T(p[pi::s3]);
  const T eta = 1 - rho0 / rho;
  const T s = s1 * eta + s2 * (eta * eta) + s3 * (eta * (eta * eta));
  const T ds = s1 + 2 * s2 * eta + 3 * s3 * (eta * eta);
  const T deta = rho0 / (rho * rho);
  const T dGam = (T(p[pi::b]) - T(p[pi::G0])) * deta;
  const T C02 = C0 * C0;
  const T oms2 = (1 - s) * (1 - s);
  const T P_H = P0 + C02 * rho0 * eta / oms2;
  const T dP_H = C02 * rho0 / oms2 * deta * (1 + 2 * eta * ds / (1 - s));
  const T E_H = (P_H + P0) * eta / rho0 / T(2.);
  const T dE_H = deta * (P_H + P0) / rho0 / T(2.) + eta / rho0 / 2 * dP_H;
  const T G = gru_gamma<T>(e, rho);
  return dP_H + G * (sie - E_H) + rho * dGam * (sie - E_H) - rho * G * dE_H;
}
template <typename T> SGX_HD T gru_e_rho_T(const sgx_eos &e, const T temp) {
  return T(e.p[pi::gCv]) * (temp - T(e.p[pi::T0]));
}
template <typename T> SGX_HD T gru_B_rho_e(const sgx_eos &e, const T rho_in, const T sie) {
  const double *p = e.p;
  const T rho = smin(rho_in, T(p[pi::rho_max]));
  const T C0 = T(p[pi::C0]);
  if (rho < T(p[pi::rho0])) {
    return rho * (C0 * C0) + T(p[pi::G0]) * (rho * sie + gru_P_rho_e<T>(e, rho, sie));
  }
  const T dPdr_e = gru_dPdrho_e<T>(e, rho, sie);
  const T dPde_r = rho * gru_gamma<T>(e, rho);
  return rho * dPdr_e + gru_P_rho_e<T>(e, rho, sie) / rho * dPde_r;
}

// MaxStableDensityAtTemperature (eos_gruneisen.hpp:423-477). A reference
// abort (pressure decreasing at rho0) becomes *err = 1 and rho0 is returned.
SGX_HDN double gru_max_stable_density(const sgx_eos &e, const double T, int *err) {
  const double *p = e.p;
  const double slope_max = gru_dPdrho_e(e, p[pi::rho_max], gru_e_rho_T(e, T));
  const double slope_ref = gru_dPdrho_e(e, p[pi::rho0], gru_e_rho_T(e, T));
  if (slope_max >= 0) return p[pi::rho_max];
  if (slope_ref < 0) {
    if (err) *err = 1;
    return p[pi::rho0];
  }
  auto dPdrho_T = [&](const double r) { return gru_dPdrho_e(e, r, gru_e_rho_T(e, T)); };
  const double rho_lower = p[pi::rho0];
  const double rho_upper = smin(p[pi::rho_max], 1.0e4);
  const double rho_guess = (rho_lower + rho_upper) / 2.;
  double root = rho_guess;
  if (regula_falsi(dPdrho_T, 0., rho_guess, rho_lower, rho_upper, 1.0e-8, 1.0e-8, root) !=
          RootStatus::SUCCESS &&
      err)
    *err = 2;
  return root;
}

// DensityEnergyFromPressureTemperature (eos_gruneisen.hpp:478-526).
SGX_HDN void gru_rho_sie_from_PT(const sgx_eos &e, const double press, const double temp,
                                 double &rho, double &sie, int *err) {
  const double *p = e.p;
  auto PofRatT = [&](const double r) { return gru_P_rho_e(e, smin(r, p[pi::rho_max]), gru_e_rho_T(e, temp)); };
  const double Pref = PofRatT(p[pi::rho0]);
  double rho_lower, rho_upper, rho_guess, p_used = press;
  if (press < Pref) {
    rho_lower = 0.;
    rho_upper = 1.1 * p[pi::rho0];
    rho_guess = p[pi::rho0];
  } else {
    rho_lower = 0.9 * p[pi::rho0];
    rho_upper = gru_max_stable_density(e, temp, err);
    const double pres_max = PofRatT(rho_upper);
    if (press > pres_max) p_used = pres_max;
    const double slope = (rho_upper - p[pi::rho0]) / (pres_max - Pref);
    rho_guess = p[pi::rho0] + slope * (p_used - Pref);
  }
  if (regula_falsi(PofRatT, p_used, rho_guess, rho_lower, rho_upper, 1.0e-8, 1.0e-8, rho) !=
          RootStatus::SUCCESS &&
      err)
    *err = 3;
  sie = gru_e_rho_T(e, temp);
}

// ---------------------------------------------------------------------------
// Scalar member functions, dispatched on the model code.

SGX_HD unsigned preferred_input(const sgx_eos &e) {
  // IdealGas prefers pressure too (eos_ideal.hpp:227-229); the tabulated
  // models prefer rho, T (eos_spiner_rho_temp.hpp:182-183,
  // eos_spiner_rho_sie.hpp:350-351); the others rho, sie.
  if (e.type == SGX_IDEAL_GAS) return Q_DENSITY | Q_SIE | Q_TEMPERATURE | Q_PRESSURE;
  if (e.type == SGX_SPINER_RHOT || e.type == SGX_SPINER_RHOSIE) return Q_DENSITY | Q_TEMPERATURE;
  return Q_DENSITY | Q_SIE;
}

template <typename T>
SGX_HD T eos_T_from_rho_sie(const sgx_eos &e, const T rho, const T sie) {
  const T gm1 = T(e.p[pi::gm1]), Cv = T(e.p[pi::Cv]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return mymax(T(0), sie / Cv);
  case SGX_STIFF_GAS:
    return smax(lim<T>::small, ratio(rho * (sie - T(e.p[pi::qq])) - T(e.p[pi::Pinf]), rho * Cv));
  case SGX_NOBLE_ABEL:
    return smax(lim<T>::small, (sie - T(e.p[pi::qq])) / Cv);
  case SGX_GRUNEISEN:
    return T(e.p[pi::T0]) + sie / T(e.p[pi::gCv]);
  }
  (void)gm1;
  return T(0);
}

template <typename T>
SGX_HD T eos_sie_from_rho_T(const sgx_eos &e, const T rho, const T temp) {
  const T Cv = T(e.p[pi::Cv]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return mymax(T(0), Cv * temp);
  case SGX_STIFF_GAS: {
    const T qq = T(e.p[pi::qq]);
    return smax(qq, ratio(rho * Cv * temp + T(e.p[pi::Pinf]), rho) + qq);
  }
  case SGX_NOBLE_ABEL: {
    const T qq = T(e.p[pi::qq]);
    return smax(qq, Cv * temp + qq);
  }
  case SGX_GRUNEISEN:
    return T(e.p[pi::gCv]) * (temp - T(e.p[pi::T0]));
  }
  return T(0);
}

template <typename T>
SGX_HD T eos_P_from_rho_sie(const sgx_eos &e, const T rho, const T sie) {
  const T gm1 = T(e.p[pi::gm1]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return mymax(T(0), gm1 * rho * sie);
  case SGX_STIFF_GAS: {
    const T Pinf = T(e.p[pi::Pinf]);
    return smax(-Pinf, gm1 * rho * (sie - T(e.p[pi::qq])) - (gm1 + T(1.0)) * Pinf);
  }
  case SGX_NOBLE_ABEL:
    return smax(lim<T>::small,
                ratio(gm1 * rho * (sie - T(e.p[pi::qq])), T(1.0) - T(e.p[pi::bb]) * rho));
  case SGX_GRUNEISEN:
    return gru_P_rho_e<T>(e, rho, sie);
  }
  return T(0);
}

template <typename T>
SGX_HD T eos_P_from_rho_T(const sgx_eos &e, const T rho, const T temp) {
  const T gm1 = T(e.p[pi::gm1]), Cv = T(e.p[pi::Cv]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return mymax(T(0), gm1 * rho * Cv * temp);
  case SGX_STIFF_GAS: {
    const T Pinf = T(e.p[pi::Pinf]);
    return smax(-Pinf, gm1 * rho * Cv * temp - Pinf);
  }
  case SGX_NOBLE_ABEL:
    return smax(lim<T>::small, ratio(gm1 * rho * Cv * temp, T(1.0) - T(e.p[pi::bb]) * rho));
  case SGX_GRUNEISEN: {
    const T r = smin(rho, T(e.p[pi::rho_max]));
    return gru_P_rho_e<T>(e, r, gru_e_rho_T<T>(e, temp));
  }
  }
  return T(0);
}

template <typename T> SGX_HD T eos_cv(const sgx_eos &e) {
  return T(e.type == SGX_GRUNEISEN ? e.p[pi::gCv] : e.p[pi::Cv]);
}

template <typename T>
SGX_HD T eos_B_from_rho_sie(const sgx_eos &e, const T rho, const T sie) {
  const T gm1 = T(e.p[pi::gm1]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return mymax(T(0), (gm1 + 1) * gm1 * rho * sie);
  case SGX_STIFF_GAS:
    return smax(lim<T>::small, gm1 * (gm1 + T(1.0)) *
                                   (rho * (sie - T(e.p[pi::qq])) - T(e.p[pi::Pinf])));
  case SGX_NOBLE_ABEL: {
    const T omb = T(1.0) - T(e.p[pi::bb]) * rho;
    return smax(lim<T>::small,
                ratio(gm1 * (gm1 + T(1.0)) * rho * (sie - T(e.p[pi::qq])), omb * omb));
  }
  case SGX_GRUNEISEN:
    return gru_B_rho_e<T>(e, rho, sie);
  }
  return T(0);
}

template <typename T>
SGX_HD T eos_B_from_rho_T(const sgx_eos &e, const T rho, const T temp) {
  const T gm1 = T(e.p[pi::gm1]), Cv = T(e.p[pi::Cv]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return mymax(T(0), (gm1 + 1) * gm1 * rho * Cv * temp);
  case SGX_STIFF_GAS:
    return smax(lim<T>::small, gm1 * (gm1 + T(1.0)) * rho * Cv * temp);
  case SGX_NOBLE_ABEL: {
    const T omb = T(1.0) - T(e.p[pi::bb]) * rho;
    return smax(lim<T>::small, ratio(gm1 * (gm1 + T(1.0)) * rho * Cv * temp, omb * omb));
  }
  case SGX_GRUNEISEN: {
    const T r = smin(rho, T(e.p[pi::rho_max]));
    return gru_B_rho_e<T>(e, r, gru_e_rho_T<T>(e, temp));
  }
  }
  return T(0);
}

template <typename T> SGX_HD T eos_gamma(const sgx_eos &e, const T rho) {
  switch (e.type) {
  case SGX_IDEAL_GAS:
  case SGX_STIFF_GAS:
    return T(e.p[pi::gm1]);
  case SGX_NOBLE_ABEL:
    return ratio(T(e.p[pi::gm1]), (T(1.0) - T(e.p[pi::bb]) * rho));
  case SGX_GRUNEISEN:
    return gru_gamma<T>(e, smin(rho, T(e.p[pi::rho_max])));
  }
  return T(0);
}

template <typename T> SGX_HD T eos_min_sie(const sgx_eos &e, const T rho) {
  switch (e.type) {
  case SGX_IDEAL_GAS:
    return T(0);
  case SGX_NOBLE_ABEL:
    return T(e.p[pi::qq]);
  case SGX_STIFF_GAS:
    return eos_sie_from_rho_T<T>(e, rho, T(0.));
  case SGX_GRUNEISEN:
    return gru_e_rho_T<T>(e, T(0.));
  }
  return T(0);
}

// Partial derivatives of sie(rho, T) and P(rho, T) of the analytic models,
// for the Jacobian of the mixed-precision solver, where finite differences in
// FP32 cannot resolve a thermal energy that is small against a cold one.
// Returns false for tabulated and modified models.
//   IdealGas  e = Cv T, P = gm1 rho Cv T
//   StiffGas  e = Cv T + Pinf/rho + q, P = gm1 rho Cv T - Pinf
//   NobleAbel e = Cv T + q, P = gm1 rho Cv T / (1 - b rho)
//   Gruneisen e = Cv (T - T0), P = P(rho, e) (eos_gruneisen.hpp:331-371)
template <typename T>
SGX_HD bool eos_derivs(const sgx_eos &e, const T rho, const T temp, T &de_drho, T &de_dT,
                       T &dP_drho, T &dP_dT) {
  if (e.mods) return false; // modified models differentiate by finite differences
  const T gm1 = T(e.p[pi::gm1]), Cv = T(e.p[pi::Cv]);
  switch (e.type) {
  case SGX_IDEAL_GAS:
    de_drho = T(0);
    de_dT = Cv;
    dP_drho = gm1 * Cv * temp;
    dP_dT = gm1 * rho * Cv;
    return true;
  case SGX_STIFF_GAS:
    de_drho = -T(e.p[pi::Pinf]) / (rho * rho);
    de_dT = Cv;
    dP_drho = gm1 * Cv * temp;
    dP_dT = gm1 * rho * Cv;
    return true;
  case SGX_NOBLE_ABEL: {
    const T omb = T(1) - T(e.p[pi::bb]) * rho;
    de_drho = T(0);
    de_dT = Cv;
    dP_drho = gm1 * Cv * temp / (omb * omb);
    dP_dT = gm1 * rho * Cv / omb;
    return true;
  }
  case SGX_GRUNEISEN: {
    const T gCv = T(e.p[pi::gCv]);
    const T r = smin(rho, T(e.p[pi::rho_max]));
    const T sie = gru_e_rho_T<T>(e, temp);
    de_drho = T(0);
    de_dT = gCv;
    dP_drho = gru_dPdrho_e<T>(e, r, sie);
    dP_dT = gru_gamma<T>(e, r) * r * gCv;
    return true;
  }
  }
  return false;
}

// Bounds introspection (eos_base.hpp:594-613 defaults; Gruneisen overrides
// at eos_gruneisen.hpp:176-183).
SGX_HD double eos_min_temperature(const sgx_eos &) { return 0; }
SGX_HD double eos_max_density(const sgx_eos &e) {
  return e.type == SGX_GRUNEISEN ? e.p[pi::rho_max] : 1e100;
}
SGX_HD double eos_rho_pmin(const sgx_eos &, const double) { return 0.0; }
SGX_HD double eos_min_pressure(const sgx_eos &e) {
  return e.type == SGX_GRUNEISEN ? gru_P_rho_e<double>(e, 0.0, 0.0) : 0;
}
// Gruneisen returns MaxStableDensityAtTemperature here, as the reference does
// (eos_gruneisen.hpp:180-182).
SGX_HDI double eos_max_pressure_at_T(const sgx_eos &e, const double T, int *err) {
  return e.type == SGX_GRUNEISEN ? gru_max_stable_density(e, T, err) : 1e100;
}

// DensityEnergyFromPressureTemperature per model.
SGX_HDI void eos_rho_sie_from_PT(const sgx_eos &e, const double press, const double temp,
                                 double &rho, double &sie, int *err) {
  const double gm1 = e.p[pi::gm1], Cv = e.p[pi::Cv];
  switch (e.type) {
  case SGX_IDEAL_GAS:
    sie = mymax(0.0, Cv * temp);
    rho = mymax(0.0, press / (gm1 * sie));
    return;
  case SGX_STIFF_GAS: {
    const double Pinf = e.p[pi::Pinf], qq = e.p[pi::qq];
    sie = smax(qq, ratio(press + (gm1 + 1.0) * Pinf, press + Pinf) * Cv * temp + qq);
    rho = smax(lim<double>::small, ratio(press + Pinf, gm1 * Cv * temp));
    return;
  }
  case SGX_NOBLE_ABEL: {
    const double qq = e.p[pi::qq];
    sie = smax(qq, Cv * temp + qq);
    rho = smax(lim<double>::small, ratio(press, gm1 * Cv * temp + e.p[pi::bb] * press));
    return;
  }
  case SGX_GRUNEISEN:
    gru_rho_sie_from_PT(e, press, temp, rho, sie, err);
    return;
  }
}

} // namespace sgx
