// Tabulated EOS on (rho, T) and (rho, sie) grids (singularity-eos
// SpinerEOSDependsRhoSie, eos/eos_spiner_rho_sie.hpp, with the default
// NullTransform of eos_spiner_sie_transforms.hpp:40-55) on a device-resident
// table image.
//
// Unlike the rho-T model, every function of (rho, sie) is a direct bilinear
// interpolation on the table's (lRho, lE) grid -- no root find -- and every
// function of (rho, T) one on its (lRho, lT) grid. Off the grids the
// interpolation extrapolates linearly (the cell index is clamped, the
// weights are not), as the reference's DataBox::interpToReal does.
//
// Layout in device memory (one allocation, 256-byte aligned sections):
//   SieTable header (this struct, copied by value into kernels)
//   2-D fields of the rho-T group [nRhoT][nT], T index fastest:
//     sie, P, bMod (recomputed at load), dPdE, dTdE
//   2-D fields of the rho-sie group [nRhoE][nE], sie index fastest:
//     T, P, bMod (recomputed at load), dPdE, dTdE
//   1-D: sieCold on the cold-curve grid; PlRhoMax, dPdRhoMax and rho_at_pmin
//     on the T grid.
#pragma once

#include "sgx_spiner.cuh"

namespace sgx {

enum SieField2D { ST_SIE = 0, ST_P, ST_BMOD, ST_DPDE, ST_DTDE, NST2D };
enum SieFieldE2D { SE_T = 0, SE_P, SE_BMOD, SE_DPDE, SE_DTDE, NSE2D };

// One (lRho, lE) cell of the rho-sie group for the float-float FillEos: the
// four fields it outputs in difference form (FfRec: f = x + a dE + b dR +
// a b dRE over the cell's unit square, a the lE weight, b the density
// weight), 128 bytes, one cache line per query.
struct alignas(128) SieCellFF {
  FfRec T, P, dTdE, bMod;
};

struct SieTable {
  Grid1D gT, gRhoT;  // rho-T group: T grid (fastest), density grid
  Grid1D gE, gRhoE;  // rho-sie group: lE grid (fastest), density grid
  Grid1D gCold;      // cold curve (sieCold)
  double lRhoOffset, lTOffset, lEOffset;
  double lRhoMin, lRhoMax, rhoMax, PMin;
  // ValuesAtReferenceState (eos_spiner_rho_sie.hpp:528-548, 901-915)
  double rhoNormal, TNormal, sieNormal, PNormal, CvNormal, bModNormal, dPdENormal,
      dVdTNormal;
  int nRhoT, nT, nRhoE, nE;
  int reproducible, pad;
  const double *fT[NST2D]; // rho-T group
  const double *fE[NSE2D]; // rho-sie group
  const double *sieCold, *PlRhoMax, *dPdRhoMax, *rho_at_pmin;
  // float-float FillEos from (rho, sie): the cells [nRhoE-1][nE-1] (null when
  // a value lies outside the float range) and, per axis (0 density, 1
  // energy), the cell coordinate u = (lX - min) / dx in fixed point from
  // the NQT log's integer v (lX = v scale_down log10(2)):
  // u 2^fxF = mulhi64(v, fxM) - fxOff
  const SieCellFF *cellsE;
  long long fxM[2], fxOff[2];
  int fxF[2];
};

// DataBox::interpToReal(x2 = lRho, x1 = fast coordinate) on one group.
SGX_HD double sie_interp2(const Grid1D &gx, const Grid1D &gr, const int nx, const double *d,
                          const double lRho, const double x) {
  int i, j;
  double a0, a1, b0, b1;
  gx.weights(x, i, a0, a1);
  gr.weights(lRho, j, b0, b1);
  const double *r0 = d + j * nx + i;
  const double *r1 = r0 + nx;
  return b0 * (a0 * r0[0] + a1 * r0[1]) + b1 * (a0 * r1[0] + a1 * r1[1]);
}
SGX_HD double st_interp(const SieTable &t, const int f, const double lRho, const double lT) {
  return sie_interp2(t.gT, t.gRhoT, t.nT, t.fT[f], lRho, lT);
}
SGX_HD double se_interp(const SieTable &t, const int f, const double lRho, const double lE) {
  return sie_interp2(t.gE, t.gRhoE, t.nE, t.fE[f], lRho, lE);
}

// Coordinates (spiner_common::to_log / from_log, eos_spiner_common.hpp:52-57)
SGX_HD double ss_lRho(const SieTable &t, const double rho) { return to_log(rho, t.lRhoOffset); }
SGX_HD double ss_lT(const SieTable &t, const double T) { return to_log(T, t.lTOffset); }
// NullTransform: the energy coordinate is the energy itself
SGX_HD double ss_lE(const SieTable &t, const double sie) { return to_log(sie, t.lEOffset); }

// interpRhoT_ / interpRhoSie_ (:917-941): both write the lambda cache lRho.
SGX_HD double ss_rhoT(const SieTable &t, const int f, const double rho, const double T,
                      double *lam) {
  const double lRho = ss_lRho(t, rho);
  const double lT = ss_lT(t, T);
  if (lam != nullptr) lam[0] = lRho;
  return st_interp(t, f, lRho, lT);
}
SGX_HD double ss_rhoE(const SieTable &t, const int f, const double rho, const double sie,
                      double *lam) {
  const double lRho = ss_lRho(t, rho);
  const double lE = ss_lE(t, sie);
  if (lam != nullptr) lam[0] = lRho;
  return se_interp(t, f, lRho, lE);
}

// Public scalar member functions (:654-759)
SGX_HDN double ss_T_from_rho_sie(const SieTable &t, const double rho, const double sie,
                                 double *lam) {
  return ss_rhoE(t, SE_T, rho, sie, lam);
}
SGX_HDN double ss_sie_from_rho_T(const SieTable &t, const double rho, const double T,
                                 double *lam) {
  return ss_rhoT(t, ST_SIE, rho, T, lam);
}
SGX_HDN double ss_P_from_rho_T(const SieTable &t, const double rho, const double T, double *lam) {
  return ss_rhoT(t, ST_P, rho, T, lam);
}
SGX_HDN double ss_P_from_rho_sie(const SieTable &t, const double rho, const double sie,
                                 double *lam) {
  return ss_rhoE(t, SE_P, rho, sie, lam);
}
SGX_HDN double ss_min_sie(const SieTable &t, const double rho) {
  return interp1(t.gCold, t.sieCold, ss_lRho(t, rho));
}
SGX_HDN double ss_cv_from_rho_T(const SieTable &t, const double rho, const double T, double *lam) {
  return 1. / ss_rhoT(t, ST_DTDE, rho, T, lam);
}
SGX_HDN double ss_cv_from_rho_sie(const SieTable &t, const double rho, const double sie,
                                  double *lam) {
  return 1. / ss_rhoE(t, SE_DTDE, rho, sie, lam);
}
SGX_HDN double ss_bmod_from_rho_T(const SieTable &t, const double rho, const double T,
                                  double *lam) {
  return ss_rhoT(t, ST_BMOD, rho, T, lam);
}
SGX_HDN double ss_bmod_from_rho_sie(const SieTable &t, const double rho, const double sie,
                                    double *lam) {
  return ss_rhoE(t, SE_BMOD, rho, sie, lam);
}
SGX_HDN double ss_gamma_from_rho_T(const SieTable &t, const double rho, const double T,
                                   double *lam) {
  const double dpde = ss_rhoT(t, ST_DPDE, rho, T, lam);
  return dpde / rho;
}
// GruneisenParamFromDensityInternalEnergy (:753-762) leaves the cache alone.
SGX_HDN double ss_gamma_from_rho_sie(const SieTable &t, const double rho, const double sie,
                                     double *) {
  const double dpde = se_interp(t, SE_DPDE, ss_lRho(t, rho), ss_lE(t, sie));
  return dpde / rho;
}
// RhoPmin (:267-270): rho_at_pmin at lT, extrapolated like any 1-D box.
SGX_HDN double ss_rho_pmin(const SieTable &t, const double T) {
  return interp1(t.gT, t.rho_at_pmin, ss_lT(t, T));
}
// lRhoFromPlT_ (:942-987): past the table's densest row (where P rises with
// density) linear in rho; otherwise regula falsi on P(lRho, lT) over
// [lRho(rho_at_pmin), lRhoMax], from the cache when it lies in that range.
SGX_HD double ss_lRho_from_P_lT(const SieTable &t, const double P, const double lT,
                                double *lam) {
  const double rhopmin = ss_lRho(t, interp1(t.gT, t.rho_at_pmin, lT));
  double lRho;
  const double dPdRhoMax = interp1(t.gT, t.dPdRhoMax, lT);
  const double PMax = interp1(t.gT, t.PlRhoMax, lT);
  if (dPdRhoMax > 0 && P > PMax) {
    const double rho = (P - PMax) / dPdRhoMax + t.rhoMax;
    lRho = ss_lRho(t, rho);
  } else {
    double lRhoGuess = t.reproducible ? t.lRhoMax : 0.5 * (rhopmin + t.lRhoMax);
    if (lam != nullptr) {
      const double c = lam[0];
      if ((rhopmin <= c) && (c <= t.lRhoMax)) lRhoGuess = c;
    }
    auto PFunc = [&](const double x) { return st_interp(t, ST_P, x, lT); };
    const RootStatus st = regula_falsi(PFunc, P, lRhoGuess, rhopmin, t.lRhoMax,
                                       lim<double>::eps, lim<double>::eps, lRho);
    if (st != RootStatus::SUCCESS) lRho = t.reproducible ? t.lRhoMax : lRhoGuess;
  }
  if (lam != nullptr) lam[0] = lRho;
  return lRho;
}
// DensityEnergyFromPressureTemperature (:834-842)
SGX_HDN void ss_rho_sie_from_PT(const SieTable &t, const double P, const double T, double &rho,
                                double &sie, double *lam) {
  const double lT = ss_lT(t, T);
  const double lRho = ss_lRho_from_P_lT(t, P, lT, lam);
  rho = from_log(lRho, t.lRhoOffset);
  sie = st_interp(t, ST_SIE, lRho, lT);
}

} // namespace sgx
