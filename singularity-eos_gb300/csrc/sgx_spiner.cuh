// Tabulated rho-T EOS (singularity-eos SpinerEOSDependsRhoT,
// eos/eos_spiner_rho_temp.hpp) on a device-resident table image.
//
// Layout in device memory (one allocation, 256-byte aligned sections):
//   SpinerTable header (this struct, copied by value into kernels)
//   2-D fields [nRho][nT], T index fastest (the reference's P_(jRho, iT)):
//     P, sie, bMod, dPdRho, dPdE, dTdRho, dTdE, dEdRho, dEdT
//   1-D fields on the density grid [nRho]: PMax, sielTMax, dEdTMax, gm1Max
//   1-D fields on the cold-curve grid [nRho]: lTColdCrit, PCold, sieCold,
//     bModCold, dPdRhoCold, dPdECold, dTdRhoCold, dTdECold, dEdTCold
//   1-D field on the temperature grid [nT]: rho_at_pmin
//   corner-packed copies for the lookup hot loop: for each cell (j, i) of the
//     grid the four corner values {f(j,i), f(j,i+1), f(j+1,i), f(j+1,i+1)}
//     as one 32-byte dq4 (sie, P, bMod) and one 16-byte fq4 (sie, for
//     the FP32 search), so one bilinear evaluation is one aligned sector load.
//
// Interpolation follows the spiner-lite formula used by the oracle (uniform
// grid, cell index clamped to [0, N-2], weights w1 = (x - x_i)/dx,
// w0 = 1 - w1), with the same operation order.
#pragma once

#include "sgx_math.cuh"

namespace sgx {

// 32- and 16-byte aligned quads (a corner-packed interpolation cell).
struct alignas(32) dq4 {
  double x, y, z, w;
};
struct alignas(16) fq4 {
  float x, y, z, w;
};
// One interpolation cell in difference form, for the float-float lookup:
// f(a, b) = x + a dT + b dR + a b dRT over the cell's unit square (a: T
// weight, b: density weight), the differences formed in FP64 on the host.
// sie keeps FP64 (the root's numerator sie - x - b dR cancels where the cold
// energy dominates); the other fields are float pairs (hi, lo).
struct alignas(32) SieRec {
  double x, dT, dR, dRT;
};
struct alignas(16) FfRec {
  float x[2], dT[2], dR[2], dRT[2];
};

struct Grid1D {
  double min, max, dx, inv_dx;
  int n, pad;
  SGX_HD int index(const double x) const {
    const double u = (x - min) * inv_dx;
    if (!(u >= 0)) return 0;
    if (u > static_cast<double>(n - 2)) return n - 2;
    return static_cast<int>(u);
  }
  SGX_HD void weights(const double x, int &ix, double &w0, double &w1) const {
    ix = index(x);
    const double xl = min + ix * dx;
    w1 = (x - xl) * inv_dx;
    w0 = 1 - w1;
  }
  SGX_HD double x(const int i) const { return min + i * dx; }
};

enum SpinerField2D { F_P = 0, F_SIE, F_BMOD, F_DPDRHO, F_DPDE, F_DTDRHO, F_DTDE, F_DEDRHO, F_DEDT, NF2D };
enum SpinerField1D {
  F_PMAX = 0, F_SIELTMAX, F_DEDTMAX, F_GM1MAX, // density grid
  F_LTCOLDCRIT, F_PCOLD, F_SIECOLD, F_BMODCOLD, F_DPDRHOCOLD, F_DPDECOLD, F_DTDRHOCOLD,
  F_DTDECOLD, F_DEDTCOLD, // cold-curve grid
  F_RHO_AT_PMIN,          // temperature grid
  NF1D
};

struct SpinerTable {
  Grid1D gT, gRho, gCold; // T grid (fastest), rho grid, cold-curve grid
  double lRhoMin, lRhoMax, rhoMax, lTMin, lTMax, TMax, PMin, lRhoOffset, lTOffset;
  double TNormal; // reference-state temperature (ValuesAtReferenceState)
  // reference-state density, pressure and bulk modulus (:663-684)
  double rhoNormal, PNormal, bModNormal;
  double TatlTMin; // T_(lTMin_): the temperature returned off the table's bottom
  int nRho, nT;
  int reproducible;
  // 1 when sie increases strictly along T in every density row, which makes
  // T(rho, sie) a unique root that a bracketing search can locate directly.
  int sie_monotone_T;
  const double *f2[NF2D];
  const double *f1[NF1D];
  const dq4 *sie4, *P4, *bmod4; // corner-packed [nRho-1][nT-1]
  const fq4 *sie4f;               // corner-packed FP32 copy of sie
  const float *sieCold32, *sielTMax32; // FP32 copies of the on-table bounds
  // float-float records [nRho-1][nT-1]; ff_ok = 0 when a value is outside
  // the float exponent range (the lookups then take the FP64 iteration)
  const SieRec *sieR;
  const FfRec *PR, *bmodR;
  const double *rhoNodes; // Grid1D node positions min + j * dx, rounded as weights() rounds them
  // every coarse_stride-th T node of each density cell's two rows
  // ([nRho-1][SP_COARSE_ROW], (sie(j, i), sie(j+1, i)), +inf past the last
  // cell and in the row padding), staged in shared memory by the lookup to
  // shorten its search
  const float2 *sieCoarse;
  int coarse_stride;
  int ff_ok;
  // Thermal-energy bin index of each density row (null when the table does
  // not allow one): for the thermal part t_r(i) = sie(r, i) - sieCold(r),
  // bins log-spaced by the float bit pattern (bin = (bits(t) >> therm_shift)
  // - therm_base, therm_bins of them, finer than the T cells), therm_idx[r *
  // therm_bins + k] is the last T cell whose lower node lies at or below the
  // bin's lower edge. The root of a density blend of rows r and r + 1 lies
  // between the two rows' cells for the blended thermal target.
  const uint16_t *therm_idx;
  int therm_bins, therm_shift, therm_base;
};
constexpr int SP_COARSE = 16;
// Row length of the coarse index in memory: 16 entries and 2 of padding,
// 144 bytes, so that rows and the whole index are multiples of 16 bytes (a
// bulk copy's unit) and lanes probing the same entry of different rows
// spread over the banks.
constexpr int SP_COARSE_ROW = SP_COARSE + 2;

// ---- interpolation (DataBox::interpToReal) ----
SGX_HD double interp1(const Grid1D &g, const double *d, const double x) {
  int i;
  double w0, w1;
  g.weights(x, i, w0, w1);
  return w0 * d[i] + w1 * d[i + 1];
}
SGX_HD double interp2(const SpinerTable &t, const double *d, const double lRho,
                      const double lT) {
  int i, j;
  double a0, a1, b0, b1;
  t.gT.weights(lT, i, a0, a1);
  t.gRho.weights(lRho, j, b0, b1);
  const double *r0 = d + j * t.nT + i;
  const double *r1 = r0 + t.nT;
  return b0 * (a0 * r0[0] + a1 * r0[1]) + b1 * (a0 * r1[0] + a1 * r1[1]);
}
// Same value from a corner-packed field: one 32-byte load.
SGX_HD double interp2_packed(const SpinerTable &t, const dq4 *d4, const double lRho,
                             const double lT) {
  int i, j;
  double a0, a1, b0, b1;
  t.gT.weights(lT, i, a0, a1);
  t.gRho.weights(lRho, j, b0, b1);
  const dq4 c = d4[j * (t.nT - 1) + i];
  return b0 * (a0 * c.x + a1 * c.y) + b1 * (a0 * c.z + a1 * c.w);
}

// ---- coordinate transforms (eos_spiner_rho_temp.hpp:142-156) ----
SGX_HD double sp_lRho(const SpinerTable &t, const double rho) { return to_log(rho, t.lRhoOffset); }
SGX_HD double sp_lT(const SpinerTable &t, const double T) { return to_log(T, t.lTOffset); }
SGX_HD double sp_rho(const SpinerTable &t, const double lRho) {
  const double rho = from_log(lRho, t.lRhoOffset);
  return rho < 0 ? 0 : rho;
}
SGX_HD double sp_T(const SpinerTable &t, const double lT) { return from_log(lT, t.lTOffset); }

enum class TableStatus : int { OnTable = 0, OffBottom = 1, OffTop = 2 };
constexpr double SP_ROOT_THRESH = 1e-14; // eos_spiner_rho_temp.hpp:364
constexpr double SP_SOFT_THRESH = 1e-8;  // :365

// getLocDependsRhoSie_ (:1377-1392)
SGX_HD TableStatus sp_loc_rho_sie(const SpinerTable &t, const double lRho, const double sie) {
  const double sielTMax = interp1(t.gRho, t.f1[F_SIELTMAX], lRho);
  const double sieCold = interp1(t.gCold, t.f1[F_SIECOLD], lRho);
  if (sie >= sielTMax - SP_SOFT_THRESH * sabs(sielTMax)) return TableStatus::OffTop;
  if (sie <= sieCold + SP_SOFT_THRESH * sabs(sieCold)) return TableStatus::OffBottom;
  return TableStatus::OnTable;
}
// getLocDependsRhoT_ (:1394-1404)
SGX_HD TableStatus sp_loc_rho_T(const SpinerTable &t, const double, const double lT) {
  if (lT <= (1 + SP_SOFT_THRESH) * t.lTMin) return TableStatus::OffBottom;
  if (lT >= (1 - SP_SOFT_THRESH) * t.lTMax) return TableStatus::OffTop;
  return TableStatus::OnTable;
}

// lTFromlRhoSie_ (:1192-1250). lam (nullable) is the lambda row
// {lRho, lT}; a missing cache means "no guess" (midpoint start).
SGX_HD double sp_lT_from_lRho_sie(const SpinerTable &t, const double lRho, const double sie,
                                  TableStatus &where, double *lam, int *iters = nullptr) {
  double lT;
  where = sp_loc_rho_sie(t, lRho, sie);
  if (where == TableStatus::OffBottom) {
    lT = t.lTMin;
  } else if (where == TableStatus::OffTop) {
    const double Cv = interp1(t.gRho, t.f1[F_DEDTMAX], lRho);
    const double e0 = interp1(t.gRho, t.f1[F_SIELTMAX], lRho);
    const double Tk = t.TMax + ratio(sie - e0, Cv);
    lT = sp_lT(t, Tk);
  } else {
    double lTGuess = t.reproducible ? t.lTMin : 0.5 * (t.lTMin + t.lTMax);
    if (lam != nullptr) {
      const double c = lam[1];
      if ((t.lTMin <= c) && (c <= t.lTMax)) lTGuess = c;
    }
    auto sieFunc = [&](const double x) { return interp2_packed(t, t.sie4, lRho, x); };
    const RootStatus st = regula_falsi(sieFunc, sie, lTGuess, t.lTMin, t.lTMax, SP_ROOT_THRESH,
                                       SP_ROOT_THRESH, lT, iters);
    if (st != RootStatus::SUCCESS) lT = t.reproducible ? t.lTMin : lTGuess;
  }
  if (lam != nullptr) {
    lam[0] = lRho;
    lam[1] = lT;
  }
  return lT;
}

// sieFromlRhoTlT_, PFromRholRhoTlT_, CvFromlRholT_, bModFromRholRhoTlT_
// (:1307-1375)
SGX_HD double sp_sie_from(const SpinerTable &t, const double lRho, const double Tk,
                          const double lT, const TableStatus w) {
  if (w == TableStatus::OffBottom) return interp1(t.gCold, t.f1[F_SIECOLD], lRho);
  if (w == TableStatus::OffTop) {
    const double Cv = interp1(t.gRho, t.f1[F_DEDTMAX], lRho);
    const double e0 = interp1(t.gRho, t.f1[F_SIELTMAX], lRho);
    return e0 + Cv * (Tk - t.TMax);
  }
  return interp2_packed(t, t.sie4, lRho, lT);
}
SGX_HD double sp_P_from(const SpinerTable &t, const double rho, const double lRho,
                        const double Tk, const double lT, const TableStatus w) {
  if (w == TableStatus::OffBottom) return interp1(t.gCold, t.f1[F_PCOLD], lRho);
  if (w == TableStatus::OffTop) {
    const double Cv = interp1(t.gRho, t.f1[F_DEDTMAX], lRho);
    const double gm1 = interp1(t.gRho, t.f1[F_GM1MAX], lRho);
    const double e0 = interp1(t.gRho, t.f1[F_SIELTMAX], lRho);
    const double e = e0 + Cv * (Tk - t.TMax);
    return gm1 * rho * e;
  }
  return interp2_packed(t, t.P4, lRho, lT);
}
SGX_HD double sp_cv_from(const SpinerTable &t, const double lRho, const double lT,
                         const TableStatus w) {
  double Cv;
  if (w == TableStatus::OffBottom)
    Cv = interp1(t.gCold, t.f1[F_DEDTCOLD], lRho);
  else if (w == TableStatus::OffTop)
    Cv = interp1(t.gRho, t.f1[F_DEDTMAX], lRho);
  else
    Cv = interp2(t, t.f2[F_DEDT], lRho, lT);
  return Cv > lim<double>::eps ? Cv : lim<double>::eps;
}
SGX_HD double sp_bmod_from(const SpinerTable &t, const double rho, const double lRho,
                           const double Tk, const double lT, const TableStatus w) {
  double bMod;
  if (w == TableStatus::OffBottom) {
    bMod = interp1(t.gCold, t.f1[F_BMODCOLD], lRho);
  } else if (w == TableStatus::OffTop) {
    const double Cv = interp1(t.gRho, t.f1[F_DEDTMAX], lRho);
    const double gm1 = interp1(t.gRho, t.f1[F_GM1MAX], lRho);
    const double e0 = interp1(t.gRho, t.f1[F_SIELTMAX], lRho);
    const double e = e0 + Cv * (Tk - t.TMax);
    bMod = (gm1 + 1) * gm1 * rho * e;
  } else {
    bMod = interp2_packed(t, t.bmod4, lRho, lT);
  }
  return bMod > lim<double>::eps ? bMod : lim<double>::eps;
}

// getLogsRhoT_ (:1125-1133): also writes the lambda cache.
SGX_HD void sp_logs_rho_T(const SpinerTable &t, const double rho, const double Tk,
                          double &lRho, double &lT, double *lam) {
  lRho = sp_lRho(t, rho);
  lT = sp_lT(t, Tk);
  if (lam != nullptr) {
    lam[0] = lRho;
    lam[1] = lT;
  }
}

// Public scalar member functions (:777-935)
SGX_HDN double sp_T_from_rho_sie(const SpinerTable &t, const double rho, const double sie,
                                double *lam) {
  TableStatus w;
  const double lRho = sp_lRho(t, rho);
  return sp_T(t, sp_lT_from_lRho_sie(t, lRho, sie, w, lam));
}
SGX_HDN double sp_sie_from_rho_T(const SpinerTable &t, const double rho, const double Tk,
                                double *lam) {
  double lRho, lT;
  sp_logs_rho_T(t, rho, Tk, lRho, lT, lam);
  return sp_sie_from(t, lRho, Tk, lT, sp_loc_rho_T(t, lRho, lT));
}
SGX_HDN double sp_P_from_rho_T(const SpinerTable &t, const double rho, const double Tk,
                              double *lam) {
  double lRho, lT;
  sp_logs_rho_T(t, rho, Tk, lRho, lT, lam);
  return sp_P_from(t, rho, lRho, Tk, lT, sp_loc_rho_T(t, lRho, lT));
}
SGX_HDN double sp_P_from_rho_sie(const SpinerTable &t, const double rho, const double sie,
                                double *lam) {
  TableStatus w;
  const double lRho = sp_lRho(t, rho);
  const double lT = sp_lT_from_lRho_sie(t, lRho, sie, w, lam);
  if (w == TableStatus::OffBottom) return interp1(t.gCold, t.f1[F_PCOLD], lRho);
  if (w == TableStatus::OffTop) {
    const double gm1 = interp1(t.gRho, t.f1[F_GM1MAX], lRho);
    return gm1 * rho * sie;
  }
  return interp2_packed(t, t.P4, lRho, lT);
}
SGX_HDN double sp_min_sie(const SpinerTable &t, const double rho) {
  return interp1(t.gCold, t.f1[F_SIECOLD], sp_lRho(t, rho));
}
SGX_HDN double sp_cv_from_rho_T(const SpinerTable &t, const double rho, const double Tk,
                               double *lam) {
  double lRho, lT;
  sp_logs_rho_T(t, rho, Tk, lRho, lT, lam);
  return sp_cv_from(t, lRho, lT, sp_loc_rho_T(t, lRho, lT));
}
SGX_HDN double sp_cv_from_rho_sie(const SpinerTable &t, const double rho, const double sie,
                                 double *lam) {
  TableStatus w;
  const double lRho = sp_lRho(t, rho);
  const double lT = sp_lT_from_lRho_sie(t, lRho, sie, w, lam);
  double Cv;
  if (w == TableStatus::OffBottom)
    Cv = interp1(t.gCold, t.f1[F_DEDTCOLD], lRho);
  else if (w == TableStatus::OffTop)
    Cv = interp1(t.gRho, t.f1[F_DEDTMAX], lRho);
  else
    Cv = interp2(t, t.f2[F_DEDT], lRho, lT);
  return Cv > lim<double>::eps ? Cv : lim<double>::eps;
}
SGX_HDN double sp_bmod_from_rho_T(const SpinerTable &t, const double rho, const double Tk,
                                 double *lam) {
  double lRho, lT;
  sp_logs_rho_T(t, rho, Tk, lRho, lT, lam);
  return sp_bmod_from(t, rho, lRho, Tk, lT, sp_loc_rho_T(t, lRho, lT));
}
SGX_HDN double sp_bmod_from_rho_sie(const SpinerTable &t, const double rho, const double sie,
                                   double *lam) {
  TableStatus w;
  const double lRho = sp_lRho(t, rho);
  const double lT = sp_lT_from_lRho_sie(t, lRho, sie, w, lam);
  if (w == TableStatus::OffBottom) return interp1(t.gCold, t.f1[F_BMODCOLD], lRho);
  if (w == TableStatus::OffTop) {
    const double gm1 = interp1(t.gRho, t.f1[F_GM1MAX], lRho);
    return (gm1 + 1) * gm1 * rho * sie;
  }
  return interp2_packed(t, t.bmod4, lRho, lT);
}
// Gruneisen parameter (:878-935): |dPdE| / |rho| on table and cold curve.
SGX_HD double sp_gamma_from(const SpinerTable &t, const double rho, const double lRho,
                            const double lT, const TableStatus w) {
  if (w == TableStatus::OffBottom)
    return ratio(sabs(interp1(t.gCold, t.f1[F_DPDECOLD], lRho)), sabs(rho));
  if (w == TableStatus::OffTop) return interp1(t.gRho, t.f1[F_GM1MAX], lRho);
  return ratio(sabs(interp2(t, t.f2[F_DPDE], lRho, lT)), sabs(rho));
}
SGX_HDN double sp_gamma_from_rho_T(const SpinerTable &t, const double rho, const double Tk,
                                  double *lam) {
  double lRho, lT;
  sp_logs_rho_T(t, rho, Tk, lRho, lT, lam);
  return sp_gamma_from(t, rho, lRho, lT, sp_loc_rho_T(t, lRho, lT));
}
SGX_HDN double sp_gamma_from_rho_sie(const SpinerTable &t, const double rho, const double sie,
                                    double *lam) {
  TableStatus w;
  const double lRho = sp_lRho(t, rho);
  const double lT = sp_lT_from_lRho_sie(t, lRho, sie, w, lam);
  return sp_gamma_from(t, rho, lRho, lT, w);
}
// RhoPmin (:1117-1123)
SGX_HDN double sp_rho_pmin(const SpinerTable &t, const double Tk) {
  const double lT = sp_lT(t, Tk);
  if (lT <= t.lTMin) return t.f1[F_RHO_AT_PMIN][0];
  if (lT >= t.lTMax) return 0.0;
  return interp1(t.gT, t.f1[F_RHO_AT_PMIN], lT);
}
// lRhoFromPlT_ (:1135-1190), only the on-table and two off-table branches;
// the 1-D callables are r_interp/l_interp/prod_interp_1d
// (eos_spiner_common.hpp:222-274).
SGX_HD double sp_lRho_from_P_lT(const SpinerTable &t, const double P, const double lT,
                                TableStatus &w, double *lam) {
  const double rhopmin = sp_lRho(t, interp1(t.gT, t.f1[F_RHO_AT_PMIN], lT));
  double lRho;
  double lRhoGuess = t.reproducible ? t.lRhoMax : 0.5 * (rhopmin + t.lRhoMax);
  if (lam != nullptr) {
    const double c = lam[0];
    if ((rhopmin <= c) && (c <= t.lRhoMax)) lRhoGuess = c;
  }
  RootStatus st;
  if (lT <= t.lTMin) {
    w = TableStatus::OffBottom;
    auto PFunc = [&](const double x) { return interp1(t.gCold, t.f1[F_PCOLD], x); };
    st = regula_falsi(PFunc, P, lRhoGuess, rhopmin, t.lRhoMax, SP_ROOT_THRESH, SP_ROOT_THRESH,
                      lRho);
  } else if (lT >= t.lTMax) {
    w = TableStatus::OffTop;
    auto PFunc = [&](const double x) {
      return interp1(t.gRho, t.f1[F_GM1MAX], x) * interp1(t.gRho, t.f1[F_DEDTMAX], x) * lT * x;
    };
    st = regula_falsi(PFunc, P, lRhoGuess, rhopmin, t.lRhoMax, SP_ROOT_THRESH, SP_ROOT_THRESH,
                      lRho);
  } else {
    w = TableStatus::OnTable;
    auto PFunc = [&](const double x) { return interp2(t, t.f2[F_P], x, lT); };
    st = regula_falsi(PFunc, P, lRhoGuess, rhopmin, t.lRhoMax, SP_ROOT_THRESH, SP_ROOT_THRESH,
                      lRho);
  }
  if (st != RootStatus::SUCCESS) lRho = t.reproducible ? t.lRhoMax : lRhoGuess;
  if (lam != nullptr) {
    lam[0] = lRho;
    lam[1] = lT;
  }
  return lRho;
}
// DensityEnergyFromPressureTemperature (:1006-1014)
SGX_HDN void sp_rho_sie_from_PT(const SpinerTable &t, const double P, const double Tk,
                               double &rho, double &sie, double *lam) {
  TableStatus w;
  const double lT = sp_lT(t, Tk);
  const double lRho = sp_lRho_from_P_lT(t, P, lT, w, lam);
  rho = sp_rho(t, lRho);
  sie = sp_sie_from_rho_T(t, rho, Tk, lam);
}

} // namespace sgx
