// The Helmholtz EOS (Timmes & Swesty 2000) on the device: radiation, ideal
// ions, the tabulated electron-positron free energy (biquintic Hermite for F
// and its first derivatives, bicubic for dP/dDe, eta and the pair density)
// and Coulomb corrections, combined into P, e, s and their derivatives; the
// inversion T(rho, e) by Newton-Raphson with regula-falsi and analytic
// fallbacks. Follows singularity-eos eos/eos_helmholtz.hpp operation by
// operation (with --fmad=false the only differences from the host are the
// last bits of log/log10/exp/cbrt).
//
// Table layout (built by sgx_table.cu): one record of 84 doubles per table
// cell (jT, iRho) -- the 36 biquintic coefficients in the order the
// reference's fi[] cache uses, then the 16 bicubic coefficients of each of
// dP/dDe, eta and the pair density -- so one evaluation reads 2 x 288 bytes
// of contiguous, L2-resident memory instead of 84 scattered doubles.
#pragma once

#include <cuda_runtime.h>

#include "sgx_eos.cuh"
#include "sgx_math.cuh"

namespace sgx {

constexpr int HELM_NT = 101;
constexpr int HELM_NRHO = 271;
constexpr int HELM_REC = 84;

// Option bits of sgx_eos.flags for SGX_HELMHOLTZ.
enum : int {
  HELM_RAD = 1,
  HELM_GAS = 2,
  HELM_COUL = 4,
  HELM_ION = 8,
  HELM_ELE = 16,
  HELM_REGULA_FALSI = 32,  // Options::USE_NEWTON_RAPHSON = false
  HELM_CACHE_READBACK = 64 // reproduce the reference's lT cache read-back
};

struct HelmTable {
  const double *cells; // [HELM_NT - 1][HELM_NRHO - 1][HELM_REC]
  // FP32 copy of each cell's biquintic free-energy coefficients in the
  // cell's normalised coordinates ([HELM_NT - 1][HELM_NRHO - 1][36], the
  // 6 x 6 products of T and density Hermite weights, T-major), for the
  // FP32 Newton phase of the mixed-precision inversion; null when a
  // coefficient lies outside the float range
  const float *cells32;
  const double *rho;   // [HELM_NRHO] node densities 10^lRho
  const double *T;     // [HELM_NT] node temperatures 10^lT
  // RegularGrid1D of lRho (range(0)) and lT (range(1))
  double lRhoMin, lRhoMax, dlRho, inv_dlRho;
  double lTMin, lTMax, dlT, inv_dlT;
  double rhoMin, rhoMax;
  // The FP32 phase's copies, rounded to float at load (a double-to-float
  // conversion issues on the FP64 pipe): the nodes (with cells32) and the
  // grid constants
  const float *rho32, *T32;
  float f_lRhoMin, f_lRhoMax, f_inv_dlRho, f_lTMin, f_inv_dlT, f_rhoMin, f_rhoMax;
};

namespace helm {

// Physical constants as the reference states them (eos_helmholtz.hpp:280-340).
constexpr double STEFAN_BOLTZMANN = 5.67040047374e-5;
constexpr double CL = 2.99792458e10;
constexpr double SIG_O_C = STEFAN_BOLTZMANN / CL;
constexpr double RAD_PREFACTOR = (4. / 3.) * SIG_O_C;
constexpr double KB = 1.3806504e-16;
constexpr double NA = 6.02214199e23;
constexpr double KBNA = KB * NA;
constexpr double KBi = 1.0 / KB;
constexpr double LSWOT15 = 46.682612633059801;
constexpr double LN10 = 2.30258509299405e+00;
constexpr double ELECTRON_CHARGE_ESU = 4.80320427e-10;
constexpr double PI = 3.14159265358979323846;
constexpr double E_CONST = 2.7182818284590452354;
constexpr double ROOT_THRESH = 1e-14;
constexpr double HELM_EOS_EPS = 1e-10;
constexpr int NEWTON_MAX_ITER = 100; // NEWTON_RAPHSON_NITER_MAX
enum { VAL = 0, DDR = 1, DDT = 2, DDA = 3, DDZ = 4 };

// math_utils::pow<P> (base/math_utils.hpp:31-49): the same recursion, so
// the products round the same way.
template <int P> struct IPow {
  static SGX_HDI double of(const double x) {
    if constexpr (P == 0)
      return 1.0;
    else if constexpr (P == 1)
      return x;
    else if constexpr (P % 2)
      return x * IPow<P - 1>::of(x);
    else
      return IPow<P / 2>::of(x) * IPow<P / 2>::of(x);
  }
};

// math_utils::pow10 (:56-59)
SGX_HDI double pow10e(const double x) {
#if defined(__CUDA_ARCH__)
  return exp(LN10 * x);
#else
  return __builtin_exp(LN10 * x);
#endif
}

// Hermite basis functions (base/hermite.hpp:25-94).
SGX_HDI double psi0(double z) { return z * z * z * (z * (-6.0 * z + 15.0) - 10.0) + 1.0; }
SGX_HDI double dpsi0(double z) { return z * z * (z * (-30.0 * z + 60.0) - 30.0); }
SGX_HDI double ddpsi0(double z) { return z * (z * (-120.0 * z + 180.0) - 60.0); }
SGX_HDI double psi1(double z) { return z * (z * z * (z * (-3.0 * z + 8.0) - 6.0) + 1.0); }
SGX_HDI double dpsi1(double z) { return z * z * (z * (-15.0 * z + 32.0) - 18.0) + 1.0; }
SGX_HDI double ddpsi1(double z) { return z * (z * (-60.0 * z + 96.0) - 36.0); }
SGX_HDI double psi2(double z) { return 0.5 * z * z * (z * (z * (-z + 3.0) - 3.0) + 1.0); }
SGX_HDI double dpsi2(double z) { return 0.5 * z * (z * (z * (-5.0 * z + 12.0) - 9.0) + 2.0); }
SGX_HDI double ddpsi2(double z) { return 0.5 * (z * (z * (-20.0 * z + 36.0) - 18.0) + 2.0); }
SGX_HDI double xpsi0(double z) { return z * z * (2.0 * z - 3.0) + 1.0; }
SGX_HDI double xdpsi0(double z) { return z * (6.0 * z - 6.0); }
SGX_HDI double xpsi1(double z) { return z * (z * (z - 2.0) + 1.0); }
SGX_HDI double xdpsi1(double z) { return z * (3.0 * z - 4.0) + 1.0; }

// The density and T weight of each of the 36 biquintic terms, in the
// reference's order (hermite.hpp h5): (d0,t0) (d0m,t0) (d0,t0m) (d0m,t0m)
// then t1, t2 with d0; then d1, d2 with t0; d1, d2 with t1; d1, d2 with t2.
// Weight index: 0 psi0(x), 1 psi0(1-x), 2 psi1(x) dx, 3 -psi1(1-x) dx,
// 4 psi2(x) dx^2, 5 psi2(1-x) dx^2.
constexpr int H5_DI[36] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 2, 3, 2, 3, 4, 5,
                           4, 5, 2, 3, 2, 3, 4, 5, 4, 5, 2, 3, 2, 3, 4, 5, 4, 5};
constexpr int H5_TI[36] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 0, 0, 1, 1, 0, 0,
                           1, 1, 2, 2, 3, 3, 2, 2, 3, 3, 4, 4, 5, 5, 4, 4, 5, 5};

// Biquintic sum over the 36 coefficients (hermite.hpp h5), left to right.
SGX_HDI double h5(const double *fi, double w0t, double w1t, double w2t, double w0mt,
                  double w1mt, double w2mt, double w0d, double w1d, double w2d, double w0md,
                  double w1md, double w2md) {
  const double wd[6] = {w0d, w0md, w1d, w1md, w2d, w2md};
  const double wt[6] = {w0t, w0mt, w1t, w1mt, w2t, w2mt};
  // term k pairs a density weight and a temperature weight; the 36 pairs in
  // the reference's order: (d0,t0) (d0m,t0) (d0,t0m) (d0m,t0m) then t1, t2
  // with d0; then d1, d2 with t0; d1, d2 with t1; d1, d2 with t2.
  constexpr int di[36] = {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 2, 3, 2, 3, 4, 5,
                          4, 5, 2, 3, 2, 3, 4, 5, 4, 5, 2, 3, 2, 3, 4, 5, 4, 5};
  constexpr int ti[36] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 0, 0, 1, 1, 0, 0,
                          1, 1, 2, 2, 3, 3, 2, 2, 3, 3, 4, 4, 5, 5, 4, 4, 5, 5};
  double s = fi[0] * wd[0] * wt[0];
#pragma unroll
  for (int k = 1; k < 36; ++k)
    s = s + fi[k] * wd[di[k]] * wt[ti[k]];
  return s;
}

// Bicubic sum over 16 coefficients (hermite.hpp h3), left to right.
SGX_HDI double h3(const double *fi, double w0t, double w1t, double w0mt, double w1mt,
                  double w0d, double w1d, double w0md, double w1md) {
  const double wd[4] = {w0d, w0md, w1d, w1md};
  const double wt[4] = {w0t, w0mt, w1t, w1mt};
  constexpr int di[16] = {0, 1, 0, 1, 0, 1, 0, 1, 2, 3, 2, 3, 2, 3, 2, 3};
  constexpr int ti[16] = {0, 0, 1, 1, 2, 2, 3, 3, 0, 0, 1, 1, 2, 2, 3, 3};
  double s = fi[0] * wd[0] * wt[0];
#pragma unroll
  for (int k = 1; k < 16; ++k)
    s = s + fi[k] * wd[di[k]] * wt[ti[k]];
  return s;
}

SGX_HDI int grid_index(const double x, const double xmin, const double inv_dx, const int n) {
  const double u = (x - xmin) * inv_dx;
  if (!(u >= 0)) return 0;
  if (u > static_cast<double>(n - 2)) return n - 2;
  return static_cast<int>(u);
}

// Per-cell inputs shared by every evaluation (GetElectronDensities_,
// :717-726).
struct Cell {
  double rho, abar, zbar, ytot, ye, ywot, De, lDe;
};

// HelmElectrons::GetFromDensityTemperature (:996-1278).
SGX_HDN void electrons(const HelmTable &t, double rho, const double lT, const double Ye,
                       const double Ytot, double De, double lDe, double pele[5],
                       double eele[5], double sele[5], double etaele[5], double xne[5],
                       const bool only_e) {
  rho = smin(t.rhoMax, smax(t.rhoMin, rho));
  De = smin(t.rhoMax, smax(t.rhoMin, De));
  lDe = smin(t.lRhoMax, smax(t.lRhoMin, lDe));
  const double T = pow10e(lT);
  const int iat = grid_index(lDe, t.lRhoMin, t.inv_dlRho, HELM_NRHO);
  const int jat = grid_index(lT, t.lTMin, t.inv_dlT, HELM_NT);
  const double dth = t.T[jat + 1] - t.T[jat];
  const double dt2 = dth * dth;
  const double dti = ratio(1.0, dth);
  const double dt2i = dti * dti;
  const double dd = t.rho[iat + 1] - t.rho[iat];
  const double dd2 = dd * dd;
  const double ddi = ratio(1.0, dd);
  const double *fi = t.cells + (static_cast<long long>(jat) * (HELM_NRHO - 1) + iat) * HELM_REC;

  const double xt = smax(0.0, (T - t.T[jat]) * dti);
  const double xd = smax(0.0, (De - t.rho[iat]) * ddi);
  const double mxt = 1. - xt;
  const double mxd = 1. - xd;

  double si0t = psi0(xt);
  double si1t = psi1(xt) * dth;
  const double si2t = psi2(xt) * dt2;
  double si0mt = psi0(mxt);
  double si1mt = -psi1(mxt) * dth;
  const double si2mt = psi2(mxt) * dt2;
  double si0d = psi0(xd);
  double si1d = psi1(xd) * dd;
  const double si2d = psi2(xd) * dd2;
  double si0md = psi0(mxd);
  double si1md = -psi1(mxd) * dd;
  const double si2md = psi2(mxd) * dd2;

  double dsi0t = dpsi0(xt) * dti;
  double dsi1t = dpsi1(xt);
  const double dsi2t = dpsi2(xt) * dth;
  double dsi0mt = -dpsi0(mxt) * dti;
  double dsi1mt = dpsi1(mxt);
  const double dsi2mt = -dpsi2(mxt) * dth;
  double dsi0d = dpsi0(xd) * ddi;
  double dsi1d = dpsi1(xd);
  const double dsi2d = dpsi2(xd) * dd;
  double dsi0md = -dpsi0(mxd) * ddi;
  double dsi1md = dpsi1(mxd);
  const double dsi2md = -dpsi2(mxd) * dd;

  const double ddsi0t = ddpsi0(xt) * dt2i;
  const double ddsi1t = ddpsi1(xt) * dti;
  const double ddsi2t = ddpsi2(xt);
  const double ddsi0mt = ddpsi0(mxt) * dt2i;
  const double ddsi1mt = -ddpsi1(mxt) * dti;
  const double ddsi2mt = ddpsi2(mxt);

  const double free_en =
      h5(fi, si0t, si1t, si2t, si0mt, si1mt, si2mt, si0d, si1d, si2d, si0md, si1md, si2md);
  const double df_t = h5(fi, dsi0t, dsi1t, dsi2t, dsi0mt, dsi1mt, dsi2mt, si0d, si1d, si2d,
                         si0md, si1md, si2md);
  const double df_tt = h5(fi, ddsi0t, ddsi1t, ddsi2t, ddsi0mt, ddsi1mt, ddsi2mt, si0d, si1d,
                          si2d, si0md, si1md, si2md);
  if (only_e) {
    eele[0] = Ye * free_en + T * (-df_t) * Ye;
    eele[2] = T * (-df_tt) * Ye;
    return;
  }
  const double df_d = h5(fi, si0t, si1t, si2t, si0mt, si1mt, si2mt, dsi0d, dsi1d, dsi2d,
                         dsi0md, dsi1md, dsi2md);
  const double df_dt = h5(fi, dsi0t, dsi1t, dsi2t, dsi0mt, dsi1mt, dsi2mt, dsi0d, dsi1d,
                          dsi2d, dsi0md, dsi1md, dsi2md);

  // cubic weights for dP/dDe, eta and the pair density
  si0t = xpsi0(xt);
  si1t = xpsi1(xt) * dth;
  si0mt = xpsi0(mxt);
  si1mt = -xpsi1(mxt) * dth;
  si0d = xpsi0(xd);
  si1d = xpsi1(xd) * dd;
  si0md = xpsi0(mxd);
  si1md = -xpsi1(mxd) * dd;
  dsi0t = xdpsi0(xt) * dti;
  dsi1t = xdpsi1(xt);
  dsi0mt = -xdpsi0(mxt) * dti;
  dsi1mt = xdpsi1(mxt);
  dsi0d = xdpsi0(xd) * ddi;
  dsi1d = xdpsi1(xd);
  dsi0md = -xdpsi0(mxd) * ddi;
  dsi1md = xdpsi1(mxd);

  const double *fp = fi + 36;
  pele[1] = smax(0.0, Ye * h3(fp, si0t, si1t, si0mt, si1mt, si0d, si1d, si0md, si1md));

  const double *fe = fi + 52;
  etaele[0] = h3(fe, si0t, si1t, si0mt, si1mt, si0d, si1d, si0md, si1md);
  double x = h3(fe, si0t, si1t, si0mt, si1mt, dsi0d, dsi1d, dsi0md, dsi1md);
  etaele[1] = Ye * x;
  etaele[2] = h3(fe, dsi0t, dsi1t, dsi0mt, dsi1mt, si0d, si1d, si0md, si1md);
  etaele[3] = -x * De * Ytot;
  etaele[4] = x * rho * Ytot;

  const double *fx = fi + 68;
  xne[0] = h3(fx, si0t, si1t, si0mt, si1mt, si0d, si1d, si0md, si1md);
  x = smax(0.0, h3(fx, si0t, si1t, si0mt, si1mt, dsi0d, dsi1d, dsi0md, dsi1md));
  xne[1] = Ye * x;
  xne[2] = h3(fx, dsi0t, dsi1t, dsi0mt, dsi1mt, si0d, si1d, si0md, si1md);
  xne[3] = -x * De * Ytot;
  xne[4] = x * rho * Ytot;

  x = De * De;
  pele[0] = x * df_d;
  pele[2] = x * df_dt;
  const double s = pele[1] / Ye - 2.0 * De * df_d;
  pele[3] = -Ytot * (2.0 * pele[0] + s * De);
  pele[4] = rho * Ytot * (2.0 * De * df_d + s);

  x = Ye * Ye;
  sele[0] = -df_t * Ye;
  sele[2] = -df_tt * Ye;
  sele[1] = -df_dt * x;
  sele[3] = Ytot * (Ye * df_dt * De - sele[0]);
  sele[4] = -Ytot * (Ye * df_dt * rho + df_t);

  eele[0] = Ye * free_en + T * sele[0];
  eele[2] = T * sele[2];
  eele[1] = x * df_d + T * sele[1];
  eele[3] = -Ye * Ytot * (free_en + df_d * De) + T * sele[3];
  eele[4] = Ytot * (free_en + Ye * df_d * rho) + T * sele[4];
}

// HelmRad::GetFromDensityTemperature (:1280-1320).
SGX_HDI void radiation(const double rho, const double temp, double prad[5], double erad[5],
                       double srad[5]) {
  const double rhoi = ratio(1.0, rho);
  const double tempi = ratio(1.0, temp);
  const double T3 = IPow<3>::of(temp);
  const double T4 = T3 * temp;
  const double P = RAD_PREFACTOR * T4;
  const double dPdT = 4.0 * RAD_PREFACTOR * T3;
  prad[VAL] = P;
  prad[DDR] = 0;
  prad[DDT] = dPdT;
  prad[DDA] = 0;
  prad[DDZ] = 0;
  const double PoR = P * rhoi;
  const double e = 3.0 * PoR;
  const double dedR = -e * rhoi;
  const double dedT = 3.0 * dPdT * rhoi;
  erad[VAL] = e;
  erad[DDR] = dedR;
  erad[DDT] = dedT;
  erad[DDA] = 0;
  erad[DDZ] = 0;
  constexpr double dPdR = 0;
  const double dEdR = erad[DDR];
  const double s = (PoR + e) * tempi;
  const double dsdR = ((dPdR - PoR) * rhoi + dEdR) * tempi;
  const double dsdT = (dPdT * rhoi + dedT - s) * tempi;
  srad[VAL] = s;
  srad[DDR] = dsdR;
  srad[DDT] = dsdT;
  srad[DDA] = 0;
  srad[DDZ] = 0;
}

// HelmIon::GetFromDensityTemperature (:1322-1367).
SGX_HDI void ions(const double rho, const double temp, const double y, const double ytot,
                  const double xni, const double dxnidd, const double dxnida, double pion[5],
                  double eion[5], double sion[5]) {
  const double kbT = KB * temp;
  const double P = xni * kbT;
  const double dPdR = dxnidd * kbT;
  const double dPdT = xni * KB;
  const double dPdA = dxnida * kbT;
  pion[VAL] = P;
  pion[DDR] = dPdR;
  pion[DDT] = dPdT;
  pion[DDA] = dPdA;
  pion[DDZ] = 0;
  const double rhoi = ratio(1.0, rho);
  const double PoR = P * rhoi;
  const double e = 1.5 * PoR;
  const double dedR = (1.5 * dPdR - e) * rhoi;
  const double dedT = 1.5 * dPdT * rhoi;
  const double dedA = 1.5 * dPdA * rhoi;
  eion[VAL] = e;
  eion[DDR] = dedR;
  eion[DDT] = dedT;
  eion[DDA] = dedA;
  eion[DDZ] = 0;
  const double tempi = ratio(1.0, temp);
  const double KBNAY = KBNA * ytot;
  const double s = (PoR + e) * tempi + KBNAY * y;
  const double dsdR = (dPdR * rhoi - P * rhoi * rhoi + dedR) * tempi - KBNAY * rhoi;
  const double dsdT =
      (dPdT * rhoi + dedT) * tempi - (PoR + e) * tempi * tempi + 1.5 * KBNAY * tempi;
  const double dsdA = (dPdA * rhoi + dedA) * tempi + KBNAY * ytot * (2.5 - y);
  sion[VAL] = s;
  sion[DDR] = dsdR;
  sion[DDT] = dsdT;
  sion[DDA] = dsdA;
  sion[DDZ] = 0;
}

template <int n>
SGX_HDI void butterworth(const double freq, const double cfreq, double &g, double &dgdf) {
  g = ratio(1.0, 1.0 + IPow<2 * n>::of(ratio(freq, cfreq)));
  dgdf = ratio(-IPow<2>::of(g) * 2 * n, IPow<2 * n>::of(cfreq)) * IPow<2 * n - 1>::of(freq);
}

// HelmCoulomb::GetFromDensityTemperature (:1369-1504).
SGX_HDN void coulomb(const double rho, const double temp, const double ytot, const double abar,
                     const double zbar, const double xni, const double dxnidd,
                     const double dxnida, double pcoul[5], double ecoul[5], double scoul[5]) {
  constexpr double a1 = -0.898004, b1 = 0.96786, c1 = 0.220703, d1 = -0.86097, e1 = 2.5269;
  constexpr double a2 = 0.29561, b2 = 1.9885, c2 = 0.288675;
  const double kbT = KB * temp;
  const double pion = xni * kbT;
  const double dpiondd = dxnidd * kbT;
  const double dpiondt = xni * KB;
  const double dpionda = dxnida * kbT;
  constexpr double dpiondz = 0.0;
  constexpr double four_thirds = 4.0 / 3.0;
  constexpr double ftpi = four_thirds * PI;
  double s = ftpi * xni;
  const double dsdd = ftpi * dxnidd;
  const double dsda = ftpi * dxnida;
  constexpr double one_third = 1.0 / 3.0;
  const double si = ratio(1.0, s);
  const double lami = ratio(1.0, cbrt(s));
  const double lamidd = -lami * one_third * dsdd * si;
  const double lamida = -lami * one_third * dsda * si;
  const double plasg = IPow<2>::of(ELECTRON_CHARGE_ESU * zbar) / (kbT * lami);
  const double plasg_o_lami = ratio(plasg, lami);
  const double plasgdd = -plasg_o_lami * lamidd;
  const double plasgda = -plasg_o_lami * lamida;
  const double plasgdt = -ratio(plasg, temp);
  const double plasgdz = 2.0 * ratio(plasg, zbar);
  const double abari = ratio(1.0, abar);
  if (plasg >= 0) {
    const double x = sqrt(sqrt(plasg));
    double y = KBNA * ytot;
    const double c1_o_x = ratio(c1, x);
    ecoul[VAL] = y * temp * (a1 * plasg + b1 * x + c1_o_x + d1);
    pcoul[VAL] = one_third * rho * ecoul[0];
    scoul[VAL] = -y * (3.0 * b1 * x - 5.0 * c1_o_x + d1 * (log(plasg) - 1.0) - e1);
    y = KBNA * temp * ytot * (a1 + ratio(0.25, plasg) * (b1 * x - c1_o_x));
    ecoul[DDR] = y * plasgdd;
    ecoul[DDT] = y * plasgdt + ratio(ecoul[0], temp);
    ecoul[DDA] = y * plasgda - ecoul[0] * abari;
    ecoul[DDZ] = y * plasgdz;
    y = one_third * rho;
    pcoul[DDR] = one_third * ecoul[0] + y * ecoul[1];
    pcoul[DDT] = y * ecoul[2];
    pcoul[DDA] = y * ecoul[3];
    pcoul[DDZ] = y * ecoul[4];
    y = -KBNA * plasg * abari * (0.75 * b1 * x + 1.25 * c1_o_x + d1);
    scoul[DDR] = y * plasgdd;
    scoul[DDT] = y * plasgdt;
    scoul[DDA] = y * plasgda - scoul[0] * abari;
    scoul[DDZ] = y * plasgdz;
  } else {
    const double x = plasg * sqrt(sabs(plasg));
    const double y = pow(plasg, b2);
    const double z = c2 * x - one_third * a2 * y;
    const double plasgi = ratio(1., plasg);
    const double rhoi = ratio(1.0, rho);
    pcoul[VAL] = -pion * z;
    ecoul[VAL] = 3.0 * pcoul[0] * rhoi;
    scoul[VAL] = -KBNA * abari * (c2 * x - a2 * ratio(b2 - 1.0, b2) * y);
    s = 1.5 * c2 * x * plasgi - one_third * a2 * b2 * y * plasgi;
    pcoul[DDR] = -dpiondd * z - pion * s * plasgdd;
    pcoul[DDT] = -dpiondt * z - pion * s * plasgdt;
    pcoul[DDA] = -dpionda * z - pion * s * plasgda;
    pcoul[DDZ] = -dpiondz * z - pion * s * plasgdz;
    s = 3.0 * rhoi;
    ecoul[DDR] = s * pcoul[1] - ecoul[0] * rhoi;
    ecoul[DDT] = s * pcoul[2];
    ecoul[DDA] = s * pcoul[3];
    ecoul[DDZ] = s * pcoul[4];
    s = -KBNA * abari * plasgi * (1.5 * c2 * x - a2 * (b2 - 1.0) * y);
    scoul[DDR] = s * plasgdd;
    scoul[DDT] = s * plasgdt;
    scoul[DDA] = s * plasgda - scoul[0] * abari;
    scoul[DDZ] = s * plasgdz;
  }
  double g_r, dgdf_r, g_t, dgdf_t;
  butterworth<12>(log10(temp) - 4.5, 3.0, g_r, dgdf_r);
  butterworth<12>(log10(rho) + 1.0, 6.0, g_t, dgdf_t);
  const double gain = (1.0 - g_t * g_r);
  const double dgaindt = -ratio(g_r * dgdf_t, temp * LN10);
  const double dgaindd = -ratio(g_t * dgdf_r, rho * LN10);
  pcoul[VAL] = pcoul[VAL] * gain;
  ecoul[VAL] = ecoul[VAL] * gain;
  scoul[VAL] = scoul[VAL] * gain;
  pcoul[DDR] = gain * pcoul[DDR] + ratio(pcoul[VAL] * dgaindd, gain);
  pcoul[DDT] = gain * pcoul[DDT] + ratio(pcoul[VAL] * dgaindt, gain);
  pcoul[DDA] = gain * pcoul[DDA];
  pcoul[DDZ] = gain * pcoul[DDZ];
  ecoul[DDR] = gain * ecoul[DDR] + ratio(ecoul[VAL] * dgaindd, gain);
  ecoul[DDT] = gain * ecoul[DDT] + ratio(ecoul[VAL] * dgaindt, gain);
  ecoul[DDA] = gain * ecoul[DDA];
  ecoul[DDZ] = gain * ecoul[DDZ];
  scoul[DDR] = gain * scoul[DDR] + ratio(scoul[VAL] * dgaindd, gain);
  scoul[DDT] = gain * scoul[DDT] + ratio(scoul[VAL] * dgaindt, gain);
  scoul[DDA] = gain * scoul[DDA];
  scoul[DDZ] = gain * scoul[DDZ];
}

// GetMassFractions (:506-512)
SGX_HDI void mass_fractions(const double rho, const double ytot, double &xni, double &dxnidd,
                            double &dxnida) {
  xni = NA * ytot * rho;
  dxnidd = NA * ytot;
  dxnida = -xni * ytot;
}

// Helmholtz::GetFromDensityLogTemperature_ (:1506-1572): the sum of the
// enabled components.
SGX_HDN void evaluate(const HelmTable &t, const int opt, const Cell &c, const double T,
                      double p[5], double e[5], double s[5], double etaele[5], double nep[5],
                      const bool only_e) {
  double prad[5] = {0}, pion[5] = {0}, pele[5] = {0}, pcoul[5] = {0};
  double erad[5] = {0}, eion[5] = {0}, eele[5] = {0}, ecoul[5] = {0};
  double srad[5] = {0}, sion[5] = {0}, sele[5] = {0}, scoul[5] = {0};
  for (int i = 0; i < 5; ++i)
    etaele[i] = nep[i] = 0;
  const double lT = log10(T);
  const double log10e = log10(E_CONST);
  const double lnT = lT / log10e;
  const double rho = c.rho;
  if (opt & HELM_RAD) radiation(rho, T, prad, erad, srad);
  if (opt & HELM_GAS) {
    const bool ionized = (opt & HELM_ION) != 0, degenerate = (opt & HELM_ELE) != 0;
    const bool do_unmodified_ions = (ionized && degenerate) || !ionized;
    if (do_unmodified_ions) {
      double xni, dxnidd, dxnida;
      mass_fractions(rho, c.ytot, xni, dxnidd, dxnida);
      const double y = c.ywot + LSWOT15 * lnT;
      ions(rho, T, y, c.ytot, xni, dxnidd, dxnida, pion, eion, sion);
    } else {
      const double abar_ion = ratio(c.abar, c.zbar + 1);
      const double ytot_ion = ratio(1.0, abar_ion);
      const double ywot_ion = ratio(log(abar_ion * abar_ion * sqrt(abar_ion)), rho * NA);
      const double y_ion = ywot_ion + LSWOT15 * lnT;
      double xni, dxnidd, dxnida;
      mass_fractions(rho, ytot_ion, xni, dxnidd, dxnida);
      ions(rho, T, y_ion, ytot_ion, xni, dxnidd, dxnida, pion, eion, sion);
    }
    if (degenerate) {
      electrons(t, rho, lT, c.ye, c.ytot, c.De, c.lDe, pele, eele, sele, etaele, nep, only_e);
      if (opt & HELM_COUL) {
        double xni, dxnidd, dxnida;
        mass_fractions(rho, c.ytot, xni, dxnidd, dxnida);
        coulomb(rho, T, c.ytot, c.abar, c.zbar, xni, dxnidd, dxnida, pcoul, ecoul, scoul);
      }
    }
  }
  for (int i = 0; i < 5; ++i)
    e[i] = erad[i] + eion[i] + eele[i] + ecoul[i];
  if (!only_e) {
    for (int i = 0; i < 5; ++i) {
      p[i] = prad[i] + pion[i] + pele[i] + pcoul[i];
      s[i] = srad[i] + sion[i] + sele[i] + scoul[i];
    }
  }
}

// GetElectronDensities_ (:717-726)
SGX_HDI Cell cell(const double rho, const double abar, const double zbar) {
  Cell c;
  c.rho = rho;
  c.abar = abar;
  c.zbar = zbar;
  c.ytot = ratio(1.0, abar);
  c.ye = zbar * c.ytot;
  c.ywot = log(ratio(abar * abar * sqrt(abar), rho * NA));
  c.De = rho * c.ye;
  c.lDe = log10(c.De);
  return c;
}

// lTAnalytic_ (:728-731)
SGX_HDI double lT_analytic(const double rho, const double e, const double ni, const double ne) {
  return log10((2.0 / 3.0) * ratio(e * rho, ni + ne) * KBi);
}

// Gamma1 and Gamma3 (:697-715; Cox & Giuli 9.97, 9.93)
SGX_HDI double gamma1(const double rho, const double T, const double p[5], const double e[5]) {
  const double chit = ratio(T, p[0]) * p[DDT];
  const double chid = ratio(p[DDR] * rho, p[0]);
  const double x = ratio(p[0] * chit, rho * T * e[DDT]);
  return chit * x + chid;
}
SGX_HDI double gamma3(const double rho, const double T, const double p[5], const double e[5]) {
  const double chit = ratio(T, p[0]) * p[DDT];
  const double x = ratio(p[0] * chit, rho * T * e[DDT]);
  return x + 1.0;
}

// Iterations iter .. iter_end - 1 of RootFinding1D::newton_raphson
// (root_finding.hpp:246-310) on e(T), from x, with fail_on_bound_root =
// false. Resumable: returns true when the iteration stopped (converged, or
// stepped out of [a, b], which the reference then accepts), false when
// iter_end was reached first; x and iter carry the state across calls, so
// running 0..k and then k..100 gives the same result as 0..100.
SGX_HDN bool newton_e_steps(const HelmTable &t, const int opt, const Cell &c,
                            const double ytarget, const double a, const double b,
                            const double ytol, double &x, int &iter, const int iter_end) {
  for (; iter < iter_end; iter++) {
    double p[5], e[5], s[5], eta[5], nep[5];
    evaluate(t, opt, c, x, p, e, s, eta, nep, true);
    const double yg = e[VAL], dfunc = e[DDT];
    if (sabs(yg - ytarget) < sabs(ytol * ytarget)) return true;
    const double xold = x;
    x = x - (yg - ytarget) / dfunc;
    if ((x <= a && xold <= a) || (x >= b && xold >= b)) return true;
    x = smax(smin(x, b), a);
  }
  return false;
}

// One inversion T(rho, e) (lTFromRhoSie_, :867-960) between its phases.
struct Inversion {
  double e, Tguess, Ta, Tb, ni, ne, x;
  int iter;
  bool iterate; // a root find is needed (radiation, electrons or Coulomb on)
  bool newton;  // Newton-Raphson first (Options::USE_NEWTON_RAPHSON)
};

// Initial guess: the lT cache when it lies in the table, else the ideal-gas
// estimate, else 10^8 K.
SGX_HDI Inversion inversion_begin(const HelmTable &t, const int opt, const Cell &c,
                                  const double e, const double *lam) {
  Inversion v;
  v.e = e;
  const double abari = ratio(1.0, c.abar);
  v.ni = abari * c.rho * NA;
  v.ne = c.zbar * v.ni;
  v.iterate = (opt & HELM_RAD) || (opt & HELM_ELE) || (opt & HELM_COUL);
  v.newton = !(opt & HELM_REGULA_FALSI);
  v.iter = 0;
  v.Tguess = v.Ta = v.Tb = v.x = 0.0;
  if (v.iterate) {
    double lTguess = lam ? lam[2] : NAN;
    if (!((t.lTMin <= lTguess) && (lTguess <= t.lTMax))) {
      lTguess = lT_analytic(c.rho, e, v.ni, v.ne);
      if (!((t.lTMin <= lTguess) && (lTguess <= t.lTMax))) lTguess = 8;
    }
    v.Tguess = pow10e(lTguess);
    v.Ta = pow10e(t.lTMin);
    v.Tb = pow10e(t.lTMax);
    v.x = v.Tguess;
  }
  return v;
}

// After the Newton phase (newton_done: it stopped before its iteration
// limit): the regula-falsi and analytic fallbacks, the clamp to the table
// and the lT cache. The reference ends with a SafeGet of the cache, which
// with a numerically indexed lambda replaces the root by the cached guess;
// HELM_CACHE_READBACK keeps that behaviour, otherwise the root is stored
// into the cache. Returns log10 T.
SGX_HDN double inversion_end(const HelmTable &t, const int opt, const Cell &c,
                             const Inversion &v, const bool newton_done, double *lam) {
  const double ionized = (opt & HELM_ION) ? 1.0 : 0.0;
  double lT, T = 0.0;
  if (v.iterate) {
    auto e_of_T = [&](const double x) {
      double p[5], ee[5], s[5], eta[5], nep[5];
      evaluate(t, opt, c, x, p, ee, s, eta, nep, true);
      return ee[VAL];
    };
    bool ok;
    if (v.newton) {
      ok = newton_done;
      T = v.x;
      if (!ok)
        ok = regula_falsi(e_of_T, v.e, v.Tguess, v.Ta, v.Tb, ROOT_THRESH, ROOT_THRESH, T) ==
             RootStatus::SUCCESS;
    } else {
      ok = regula_falsi(e_of_T, v.e, v.Tguess, v.Ta, v.Tb, ROOT_THRESH, ROOT_THRESH, T) ==
           RootStatus::SUCCESS;
    }
    if (!ok) {
      lT = lT_analytic(c.rho, v.e, v.ni, ionized * v.ne);
      T = pow10e(lT);
    }
  } else {
    lT = lT_analytic(c.rho, v.e, v.ni, ionized * v.ne);
    T = pow10e(lT);
  }
  lT = log10(T);
  if (lT < t.lTMin) lT = t.lTMin;
  if (lT > t.lTMax) lT = t.lTMax;
  if (lam) {
    if (opt & HELM_CACHE_READBACK)
      lT = lam[2];
    else
      lam[2] = lT;
  }
  return lT;
}

// lTFromRhoSie_ in one pass. lam: [Abar, Zbar, lT] or null.
SGX_HDN double lT_from_rho_sie(const HelmTable &t, const int opt, const Cell &c, const double e,
                               double *lam) {
  Inversion v = inversion_begin(t, opt, c, e, lam);
  bool done = false;
  if (v.iterate && v.newton)
    done = newton_e_steps(t, opt, c, e, v.Ta, v.Tb, HELM_EOS_EPS, v.x, v.iter, NEWTON_MAX_ITER);
  return inversion_end(t, opt, c, v, done, lam);
}

// ---------------------------------------------------------------------------
// FP32 e(T) for the Newton phase of the mixed-precision inversion: the same
// components as evaluate(..., only_e) -- radiation, ions, the tabulated
// electrons and the Coulomb correction with its filter -- in float, with
// the electron free energy from the normalised FP32 coefficients. Only the
// root's neighbourhood matters here: the FP64 Newton iteration of the
// reference finishes from this phase's T. Returns false when a value left
// the float range (the FP64 iteration then starts from the reference's own
// guess).
// ---------------------------------------------------------------------------
SGX_HDI float fpsi0(float z) { return z * z * z * (z * (-6.0f * z + 15.0f) - 10.0f) + 1.0f; }
SGX_HDI float fdpsi0(float z) { return z * z * (z * (-30.0f * z + 60.0f) - 30.0f); }
SGX_HDI float fddpsi0(float z) { return z * (z * (-120.0f * z + 180.0f) - 60.0f); }
SGX_HDI float fpsi1(float z) { return z * (z * z * (z * (-3.0f * z + 8.0f) - 6.0f) + 1.0f); }
SGX_HDI float fdpsi1(float z) { return z * z * (z * (-15.0f * z + 32.0f) - 18.0f) + 1.0f; }
SGX_HDI float fddpsi1(float z) { return z * (z * (-60.0f * z + 96.0f) - 36.0f); }
SGX_HDI float fpsi2(float z) { return 0.5f * z * z * (z * (z * (-z + 3.0f) - 3.0f) + 1.0f); }
SGX_HDI float fdpsi2(float z) { return 0.5f * z * (z * (z * (-5.0f * z + 12.0f) - 9.0f) + 2.0f); }
SGX_HDI float fddpsi2(float z) { return 0.5f * (z * (z * (-20.0f * z + 36.0f) - 18.0f) + 2.0f); }

// Per-cell constants of the FP32 phase.
struct Cell32 {
  float rho, De, lDe, ye, ytot, ytot_ion, abar, zbar, lrho;
};
SGX_HDI Cell32 cell32(const Cell &c) {
  Cell32 f;
  f.rho = static_cast<float>(c.rho);
  f.De = static_cast<float>(c.De);
  f.lDe = static_cast<float>(c.lDe);
  f.ye = static_cast<float>(c.ye);
  f.ytot = static_cast<float>(c.ytot);
  f.ytot_ion = static_cast<float>(ratio(c.zbar + 1.0, c.abar));
  f.abar = static_cast<float>(c.abar);
  f.zbar = static_cast<float>(c.zbar);
  f.lrho = log10f(f.rho);
  return f;
}

__device__ __forceinline__ bool e_of_T32(const HelmTable &t, const int opt, const Cell32 &c,
                                         const float T, float &e, float &dedT) {
  e = 0.0f;
  dedT = 0.0f;
  const float lT = log10f(T);
  if (opt & HELM_RAD) {
    // 3 a/3 T^4 / rho, with T scaled by 1e-4 to stay inside the float range
    constexpr float c3 = static_cast<float>(3.0 * RAD_PREFACTOR * 1e16);
    const float s = T * 1e-4f, s3 = s * s * s;
    e += c3 * s3 * s / c.rho;
    dedT += 4.0f * c3 * s3 * 1e-4f / c.rho;
  }
  if (opt & HELM_GAS) {
    const bool ionized = (opt & HELM_ION) != 0, degenerate = (opt & HELM_ELE) != 0;
    const float y = ((ionized && degenerate) || !ionized) ? c.ytot : c.ytot_ion;
    constexpr float k15 = static_cast<float>(1.5 * KBNA);
    e += k15 * y * T;
    dedT += k15 * y;
    if (degenerate) {
      if (!t.cells32) return false;
      const float De = fminf(t.f_rhoMax, fmaxf(t.f_rhoMin, c.De));
      const float lDe = fminf(t.f_lRhoMax, fmaxf(t.f_lRhoMin, c.lDe));
      float u = (lDe - t.f_lRhoMin) * t.f_inv_dlRho;
      const int iat = !(u >= 0.0f) ? 0 : (u > HELM_NRHO - 2 ? HELM_NRHO - 2 : static_cast<int>(u));
      u = (lT - t.f_lTMin) * t.f_inv_dlT;
      const int jat = !(u >= 0.0f) ? 0 : (u > HELM_NT - 2 ? HELM_NT - 2 : static_cast<int>(u));
      const float Tj = __ldg(t.T32 + jat);
      const float dth = __ldg(t.T32 + jat + 1) - Tj;
      const float ri = __ldg(t.rho32 + iat);
      const float dd = __ldg(t.rho32 + iat + 1) - ri;
      const float xt = fmaxf(0.0f, (T - Tj) / dth), xd = fmaxf(0.0f, (De - ri) / dd);
      const float mxt = 1.0f - xt, mxd = 1.0f - xd;
      const float wd[6] = {fpsi0(xd), fpsi0(mxd), fpsi1(xd), fpsi1(mxd), fpsi2(xd), fpsi2(mxd)};
      const float wt[6] = {fpsi0(xt), fpsi0(mxt), fpsi1(xt), fpsi1(mxt), fpsi2(xt), fpsi2(mxt)};
      const float w1[6] = {fdpsi0(xt), -fdpsi0(mxt), fdpsi1(xt), -fdpsi1(mxt), fdpsi2(xt),
                           -fdpsi2(mxt)};
      const float w2[6] = {fddpsi0(xt), fddpsi0(mxt), fddpsi1(xt), fddpsi1(mxt), fddpsi2(xt),
                           fddpsi2(mxt)};
      // the cell's 6 x 6 coefficients (T weight major), 9 aligned 16-byte loads
      const float4 *c4 = reinterpret_cast<const float4 *>(
          t.cells32 + (static_cast<long long>(jat) * (HELM_NRHO - 1) + iat) * 36);
      float C[36];
#pragma unroll
      for (int q = 0; q < 9; ++q) {
        const float4 v = __ldg(c4 + q);
        C[4 * q] = v.x;
        C[4 * q + 1] = v.y;
        C[4 * q + 2] = v.z;
        C[4 * q + 3] = v.w;
      }
      // F and its first two xt derivatives: each T row summed over the
      // density weights first
      float F = 0.0f, Fx = 0.0f, Fxx = 0.0f;
#pragma unroll
      for (int ti = 0; ti < 6; ++ti) {
        float ut = 0.0f;
#pragma unroll
        for (int di = 0; di < 6; ++di)
          ut = fmaf(C[ti * 6 + di], wd[di], ut);
        F = fmaf(ut, wt[ti], F);
        Fx = fmaf(ut, w1[ti], Fx);
        Fxx = fmaf(ut, w2[ti], Fxx);
      }
      const float dti = 1.0f / dth;
      e += c.ye * (F - T * Fx * dti);
      dedT += -c.ye * T * Fxx * dti * dti;
    }
    if (degenerate && (opt & HELM_COUL)) {
      // HelmCoulomb (:1369-1504), energy and its T derivative
      constexpr float a1 = -0.898004f, b1 = 0.96786f, c1 = 0.220703f, d1 = -0.86097f;
      constexpr float a2 = 0.29561f, b2 = 1.9885f, c2 = 0.288675f;
      const float xni = static_cast<float>(NA) * c.ytot * c.rho;
      const float kbT = static_cast<float>(KB) * T;
      const float s = static_cast<float>(4.0 / 3.0 * PI) * xni;
      const float lami = 1.0f / cbrtf(s);
      const float ez = static_cast<float>(ELECTRON_CHARGE_ESU) * c.zbar;
      const float plasg = ez * ez / (kbT * lami);
      const float plasgdt = -plasg / T;
      float ec, ecdt;
      if (plasg >= 0.0f) {
        const float x = sqrtf(sqrtf(plasg));
        const float y = static_cast<float>(KBNA) * c.ytot;
        const float c1x = c1 / x;
        ec = y * T * (a1 * plasg + b1 * x + c1x + d1);
        const float y2 = static_cast<float>(KBNA) * T * c.ytot * (a1 + 0.25f / plasg * (b1 * x - c1x));
        ecdt = y2 * plasgdt + ec / T;
      } else {
        const float x = plasg * sqrtf(fabsf(plasg));
        const float y = powf(plasg, b2);
        const float z = c2 * x - a2 * y / 3.0f;
        const float pion = xni * kbT;
        const float ss = 1.5f * c2 * x / plasg - a2 * b2 * y / (3.0f * plasg);
        ec = 3.0f * (-pion * z) / c.rho;
        ecdt = 3.0f * (-xni * static_cast<float>(KB) * z - pion * ss * plasgdt) / c.rho;
      }
      // the Butterworth filters (the reference takes the T derivative of the
      // gain from the density filter's derivative; kept)
      const float fr = (lT - 4.5f) / 3.0f, ft = (c.lrho + 1.0f) / 6.0f;
      const float fr2 = fr * fr, ft2 = ft * ft;
      const float fr8 = fr2 * fr2 * fr2 * fr2, ft8 = ft2 * ft2 * ft2 * ft2;
      const float fr24 = fr8 * fr8 * fr8, ft24 = ft8 * ft8 * ft8;
      const float g_r = 1.0f / (1.0f + fr24), g_t = 1.0f / (1.0f + ft24);
      // dg/df = -24 g^2 f^23 / c^24 for the density filter (c = 6)
      const float ft23 = ft24 / ft;
      const float dgdf_t = (ft != 0.0f) ? -g_t * g_t * 24.0f * ft23 / 6.0f : 0.0f;
      const float gain = 1.0f - g_t * g_r;
      const float dgaindt = -(g_r * dgdf_t) / (T * static_cast<float>(LN10));
      const float ecg = ec * gain;
      e += ecg;
      dedT += gain * ecdt + ecg * dgaindt / gain;
    }
  }
  return isfinite(e) && isfinite(dedT) && dedT != 0.0f;
}

// The FP32 Newton phase: newton_e_steps in float from the reference's guess
// to |e - target| < 1e-6 |target| (at most 40 steps, the same bound handling).
// true with x set when it got there.
__device__ __forceinline__ bool newton_e32(const HelmTable &t, const int opt, const Cell32 &c,
                                           const double target, const double a, const double b,
                                           double &x) {
  const float tg = static_cast<float>(target), fa = static_cast<float>(a),
              fb = static_cast<float>(b);
  float xf = static_cast<float>(x);
  for (int it = 0; it < 40; ++it) {
    float ev, de;
    if (!e_of_T32(t, opt, c, xf, ev, de)) return false;
    if (fabsf(ev - tg) < 1e-6f * fabsf(tg)) {
      x = static_cast<double>(xf);
      return true;
    }
    const float xold = xf;
    xf = xf - (ev - tg) / de;
    if ((xf <= fa && xold <= fa) || (xf >= fb && xold >= fb)) return false;
    xf = fmaxf(fminf(xf, fb), fa);
    if (!isfinite(xf)) return false;
  }
  return false;
}

} // namespace helm

// The end of Helmholtz::FillEos (:847-864): the full evaluation at temp and
// the requested outputs.
SGX_HDN void helm_fill_tail(const HelmTable &t, const int opt, const helm::Cell &c,
                            const double temp, double &energy, double &press, double &cv,
                            double &bmod, const unsigned output) {
  using namespace helm;
  double p[5], e[5], s[5], eta[5], nep[5];
  evaluate(t, opt, c, temp, p, e, s, eta, nep, false);
  if (output & Q_SIE) energy = e[0];
  if (output & Q_PRESSURE) press = p[0];
  if (output & Q_CV) cv = e[DDT];
  if (output & Q_BMOD) bmod = smax(lim<double>::eps, p[0] * gamma1(c.rho, temp, p, e));
}

// Helmholtz::FillEos (:818-865) for one element; lam = [Abar, Zbar, lT].
// err: 1 = an output combination the reference rejects, 2 = no lambda.
SGX_HDN void helm_fill(const HelmTable &t, const int opt, double rho, double &temp,
                       double &energy, double &press, double &cv, double &bmod,
                       const unsigned output, double *lam, int *err) {
  using namespace helm;
  const bool need_temp = (output & Q_TEMPERATURE) != 0;
  const bool need_sie = (output & Q_SIE) != 0;
  if ((output & Q_DENSITY) || (need_temp && need_sie)) {
    *err = 1;
    return;
  }
  if (!lam) {
    *err = 2;
    return;
  }
  const Cell c = cell(rho, lam[0], lam[1]);
  if (need_temp) {
    temp = pow10e(lT_from_rho_sie(t, opt, c, energy, lam));
  } else {
    lam[2] = log10(temp);
  }
  helm_fill_tail(t, opt, c, temp, energy, press, cv, bmod, output);
}

} // namespace sgx
