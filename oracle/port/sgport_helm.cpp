// Helmholtz electron-positron EOS: this project's CPU restatement of
// singularity-eos eos/eos_helmholtz.hpp (Timmes & Swesty 2000), for the
// oracle's C surface. TEST INFRASTRUCTURE ONLY: the GPU library never links
// it; tests and bench.py's CPU-baseline leg call it through
// oracle/refbind.py. tests/test_oracle.py pins it to the fixture the
// compiled reference made (tests/golden/helmholtz.npz). Included at the end
// of sgport.cpp (one translation unit), so it shares the port's robust
// ratio and root finders.
//
// Each function names the reference lines it follows. The table is read
// from the reference's ASCII layout (SetTablesFromFile, :962-989); the node
// values use math_utils::pow10 (base/math_utils.hpp:56-59). Compile with
// -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

namespace helm_port {

using port::ratio;
using port::regula_falsi;

constexpr int NT = 101, NR = 271;
constexpr int VAL = 0, DDR = 1, DDT = 2, DDA = 3, DDZ = 4;
// physical constants as the reference states them (:280-340)
constexpr double STEFAN_BOLTZMANN = 5.67040047374e-5;
constexpr double CL = 2.99792458e10;
constexpr double PREFACTOR = (4. / 3.) * (STEFAN_BOLTZMANN / CL);
constexpr double KB = 1.3806504e-16;
constexpr double NA = 6.02214199e23;
constexpr double KBNA = KB * NA;
constexpr double KBi = 1.0 / KB;
constexpr double LSWOT15 = 46.682612633059801;
constexpr double LN10 = 2.30258509299405e+00;
constexpr double ELECTRON_CHARGE_ESU = 4.80320427e-10;
constexpr double ROOT_THRESH = 1e-14;
constexpr double HELM_EOS_EPS = 1e-10;
constexpr double EPS = port::EPS;

inline double pow10(double x) { return std::exp(LN10 * x); }
template <int P> inline double ipow(double x) {
  if constexpr (P == 0)
    return 1.0;
  else if constexpr (P == 1)
    return x;
  else if constexpr (P % 2)
    return x * ipow<P - 1>(x);
  else
    return ipow<P / 2>(x) * ipow<P / 2>(x);
}

// hermite.hpp:25-94
inline double psi0(double z) { return z * z * z * (z * (-6.0 * z + 15.0) - 10.0) + 1.0; }
inline double dpsi0(double z) { return z * z * (z * (-30.0 * z + 60.0) - 30.0); }
inline double ddpsi0(double z) { return z * (z * (-120.0 * z + 180.0) - 60.0); }
inline double psi1(double z) { return z * (z * z * (z * (-3.0 * z + 8.0) - 6.0) + 1.0); }
inline double dpsi1(double z) { return z * z * (z * (-15.0 * z + 32.0) - 18.0) + 1.0; }
inline double ddpsi1(double z) { return z * (z * (-60.0 * z + 96.0) - 36.0); }
inline double psi2(double z) { return 0.5 * z * z * (z * (z * (-z + 3.0) - 3.0) + 1.0); }
inline double dpsi2(double z) { return 0.5 * z * (z * (z * (-5.0 * z + 12.0) - 9.0) + 2.0); }
inline double ddpsi2(double z) { return 0.5 * (z * (z * (-20.0 * z + 36.0) - 18.0) + 2.0); }
inline double xpsi0(double z) { return z * z * (2.0 * z - 3.0) + 1.0; }
inline double xdpsi0(double z) { return z * (6.0 * z - 6.0); }
inline double xpsi1(double z) { return z * (z * (z - 2.0) + 1.0); }
inline double xdpsi1(double z) { return z * (3.0 * z - 4.0) + 1.0; }

// hermite.hpp h5: the 36 terms in the order the reference writes them
inline double h5(const double *fi, double w0t, double w1t, double w2t, double w0mt,
                 double w1mt, double w2mt, double w0d, double w1d, double w2d, double w0md,
                 double w1md, double w2md) {
  return fi[0] * w0d * w0t + fi[1] * w0md * w0t + fi[2] * w0d * w0mt + fi[3] * w0md * w0mt +
         fi[4] * w0d * w1t + fi[5] * w0md * w1t + fi[6] * w0d * w1mt + fi[7] * w0md * w1mt +
         fi[8] * w0d * w2t + fi[9] * w0md * w2t + fi[10] * w0d * w2mt + fi[11] * w0md * w2mt +
         fi[12] * w1d * w0t + fi[13] * w1md * w0t + fi[14] * w1d * w0mt +
         fi[15] * w1md * w0mt + fi[16] * w2d * w0t + fi[17] * w2md * w0t +
         fi[18] * w2d * w0mt + fi[19] * w2md * w0mt + fi[20] * w1d * w1t +
         fi[21] * w1md * w1t + fi[22] * w1d * w1mt + fi[23] * w1md * w1mt +
         fi[24] * w2d * w1t + fi[25] * w2md * w1t + fi[26] * w2d * w1mt +
         fi[27] * w2md * w1mt + fi[28] * w1d * w2t + fi[29] * w1md * w2t +
         fi[30] * w1d * w2mt + fi[31] * w1md * w2mt + fi[32] * w2d * w2t +
         fi[33] * w2md * w2t + fi[34] * w2d * w2mt + fi[35] * w2md * w2mt;
}
// hermite.hpp h3
inline double h3(const double *fi, double w0t, double w1t, double w0mt, double w1mt,
                 double w0d, double w1d, double w0md, double w1md) {
  return fi[0] * w0d * w0t + fi[1] * w0md * w0t + fi[2] * w0d * w0mt + fi[3] * w0md * w0mt +
         fi[4] * w0d * w1t + fi[5] * w0md * w1t + fi[6] * w0d * w1mt + fi[7] * w0md * w1mt +
         fi[8] * w1d * w0t + fi[9] * w1md * w0t + fi[10] * w1d * w0mt + fi[11] * w1md * w0mt +
         fi[12] * w1d * w1t + fi[13] * w1md * w1t + fi[14] * w1d * w1mt + fi[15] * w1md * w1mt;
}

// HelmElectrons tables (:279-292): field[j * NR + i], j = T node, i = density node
struct Table {
  std::vector<double> f, fd, ft, fdd, ftt, fdt, fddt, fdtt, fddtt;
  std::vector<double> dpdf, dpdfd, dpdft, dpdfdt, ef, efd, eft, efdt, xf, xfd, xft, xfdt;
  std::vector<double> rho, T;
  double lRhoMin = -12, lRhoMax = 15, lTMin = 3, lTMax = 13;
  double dlRho = 27.0 / (NR - 1), dlT = 10.0 / (NT - 1);
  double rhoMin = 1e-12, rhoMax = 1e15;
  double at(const std::vector<double> &v, int j, int i) const { return v[j * NR + i]; }
};

// SetTablesFromFile (:962-989): for each T row, for each density, the
// block's fields in the file's column order
bool load(const char *path, Table &t) {
  std::ifstream file(path);
  if (!file.is_open()) return false;
  std::stringstream ss;
  ss << file.rdbuf();
  const std::string text = ss.str();
  const char *cur = text.c_str();
  std::vector<double> *b1[9] = {&t.f, &t.fd, &t.ft, &t.fdd, &t.ftt, &t.fdt, &t.fddt, &t.fdtt,
                                &t.fddtt};
  std::vector<double> *b2[4] = {&t.dpdf, &t.dpdfd, &t.dpdft, &t.dpdfdt};
  std::vector<double> *b3[4] = {&t.ef, &t.efd, &t.eft, &t.efdt};
  std::vector<double> *b4[4] = {&t.xf, &t.xfd, &t.xft, &t.xfdt};
  std::vector<double> **blocks[4] = {b1, b2, b3, b4};
  const int nper[4] = {9, 4, 4, 4};
  for (int b = 0; b < 4; ++b) {
    for (int k = 0; k < nper[b]; ++k)
      blocks[b][k]->assign(static_cast<size_t>(NT) * NR, 0.0);
    for (int j = 0; j < NT; ++j)
      for (int i = 0; i < NR; ++i)
        for (int k = 0; k < nper[b]; ++k) {
          char *end = nullptr;
          const double v = std::strtod(cur, &end);
          if (end == cur) return false;
          (*blocks[b][k])[static_cast<size_t>(j) * NR + i] = v;
          cur = end;
        }
  }
  t.rho.resize(NR);
  t.T.resize(NT);
  for (int i = 0; i < NR; ++i)
    t.rho[i] = pow10(t.lRhoMin + i * t.dlRho);
  for (int j = 0; j < NT; ++j)
    t.T[j] = pow10(t.lTMin + j * t.dlT);
  return true;
}

// RegularGrid1D::index, bounded to the last cell
inline int index(double x, double xmin, double dx, int n) {
  const double u = (x - xmin) * (1 / dx);
  if (!(u >= 0)) return 0;
  if (u > n - 2) return n - 2;
  return static_cast<int>(u);
}

// HelmElectrons::GetFromDensityTemperature (:997-1278)
void electrons(const Table &t, double rho, double lT, double Ye, double Ytot, double De,
               double lDe, double pele[5], double eele[5], double sele[5], double etaele[5],
               double xne[5], bool only_e) {
  rho = std::min(t.rhoMax, std::max(t.rhoMin, rho));
  De = std::min(t.rhoMax, std::max(t.rhoMin, De));
  lDe = std::min(t.lRhoMax, std::max(t.lRhoMin, lDe));
  const double T = pow10(lT);
  const int iat = index(lDe, t.lRhoMin, t.dlRho, NR);
  const int jat = index(lT, t.lTMin, t.dlT, NT);
  const double dth = t.T[jat + 1] - t.T[jat], dt2 = dth * dth, dti = ratio(1.0, dth),
               dt2i = dti * dti;
  const double dd = t.rho[iat + 1] - t.rho[iat], dd2 = dd * dd, ddi = ratio(1.0, dd);
  auto corners = [&](double *o, const std::vector<double> &v) {
    o[0] = t.at(v, jat, iat);
    o[1] = t.at(v, jat, iat + 1);
    o[2] = t.at(v, jat + 1, iat);
    o[3] = t.at(v, jat + 1, iat + 1);
  };
  double fi[36];
  const std::vector<double> *order[9] = {&t.f,   &t.ft,   &t.ftt,  &t.fd,   &t.fdd,
                                         &t.fdt, &t.fddt, &t.fdtt, &t.fddtt};
  for (int k = 0; k < 9; ++k)
    corners(fi + 4 * k, *order[k]);
  const double xt = std::max(0.0, (T - t.T[jat]) * dti);
  const double xd = std::max(0.0, (De - t.rho[iat]) * ddi);
  const double mxt = 1. - xt, mxd = 1. - xd;
  double si0t = psi0(xt), si1t = psi1(xt) * dth;
  const double si2t = psi2(xt) * dt2;
  double si0mt = psi0(mxt), si1mt = -psi1(mxt) * dth;
  const double si2mt = psi2(mxt) * dt2;
  double si0d = psi0(xd), si1d = psi1(xd) * dd;
  const double si2d = psi2(xd) * dd2;
  double si0md = psi0(mxd), si1md = -psi1(mxd) * dd;
  const double si2md = psi2(mxd) * dd2;
  double dsi0t = dpsi0(xt) * dti, dsi1t = dpsi1(xt);
  const double dsi2t = dpsi2(xt) * dth;
  double dsi0mt = -dpsi0(mxt) * dti, dsi1mt = dpsi1(mxt);
  const double dsi2mt = -dpsi2(mxt) * dth;
  double dsi0d = dpsi0(xd) * ddi, dsi1d = dpsi1(xd);
  const double dsi2d = dpsi2(xd) * dd;
  double dsi0md = -dpsi0(mxd) * ddi, dsi1md = dpsi1(mxd);
  const double dsi2md = -dpsi2(mxd) * dd;
  const double ddsi0t = ddpsi0(xt) * dt2i, ddsi1t = ddpsi1(xt) * dti, ddsi2t = ddpsi2(xt);
  const double ddsi0mt = ddpsi0(mxt) * dt2i, ddsi1mt = -ddpsi1(mxt) * dti,
               ddsi2mt = ddpsi2(mxt);
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
  corners(fi, t.dpdf);
  corners(fi + 4, t.dpdft);
  corners(fi + 8, t.dpdfd);
  corners(fi + 12, t.dpdfdt);
  pele[1] = std::max(0.0, Ye * h3(fi, si0t, si1t, si0mt, si1mt, si0d, si1d, si0md, si1md));
  corners(fi, t.ef);
  corners(fi + 4, t.eft);
  corners(fi + 8, t.efd);
  corners(fi + 12, t.efdt);
  etaele[0] = h3(fi, si0t, si1t, si0mt, si1mt, si0d, si1d, si0md, si1md);
  double x = h3(fi, si0t, si1t, si0mt, si1mt, dsi0d, dsi1d, dsi0md, dsi1md);
  etaele[1] = Ye * x;
  etaele[2] = h3(fi, dsi0t, dsi1t, dsi0mt, dsi1mt, si0d, si1d, si0md, si1md);
  etaele[3] = -x * De * Ytot;
  etaele[4] = x * rho * Ytot;
  corners(fi, t.xf);
  corners(fi + 4, t.xft);
  corners(fi + 8, t.xfd);
  corners(fi + 12, t.xfdt);
  xne[0] = h3(fi, si0t, si1t, si0mt, si1mt, si0d, si1d, si0md, si1md);
  x = std::max(0.0, h3(fi, si0t, si1t, si0mt, si1mt, dsi0d, dsi1d, dsi0md, dsi1md));
  xne[1] = Ye * x;
  xne[2] = h3(fi, dsi0t, dsi1t, dsi0mt, dsi1mt, si0d, si1d, si0md, si1md);
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

// HelmRad::GetFromDensityTemperature (:1280-1320)
void radiation(double rho, double temp, double p[5], double e[5], double s[5]) {
  const double rhoi = ratio(1.0, rho), tempi = ratio(1.0, temp);
  const double T3 = ipow<3>(temp), T4 = T3 * temp;
  const double P = PREFACTOR * T4, dPdT = 4.0 * PREFACTOR * T3;
  p[VAL] = P;
  p[DDR] = 0;
  p[DDT] = dPdT;
  p[DDA] = p[DDZ] = 0;
  const double PoR = P * rhoi;
  const double ev = 3.0 * PoR;
  const double dedT = 3.0 * dPdT * rhoi;
  e[VAL] = ev;
  e[DDR] = -ev * rhoi;
  e[DDT] = dedT;
  e[DDA] = e[DDZ] = 0;
  const double sv = (PoR + ev) * tempi;
  s[VAL] = sv;
  s[DDR] = ((0.0 - PoR) * rhoi + e[DDR]) * tempi;
  s[DDT] = (dPdT * rhoi + dedT - sv) * tempi;
  s[DDA] = s[DDZ] = 0;
}

// HelmIon::GetFromDensityTemperature (:1322-1367)
void ions(double rho, double temp, double y, double ytot, double xni, double dxnidd,
          double dxnida, double p[5], double e[5], double s[5]) {
  const double kbT = KB * temp;
  const double P = xni * kbT, dPdR = dxnidd * kbT, dPdT = xni * KB, dPdA = dxnida * kbT;
  p[VAL] = P;
  p[DDR] = dPdR;
  p[DDT] = dPdT;
  p[DDA] = dPdA;
  p[DDZ] = 0;
  const double rhoi = ratio(1.0, rho);
  const double PoR = P * rhoi;
  const double ev = 1.5 * PoR;
  const double dedR = (1.5 * dPdR - ev) * rhoi, dedT = 1.5 * dPdT * rhoi,
               dedA = 1.5 * dPdA * rhoi;
  e[VAL] = ev;
  e[DDR] = dedR;
  e[DDT] = dedT;
  e[DDA] = dedA;
  e[DDZ] = 0;
  const double tempi = ratio(1.0, temp);
  const double KBNAY = KBNA * ytot;
  s[VAL] = (PoR + ev) * tempi + KBNAY * y;
  s[DDR] = (dPdR * rhoi - P * rhoi * rhoi + dedR) * tempi - KBNAY * rhoi;
  s[DDT] = (dPdT * rhoi + dedT) * tempi - (PoR + ev) * tempi * tempi + 1.5 * KBNAY * tempi;
  s[DDA] = (dPdA * rhoi + dedA) * tempi + KBNAY * ytot * (2.5 - y);
  s[DDZ] = 0;
}

// Butterworth filter of order n: g = 1 / (1 + (f/c)^2n) and dg/df
template <int n> void butterworth(double freq, double cfreq, double &g, double &dgdf) {
  g = ratio(1.0, 1.0 + ipow<2 * n>(ratio(freq, cfreq)));
  dgdf = ratio(-ipow<2>(g) * 2 * n, ipow<2 * n>(cfreq)) * ipow<2 * n - 1>(freq);
}

// HelmCoulomb::GetFromDensityTemperature (:1369-1504)
void coulomb(double rho, double temp, double ytot, double abar, double zbar, double xni,
             double dxnidd, double dxnida, double p[5], double e[5], double s[5]) {
  constexpr double a1 = -0.898004, b1 = 0.96786, c1 = 0.220703, d1 = -0.86097, e1 = 2.5269;
  constexpr double a2 = 0.29561, b2 = 1.9885, c2 = 0.288675;
  const double kbT = KB * temp;
  const double pion = xni * kbT, dpiondd = dxnidd * kbT, dpiondt = xni * KB,
               dpionda = dxnida * kbT, dpiondz = 0.0;
  constexpr double ftpi = (4.0 / 3.0) * M_PI;
  double sv = ftpi * xni;
  const double dsdd = ftpi * dxnidd, dsda = ftpi * dxnida;
  constexpr double third = 1.0 / 3.0;
  const double si = ratio(1.0, sv);
  const double lami = ratio(1.0, std::cbrt(sv));
  const double lamidd = -lami * third * dsdd * si, lamida = -lami * third * dsda * si;
  const double plasg = ipow<2>(ELECTRON_CHARGE_ESU * zbar) / (kbT * lami);
  const double pol = ratio(plasg, lami);
  const double plasgdd = -pol * lamidd, plasgda = -pol * lamida;
  const double plasgdt = -ratio(plasg, temp), plasgdz = 2.0 * ratio(plasg, zbar);
  const double abari = ratio(1, abar);
  if (plasg >= 0) {
    const double x = std::sqrt(std::sqrt(plasg));
    double y = KBNA * ytot;
    const double c1x = ratio(c1, x);
    e[VAL] = y * temp * (a1 * plasg + b1 * x + c1x + d1);
    p[VAL] = third * rho * e[0];
    s[VAL] = -y * (3.0 * b1 * x - 5.0 * c1x + d1 * (std::log(plasg) - 1.0) - e1);
    y = KBNA * temp * ytot * (a1 + ratio(0.25, plasg) * (b1 * x - c1x));
    e[DDR] = y * plasgdd;
    e[DDT] = y * plasgdt + ratio(e[0], temp);
    e[DDA] = y * plasgda - e[0] * abari;
    e[DDZ] = y * plasgdz;
    y = third * rho;
    p[DDR] = third * e[0] + y * e[1];
    p[DDT] = y * e[2];
    p[DDA] = y * e[3];
    p[DDZ] = y * e[4];
    y = -KBNA * plasg * abari * (0.75 * b1 * x + 1.25 * c1x + d1);
    s[DDR] = y * plasgdd;
    s[DDT] = y * plasgdt;
    s[DDA] = y * plasgda - s[0] * abari;
    s[DDZ] = y * plasgdz;
  } else {
    const double x = plasg * std::sqrt(std::abs(plasg));
    const double y = std::pow(plasg, b2);
    const double z = c2 * x - third * a2 * y;
    const double plasgi = ratio(1., plasg), rhoi = ratio(1.0, rho);
    p[VAL] = -pion * z;
    e[VAL] = 3.0 * p[0] * rhoi;
    s[VAL] = -KBNA * abari * (c2 * x - a2 * ratio(b2 - 1.0, b2) * y);
    sv = 1.5 * c2 * x * plasgi - third * a2 * b2 * y * plasgi;
    p[DDR] = -dpiondd * z - pion * sv * plasgdd;
    p[DDT] = -dpiondt * z - pion * sv * plasgdt;
    p[DDA] = -dpionda * z - pion * sv * plasgda;
    p[DDZ] = -dpiondz * z - pion * sv * plasgdz;
    sv = 3.0 * rhoi;
    e[DDR] = sv * p[1] - e[0] * rhoi;
    e[DDT] = sv * p[2];
    e[DDA] = sv * p[3];
    e[DDZ] = sv * p[4];
    sv = -KBNA * abari * plasgi * (1.5 * c2 * x - a2 * (b2 - 1.0) * y);
    s[DDR] = sv * plasgdd;
    s[DDT] = sv * plasgdt;
    s[DDA] = sv * plasgda - s[0] * abari;
    s[DDZ] = sv * plasgdz;
  }
  double g_r, dgdf_r, g_t, dgdf_t;
  butterworth<12>(std::log10(temp) - 4.5, 3.0, g_r, dgdf_r);
  butterworth<12>(std::log10(rho) + 1.0, 6.0, g_t, dgdf_t);
  const double gain = (1.0 - g_t * g_r);
  const double dgaindt = -ratio(g_r * dgdf_t, temp * LN10);
  const double dgaindd = -ratio(g_t * dgdf_r, rho * LN10);
  double *arr[3] = {p, e, s};
  for (double *a : arr) {
    a[VAL] = a[VAL] * gain;
    a[DDR] = gain * a[DDR] + ratio(a[VAL] * dgaindd, gain);
    a[DDT] = gain * a[DDT] + ratio(a[VAL] * dgaindt, gain);
    a[DDA] = gain * a[DDA];
    a[DDZ] = gain * a[DDZ];
  }
}

// Options (:420-441), as the library's option bits
struct Opt {
  bool rad, gas, coul, ion, ele, newton;
};

// The per-cell electron quantities (GetElectronDensities_, :745-753)
struct Cell {
  double rho, abar, zbar, ytot, ye, ywot, De, lDe;
};
Cell cell(double rho, double abar, double zbar) {
  Cell c;
  c.rho = rho;
  c.abar = abar;
  c.zbar = zbar;
  c.ytot = ratio(1.0, abar);
  c.ye = zbar * c.ytot;
  c.ywot = std::log(ratio(abar * abar * std::sqrt(abar), rho * NA));
  c.De = rho * c.ye;
  c.lDe = std::log10(c.De);
  return c;
}

// Helmholtz::GetFromDensityLogTemperature_ (:1506-1572)
void evaluate(const Table &t, const Opt &o, const Cell &c, double T, double p[5], double e[5],
              double s[5], bool only_e) {
  double prad[5] = {0}, pion[5] = {0}, pele[5] = {0}, pcoul[5] = {0};
  double erad[5] = {0}, eion[5] = {0}, eele[5] = {0}, ecoul[5] = {0};
  double srad[5] = {0}, sion[5] = {0}, sele[5] = {0}, scoul[5] = {0};
  double etaele[5] = {0}, nep[5] = {0};
  const double lT = std::log10(T);
  const double lnT = lT / std::log10(M_E);
  const double rho = c.rho;
  if (o.rad) radiation(rho, T, prad, erad, srad);
  if (o.gas) {
    const bool unmodified = (o.ion && o.ele) || !o.ion;
    if (unmodified) {
      const double xni = NA * c.ytot * rho, dxnidd = NA * c.ytot, dxnida = -xni * c.ytot;
      ions(rho, T, c.ywot + LSWOT15 * lnT, c.ytot, xni, dxnidd, dxnida, pion, eion, sion);
    } else {
      const double abar_ion = ratio(c.abar, c.zbar + 1);
      const double ytot_ion = ratio(1.0, abar_ion);
      const double ywot_ion =
          ratio(std::log(abar_ion * abar_ion * std::sqrt(abar_ion)), rho * NA);
      const double xni = NA * ytot_ion * rho, dxnidd = NA * ytot_ion,
                   dxnida = -xni * ytot_ion;
      ions(rho, T, ywot_ion + LSWOT15 * lnT, ytot_ion, xni, dxnidd, dxnida, pion, eion, sion);
    }
    if (o.ele) {
      electrons(t, rho, lT, c.ye, c.ytot, c.De, c.lDe, pele, eele, sele, etaele, nep, only_e);
      if (o.coul) {
        const double xni = NA * c.ytot * rho, dxnidd = NA * c.ytot, dxnida = -xni * c.ytot;
        coulomb(rho, T, c.ytot, c.abar, c.zbar, xni, dxnidd, dxnida, pcoul, ecoul, scoul);
      }
    }
  }
  for (int i = 0; i < 5; ++i)
    e[i] = erad[i] + eion[i] + eele[i] + ecoul[i];
  if (!only_e)
    for (int i = 0; i < 5; ++i) {
      p[i] = prad[i] + pion[i] + pele[i] + pcoul[i];
      s[i] = srad[i] + sion[i] + sele[i] + scoul[i];
    }
}

// RootFinding1D::newton_raphson (root_finding.hpp:246-310) with
// fail_on_bound_root false: true on SUCCESS
template <typename F>
bool newton(const F &f, double ytarget, double guess, double a, double b, double ytol,
            double &xroot) {
  double x = guess, xold = 0.0;
  int iter;
  for (iter = 0; iter < 100; iter++) {
    double yg, dfunc;
    f(x, yg, dfunc);
    if (std::abs(yg - ytarget) < std::abs(ytol * ytarget)) break;
    xold = x;
    x = x - (yg - ytarget) / dfunc;
    if ((x <= a && xold <= a) || (x >= b && xold >= b)) break;
    x = std::max(std::min(x, b), a);
  }
  xroot = x;
  return iter < 100;
}

// lTAnalytic_ (:756-758)
inline double lT_analytic(double rho, double e, double ni, double ne) {
  return std::log10((2.0 / 3.0) * ratio(e * rho, ni + ne) * KBi);
}

// lTFromRhoSie_ (:867-960); lam = [Abar, Zbar, lT]; the cache receives the
// root (as the library's default mode keeps it)
double lT_from_rho_sie(const Table &t, const Opt &o, const Cell &c, double e, double *lam) {
  const double ni = ratio(1.0, c.abar) * c.rho * NA, ne = c.zbar * ni;
  double T = 0.0;
  if (o.rad || o.ele || o.coul) {
    double lTguess = lam ? lam[2] : NAN;
    if (!((t.lTMin <= lTguess) && (lTguess <= t.lTMax))) {
      lTguess = lT_analytic(c.rho, e, ni, ne);
      if (!((t.lTMin <= lTguess) && (lTguess <= t.lTMax))) lTguess = 8;
    }
    const double Tguess = pow10(lTguess), Ta = pow10(t.lTMin), Tb = pow10(t.lTMax);
    auto e_and_dedt = [&](double x, double &y, double &dy) {
      double p[5], ee[5], s[5];
      evaluate(t, o, c, x, p, ee, s, true);
      y = ee[VAL];
      dy = ee[DDT];
    };
    auto e_of = [&](double x) {
      double p[5], ee[5], s[5];
      evaluate(t, o, c, x, p, ee, s, true);
      return ee[VAL];
    };
    bool ok = o.newton ? newton(e_and_dedt, e, Tguess, Ta, Tb, HELM_EOS_EPS, T) : false;
    if (!ok) ok = regula_falsi(e_of, e, Tguess, Ta, Tb, ROOT_THRESH, ROOT_THRESH, T);
    if (!ok) T = pow10(lT_analytic(c.rho, e, ni, (o.ion ? 1.0 : 0.0) * ne));
  } else {
    T = pow10(lT_analytic(c.rho, e, ni, (o.ion ? 1.0 : 0.0) * ne));
  }
  double lT = std::log10(T);
  lT = std::max(t.lTMin, std::min(t.lTMax, lT));
  if (lam) lam[2] = lT;
  return lT;
}

std::mutex g_mu;
std::map<std::string, Table> g_tables;
const Table *table(const char *path) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(path);
  if (it != g_tables.end()) return &it->second;
  Table t;
  if (!load(path, t)) return nullptr;
  return &g_tables.emplace(path, std::move(t)).first->second;
}

} // namespace helm_port

extern "C" {

// Helmholtz::FillEos (:818-865) over n elements, OpenMP over all host
// threads; lam rows [Abar, Zbar, lT] (stride 3, required). options: the
// library's bits (1 rad, 2 gas, 4 coulomb, 8 ionized, 16 degenerate, 32
// regula falsi only). output: thermalqs bits (T or sie is the input).
int sgport_helm_fill(const char *path, int options, int n, const double *rho, double *temp,
                     double *sie, double *press, double *cv, double *bmod, unsigned output,
                     double *lam) {
  using namespace helm_port;
  const Table *t = table(path);
  if (!t || !lam) return 1;
  const Opt o{(options & 1) != 0,  (options & 2) != 0,  (options & 4) != 0,
              (options & 8) != 0,  (options & 16) != 0, (options & 32) == 0};
  const bool need_temp = (output & 8) != 0;
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    double *l = lam + 3 * static_cast<long>(i);
    const Cell c = cell(rho[i], l[0], l[1]);
    double T;
    if (need_temp) {
      T = pow10(lT_from_rho_sie(*t, o, c, sie[i], l));
      temp[i] = T;
    } else {
      T = temp[i];
      l[2] = std::log10(T);
    }
    double p[5], e[5], s[5];
    evaluate(*t, o, c, T, p, e, s, false);
    if ((output & 2) && sie) sie[i] = e[0];
    if ((output & 4) && press) press[i] = p[0];
    if ((output & 16) && cv) cv[i] = e[DDT];
    if ((output & 32) && bmod) {
      // ComputeGamma1_ (:724-732) times P
      const double chit = ratio(T, p[0]) * p[DDT];
      const double chid = ratio(p[DDR] * c.rho, p[0]);
      const double x = ratio(p[0] * chit, c.rho * T * e[DDT]);
      bmod[i] = std::max(EPS, p[0] * (chit * x + chid));
    }
  }
  return 0;
}

} // extern "C"
