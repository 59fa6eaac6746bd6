// sgport: a plain C++ restatement of singularity-eos's closure hot path.
//
// TEST INFRASTRUCTURE ONLY: the oracle. Built by oracle/build_port.sh into
// oracle/_build/libsgport.so on every machine (including the GPU machine, where
// the reference sources are absent), it exposes the same C surface as
// oracle/sgref.cpp (the reference's own headers compiled against shims).
// tests/ pin this restatement to the compiled reference through the golden
// fixtures; the GPU tests, __graft_entry__.smoke() and bench.py's CPU
// baseline then use it as the checker and the timed CPU path. The product
// library never links it.
//
// Each function cites the reference file:line it restates (paths inside
// lanl/singularity-eos). Compile with -ffp-contract=off: the arithmetic
// follows the reference's operation order so results agree bit for bit.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <string>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace port {

// ---- robust_utils.hpp:26-61 -------------------------------------------------
constexpr double SMALL = 10 * DBL_MIN;
constexpr double EPS = 10 * DBL_EPSILON;
inline int sgn(double v) { return (0.0 <= v) - (v < 0.0); }
inline double ratio(double a, double b) { return a / (b + sgn(b) * SMALL); }

// ---- fast-math/logs.hpp:113-125, 188-214, 282-292 ---------------------------
inline int64_t as_int(double f) {
  int64_t i;
  std::memcpy(&i, &f, 8);
  return i;
}
inline double as_double(int64_t i) {
  double f;
  std::memcpy(&f, &i, 8);
  return f;
}
constexpr int64_t ONE_AS_INT = (int64_t(1) << 62) - (int64_t(1) << 52);
inline double lg(double x) {
  const int64_t xi = as_int(x) - ONE_AS_INT;
  const int64_t frac = xi & ((int64_t(1) << 52) - 1);
  const int64_t hi = frac >> 26, lo = frac & ((int64_t(1) << 26) - 1);
  const int64_t fsq = hi * hi + ((hi * lo) >> 25);
  return static_cast<double>(xi + ((frac - fsq) / 3)) * 2.22044604925031e-16;
}
inline double pow2(double x) {
  const int64_t xi = static_cast<int64_t>(x * static_cast<double>(int64_t(1) << 52));
  const int64_t frac = xi & ((int64_t(1) << 52) - 1);
  const int64_t fsqrt = static_cast<int64_t>(
      67108864.0 * std::sqrt(static_cast<double>(int64_t(18014398509481984) - 3 * frac)));
  return as_double(xi + int64_t(9007199254740992) - fsqrt - frac + ONE_AS_INT);
}
inline double log10(double x) { return 0.301029995663981195 * lg(x); }
inline double pow10(double x) { return pow2(3.321928094887362626 * x); }
// eos_spiner_common.hpp:52-57
inline double to_log(double x, double off) {
  return log10(std::abs(std::max(x, -off) + off) + EPS);
}
inline double from_log(double lx, double off) { return pow10(lx) - off; }

// ---- root_finding.hpp:114-240 -----------------------------------------------
template <typename F>
bool set_bracket(const F &f, double &a, double guess, double &b, double &ya, double yg,
                 double &yb) {
  const double dx = b - a;
  for (std::size_t level = 0; level < 6; level++) {
    const std::size_t nlev = std::size_t(1) << level;
    for (std::size_t i = 0; i < nlev; i++) {
      const double x = a + (i + 0.5) * dx;
      const double yx = f(x);
      if (yx * yg <= 0.0) {
        if (x < guess) {
          a = x, ya = yx, b = guess, yb = yg;
        } else {
          a = guess, ya = yg, b = x, yb = yx;
        }
        return true;
      }
    }
  }
  return false;
}
// returns true on success
template <typename F>
bool regula_falsi(const F &f, double ytarget, double guess, double a, double b, double xtol,
                  double ytol, double &xroot) {
  auto func = [&](double x) { return f(x) - ytarget; };
  double ya = func(a), yg = func(guess), yb;
  if (ya * yg <= 0.0) {
    b = guess, yb = yg;
  } else {
    yb = func(b);
    if (yg * yb <= 0.0) {
      a = guess, ya = yg;
    } else if (!set_bracket(func, a, guess, b, ya, yg, yb)) {
      return false;
    }
  }
  const double sign = ya < 0 ? 1.0 : -1.0;
  ya *= sign;
  yb *= sign;
  std::size_t b1 = 0, b2 = 0, it = 0;
  while (b - a > 2.0 * xtol && (std::abs(ya) > ytol || std::abs(yb) > ytol) && it < 1000) {
    const double c = (a * yb - b * ya) / (yb - ya);
    if (c == a) {
      b = a;
      continue;
    }
    if (c == b) {
      a = b;
      continue;
    }
    const double yc = sign * func(c);
    if (yc > 0.0) {
      b = c, yb = yc, b1++;
      ya *= (b1 > 1 ? 0.5 : 1.0);
      b2 = 0;
    } else if (yc < 0.0) {
      a = c, ya = yc, b2++;
      yb *= (b2 > 1 ? 0.5 : 1.0);
      b1 = 0;
    } else {
      a = c, b = c;
    }
    it++;
  }
  xroot = 0.5 * (a + b);
  return it != 1000;
}

// ---- spiner-lite interpolation (the formula the oracle shims define) --------
struct Grid {
  double min = 0, max = 0, dx = 0, idx = 0;
  int n = 0;
  Grid() = default;
  Grid(double a, double b, int N) : min(a), max(b), dx((b - a) / double(N - 1)), n(N) {
    idx = 1 / dx;
  }
  double x(int i) const { return min + i * dx; }
  void w(double x, int &i, double &w0, double &w1) const {
    const double u = (x - min) * idx;
    i = !(u >= 0) ? 0 : (u > double(n - 2) ? n - 2 : int(u));
    w1 = (x - (min + i * dx)) * idx;
    w0 = 1 - w1;
  }
};
inline double lin(const Grid &g, const std::vector<double> &d, double x) {
  int i;
  double w0, w1;
  g.w(x, i, w0, w1);
  return w0 * d[i] + w1 * d[i + 1];
}
inline double bilin(const Grid &gT, const Grid &gR, const std::vector<double> &d, double lRho,
                    double lT) {
  int i, j;
  double a0, a1, b0, b1;
  gT.w(lT, i, a0, a1);
  gR.w(lRho, j, b0, b1);
  const double *r0 = d.data() + j * gT.n + i, *r1 = r0 + gT.n;
  return b0 * (a0 * r0[0] + a1 * r0[1]) + b1 * (a0 * r1[0] + a1 * r1[1]);
}

// ---- SpinerEOSDependsRhoT table (eos_spiner_rho_temp.hpp:545-775) ---------
struct Table {
  Grid gT, gR, gC;
  int nR = 0, nT = 0;
  double lRhoOff = 0, lTOff = 0, lRhoMin = 0, lRhoMax = 0, rhoMax = 0, lTMin = 0, lTMax = 0,
         TMax = 0, PMin = 0;
  bool reproducible = false;
  std::vector<double> P, sie, bMod, dPdRho, dPdE, dTdRho, dTdE, dEdRho, dEdT;
  std::vector<double> PMax, sielTMax, dEdTMax, gm1Max, lTColdCrit, PCold, sieCold, bModCold,
      dPdRhoCold, dPdECold, dTdRhoCold, dTdECold, dEdTCold, rho_at_pmin;
  double lRho(double r) const { return to_log(r, lRhoOff); }
  double lT(double t) const { return to_log(t, lTOff); }
  double rho(double l) const {
    const double r = from_log(l, lRhoOff);
    return r < 0 ? 0 : r;
  }
  double T(double l) const { return from_log(l, lTOff); }
  double f2(const std::vector<double> &d, double lr, double lt) const {
    return bilin(gT, gR, d, lr, lt);
  }
};

// Reads an sp5-lite image (format documented in sgx/sp5lite.py).
bool load_table(const char *path, int matid, Table &t) {
  FILE *f = std::fopen(path, "rb");
  if (!f) return false;
  auto rd = [&](void *p, size_t n) { return std::fread(p, 1, n, f) == n; };
  auto rds = [&](std::string &s) {
    uint32_t n;
    if (!rd(&n, 4)) return false;
    s.resize(n);
    return n == 0 || rd(&s[0], n);
  };
  char magic[8];
  uint32_t ver, nrec;
  bool ok = rd(magic, 8) && rd(&ver, 4) && rd(&nrec, 4) && std::memcmp(magic, "SGXSP5L", 8) == 0;
  std::map<std::string, double> attr;
  std::map<std::string, std::pair<std::vector<double>, std::vector<double>>> ds;
  for (uint32_t k = 0; ok && k < nrec; ++k) {
    uint32_t kind;
    std::string p, n;
    ok = rd(&kind, 4) && rds(p) && rds(n);
    if (kind == 1) {
      double v;
      ok = ok && rd(&v, 8);
      attr[p + "@" + n] = v;
    } else if (kind == 2) {
      int32_t v;
      ok = ok && rd(&v, 4);
    } else if (kind == 4) {
      std::string v;
      ok = ok && rds(v);
    } else if (kind == 3) {
      uint32_t r;
      ok = ok && rd(&r, 4);
      std::vector<double> meta;
      size_t tot = 1;
      for (uint32_t q = 0; ok && q < r; ++q) {
        int32_t nn;
        double a, b;
        ok = rd(&nn, 4) && rd(&a, 8) && rd(&b, 8);
        meta.insert(meta.end(), {double(nn), a, b});
        tot *= size_t(nn);
      }
      std::vector<double> d(tot);
      ok = ok && rd(d.data(), tot * 8);
      ds[p] = {meta, d};
    }
  }
  std::fclose(f);
  if (!ok) return false;
  const std::string g = "/" + std::to_string(matid);
  auto get2 = [&](const char *name, std::vector<double> &out) {
    auto it = ds.find(g + "/dependsLogRhoLogT/" + name);
    if (it == ds.end()) return false;
    out = it->second.second;
    const auto &m = it->second.first;
    t.nT = int(m[0]);
    t.nR = int(m[3]);
    t.gT = Grid(m[1], m[2], t.nT);
    t.gR = Grid(m[4], m[5], t.nR);
    return true;
  };
  auto get1 = [&](const char *name, std::vector<double> &out) {
    auto it = ds.find(g + "/coldCurve/" + name);
    if (it == ds.end()) return false;
    out = it->second.second;
    const auto &m = it->second.first;
    t.gC = Grid(m[1], m[2], int(m[0]));
    return true;
  };
  ok = get2("pressure", t.P) && get2("specific internal energy", t.sie) &&
       get2("bulk modulus", t.bMod) && get2("dPdRho", t.dPdRho) && get2("dPdE", t.dPdE) &&
       get2("dTdRho", t.dTdRho) && get2("dTdE", t.dTdE) && get2("dEdRho", t.dEdRho) &&
       get2("dEdT", t.dEdT) && get1("pressure", t.PCold) &&
       get1("specific internal energy", t.sieCold) && get1("bulk modulus", t.bModCold) &&
       get1("dPdRho", t.dPdRhoCold);
  if (!ok || !attr.count(g + "@rhoOffset") || !attr.count(g + "@TOffset")) return false;
  t.lRhoOff = std::abs(attr[g + "@rhoOffset"]);
  t.lTOff = std::abs(attr[g + "@TOffset"]);
  const int nR = t.nR, nT = t.nT;
  // bounds (:601-608)
  t.lRhoMin = t.gR.min, t.lRhoMax = t.gR.max, t.rhoMax = from_log(t.lRhoMax, t.lRhoOff);
  t.lTMin = t.gT.min, t.lTMax = t.gT.max, t.TMax = from_log(t.lTMax, t.lTOff);
  // fixBulkModulus_ (:689-714)
  for (int j = 0; j < nR; j++) {
    const double lr = t.gR.x(j), r = t.rho(lr);
    for (int i = 0; i < nT; i++) {
      const double lt = t.gT.x(i);
      const double press = t.f2(t.P, lr, lt), DPDR_E = t.f2(t.dPdRho, lr, lt),
                   DPDE_R = t.f2(t.dPdE, lr, lt), DEDR_T = t.f2(t.dEdRho, lr, lt);
      const double DPDR_T = DPDR_E + DPDE_R * DEDR_T;
      double b;
      if (DPDE_R > 0.0 && r > 0.0)
        b = r * DPDR_E + DPDE_R * (press / r);
      else if (r > 0.0)
        b = std::max(r * DPDR_T, 0.0);
      else
        b = 0.0;
      t.bMod[j * nT + i] = std::max(b, std::abs(EPS));
    }
  }
  // setlTColdCrit_ (:716-775)
  t.lTColdCrit.assign(nR, 0.0);
  for (int j = 0; j < nR; j++) {
    const double lr = t.gC.x(j), sc = lin(t.gC, t.sieCold, lr);
    std::vector<int> cross;
    int last_pos = -1;
    for (int i = 0; i < nT - 1; i++) {
      const double c0 = t.sie[j * nT + i] - sc, c1 = t.sie[j * nT + i + 1] - sc;
      if (c0 < 0 && c1 > 0) {
        cross.push_back(i);
        last_pos = int(cross.size()) - 1;
      } else if (c0 > 0 && c1 < 0) {
        cross.push_back(i);
      }
    }
    double lt;
    if (last_pos <= 0) {
      lt = t.lTMin;
    } else {
      const int il = cross[last_pos];
      const double lo = t.gT.x(il) - 1.0e-14, hi = t.gT.x(il + 1) + 1.0e-14;
      const double guess = 0.5 * (lo + hi);
      auto fs = [&](double x) { return t.f2(t.sie, lr, x); };
      if (!regula_falsi(fs, sc, guess, lo, hi, 1e-14, 1e-14, lt)) lt = guess;
    }
    t.lTColdCrit[j] = std::max(t.lTMin, lt);
  }
  // SetRhoPMin (eos_spiner_common.hpp:59-109), vapor dome not excluded
  t.rho_at_pmin.assign(nT, 0.0);
  double PMin = std::numeric_limits<double>::max();
  for (int i = 0; i < nT; ++i) {
    double pm = std::numeric_limits<double>::max();
    int jm = 0;
    for (int j = 0; j < nR; ++j)
      if (t.P[j * nT + i] < pm) pm = t.P[j * nT + i], jm = j;
    if (pm > 0) {
      t.rho_at_pmin[i] = 0, pm = 0;
    } else {
      t.rho_at_pmin[i] = from_log(t.gR.x(jm), t.lRhoOff);
    }
    PMin = std::min(pm, PMin);
  }
  t.PMin = PMin;
  // cold-curve and maximum-temperature tables (:629-656)
  for (auto *v : {&t.dPdECold, &t.dTdRhoCold, &t.dTdECold, &t.dEdTCold})
    v->assign(nR, 0.0);
  for (int j = 0; j < nR; j++) {
    const double lr = t.gC.x(j), lt = t.lTColdCrit[j];
    t.bModCold[j] = t.f2(t.bMod, lr, lt);
    t.dPdECold[j] = t.f2(t.dPdE, lr, lt);
    t.dTdRhoCold[j] = t.f2(t.dTdRho, lr, lt);
    t.dTdECold[j] = t.f2(t.dTdE, lr, lt);
    t.dEdTCold[j] = t.f2(t.dEdT, lr, lt);
  }
  for (auto *v : {&t.PMax, &t.sielTMax, &t.dEdTMax, &t.gm1Max})
    v->assign(nR, 0.0);
  for (int j = 0; j < nR; j++) {
    const double r = t.rho(t.gR.x(j));
    t.PMax[j] = t.P[j * nT + nT - 1];
    t.dEdTMax[j] = t.dEdT[j * nT + nT - 1];
    t.gm1Max[j] = ratio(t.dPdE[j * nT + nT - 1], r);
    t.sielTMax[j] = t.sie[j * nT + nT - 1];
  }
  return true;
}

enum Where { OnTable = 0, OffBottom = 1, OffTop = 2 };

// ---- EOS models ---------------------------------------------------------------
struct Eos {
  int type = 0;
  double p[16] = {};
  const Table *tab = nullptr;
  static constexpr unsigned DENS = 1, SIE = 2, PRES = 4, TEMP = 8, CV = 16, BMOD = 32;

  unsigned preferred() const {
    if (type == 1) return DENS | SIE | TEMP | PRES; // eos_ideal.hpp:227-229
    if (type == 5) return DENS | TEMP;              // eos_spiner_rho_temp.hpp:182
    return DENS | SIE;
  }
  // Gruneisen (eos_gruneisen.hpp:191-195, 331-371, 478-526)
  double gGamma(double rin) const {
    const double r = std::min(rin, p[11]);
    return r < p[6] ? p[4] : p[4] * p[6] / r + p[5] * (1 - p[6] / r);
  }
  double gP(double rin, double e) const {
    const double r = std::min(rin, p[11]);
    double PH, EH;
    if (r >= p[6]) {
      const double eta = 1 - p[6] / r;
      const double s = p[1] * eta + p[2] * (eta * eta) + p[3] * (eta * (eta * eta));
      PH = p[8] + (p[0] * p[0]) * p[6] * eta / ((1 - s) * (1 - s));
      EH = (PH + p[8]) * eta / p[6] / 2.;
    } else {
      PH = p[8] + (p[0] * p[0]) * (r - p[6]);
      EH = 0.;
    }
    return PH + gGamma(r) * r * (e - EH);
  }
  double gdPdr(double rin, double e) const {
    const double r = std::min(rin, p[11]);
    if (r < p[6]) return (p[0] * p[0]) + gGamma(r) * e;
    const double eta = 1 - p[6] / r;
    const double s = p[1] * eta + p[2] * (eta * eta) + p[3] * (eta * (eta * eta));
    const double ds = p[1] + 2 * p[2] * eta + 3 * p[3] * (eta * eta);
    const double deta = p[6] / (r * r), dGam = (p[5] - p[4]) * deta;
    const double PH = p[8] + (p[0] * p[0]) * p[6] * eta / ((1 - s) * (1 - s));
    const double dPH = (p[0] * p[0]) * p[6] / ((1 - s) * (1 - s)) * deta * (1 + 2 * eta * ds / (1 - s));
    const double EH = (PH + p[8]) * eta / p[6] / 2.;
    const double dEH = deta * (PH + p[8]) / p[6] / 2. + eta / p[6] / 2 * dPH;
    return dPH + gGamma(r) * (e - EH) + r * dGam * (e - EH) - r * gGamma(r) * dEH;
  }
  double gE(double T) const { return p[9] * (T - p[7]); }
  double gB(double rin, double e) const {
    const double r = std::min(rin, p[11]);
    if (r < p[6]) return r * (p[0] * p[0]) + p[4] * (r * e + gP(r, e));
    return r * gdPdr(r, e) + gP(r, e) / r * (r * gGamma(r));
  }
  double gMaxStable(double T) const { // :423-477
    if (gdPdr(p[11], gE(T)) >= 0) return p[11];
    const double lo = p[6], hi = std::min(p[11], 1.0e4), guess = (lo + hi) / 2.;
    double root = guess;
    regula_falsi([&](double r) { return gdPdr(r, gE(T)); }, 0., guess, lo, hi, 1e-8, 1e-8, root);
    return root;
  }

  // spiner helpers (:1192-1404)
  Where locRhoSie(double lr, double e) const {
    const double stm = lin(tab->gR, tab->sielTMax, lr), sc = lin(tab->gC, tab->sieCold, lr);
    if (e >= stm - 1e-8 * std::abs(stm)) return OffTop;
    if (e <= sc + 1e-8 * std::abs(sc)) return OffBottom;
    return OnTable;
  }
  Where locRhoT(double lt) const {
    if (lt <= (1 + 1e-8) * tab->lTMin) return OffBottom;
    if (lt >= (1 - 1e-8) * tab->lTMax) return OffTop;
    return OnTable;
  }
  double lTFromlRhoSie(double lr, double e, Where &w, double *lam) const {
    const Table &t = *tab;
    double lt;
    w = locRhoSie(lr, e);
    if (w == OffBottom) {
      lt = t.lTMin;
    } else if (w == OffTop) {
      lt = t.lT(t.TMax + ratio(e - lin(t.gR, t.sielTMax, lr), lin(t.gR, t.dEdTMax, lr)));
    } else {
      double guess = t.reproducible ? t.lTMin : 0.5 * (t.lTMin + t.lTMax);
      if (lam && t.lTMin <= lam[1] && lam[1] <= t.lTMax) guess = lam[1];
      if (!regula_falsi([&](double x) { return t.f2(t.sie, lr, x); }, e, guess, t.lTMin,
                        t.lTMax, 1e-14, 1e-14, lt))
        lt = t.reproducible ? t.lTMin : guess;
    }
    if (lam) lam[0] = lr, lam[1] = lt;
    return lt;
  }
  double sieFrom(double lr, double T, double lt, Where w) const {
    const Table &t = *tab;
    if (w == OffBottom) return lin(t.gC, t.sieCold, lr);
    if (w == OffTop) return lin(t.gR, t.sielTMax, lr) + lin(t.gR, t.dEdTMax, lr) * (T - t.TMax);
    return t.f2(t.sie, lr, lt);
  }
  double PFrom(double r, double lr, double T, double lt, Where w) const {
    const Table &t = *tab;
    if (w == OffBottom) return lin(t.gC, t.PCold, lr);
    if (w == OffTop) {
      const double Cv = lin(t.gR, t.dEdTMax, lr), gm1 = lin(t.gR, t.gm1Max, lr);
      return gm1 * r * (lin(t.gR, t.sielTMax, lr) + Cv * (T - t.TMax));
    }
    return t.f2(t.P, lr, lt);
  }
  double CvFrom(double lr, double lt, Where w) const {
    const Table &t = *tab;
    double c = w == OffBottom ? lin(t.gC, t.dEdTCold, lr)
               : w == OffTop  ? lin(t.gR, t.dEdTMax, lr)
                              : t.f2(t.dEdT, lr, lt);
    return c > EPS ? c : EPS;
  }
  double BFrom(double r, double lr, double T, double lt, Where w) const {
    const Table &t = *tab;
    double b;
    if (w == OffBottom) {
      b = lin(t.gC, t.bModCold, lr);
    } else if (w == OffTop) {
      const double Cv = lin(t.gR, t.dEdTMax, lr), gm1 = lin(t.gR, t.gm1Max, lr);
      b = (gm1 + 1) * gm1 * r * (lin(t.gR, t.sielTMax, lr) + Cv * (T - t.TMax));
    } else {
      b = t.f2(t.bMod, lr, lt);
    }
    return b > EPS ? b : EPS;
  }
  double GFrom(double r, double lr, double lt, Where w) const {
    const Table &t = *tab;
    if (w == OffBottom) return ratio(std::abs(lin(t.gC, t.dPdECold, lr)), std::abs(r));
    if (w == OffTop) return lin(t.gR, t.gm1Max, lr);
    return ratio(std::abs(t.f2(t.dPdE, lr, lt)), std::abs(r));
  }
  void logsRhoT(double r, double T, double &lr, double &lt, double *lam) const {
    lr = tab->lRho(r), lt = tab->lT(T);
    if (lam) lam[0] = lr, lam[1] = lt;
  }
  double lRhoFromPlT(double P, double lt, double *lam) const { // :1135-1190
    const Table &t = *tab;
    const double rpm = t.lRho(lin(t.gT, t.rho_at_pmin, lt));
    double guess = t.reproducible ? t.lRhoMax : 0.5 * (rpm + t.lRhoMax), lr;
    if (lam && rpm <= lam[0] && lam[0] <= t.lRhoMax) guess = lam[0];
    bool ok;
    if (lt <= t.lTMin)
      ok = regula_falsi([&](double x) { return lin(t.gC, t.PCold, x); }, P, guess, rpm,
                        t.lRhoMax, 1e-14, 1e-14, lr);
    else if (lt >= t.lTMax)
      ok = regula_falsi(
          [&](double x) { return lin(t.gR, t.gm1Max, x) * lin(t.gR, t.dEdTMax, x) * lt * x; }, P,
          guess, rpm, t.lRhoMax, 1e-14, 1e-14, lr);
    else
      ok = regula_falsi([&](double x) { return t.f2(t.P, x, lt); }, P, guess, rpm, t.lRhoMax,
                        1e-14, 1e-14, lr);
    if (!ok) lr = t.reproducible ? t.lRhoMax : guess;
    if (lam) lam[0] = lr, lam[1] = lt;
    return lr;
  }

  // ---- scalar API (model files cited in sgx_eos.cuh's order) ----
  double T_re(double r, double e, double *lam) const {
    switch (type) {
    case 1: { const double v = e / p[1]; return 0.0 > v ? 0.0 : v; }
    case 2: return std::max(SMALL, ratio(r * (e - p[3]) - p[2], r * p[1]));
    case 3: return std::max(SMALL, (e - p[3]) / p[1]);
    case 4: return p[7] + e / p[9];
    case 5: { Where w; return tab->T(lTFromlRhoSie(tab->lRho(r), e, w, lam)); }
    }
    return 0;
  }
  double e_rT(double r, double T, double *lam) const {
    switch (type) {
    case 1: { const double v = p[1] * T; return 0.0 > v ? 0.0 : v; }
    case 2: return std::max(p[3], ratio(r * p[1] * T + p[2], r) + p[3]);
    case 3: return std::max(p[3], p[1] * T + p[3]);
    case 4: return gE(T);
    case 5: { double lr, lt; logsRhoT(r, T, lr, lt, lam); return sieFrom(lr, T, lt, locRhoT(lt)); }
    }
    return 0;
  }
  double P_rT(double r, double T, double *lam) const {
    switch (type) {
    case 1: { const double v = p[0] * r * p[1] * T; return 0.0 > v ? 0.0 : v; }
    case 2: return std::max(-p[2], p[0] * r * p[1] * T - p[2]);
    case 3: return std::max(SMALL, ratio(p[0] * r * p[1] * T, 1.0 - p[2] * r));
    case 4: { const double rr = std::min(r, p[11]); return gP(rr, gE(T)); }
    case 5: { double lr, lt; logsRhoT(r, T, lr, lt, lam); return PFrom(r, lr, T, lt, locRhoT(lt)); }
    }
    return 0;
  }
  double P_re(double r, double e, double *lam) const {
    switch (type) {
    case 1: { const double v = p[0] * r * e; return 0.0 > v ? 0.0 : v; }
    case 2: return std::max(-p[2], p[0] * r * (e - p[3]) - (p[0] + 1.0) * p[2]);
    case 3: return std::max(SMALL, ratio(p[0] * r * (e - p[3]), 1.0 - p[2] * r));
    case 4: return gP(r, e);
    case 5: {
      Where w;
      const double lr = tab->lRho(r), lt = lTFromlRhoSie(lr, e, w, lam);
      if (w == OffBottom) return lin(tab->gC, tab->PCold, lr);
      if (w == OffTop) return lin(tab->gR, tab->gm1Max, lr) * r * e;
      return tab->f2(tab->P, lr, lt);
    }
    }
    return 0;
  }
  double Cv_rT(double r, double T, double *lam) const {
    if (type == 5) { double lr, lt; logsRhoT(r, T, lr, lt, lam); return CvFrom(lr, lt, locRhoT(lt)); }
    return type == 4 ? p[9] : p[1];
  }
  double Cv_re(double r, double e, double *lam) const {
    if (type == 5) { Where w; const double lr = tab->lRho(r), lt = lTFromlRhoSie(lr, e, w, lam); return CvFrom(lr, lt, w); }
    return type == 4 ? p[9] : p[1];
  }
  double B_rT(double r, double T, double *lam) const {
    switch (type) {
    case 1: { const double v = (p[0] + 1) * p[0] * r * p[1] * T; return 0.0 > v ? 0.0 : v; }
    case 2: return std::max(SMALL, p[0] * (p[0] + 1.0) * r * p[1] * T);
    case 3: return std::max(SMALL, ratio(p[0] * (p[0] + 1.0) * r * p[1] * T, (1.0 - p[2] * r) * (1.0 - p[2] * r)));
    case 4: { const double rr = std::min(r, p[11]); return gB(rr, gE(T)); }
    case 5: { double lr, lt; logsRhoT(r, T, lr, lt, lam); return BFrom(r, lr, T, lt, locRhoT(lt)); }
    }
    return 0;
  }
  double B_re(double r, double e, double *lam) const {
    switch (type) {
    case 1: { const double v = (p[0] + 1) * p[0] * r * e; return 0.0 > v ? 0.0 : v; }
    case 2: return std::max(SMALL, p[0] * (p[0] + 1.0) * (r * (e - p[3]) - p[2]));
    case 3: return std::max(SMALL, ratio(p[0] * (p[0] + 1.0) * r * (e - p[3]), (1.0 - p[2] * r) * (1.0 - p[2] * r)));
    case 4: return gB(r, e);
    case 5: {
      Where w;
      const double lr = tab->lRho(r), lt = lTFromlRhoSie(lr, e, w, lam);
      if (w == OffBottom) return lin(tab->gC, tab->bModCold, lr);
      if (w == OffTop) { const double g = lin(tab->gR, tab->gm1Max, lr); return (g + 1) * g * r * e; }
      return tab->f2(tab->bMod, lr, lt);
    }
    }
    return 0;
  }
  double G_rT(double r, double T, double *lam) const {
    if (type == 5) { double lr, lt; logsRhoT(r, T, lr, lt, lam); return GFrom(r, lr, lt, locRhoT(lt)); }
    if (type == 3) return ratio(p[0], 1.0 - p[2] * r);
    if (type == 4) return gGamma(std::min(r, p[11]));
    return p[0];
  }
  double G_re(double r, double e, double *lam) const {
    if (type == 5) { Where w; const double lr = tab->lRho(r), lt = lTFromlRhoSie(lr, e, w, lam); return GFrom(r, lr, lt, w); }
    return G_rT(r, 0, lam);
  }
  double minE(double r) const {
    switch (type) {
    case 1: return 0.0;
    case 2: return e_rT(r, 0., nullptr);
    case 3: return p[3];
    case 4: return gE(0.);
    case 5: return lin(tab->gC, tab->sieCold, tab->lRho(r));
    }
    return 0;
  }
  // bounds (eos_base.hpp:594-613 and overrides)
  double minT() const { return type == 5 ? tab->T(tab->lTMin) : 0; }
  double maxRho() const { return type == 4 ? p[11] : type == 5 ? tab->rhoMax : 1e100; }
  double minP() const { return type == 4 ? gP(0, 0) : type == 5 ? tab->PMin : 0; }
  double maxPAtT(double T) const { return type == 4 ? gMaxStable(T) : 1e100; }
  double rhoPmin(double T) const {
    if (type != 5) return 0.0;
    const double lt = tab->lT(T);
    if (lt <= tab->lTMin) return tab->rho_at_pmin[0];
    if (lt >= tab->lTMax) return 0.0;
    return lin(tab->gT, tab->rho_at_pmin, lt);
  }
  void rhoSieFromPT(double P, double T, double *lam, double &r, double &e) const {
    switch (type) {
    case 1: { const double s = p[1] * T; e = 0.0 > s ? 0.0 : s; const double q = P / (p[0] * e); r = 0.0 > q ? 0.0 : q; return; }
    case 2:
      e = std::max(p[3], ratio(P + (p[0] + 1.0) * p[2], P + p[2]) * p[1] * T + p[3]);
      r = std::max(SMALL, ratio(P + p[2], p[0] * p[1] * T));
      return;
    case 3:
      e = std::max(p[3], p[1] * T + p[3]);
      r = std::max(SMALL, ratio(P, p[0] * p[1] * T + p[2] * P));
      return;
    case 4: { // eos_gruneisen.hpp:478-526
      auto PofR = [&](double x) { return P_rT(x, T, nullptr); };
      const double Pref = PofR(p[6]);
      double lo, hi, guess, pu = P;
      if (P < Pref) {
        lo = 0., hi = 1.1 * p[6], guess = p[6];
      } else {
        lo = 0.9 * p[6];
        hi = gMaxStable(T);
        const double pmax = PofR(hi);
        if (P > pmax) pu = pmax;
        guess = p[6] + (hi - p[6]) / (pmax - Pref) * (pu - Pref);
      }
      regula_falsi(PofR, pu, guess, lo, hi, 1e-8, 1e-8, r);
      e = gE(T);
      return;
    }
    case 5: {
      const double lt = tab->lT(T);
      r = tab->rho(lRhoFromPlT(P, lt, lam));
      e = e_rT(r, T, lam);
      return;
    }
    }
  }
  // FillEos per model (eos_ideal.hpp:236-262 and siblings; spiner :1052-1101)
  bool fill(double &r, double &T, double &e, double &P, double &cv, double &B, unsigned out,
            double *lam) const {
    if (type <= 3) {
      if ((out & DENS) && (out & SIE)) {
        if ((out & PRES) || (out & TEMP)) return false;
        rhoSieFromPT(P, T, lam, r, e);
      }
      if ((out & PRES) && (out & SIE)) {
        if ((out & DENS) || (out & TEMP)) return false;
        e = e_rT(r, T, lam);
      }
      if ((out & TEMP) && (out & SIE)) {
        e = type == 1 ? P / (p[0] * r)
            : type == 2 ? ratio(P + (p[0] + 1.0) * p[2], p[0] * r) + p[3]
                        : P * (1.0 - p[2] * r) / p[0] + p[3];
      }
      if (out & PRES) P = P_re(r, e, lam);
      if (out & TEMP) T = T_re(r, e, lam);
      if (out & BMOD) B = B_re(r, e, lam);
      if (out & CV) cv = p[1];
      return true;
    }
    if (type == 4) {
      const unsigned in = ~out;
      if ((TEMP & in) && (PRES & in))
        rhoSieFromPT(P, T, lam, r, e);
      else if ((DENS & out) || (SIE & out))
        return false;
      const double rr = std::min(r, p[11]);
      if (out & PRES) P = gP(rr, e);
      if (out & TEMP) T = p[7] + e / p[9];
      if (out & BMOD) B = gB(rr, e);
      if (out & CV) cv = p[9];
      return true;
    }
    const Table &t = *tab;
    const unsigned in = ~out;
    double lr, lt;
    Where w;
    if (out == 0) return false;
    if (out & DENS) {
      if (!((in & PRES) && (in & TEMP))) return false;
      lt = t.lT(T);
      lr = lRhoFromPlT(P, lt, lam);
      r = t.rho(lr);
    } else {
      lr = t.lRho(r);
    }
    if (out & TEMP) {
      if (!((in & DENS) && (in & SIE))) return false;
      lt = lTFromlRhoSie(lr, e, w, lam);
      T = t.T(lt);
    } else {
      lt = t.lT(T);
    }
    w = locRhoT(lt);
    if (out & SIE) e = sieFrom(lr, T, lt, w);
    if (out & PRES) P = PFrom(r, lr, T, lt, w);
    if (out & CV) cv = CvFrom(lr, lt, w);
    if (out & BMOD) B = BFrom(r, lr, T, lt, w);
    if (lam) lam[0] = lr, lam[1] = lt;
    return true;
  }
};

// ---- closure/mixed_cell_models.hpp ------------------------------------------
struct Mix {
  bool iterate_t_guess;
  double derivative_eps, tol_p, tol_e, tol_v, abs_p, slow, tol_p_s, tol_e_s, tol_v_s, abs_p_s;
  std::size_t max_iter_per_mat, ls_max_iter, small_step_tries;
  double ls_alpha, ls_fac, vsafety, Tlimit, Tguess0, small_step_thresh, max_dpdv;
  int64_t exclude;
};

inline bool finite_(double a) { return (a == a) && ((a == 0) || (a != 2 * a)); } // :155-157

// solve_Ax_b_wscr (:176-278); n >= 3 by column-pivoted Householder QR with
// Eigen's reflector convention (the Eigen-lite restatement in oracle/shims).
bool solve(std::size_t n, double *a, double *b, double *scr) {
  for (std::size_t row = 0; row < n; ++row) {
    double mx = 0;
    for (std::size_t c = 0; c < n; ++c)
      mx = std::max(std::abs(a[row * n + c]), mx);
    if (mx == 0) return false;
    for (std::size_t c = 0; c < n; ++c)
      a[row * n + c] /= mx;
    b[row] /= mx;
  }
  if (n == 1) {
    b[0] = ratio(b[0], a[0]);
  } else if (n == 2) {
    const double det = a[0] * a[3] - a[1] * a[2];
    scr[0] = ratio(a[3] * b[0] - a[1] * b[1], det);
    scr[1] = ratio(a[0] * b[1] - a[2] * b[0], det);
    b[0] = scr[0], b[1] = scr[1];
  } else {
    const int N = int(n);
    std::vector<double> R(a, a + n * n);
    std::vector<int> perm(n);
    for (int j = 0; j < N; ++j)
      perm[j] = j;
    for (int k = 0; k < N; ++k) {
      int pv = k;
      double cmax = -1.0;
      for (int j = k; j < N; ++j) {
        double c = 0.0;
        for (int i = k; i < N; ++i)
          c += R[i * N + j] * R[i * N + j];
        if (c > cmax) cmax = c, pv = j;
      }
      if (pv != k) {
        for (int i = 0; i < N; ++i)
          std::swap(R[i * N + k], R[i * N + pv]);
        std::swap(perm[k], perm[pv]);
      }
      double sigma = 0.0;
      for (int i = k + 1; i < N; ++i)
        sigma += R[i * N + k] * R[i * N + k];
      if (sigma == 0.0) continue;
      const double x0 = R[k * N + k], mu = std::sqrt(x0 * x0 + sigma);
      const double beta = x0 >= 0.0 ? -mu : mu, v0 = x0 - beta, tau = (beta - x0) / beta;
      for (int i = k + 1; i < N; ++i)
        R[i * N + k] = R[i * N + k] / v0;
      R[k * N + k] = beta;
      for (int j = k + 1; j < N; ++j) {
        double s = R[k * N + j];
        for (int i = k + 1; i < N; ++i)
          s += R[i * N + k] * R[i * N + j];
        s = s * tau;
        R[k * N + j] -= s;
        for (int i = k + 1; i < N; ++i)
          R[i * N + j] -= s * R[i * N + k];
      }
      double s = b[k];
      for (int i = k + 1; i < N; ++i)
        s += R[i * N + k] * b[i];
      s = s * tau;
      b[k] -= s;
      for (int i = k + 1; i < N; ++i)
        b[i] -= s * R[i * N + k];
    }
    std::vector<double> z(n);
    for (int i = N - 1; i >= 0; --i) {
      double s = b[i];
      for (int j = i + 1; j < N; ++j)
        s -= R[i * N + j] * z[j];
      z[i] = R[i * N + i] == 0.0 ? 0.0 : s / R[i * N + i];
    }
    for (int i = 0; i < N; ++i)
      b[perm[i]] = z[i];
  }
  for (std::size_t i = 0; i < n; ++i)
    if (!finite_(b[i])) return false;
  return true;
}

template <typename D> double neumaier(const D &d, std::size_t n, std::size_t off = 0, int skip = -1, bool sq = false) {
  double sum = 0, c = 0; // :287-305
  for (std::size_t i = 0; i < n; ++i) {
    if (skip >= 0 && i == std::size_t(skip)) continue;
    const double x = sq ? d[i + off] * d[i + off] : d[i + off];
    const double t = sum + x;
    if (std::abs(sum) >= std::abs(x))
      c += (sum - t) + x;
    else
      c += (x - t) + sum;
    sum = t;
  }
  return sum + c;
}
inline bool bad(double v) { // error_utils.hpp:29-36
  auto normal = [](double x) { return std::isnormal(x); };
  return !(v == 0 || (normal(1.0e10 * v) && normal(v)));
}

// PTESolverBase + PTESolverRhoT + PTESolverPT in one struct; `pt` selects.
struct Solver {
  bool pt;
  std::size_t n, neq, niter = 0;
  const Mix &mp;
  std::vector<const Eos *> eos;
  double *rho, *vfrac, *sie, *temp, *press;
  std::vector<double *> lam;
  double vtot, etot, rho_total = 0, uscale = 0, uts = 0, Tnorm = 0, Teq = 0, Ttmp = 0,
                     Peq = 0, Ptmp = 0;
  std::size_t ms = 0;
  std::vector<double> J, dx, scr, res, u, rhobar, dpdv, dedv, dpdT, vtmp;

  Solver(bool pt_, std::size_t n_, const Mix &m) : pt(pt_), n(n_), neq(pt_ ? 2 : n_), mp(m) {
    J.assign(neq * neq, 0), dx.assign(neq, 0), scr.assign(2 * neq, 0), res.assign(neq, 0);
    u.assign(n, 0), rhobar.assign(n, 0), dpdv.assign(n, 0), dedv.assign(n, 0), dpdT.assign(n, 0),
        vtmp.assign(n, 0);
  }
  double Ppref(std::size_t m, double r, double T, double e) const { // :583-597
    return (eos[m]->preferred() & Eos::SIE) ? eos[m]->P_re(r, e, lam[m]) : eos[m]->P_rT(r, T, lam[m]);
  }
  void normalize() {
    const double s = neumaier(vfrac, n);
    for (std::size_t m = 0; m < n; ++m)
      vfrac[m] *= ratio(vtot, s);
  }
  double vmax(std::size_t m, double T) const {
    return std::min(0.9 * ratio(rhobar[m], eos[m]->rhoPmin(T)), 1.0);
  }
  bool setVfracFromT(double T) { // :423-498, true = FAIL
    double vms = 0;
    for (std::size_t m = 0; m < n; ++m) {
      const double v = vmax(m, T);
      if (vfrac[m] <= 0) vfrac[m] = v;
      vms += v;
    }
    if (vms < vtot) return true;
    normalize();
    for (std::size_t it = 0; it < n; ++it) {
      double rem = 0;
      std::size_t nun = n;
      for (std::size_t m = 0; m < n; ++m) {
        const double dv = vfrac[m] - std::min(vmax(m, T), vfrac[m]);
        vfrac[m] -= dv;
        rem += dv;
        nun -= (dv > 1e-12);
      }
      if (std::abs(rem) < 1e-12) break;
      for (std::size_t m = 0; m < n; ++m)
        if ((vmax(m, T) - vfrac[m]) > 1e-12) vfrac[m] += rem / double(nun);
    }
    normalize();
    return false;
  }
  double tguess() { // :500-581
    double Tg;
    if (Tnorm > 0.0) {
      Tg = Tnorm;
    } else {
      Tg = mp.Tguess0;
      for (std::size_t m = 0; m < n; ++m)
        Tg = std::max(Tg, temp[m]);
    }
    auto newton = [&](double T) {
      double dudt = 0, usum = 0;
      for (std::size_t m = 0; m < n; ++m) {
        const Eos &e = *eos[m];
        double r = std::min(rho[m], e.maxRho()), s, cv;
        if (e.preferred() & Eos::PRES) { // :599-620
          const double Pmin = e.minP(), Pmax = e.maxPAtT(T);
          const double Pg = bad(press[m]) ? 0.5 * (Pmin + Pmax) : std::max(Pmin, std::min(Pmax, press[m]));
          e.rhoSieFromPT(Pg, T, lam[m], r, s);
          cv = e.Cv_re(r, s, lam[m]);
        } else {
          s = e.e_rT(r, T, lam[m]);
          cv = e.Cv_rT(r, T, lam[m]);
        }
        usum += rhobar[m] * s;
        dudt += rhobar[m] * cv;
      }
      return T - ratio((usum - uts * uscale), dudt);
    };
    bool badg = false;
    for (std::size_t i = 0; i < 3; i++) {
      if (mp.iterate_t_guess) Tg = std::min(mp.Tlimit, std::max(Tg, newton(Tg)));
      for (std::size_t m = 0; m < n; ++m)
        Tg = std::max(eos[m]->minT(), Tg);
      badg = setVfracFromT(Tg);
      if (badg) {
        Tg *= 10.0;
        continue;
      }
      for (std::size_t m = 0; m < n; ++m)
        rho[m] = ratio(rhobar[m], vfrac[m]);
      badg = false;
      for (std::size_t m = 0; m < n; ++m)
        if (rho[m] < eos[m]->rhoPmin(Tg)) {
          badg = true;
          Tg *= 10.0;
          break;
        }
      if (!badg) break;
    }
    return Tg;
  }
  void initBase() { // :627-662
    for (std::size_t m = 0; m < n; ++m)
      rhobar[m] = rho[m] * vfrac[m];
    rho_total = neumaier(rhobar, n);
    const double ut = rho_total * etot;
    uscale = std::max(std::abs(ut), 1.0e-14);
    uts = ratio(ut, uscale);
    const double Tg = tguess();
    Tnorm = Tg;
    for (std::size_t m = 0; m < n; m++) {
      temp[m] = 1.0;
      sie[m] = eos[m]->e_rT(rho[m], Tg, lam[m]);
      if ((eos[m]->preferred() & Eos::PRES) && !bad(press[m]))
        press[m] = ratio(press[m], uscale);
      else
        press[m] = ratio(Ppref(m, rho[m], Tg, sie[m]), uscale);
    }
    for (std::size_t m = 0; m < n; ++m)
      u[m] = sie[m] * ratio(rhobar[m], uscale);
  }
  double resNorm() const { return 0.5 * neumaier(res, neq, 0, -1, true); }
  void residual() {
    if (pt) { // :1314-1320
      res[0] = vtot - neumaier(vfrac, n);
      res[1] = uts - neumaier(u, n);
      return;
    }
    res[0] = uts - neumaier(u, n); // :1010-1019
    std::size_t r = 1;
    for (std::size_t m = 0; m < n; ++m)
      if (m != ms) res[r++] = press[ms] - press[m];
  }
  double init() {
    initBase();
    if (pt) { // :1265-1297
      residual();
      Peq = 0;
      for (std::size_t m = 0; m < n; ++m)
        Peq += std::abs(press[m]) * vfrac[m];
      Peq /= neumaier(vfrac, n);
      Teq = 1;
      for (std::size_t m = 0; m < n; ++m) {
        eos[m]->rhoSieFromPT(Peq * uscale, Teq * Tnorm, lam[m], rho[m], sie[m]);
        vfrac[m] = ratio(rhobar[m], rho[m]);
        u[m] = ratio(sie[m] * rhobar[m], uscale);
        temp[m] = Teq;
      }
      residual();
      return resNorm();
    }
    if (mp.exclude >= 0) { // :947-984
      ms = std::size_t(mp.exclude);
    } else {
      ms = 0;
      double xmax = 0;
      for (std::size_t m = 0; m < n; ++m) {
        const double x = ratio(rhobar[m], rho_total);
        if (x > xmax) xmax = x, ms = m;
      }
    }
    residual();
    Teq = temp[0];
    return resNorm();
  }
  void fixup() { // :986-1008
    if (pt || mp.exclude >= 0) return;
    double amax = 0;
    ms = 0;
    for (std::size_t m = 0; m < n; ++m)
      if (vfrac[m] > amax) amax = vfrac[m], ms = m;
    residual();
  }
  std::pair<bool, bool> check() const {
    if (pt) { // :1322-1334
      const double ev = std::abs(res[0]), eu = std::abs(res[1]);
      return {ev < mp.tol_v && eu < mp.tol_e, eu < mp.tol_e_s && ev < mp.tol_v_s};
    }
    double mean_p = 0; // :1021-1040
    for (std::size_t m = 0; m < n; ++m)
      mean_p += vfrac[m] * press[m];
    const double ep = std::sqrt(neumaier(res, neq - 1, 1, -1, true)), eu = std::abs(res[0]);
    const bool cp = ep < mp.tol_p * std::abs(mean_p) || ep < mp.abs_p, cu = eu < mp.tol_e;
    const bool ap = ep < mp.tol_p_s * std::abs(mean_p) || ep < mp.abs_p_s, au = eu < mp.tol_e_s;
    return {cp && cu, ap && au};
  }
  void jacobian() {
    if (pt) { // :1336-1385
      double dudT = 0, dudP = 0, rT = 0, rP = 0;
      for (std::size_t m = 0; m < n; ++m) {
        double rp = rho[m], ep = sie[m];
        const double dp = -Peq * mp.derivative_eps;
        eos[m]->rhoSieFromPT(uscale * (Peq + dp), Tnorm * Teq, lam[m], rp, ep);
        const double drdp = ratio(rp - rho[m], dp);
        const double dudp = ratio(ratio(rhobar[m] * ep, uscale) - u[m], dp);
        rP += ratio(rhobar[m], rho[m] * rho[m]) * drdp;
        dudP += dudp;
        const double dT = Teq * mp.derivative_eps;
        eos[m]->rhoSieFromPT(uscale * Peq, Tnorm * (Teq + dT), lam[m], rp, ep);
        const double drdT = ratio(rp - rho[m], dT);
        const double dudt = ratio(ratio(rhobar[m] * ep, uscale) - u[m], dT);
        rT += ratio(rhobar[m], rho[m] * rho[m]) * drdT;
        dudT += dudt;
      }
      J[0] = -rT, J[1] = -rP, J[2] = dudT, J[3] = dudP;
      return;
    }
    double dedT = 0.0; // :1042-1105
    for (std::size_t m = 0; m < n; m++) {
      const double dv = (vfrac[m] < 0.5 ? 1.0 : -1.0) * vfrac[m] * mp.derivative_eps;
      const double rp = ratio(rhobar[m], vfrac[m] + dv);
      double ep = eos[m]->e_rT(rp, Tnorm * Teq, lam[m]);
      double pp = ratio(Ppref(m, rp, Tnorm * Teq, ep), uscale);
      dpdv[m] = std::min(ratio((pp - press[m]), dv), -std::abs(mp.max_dpdv));
      dedv[m] = ratio(rhobar[m] * ratio(ep, uscale) - u[m], dv);
      const double dT = Teq * mp.derivative_eps;
      ep = eos[m]->e_rT(rho[m], Tnorm * (Teq + dT), lam[m]);
      pp = ratio(Ppref(m, rho[m], Tnorm * (Teq + dT), ep), uscale);
      dpdT[m] = ratio((pp - press[m]), dT);
      dedT += ratio(rhobar[m] * ratio(ep, uscale) - u[m], dT);
    }
    std::fill(J.begin(), J.end(), 0.0);
    J[0] = dedT;
    std::size_t col = 1;
    for (std::size_t m = 0; m < n; ++m)
      if (m != ms) J[col++] = dedv[m] - dedv[ms];
    std::size_t row = 1;
    for (std::size_t m = 0; m < n; m++) {
      if (m == ms) continue;
      J[row * neq] = dpdT[m] - dpdT[ms];
      std::size_t c = 1;
      for (std::size_t mm = 0; mm < n; ++mm) {
        if (mm == ms) continue;
        J[row * neq + c] = (mm == m) ? dpdv[m] + dpdv[ms] : dpdv[ms];
        c++;
      }
      row++;
    }
  }
  bool solveStep() {
    for (std::size_t m = 0; m < neq; m++)
      dx[m] = res[m];
    return solve(neq, J.data(), dx.data(), scr.data());
  }
  double scaleDx() {
    double s = 1.0;
    if (pt) { // :1387-1411
      if (s * dx[0] < -0.95 * Teq) s = ratio(-0.95 * Teq, dx[0]);
      auto bounded = [&](double Pb, double d) { return ratio(ratio(Pb, uscale) - Peq, d); };
      for (std::size_t m = 0; m < n; ++m)
        s = std::min(std::abs(s), std::abs(0.95 * bounded(eos[m]->minP(), dx[1])));
      for (std::size_t m = 0; m < n; ++m) {
        const double Ttest = (Teq + s * dx[0]) * Tnorm;
        s = std::min(std::abs(s), std::abs(0.95 * bounded(eos[m]->maxPAtT(Ttest), dx[0])));
      }
    } else { // :1107-1151
      const double dskip = -neumaier(dx, n - 1, 1);
      std::size_t idx = 1;
      for (std::size_t m = 0; m < n; ++m) {
        const double d = (m == ms) ? dskip : dx[idx++];
        if (s * d < -mp.vsafety * vfrac[m]) s = std::min(s, std::abs(mp.vsafety * ratio(vfrac[m], d)));
      }
      const double Tnew = Teq + s * dx[0];
      idx = 1;
      for (std::size_t m = 0; m < n; m++) {
        const double rmin = std::max(eos[m]->rhoPmin(Tnorm * Teq), eos[m]->rhoPmin(Tnorm * Tnew));
        const double amax = std::min(1.0, ratio(rhobar[m], rmin));
        if (amax < vfrac[m]) continue;
        const double d = (m == ms) ? dskip : dx[idx++];
        if (s * d > 0.5 * (amax - vfrac[m])) s = std::min(ratio(0.5 * (amax - vfrac[m]), d), s);
      }
      if (s * dx[0] < -0.95 * Teq) s = std::min(s, ratio(-0.95 * Teq, dx[0]));
    }
    for (std::size_t i = 0; i < neq; ++i)
      dx[i] *= s;
    return s;
  }
  double testUpdate(double s, bool cache = false) {
    if (pt) { // :1415-1435
      if (cache) Ttmp = Teq, Ptmp = Peq;
      Teq = Ttmp + s * dx[0];
      Peq = Ptmp + s * dx[1];
      for (std::size_t m = 0; m < n; ++m) {
        eos[m]->rhoSieFromPT(Peq * uscale, Teq * Tnorm, lam[m], rho[m], sie[m]);
        vfrac[m] = ratio(rhobar[m], rho[m]);
        u[m] = ratio(sie[m] * rhobar[m], uscale);
        temp[m] = Teq;
        press[m] = Peq;
      }
      residual();
      return resNorm();
    }
    if (cache) { // :1155-1187
      Ttmp = Teq;
      for (std::size_t m = 0; m < n; ++m)
        vtmp[m] = vfrac[m];
    }
    Teq = Ttmp + s * dx[0];
    std::size_t idx = 1;
    for (std::size_t m = 0; m < n; ++m)
      if (ms != m) vfrac[m] = vtmp[m] + s * dx[idx++];
    vfrac[ms] = neumaier(vfrac, n, 0, int(ms));
    vfrac[ms] = 1 - vfrac[ms];
    for (std::size_t m = 0; m < n; ++m) {
      rho[m] = ratio(rhobar[m], vfrac[m]);
      u[m] = rhobar[m] * eos[m]->e_rT(rho[m], Tnorm * Teq, lam[m]);
      sie[m] = ratio(u[m], rhobar[m]);
      u[m] = ratio(u[m], uscale);
      temp[m] = Teq;
      press[m] = ratio(Ppref(m, rho[m], Tnorm * Teq, sie[m]), uscale);
    }
    residual();
    return resNorm();
  }
  void finalize() {
    for (std::size_t m = 0; m < n; m++) {
      if (pt) { // :1299-1312
        press[m] = Peq * uscale;
        temp[m] = Teq * Tnorm;
      } else { // :351-357
        temp[m] *= Tnorm;
        press[m] *= uscale;
      }
      u[m] *= uscale;
    }
  }
};

struct Status {
  bool converged = false;
  double residual = 0;
};
// PTESolver (:2188-2291)
Status solve_cell(Solver &s) {
  Status st;
  double err = s.init();
  const Mix &p = s.mp;
  bool conv = false, close = false;
  const std::size_t maxit = s.n * p.max_iter_per_mat;
  std::size_t small = 0;
  for (s.niter = 0; s.niter < maxit; ++s.niter) {
    auto c = s.check();
    conv = c.first, close = c.second;
    if (conv) break;
    s.jacobian();
    if (!s.solveStep()) {
      conv = false;
      break;
    }
    double scale = std::min(1.0, s.scaleDx());
    if (std::abs(scale) < p.small_step_thresh) small++;
    if (small >= p.small_step_tries) {
      conv = false;
      break;
    }
    const double g = -2.0 * scale * err;
    scale = 1.0;
    const double eo = err;
    err = s.testUpdate(scale, true);
    if (err > eo + p.ls_alpha * g) {
      scale = 0.5;
      const double em = s.testUpdate(scale);
      if (em < err && em < eo) scale = 0.75 + 0.5 * ratio(em - err, err - 2.0 * em + eo);
      for (std::size_t li = 0; li < p.ls_max_iter; li++) {
        err = s.testUpdate(scale);
        if (err < eo + p.ls_alpha * scale * g) break;
        scale *= p.ls_fac;
      }
    }
    s.fixup();
    if (((err > p.slow * eo) || s.niter == maxit - 1) && close) {
      conv = true;
      break;
    }
  }
  s.fixup();
  s.finalize();
  st.converged = conv;
  st.residual = err;
  return st;
}

} // namespace port

// ---- C surface (same as oracle/sgref.cpp) -------------------------------------
extern "C" {

struct sgref_eos {
  int32_t type, flags, matid, pad;
  double p[16];
  const char *path;
  // modifiers (ShiftedEOS, ScaledEOS, BilinearRampEOS); this port restates
  // bare models only and rejects a modified EOS
  int32_t mods, pad2;
  double shift, scale;
  double ramp[4];
};
struct sgref_mix_params {
  int32_t verbose, iterate_t_guess;
  double derivative_eps, pte_rel_tolerance_p, pte_rel_tolerance_t, pte_rel_tolerance_e,
      pte_rel_tolerance_v, pte_abs_tolerance_p, pte_abs_tolerance_t,
      pte_slow_convergence_thresh, pte_rel_tolerance_p_sufficient,
      pte_rel_tolerance_t_sufficient, pte_rel_tolerance_e_sufficient,
      pte_rel_tolerance_v_sufficient, pte_abs_tolerance_p_sufficient,
      pte_abs_tolerance_t_sufficient;
  int64_t pte_max_iter_per_mat;
  double line_search_alpha;
  int64_t line_search_max_iter;
  double line_search_fac, vfrac_safety_fac, temperature_limit, default_tguess, min_dtde;
  int64_t pte_small_step_tries;
  double pte_small_step_thresh, pte_max_dpdv;
  int64_t pte_reduced_system_exclude_idx;
};

}

namespace {

std::map<std::string, port::Table> &tables() {
  static std::map<std::string, port::Table> t;
  return t;
}
// Builds the EOS list; tabulated models load (and cache) their table.
bool make_eos(const sgref_eos *d, int n, std::vector<port::Eos> &out) {
  out.resize(n);
  for (int k = 0; k < n; ++k) {
    if (d[k].mods != 0) return false;
    if (d[k].type <= 3 && (d[k].flags & 2)) return false; // short constructors only
    out[k].type = d[k].type;
    for (int q = 0; q < 16; ++q)
      out[k].p[q] = d[k].p[q];
    if (d[k].type == 4) {
      // rho_max = 0.99 * ComputeRhoMax (eos_gruneisen.hpp:62-67, 231-329);
      // the linear Us-up form is the one the workloads use.
      const double s1 = d[k].p[1], s2 = d[k].p[2], s3 = d[k].p[3], rho0 = d[k].p[6];
      if (!(std::abs(s2) < port::EPS && std::abs(s3) < port::EPS && s1 > 1.)) return false;
      out[k].p[11] = 0.99 * (rho0 / ((1 - 1. / s1) + port::EPS));
    }
    if (d[k].type == 5) {
      const std::string key = std::string(d[k].path) + "#" + std::to_string(d[k].matid);
      auto it = tables().find(key);
      if (it == tables().end()) {
        port::Table t;
        if (!port::load_table(d[k].path, d[k].matid, t)) return false;
        it = tables().emplace(key, std::move(t)).first;
      }
      it->second.reproducible = (d[k].flags & 1) != 0;
      out[k].tab = &it->second;
    }
    if (d[k].type < 1 || d[k].type > 5) return false;
  }
  return true;
}

port::Mix to_mix(const sgref_mix_params &q) {
  port::Mix m;
  m.iterate_t_guess = q.iterate_t_guess != 0;
  m.derivative_eps = q.derivative_eps;
  m.tol_p = q.pte_rel_tolerance_p, m.tol_e = q.pte_rel_tolerance_e, m.tol_v = q.pte_rel_tolerance_v;
  m.abs_p = q.pte_abs_tolerance_p, m.slow = q.pte_slow_convergence_thresh;
  m.tol_p_s = q.pte_rel_tolerance_p_sufficient, m.tol_e_s = q.pte_rel_tolerance_e_sufficient;
  m.tol_v_s = q.pte_rel_tolerance_v_sufficient, m.abs_p_s = q.pte_abs_tolerance_p_sufficient;
  m.max_iter_per_mat = std::size_t(q.pte_max_iter_per_mat);
  m.ls_max_iter = std::size_t(q.line_search_max_iter);
  m.small_step_tries = std::size_t(q.pte_small_step_tries);
  m.ls_alpha = q.line_search_alpha, m.ls_fac = q.line_search_fac;
  m.vsafety = q.vfrac_safety_fac, m.Tlimit = q.temperature_limit, m.Tguess0 = q.default_tguess;
  m.small_step_thresh = q.pte_small_step_thresh, m.max_dpdv = q.pte_max_dpdv;
  m.exclude = q.pte_reduced_system_exclude_idx;
  return m;
}

} // namespace

extern "C" {

void sgport_mix_params_default(sgref_mix_params *q) {
  std::memset(q, 0, sizeof(*q));
  q->iterate_t_guess = 1;
  q->derivative_eps = 3.0e-6;
  q->pte_rel_tolerance_p = 1.0e-6, q->pte_rel_tolerance_t = 1.0e-4;
  q->pte_rel_tolerance_e = 1.0e-6, q->pte_rel_tolerance_v = 1.0e-6;
  q->pte_abs_tolerance_p = 1.0e-6, q->pte_abs_tolerance_t = 1.0e-4;
  q->pte_slow_convergence_thresh = 0.99;
  q->pte_rel_tolerance_p_sufficient = 1.e2 * q->pte_rel_tolerance_p;
  q->pte_rel_tolerance_t_sufficient = 10 * q->pte_rel_tolerance_t;
  q->pte_rel_tolerance_e_sufficient = 1.e2 * q->pte_rel_tolerance_e;
  q->pte_rel_tolerance_v_sufficient = 1.e2 * q->pte_rel_tolerance_v;
  q->pte_abs_tolerance_p_sufficient = 1.e2 * q->pte_abs_tolerance_p;
  q->pte_abs_tolerance_t_sufficient = 10 * q->pte_abs_tolerance_t;
  q->pte_max_iter_per_mat = 128, q->line_search_alpha = 1.e-2, q->line_search_max_iter = 6;
  q->line_search_fac = 0.5, q->vfrac_safety_fac = 0.95, q->temperature_limit = 1.0e15;
  q->default_tguess = 300., q->min_dtde = 1.0e-16, q->pte_small_step_tries = 2;
  q->pte_small_step_thresh = 1e-16, q->pte_max_dpdv = -1e-8;
  q->pte_reduced_system_exclude_idx = -1;
}

int sgport_pte(int solver, int nmat_max, int ncell, const sgref_eos *descs, int neos,
               const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
               double *rho, double *vfrac, double *sie, double *temp, double *press,
               double *lambda, const sgref_mix_params *params, int32_t *converged,
               int32_t *niter, double *residual, int nthreads) {
  std::vector<port::Eos> eos;
  if (!make_eos(descs, neos, eos)) return 1;
  sgref_mix_params defaults;
  sgport_mix_params_default(&defaults);
  const port::Mix mp = to_mix(params ? *params : defaults);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
#endif
  for (int i = 0; i < ncell; ++i) {
    int slot[16], n = 0;
    for (int m = 0; m < nmat_max; ++m) {
      const int ie = eos_idx ? eos_idx[size_t(m) * ncell + i] : m;
      if (ie >= 0) slot[n++] = m;
    }
    port::Solver s(solver == 1, std::size_t(n), mp);
    double r[16], v[16], e[16], t[16], p[16], cache[16 * 3];
    s.eos.resize(n), s.lam.resize(n);
    for (int q = 0; q < n; ++q) {
      const size_t k = size_t(slot[q]) * ncell + i;
      s.eos[q] = &eos[eos_idx ? eos_idx[k] : slot[q]];
      r[q] = rho[k], v[q] = vfrac[k], e[q] = sie[k], t[q] = temp[k], p[q] = press[k];
      for (int l = 0; l < 3; ++l)
        cache[q * 3 + l] = lambda ? lambda[(size_t(slot[q]) * 3 + l) * ncell + i] : 0.0;
      s.lam[q] = cache + q * 3;
    }
    s.rho = r, s.vfrac = v, s.sie = e, s.temp = t, s.press = p;
    s.vtot = vfrac_tot[i], s.etot = sie_tot[i];
    const port::Status st = port::solve_cell(s);
    for (int q = 0; q < n; ++q) {
      const size_t k = size_t(slot[q]) * ncell + i;
      rho[k] = r[q], vfrac[k] = v[q], sie[k] = e[q], temp[k] = t[q], press[k] = p[q];
      if (lambda)
        for (int l = 0; l < 3; ++l)
          lambda[(size_t(slot[q]) * 3 + l) * ncell + i] = cache[q * 3 + l];
    }
    converged[i] = st.converged;
    niter[i] = int32_t(s.niter);
    residual[i] = st.residual;
  }
  return 0;
}

// SpinerEOSDependsRhoSie (type 7) lives in sgport_sie.cpp.
int sgport_sie_eos_vec(const sgref_eos *d, int fn, int n, const double *in1, const double *in2,
                       double *out, double *lambda, int stride);
int sgport_sie_fill_eos(const sgref_eos *d, int n, double *rho, double *temp, double *sie,
                        double *press, double *cv, double *bmod, unsigned long output,
                        double *lambda, int stride);
int sgport_sie_eos_bounds(const sgref_eos *d, int what, int n, const double *x, double *out);

int sgport_eos_vec(const sgref_eos *desc, int fn, int n, const double *in1, const double *in2,
                   double *out, double *lambda, int stride) {
  if (desc->type == 7) return sgport_sie_eos_vec(desc, fn, n, in1, in2, out, lambda, stride);
  std::vector<port::Eos> v;
  if (!make_eos(desc, 1, v)) return 1;
  const port::Eos &e = v[0];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < n; ++i) {
    double *lam = lambda ? lambda + size_t(i) * stride : nullptr;
    const double a = in1[i], b = in2[i];
    double r = 0;
    switch (fn) {
    case 0: r = e.T_re(a, b, lam); break;
    case 1: r = e.e_rT(a, b, lam); break;
    case 2: r = e.P_rT(a, b, lam); break;
    case 3: r = e.P_re(a, b, lam); break;
    case 4: r = e.Cv_rT(a, b, lam); break;
    case 5: r = e.Cv_re(a, b, lam); break;
    case 6: r = e.B_rT(a, b, lam); break;
    case 7: r = e.B_re(a, b, lam); break;
    case 8: r = e.G_rT(a, b, lam); break;
    case 9: r = e.G_re(a, b, lam); break;
    case 10: r = e.minE(a); break;
    }
    out[i] = r;
  }
  return 0;
}

int sgport_fill_eos(const sgref_eos *desc, int n, double *rho, double *temp, double *sie,
                    double *press, double *cv, double *bmod, unsigned long output,
                    double *lambda, int stride) {
  if (desc->type == 7)
    return sgport_sie_fill_eos(desc, n, rho, temp, sie, press, cv, bmod, output, lambda, stride);
  std::vector<port::Eos> v;
  if (!make_eos(desc, 1, v)) return 1;
  const port::Eos &e = v[0];
  int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
  for (int i = 0; i < n; ++i) {
    double *lam = lambda ? lambda + size_t(i) * stride : nullptr;
    if (!e.fill(rho[i], temp[i], sie[i], press[i], cv[i], bmod[i], unsigned(output), lam)) bad |= 1;
  }
  return bad;
}

int sgport_rho_sie_from_pt(const sgref_eos *desc, int n, const double *P, const double *T,
                           double *rho, double *sie) {
  std::vector<port::Eos> v;
  if (!make_eos(desc, 1, v)) return 1;
  for (int i = 0; i < n; ++i)
    v[0].rhoSieFromPT(P[i], T[i], nullptr, rho[i], sie[i]);
  return 0;
}

int sgport_eos_bounds(const sgref_eos *desc, int what, int n, const double *x, double *out) {
  if (desc->type == 7) return sgport_sie_eos_bounds(desc, what, n, x, out);
  std::vector<port::Eos> v;
  if (!make_eos(desc, 1, v)) return 1;
  const port::Eos &e = v[0];
  for (int i = 0; i < n; ++i)
    out[i] = what == 0   ? (e.type == 5 ? e.tab->rho(e.tab->lRhoMin) : 0.0)
             : what == 1 ? e.minT()
             : what == 2 ? e.maxRho()
             : what == 3 ? e.minP()
             : what == 4 ? e.maxPAtT(x[i])
                         : e.rhoPmin(x[i]);
  return 0;
}

long sgport_spiner_dump(const char *path, int matid, double *out, long cap, double *scal) {
  port::Table t;
  if (!port::load_table(path, matid, t)) return -1;
  const std::vector<double> *order[] = {
      &t.P,        &t.sie,        &t.bMod,       &t.dPdRho,   &t.dPdE,       &t.dTdRho,
      &t.dTdE,     &t.dEdRho,     &t.dEdT,       &t.PMax,     &t.sielTMax,   &t.dEdTMax,
      &t.gm1Max,   &t.lTColdCrit, &t.PCold,      &t.sieCold,  &t.bModCold,   &t.dPdRhoCold,
      &t.dPdECold, &t.dTdRhoCold, &t.dTdECold,   &t.dEdTCold, &t.rho_at_pmin};
  long total = 0;
  for (auto *v : order)
    total += long(v->size());
  if (out && cap >= total) {
    long o = 0;
    for (auto *v : order) {
      std::memcpy(out + o, v->data(), v->size() * 8);
      o += long(v->size());
    }
  }
  if (scal) {
    scal[0] = t.rho(t.lRhoMin), scal[1] = t.rhoMax, scal[2] = t.T(t.lTMin), scal[3] = t.TMax;
    scal[4] = t.PMin, scal[5] = t.lRhoOff, scal[6] = t.lTOff;
  }
  return total;
}

void sgport_nqt(int which, int n, const double *x, double *y) {
  for (int i = 0; i < n; ++i)
    y[i] = which == 0 ? port::log10(x[i]) : port::pow10(x[i]);
}

} // extern "C"

// The Helmholtz model (same translation unit: it uses the port's ratio and
// root finders).
#include "sgport_helm.cpp"
// SpinerEOSDependsRhoSie.
#include "sgport_sie.cpp"
