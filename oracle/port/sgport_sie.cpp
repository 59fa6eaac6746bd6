// SpinerEOSDependsRhoSie (default NullTransform): this project's CPU
// restatement of singularity-eos eos/eos_spiner_rho_sie.hpp, for the
// oracle's C surface. TEST INFRASTRUCTURE ONLY: the GPU library never links
// it; tests and bench.py's CPU-baseline leg call it through
// oracle/refbind.py (EOS type 7 in sgport_eos_vec / sgport_fill_eos /
// sgport_eos_bounds, and sgport_spiner_sie_dump). tests/test_oracle.py pins
// it to the fixture the compiled reference made
// (tests/golden/spiner_rhosie.npz). Included at the end of sgport.cpp (one
// translation unit): it shares the port's NQT logs, grids, bilinear
// interpolation and regula falsi. Compile with -ffp-contract=off.
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace sie_port {

using port::bilin;
using port::from_log;
using port::Grid;
using port::lin;
using port::to_log;

// The tables loadDataboxes_ keeps (:433-552), one group each for (lRho, lT)
// and (lRho, lE); index [j * nx + i], the fast coordinate i.
struct Group {
  Grid gx, gr;
  std::vector<double> X, P, bMod, dPdRho, dPdE, dTdRho, dTdE, dEdRho; // X: sie_ or T_
  double f(const std::vector<double> &d, double lr, double lx) const {
    return bilin(gx, gr, d, lr, lx);
  }
};
struct SieTab {
  Group t, e;
  Grid gC;
  std::vector<double> PCold, sieCold, bModCold, dPdRhoCold, PlRhoMax, dPdRhoMax, rho_at_pmin;
  double lRhoOff = 0, lTOff = 0, lEOff = 0, lRhoMin = 0, lRhoMax = 0, rhoMax = 0, PMin = 0;
  double rhoNormal = 0, TNormal = 0, sieNormal = 0, PNormal = 0, CvNormal = 0, bModNormal = 0,
         dPdENormal = 0, dVdTNormal = 0;
  bool reproducible = false;
};

// sp5-lite image (format documented in sgx/sp5lite.py): attributes and
// datasets by path.
bool read_image(const char *path, std::map<std::string, double> &attr,
                std::map<std::string, std::pair<std::vector<double>, std::vector<double>>> &ds) {
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
    } else {
      ok = false;
    }
  }
  std::fclose(f);
  return ok;
}

// calcBMod_ (:554-578)
void calc_bmod(Group &g, double lRhoOff) {
  for (int j = 0; j < g.gr.n; j++) {
    const double r = from_log(g.gr.x(j), lRhoOff);
    for (int i = 0; i < g.gx.n; i++) {
      const size_t k = size_t(j) * g.gx.n + i;
      const double press = g.P[k], DPDR_E = g.dPdRho[k], DPDE_R = g.dPdE[k], DEDR_T = g.dEdRho[k];
      const double DPDR_T = DPDR_E + DPDE_R * DEDR_T;
      double b;
      if (DPDE_R > 0.0 && r > 0.0)
        b = r * DPDR_E + DPDE_R * (press / r);
      else if (r > 0.0)
        b = std::max(r * DPDR_T, 0.0);
      else
        b = 0.0;
      g.bMod[k] = std::max(b, port::EPS);
    }
  }
}

bool load(const char *path, int matid, SieTab &t) {
  std::map<std::string, double> attr;
  std::map<std::string, std::pair<std::vector<double>, std::vector<double>>> ds;
  if (!read_image(path, attr, ds)) return false;
  const std::string g = "/" + std::to_string(matid);
  auto get2 = [&](const char *grp, const char *name, Group &G, std::vector<double> &out) {
    auto it = ds.find(g + "/" + grp + "/" + name);
    if (it == ds.end() || it->second.first.size() != 6) return false;
    out = it->second.second;
    const auto &m = it->second.first;
    G.gx = Grid(m[1], m[2], int(m[0]));
    G.gr = Grid(m[4], m[5], int(m[3]));
    return true;
  };
  auto group = [&](const char *grp, const char *xname, Group &G) {
    return get2(grp, xname, G, G.X) && get2(grp, "pressure", G, G.P) &&
           get2(grp, "bulk modulus", G, G.bMod) && get2(grp, "dPdRho", G, G.dPdRho) &&
           get2(grp, "dPdE", G, G.dPdE) && get2(grp, "dTdRho", G, G.dTdRho) &&
           get2(grp, "dTdE", G, G.dTdE) && get2(grp, "dEdRho", G, G.dEdRho);
  };
  auto get1 = [&](const char *name, std::vector<double> &out) {
    auto it = ds.find(g + "/coldCurve/" + name);
    if (it == ds.end()) return false;
    out = it->second.second;
    const auto &m = it->second.first;
    t.gC = Grid(m[1], m[2], int(m[0]));
    return true;
  };
  if (!group("dependsLogRhoLogT", "specific internal energy", t.t) ||
      !group("dependsLogRhoLogSie", "temperature", t.e) || !get1("pressure", t.PCold) ||
      !get1("specific internal energy", t.sieCold) || !get1("bulk modulus", t.bModCold) ||
      !get1("dPdRho", t.dPdRhoCold))
    return false;
  for (const char *a : {"rhoOffset", "TOffset", "sieOffset", "normalDensity"})
    if (!attr.count(g + "@" + a)) return false;
  t.lRhoOff = std::abs(attr[g + "@rhoOffset"]);
  t.lTOff = std::abs(attr[g + "@TOffset"]);
  t.lEOff = std::abs(attr[g + "@sieOffset"]);
  calc_bmod(t.t, t.lRhoOff);
  calc_bmod(t.e, t.lRhoOff);
  const int nR = t.t.gr.n, nT = t.t.gx.n;
  t.lRhoMin = t.t.gr.min;
  t.lRhoMax = t.t.gr.max;
  t.rhoMax = from_log(t.lRhoMax, t.lRhoOff);
  // P.slice(numRho_ - 1), dPdRho.slice(numRho_ - 1) (:520-521)
  t.PlRhoMax.assign(t.t.P.begin() + size_t(nR - 1) * nT, t.t.P.begin() + size_t(nR) * nT);
  t.dPdRhoMax.assign(t.t.dPdRho.begin() + size_t(nR - 1) * nT,
                     t.t.dPdRho.begin() + size_t(nR) * nT);
  // SetRhoPMin (eos_spiner_common.hpp:59-109), no vapor dome
  t.rho_at_pmin.assign(nT, 0.0);
  t.PMin = DBL_MAX;
  for (int i = 0; i < nT; ++i) {
    double pm = DBL_MAX;
    int jm = 0;
    for (int j = 0; j < nR; ++j)
      if (t.t.P[size_t(j) * nT + i] < pm) {
        pm = t.t.P[size_t(j) * nT + i];
        jm = j;
      }
    if (pm > 0) {
      t.rho_at_pmin[i] = 0;
      pm = 0;
    } else {
      t.rho_at_pmin[i] = from_log(t.t.gr.x(jm), t.lRhoOff);
    }
    t.PMin = std::min(pm, t.PMin);
  }
  // reference state (:526-548)
  double rN = std::abs(attr[g + "@normalDensity"]);
  double lRN = to_log(rN, t.lRhoOff);
  if (!(t.lRhoMin < lRN && lRN < t.lRhoMax)) {
    lRN = 0.5 * (t.lRhoMin + t.lRhoMax);
    rN = from_log(lRN, t.lRhoOff);
  }
  double TN = 293.0, lTN = to_log(TN, t.lTOff);
  if (!(t.t.gx.min < lTN && lTN < t.t.gx.max)) {
    lTN = 0.5 * (t.t.gx.min + t.t.gx.max);
    TN = from_log(lTN, t.lTOff);
  }
  t.rhoNormal = rN;
  t.TNormal = TN;
  t.sieNormal = t.t.f(t.t.X, lRN, lTN);
  t.PNormal = t.t.f(t.t.P, lRN, lTN);
  t.CvNormal = 1. / t.t.f(t.t.dTdE, lRN, lTN);
  t.bModNormal = t.t.f(t.t.bMod, lRN, lTN);
  t.dPdENormal = t.t.f(t.t.dPdE, lRN, lTN);
  const double dPdR = t.t.f(t.t.dPdRho, lRN, lTN);
  t.dVdTNormal = t.dPdENormal * t.CvNormal / (t.rhoNormal * t.rhoNormal * dPdR);
  return true;
}

const SieTab *get(const char *path, int matid, bool reproducible) {
  static std::mutex mu;
  static std::map<std::string, SieTab> cache;
  std::lock_guard<std::mutex> lk(mu);
  const std::string key = std::string(path) + "#" + std::to_string(matid);
  auto it = cache.find(key);
  if (it == cache.end()) {
    SieTab t;
    if (!load(path, matid, t)) return nullptr;
    it = cache.emplace(key, std::move(t)).first;
  }
  it->second.reproducible = reproducible;
  return &it->second;
}

// interpRhoT_ / interpRhoSie_ (:917-941)
double rhoT(const SieTab &t, const std::vector<double> &d, double rho, double T, double *lam) {
  const double lr = to_log(rho, t.lRhoOff), lt = to_log(T, t.lTOff);
  if (lam) lam[0] = lr;
  return t.t.f(d, lr, lt);
}
double rhoE(const SieTab &t, const std::vector<double> &d, double rho, double e, double *lam) {
  const double lr = to_log(rho, t.lRhoOff), le = to_log(e, t.lEOff);
  if (lam) lam[0] = lr;
  return t.e.f(d, lr, le);
}
// lRhoFromPlT_ (:942-987)
double lRhoFromPlT(const SieTab &t, double P, double lT, double *lam) {
  const double rhopmin = to_log(lin(t.t.gx, t.rho_at_pmin, lT), t.lRhoOff);
  double lRho;
  const double dPdRhoMax = lin(t.t.gx, t.dPdRhoMax, lT), PMax = lin(t.t.gx, t.PlRhoMax, lT);
  if (dPdRhoMax > 0 && P > PMax) {
    lRho = to_log((P - PMax) / dPdRhoMax + t.rhoMax, t.lRhoOff);
  } else {
    double guess = t.reproducible ? t.lRhoMax : 0.5 * (rhopmin + t.lRhoMax);
    if (lam && rhopmin <= lam[0] && lam[0] <= t.lRhoMax) guess = lam[0];
    const bool ok = port::regula_falsi([&](double x) { return t.t.f(t.t.P, x, lT); }, P, guess,
                                       rhopmin, t.lRhoMax, port::EPS, port::EPS, lRho);
    if (!ok) lRho = t.reproducible ? t.lRhoMax : guess;
  }
  if (lam) lam[0] = lRho;
  return lRho;
}

// The vector functions 0-10 (the C surface's numbering) and 13.
double eval(const SieTab &t, int fn, double a, double b, double *lam) {
  switch (fn) {
  case 0: return rhoE(t, t.e.X, a, b, lam);
  case 1: return rhoT(t, t.t.X, a, b, lam);
  case 2: return rhoT(t, t.t.P, a, b, lam);
  case 3: return rhoE(t, t.e.P, a, b, lam);
  case 4: return 1. / rhoT(t, t.t.dTdE, a, b, lam);
  case 5: return 1. / rhoE(t, t.e.dTdE, a, b, lam);
  case 6: return rhoT(t, t.t.bMod, a, b, lam);
  case 7: return rhoE(t, t.e.bMod, a, b, lam);
  case 8: return rhoT(t, t.t.dPdE, a, b, lam) / a;
  case 9: return t.e.f(t.e.dPdE, to_log(a, t.lRhoOff), to_log(b, t.lEOff)) / a;
  case 10: return lin(t.gC, t.sieCold, to_log(a, t.lRhoOff));
  case 13: {
    // EosBase::InternalEnergyFromDensityPressure (eos_base.hpp:685-721):
    // regula falsi on P(rho, sie) between sie(rho, MinimumTemperature) and
    // sie(rho, 1e20), from the middle
    const double Tmin = from_log(t.t.gx.min, t.lTOff);
    const double smin = rhoT(t, t.t.X, a, Tmin, lam), smax = rhoT(t, t.t.X, a, 1e20, lam);
    double sie = 0.5 * (smin + smax);
    const double guess = (smin < sie && sie < smax) ? 0.5 * (smin + smax) : sie;
    port::regula_falsi([&](double s) { return rhoE(t, t.e.P, a, s, lam); }, b, guess, smin,
                       smax, port::EPS, port::EPS, sie);
    return sie;
  }
  }
  return 0.0;
}

// FillEos (:844-898); false on the reference's UNDEFINED_ERROR.
bool fill(const SieTab &t, double &rho, double &temp, double &sie, double &press, double &cv,
          double &bmod, unsigned out, double *lam) {
  constexpr unsigned DENS = 1, SIE = 2, PRES = 4, TEMP = 8, CV = 16, BMOD = 32;
  if (out == 0 || ((out & TEMP) && (out & SIE))) return false;
  double lRho;
  if (out & DENS) {
    if ((out & PRES) || (out & TEMP)) return false;
    lRho = lRhoFromPlT(t, press, to_log(temp, t.lTOff), lam);
    rho = from_log(lRho, t.lRhoOff);
  } else {
    lRho = to_log(rho, t.lRhoOff);
    if (lam) lam[0] = lRho;
  }
  if (out & TEMP) {
    const double lE = to_log(sie, t.lEOff);
    temp = t.e.f(t.e.X, lRho, lE);
    if (out & PRES) press = t.e.f(t.e.P, lRho, lE);
    if (out & CV) cv = 1. / t.e.f(t.e.dTdE, lRho, lE);
    if (out & BMOD) bmod = t.e.f(t.e.bMod, lRho, lE);
  }
  if (out & SIE) {
    const double lT = to_log(temp, t.lTOff);
    sie = t.t.f(t.t.X, lRho, lT);
    if (out & PRES) press = t.t.f(t.t.P, lRho, lT);
    if (out & CV) cv = 1. / t.t.f(t.t.dTdE, lRho, lT);
    if (out & BMOD) bmod = t.t.f(t.t.bMod, lRho, lT);
  }
  return true;
}

// MinimumDensity ... RhoPmin (:262-270)
double bound(const SieTab &t, int what, double x) {
  switch (what) {
  case 0: return from_log(t.lRhoMin, t.lRhoOff);
  case 1: return from_log(t.t.gx.min, t.lTOff);
  case 2: return t.rhoMax;
  case 3: return t.PMin;
  case 4: return 1e100;
  }
  return lin(t.t.gx, t.rho_at_pmin, to_log(x, t.lTOff));
}

} // namespace sie_port

extern "C" {

// Type-7 entry points of the port's C surface (sgport_eos_vec and friends
// forward here).
int sgport_sie_eos_vec(const sgref_eos *d, int fn, int n, const double *in1, const double *in2,
                       double *out, double *lambda, int stride) {
  const sie_port::SieTab *t = sie_port::get(d->path, d->matid, (d->flags & 1) != 0);
  if (!t || d->mods != 0) return 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < n; ++i)
    out[i] = sie_port::eval(*t, fn, in1[i], in2 ? in2[i] : 0.0,
                            lambda ? lambda + size_t(i) * stride : nullptr);
  return 0;
}

int sgport_sie_fill_eos(const sgref_eos *d, int n, double *rho, double *temp, double *sie,
                        double *press, double *cv, double *bmod, unsigned long output,
                        double *lambda, int stride) {
  const sie_port::SieTab *t = sie_port::get(d->path, d->matid, (d->flags & 1) != 0);
  if (!t || d->mods != 0) return 1;
  int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
  for (int i = 0; i < n; ++i)
    if (!sie_port::fill(*t, rho[i], temp[i], sie[i], press[i], cv[i], bmod[i], unsigned(output),
                        lambda ? lambda + size_t(i) * stride : nullptr))
      bad |= 1;
  return bad;
}

int sgport_sie_eos_bounds(const sgref_eos *d, int what, int n, const double *x, double *out) {
  const sie_port::SieTab *t = sie_port::get(d->path, d->matid, (d->flags & 1) != 0);
  if (!t) return 1;
  for (int i = 0; i < n; ++i)
    out[i] = sie_port::bound(*t, what, x[i]);
  return 0;
}

// The tables in the reference's DBLIST order (:329-336) and the scalars of
// sgref_spiner_sie_dump.
long sgport_spiner_sie_dump(const char *path, int matid, double *out, long cap, double *scal) {
  sie_port::SieTab t;
  if (!sie_port::load(path, matid, t)) return -1;
  std::vector<const std::vector<double> *> order = {&t.t.X, &t.e.X, &t.rho_at_pmin};
  for (const sie_port::Group *g : {&t.t, &t.e})
    for (const std::vector<double> *v :
         {&g->P, &g->bMod, &g->dPdRho, &g->dPdE, &g->dTdRho, &g->dTdE, &g->dEdRho})
      order.push_back(v);
  for (const std::vector<double> *v :
       {&t.PlRhoMax, &t.dPdRhoMax, &t.PCold, &t.sieCold, &t.bModCold, &t.dPdRhoCold})
    order.push_back(v);
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
    const double s[18] = {port::from_log(t.lRhoMin, t.lRhoOff), t.rhoMax,
                          port::from_log(t.t.gx.min, t.lTOff), port::from_log(t.t.gx.max, t.lTOff),
                          port::from_log(t.e.gx.min, t.lEOff), port::from_log(t.e.gx.max, t.lEOff),
                          t.PMin, t.lRhoOff, t.lTOff, t.lEOff, t.rhoNormal, t.TNormal,
                          t.sieNormal, t.PNormal, t.CvNormal, t.bModNormal, t.dPdENormal,
                          t.dVdTNormal};
    std::memcpy(scal, s, sizeof(s));
  }
  return total;
}

} // extern "C"
