// Host side of table residency.
//
// sp5-lite is this project's flat binary stand-in for the reference's SP5
// HDF5 files (HDF5 is not a dependency here). Layout, little endian:
//   char magic[8] = "SGXSP5L\0"; u32 version = 1; u32 nrecords;
//   record: u32 kind (1 attr f64, 2 attr i32, 3 dataset f64, 4 attr string);
//           u32 len, char path[len]; u32 len, char name[len];
//           kind 1: f64; kind 2: i32; kind 4: u32 len, bytes;
//           kind 3: u32 rank, per dim (fastest first) i32 n, f64 min, f64 max,
//                   then f64 data[prod n] in C order (fastest index last).
// Group and field names are the reference's SP5 keys
// (base/sp5/singularity_eos_sp5.hpp:20-75).
//
// The derivation restates SpinerEOSDependsRhoT::loadDataboxes_
// (eos/eos_spiner_rho_temp.hpp:545-687): fixBulkModulus_ (:689-714),
// setlTColdCrit_ (:716-775), SetRhoPMin (eos_spiner_common.hpp:59-109) and the
// cold-curve / maximum-temperature 1-D tables, using the same interpolation
// functions the kernels use (sgx_spiner.cuh). Host code here is compiled
// without floating-point contraction, so the derived tables equal the
// reference's bit for bit.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sgx.h"
#include "sgx_helm.cuh"
#include "sgx_spiner.cuh"
#include "sgx_spiner_sie.cuh"
#include "sgx_table.h"

namespace sgx {

namespace {

struct Dataset {
  std::vector<int> n;
  std::vector<double> mn, mx;
  std::vector<double> data;
};
struct Sp5 {
  std::map<std::string, double> f64;
  std::map<std::string, int> i32;
  std::map<std::string, Dataset> ds;
};

bool read_sp5(const char *path, Sp5 &s, std::string &msg) {
  FILE *f = std::fopen(path, "rb");
  if (!f) {
    msg = std::string("cannot open ") + path;
    return false;
  }
  auto rd = [&](void *p, size_t n) { return std::fread(p, 1, n, f) == n; };
  auto rdstr = [&](std::string &str) {
    uint32_t len;
    if (!rd(&len, 4) || len > (1u << 20)) return false;
    str.resize(len);
    return len == 0 || rd(&str[0], len);
  };
  char magic[8];
  uint32_t version = 0, nrec = 0;
  bool ok = rd(magic, 8) && std::memcmp(magic, "SGXSP5L", 8) == 0 && rd(&version, 4) &&
            version == 1 && rd(&nrec, 4);
  for (uint32_t k = 0; ok && k < nrec; ++k) {
    uint32_t kind;
    std::string p, name;
    ok = rd(&kind, 4) && rdstr(p) && rdstr(name);
    if (!ok) break;
    const std::string key = p + "@" + name;
    if (kind == 1) {
      double v;
      ok = rd(&v, 8);
      s.f64[key] = v;
    } else if (kind == 2) {
      int32_t v;
      ok = rd(&v, 4);
      s.i32[key] = v;
    } else if (kind == 4) {
      std::string v;
      ok = rdstr(v);
    } else if (kind == 3) {
      uint32_t rank;
      ok = rd(&rank, 4) && rank >= 1 && rank <= 3;
      Dataset d;
      size_t total = 1;
      for (uint32_t r = 0; ok && r < rank; ++r) {
        int32_t n;
        double a, b;
        ok = rd(&n, 4) && rd(&a, 8) && rd(&b, 8) && n >= 2 && n <= (1 << 20);
        d.n.push_back(n);
        d.mn.push_back(a);
        d.mx.push_back(b);
        total *= static_cast<size_t>(n);
      }
      if (ok && total > (size_t(1) << 31)) ok = false;
      if (ok) {
        d.data.resize(total);
        ok = rd(d.data.data(), total * 8);
      }
      s.ds[p] = std::move(d);
    } else {
      ok = false;
    }
  }
  std::fclose(f);
  if (!ok) msg = std::string("malformed sp5-lite image ") + path;
  return ok;
}

Grid1D make_grid(double mn, double mx, int n) {
  Grid1D g;
  g.min = mn;
  g.max = mx;
  g.dx = (mx - mn) / static_cast<double>(n - 1);
  g.inv_dx = 1 / g.dx;
  g.n = n;
  g.pad = 0;
  return g;
}

// Host copy of a loaded table: owning storage plus a SpinerTable whose
// pointers refer to it (used to run the shared interpolation code on host).
struct HostTable {
  int nRho = 0, nT = 0;
  std::vector<double> f2[NF2D];
  std::vector<double> f1[NF1D];
  SpinerTable t{};
  void bind() {
    for (int k = 0; k < NF2D; ++k)
      t.f2[k] = f2[k].data();
    for (int k = 0; k < NF1D; ++k)
      t.f1[k] = f1[k].data();
  }
};

struct Resident {
  void *dev = nullptr;
  size_t bytes = 0;
  int device = 0;
  HostTable host;
  std::vector<double> dump; // non-empty: the dump of a non-Spiner table
  bool sie_cells = false;   // a SpinerEOSDependsRhoSie table with float-float cells
};
std::mutex g_mu;
std::map<uint64_t, Resident> g_tables;

constexpr double VAPOR_DPDR_THRESH = 1e-8;

// The thermal-energy bin index of the float-float lookup (SpinerTable::
// therm_idx). Bins are slices of the float bit pattern of the thermal energy
// t = sie - sieCold, 2^s per octave with s chosen so that a bin is at most
// half the narrowest T cell; the index is left out (idx empty) where the
// thermal energy does not rise strictly along every row, where the table
// is coarser than the bins can hold, or where it would exceed 4 Mi entries.
void build_thermal_index(const std::vector<double> &sie, const std::vector<double> &cold,
                         const int nR, const int nT, SpinerTable &t, std::vector<uint16_t> &idx) {
  idx.clear();
  t.therm_bins = t.therm_shift = t.therm_base = 0;
  if (nR < 2 || nT < 2 || nT - 1 > 65535 || static_cast<int>(cold.size()) < nR) return;
  double tlo = INFINITY, thi = 0.0, min_step = INFINITY;
  for (int r = 0; r < nR; ++r) {
    double prev = sie[static_cast<size_t>(r) * nT] - cold[r];
    for (int i = 1; i < nT; ++i) {
      const double ti = sie[static_cast<size_t>(r) * nT + i] - cold[r];
      if (!(ti > prev)) return; // thermal energy must rise along T
      if (i == 1) tlo = std::min(tlo, ti);
      if (prev > 0.0) min_step = std::min(min_step, std::log2(ti / prev));
      thi = std::max(thi, ti);
      prev = ti;
    }
  }
  if (!(tlo > 0.0) || !(thi < 1e37) || !(min_step > 0.0)) return;
  int sub = 0; // log2 of the bins per octave
  while (sub < 7 && std::ldexp(1.0, -sub) > 0.5 * min_step)
    ++sub;
  if (std::ldexp(1.0, -sub) > 0.5 * min_step) return;
  const int shift = 23 - sub;
  auto bin_of = [shift](const float x) {
    uint32_t u;
    std::memcpy(&u, &x, sizeof(u));
    return static_cast<int>(u >> shift);
  };
  const int base = bin_of(static_cast<float>(0.5 * tlo));
  const int nbins = bin_of(static_cast<float>(thi)) - base + 2;
  if (nbins < 1 || static_cast<size_t>(nbins) * nR > (size_t(1) << 22)) return;
  idx.assign(static_cast<size_t>(nbins) * nR, 0);
  for (int r = 0; r < nR; ++r) {
    int i = 0;
    for (int k = 0; k < nbins; ++k) {
      const uint32_t u = static_cast<uint32_t>(base + k) << shift;
      float edge;
      std::memcpy(&edge, &u, sizeof(edge));
      while (i + 1 < nT - 1 && sie[static_cast<size_t>(r) * nT + i + 1] - cold[r] <= edge)
        ++i;
      idx[static_cast<size_t>(r) * nbins + k] = static_cast<uint16_t>(i);
    }
  }
  t.therm_bins = nbins;
  t.therm_shift = shift;
  t.therm_base = base;
}

// setlTColdCrit_ (eos_spiner_rho_temp.hpp:716-775) for one density node.
double cold_crit(const HostTable &h, int j, const Grid1D &gCold) {
  const SpinerTable &t = h.t;
  const double lRho = gCold.x(j);
  const double sieCold = interp1(gCold, t.f1[F_SIECOLD], lRho);
  std::vector<int> crossings;
  int last_pos_crossing = -1;
  for (int i = 0; i < h.nT - 1; i++) {
    const double sign_curr = h.f2[F_SIE][j * h.nT + i] - sieCold;
    const double sign_next = h.f2[F_SIE][j * h.nT + i + 1] - sieCold;
    if (sign_curr < 0 && sign_next > 0) {
      crossings.push_back(i);
      last_pos_crossing = static_cast<int>(crossings.size()) - 1;
    } else if (sign_curr > 0 && sign_next < 0) {
      crossings.push_back(i);
    }
  }
  double lTc;
  if (last_pos_crossing <= 0) {
    lTc = t.lTMin;
  } else {
    const int ilast = crossings[last_pos_crossing];
    const double lTlower = t.gT.x(ilast) - 1.0e-14;
    const double lTupper = t.gT.x(ilast + 1) + 1.0e-14;
    const double lTGuess = 0.5 * (lTlower + lTupper);
    auto sieFunc = [&](const double x) { return interp2(t, t.f2[F_SIE], lRho, x); };
    double lT = lTGuess;
    if (regula_falsi(sieFunc, sieCold, lTGuess, lTlower, lTupper, SP_ROOT_THRESH, SP_ROOT_THRESH,
                     lT) != RootStatus::SUCCESS)
      lT = lTGuess;
    lTc = lT;
  }
  return smax(t.lTMin, lTc);
}

} // namespace

double gruneisen_compute_rho_max(double s1, double s2, double s3, double rho0, int *err) {
  const double EPS = lim<double>::eps;
  auto poly = [=](double eta) { return 1 - s1 * eta - s2 * (eta * eta) - s3 * (eta * (eta * eta)); };
  auto near0 = [](double v, double tol) { return std::fabs(v) < tol; };
  double root = -1.;
  if (near0(s2, EPS) && near0(s3, EPS) && s1 > 1.) {
    root = 1. / s1;
  } else if (near0(s3, EPS) && !near0(s2, EPS)) {
    const double disc = (s1 * s1) + 4. * s2;
    if (disc < 0.) {
      root = -1.;
    } else {
      const double r1 = (s1 + std::sqrt(disc)) / (-2. * s2);
      const double r2 = (s1 - std::sqrt(disc)) / (-2. * s2);
      const double lo = std::min(r1, r2), hi = std::max(r1, r2);
      root = (lo > 0. && lo < 1.) ? lo : ((hi > 0. && hi < 1.) ? hi : -INFINITY);
    }
  } else if (!near0(s3, EPS)) {
    const double ms2 = -s2;
    const double disc = -18. * s3 * s2 * s1 - 4. * (ms2 * (ms2 * ms2)) + (s2 * s2) * (s1 * s1) -
                        4. * s3 * (s1 * (s1 * s1)) - 27. * (s3 * s3);
    double minbound = 0., maxbound = 1.;
    if (disc >= 0) {
      const double e1 = (s2 + std::sqrt((s2 * s2) - 3. * s3 * s1)) / (-3. * s3);
      const double e2 = (s2 - std::sqrt((s2 * s2) - 3. * s3 * s1)) / (-3. * s3);
      const double mn = std::min(e1, e2), mx = std::max(e1, e2);
      if (s3 < 0.) {
        minbound = std::max(mn, minbound);
        maxbound = std::min(std::max(mx, minbound), maxbound);
      } else if (mn > 0) {
        maxbound = std::min(mn, maxbound);
      }
    }
    if (poly(minbound) * poly(maxbound) < 0.) {
      const double xtol = 100 * EPS, ytol = 100. / 10 * EPS;
      if (regula_falsi(poly, 0., 0.001, minbound, maxbound, xtol, ytol, root) !=
          RootStatus::SUCCESS) {
        if (err) *err = 1;
      }
    } else if (near0(poly(minbound), EPS)) {
      root = minbound;
    } else if (near0(poly(maxbound), EPS)) {
      root = maxbound;
    } else {
      root = -1.;
    }
  }
  if (root > 0. && root < 1.) return rho0 / ((1 - root) + EPS);
  return INFINITY;
}

int table_load_spiner(const char *path, int matid, bool reproducible, uint64_t *handle,
                      std::string &msg) {
  Sp5 s;
  if (!read_sp5(path, s, msg)) return SGX_ERR_IO;
  const int lt = s.i32.count("/@log_type") ? s.i32["/@log_type"] : 1;
  if (lt != 2) {
    msg = "sp5-lite image was written with a log type other than NQT order 2";
    return SGX_ERR_IO;
  }
  const std::string mat = "/" + std::to_string(matid);
  const std::string lTg = mat + "/dependsLogRhoLogT/";
  const std::string cg = mat + "/coldCurve/";
  const char *names2[NF2D] = {"pressure", "specific internal energy", "bulk modulus",
                              "dPdRho",   "dPdE",                     "dTdRho",
                              "dTdE",     "dEdRho",                   "dEdT"};
  HostTable h;
  SpinerTable &t = h.t;
  std::memset(&t, 0, sizeof(t));
  for (int k = 0; k < NF2D; ++k) {
    auto it = s.ds.find(lTg + names2[k]);
    if (it == s.ds.end() || it->second.n.size() != 2) {
      msg = "missing 2-D field " + lTg + names2[k];
      return SGX_ERR_IO;
    }
    if (k == 0) {
      h.nT = it->second.n[0];
      h.nRho = it->second.n[1];
      t.gT = make_grid(it->second.mn[0], it->second.mx[0], h.nT);
      t.gRho = make_grid(it->second.mn[1], it->second.mx[1], h.nRho);
    } else if (it->second.n[0] != h.nT || it->second.n[1] != h.nRho) {
      msg = "inconsistent 2-D field shapes";
      return SGX_ERR_IO;
    }
    h.f2[k] = it->second.data;
  }
  const char *namesc[4] = {"pressure", "specific internal energy", "bulk modulus", "dPdRho"};
  const int slotc[4] = {F_PCOLD, F_SIECOLD, F_BMODCOLD, F_DPDRHOCOLD};
  for (int k = 0; k < 4; ++k) {
    auto it = s.ds.find(cg + namesc[k]);
    if (it == s.ds.end() || it->second.n.size() != 1 || it->second.n[0] != h.nRho) {
      msg = "missing or misshapen cold-curve field " + cg + namesc[k];
      return SGX_ERR_IO;
    }
    if (k == 0) t.gCold = make_grid(it->second.mn[0], it->second.mx[0], it->second.n[0]);
    h.f1[slotc[k]] = it->second.data;
  }
  auto attr = [&](const char *name, double &v) {
    auto it = s.f64.find(mat + "@" + name);
    if (it == s.f64.end()) return false;
    v = it->second;
    return true;
  };
  double rOff = 0, tOff = 0;
  if (!attr("rhoOffset", rOff) || !attr("TOffset", tOff)) {
    msg = "missing offsets on " + mat;
    return SGX_ERR_IO;
  }
  t.nRho = h.nRho;
  t.nT = h.nT;
  t.lRhoOffset = std::fabs(rOff);
  t.lTOffset = std::fabs(tOff);
  t.reproducible = reproducible ? 1 : 0;
  t.sie_monotone_T = 1;
  for (int j = 0; j < h.nRho && t.sie_monotone_T; ++j)
    for (int i = 0; i + 1 < h.nT; ++i)
      if (!(h.f2[F_SIE][j * h.nT + i + 1] > h.f2[F_SIE][j * h.nT + i])) {
        t.sie_monotone_T = 0;
        break;
      }
  for (int k = 0; k < NF1D; ++k)
    if (h.f1[k].empty()) h.f1[k].assign(k == F_RHO_AT_PMIN ? h.nT : h.nRho, 0.0);
  h.bind();
  // set bounds (:601-608)
  t.lRhoMin = t.gRho.min;
  t.lRhoMax = t.gRho.max;
  t.rhoMax = from_log(t.lRhoMax, t.lRhoOffset);
  t.lTMin = t.gT.min;
  t.lTMax = t.gT.max;
  t.TMax = from_log(t.lTMax, t.lTOffset);
  t.TatlTMin = from_log(t.lTMin, t.lTOffset);
  // reference-state temperature: room temperature if it lies inside the
  // table, else the middle of the log-T range (loadDataboxes_ :671-677)
  t.TNormal = ROOM_TEMPERATURE;
  double lTNormal = sp_lT(t, t.TNormal);
  if (!(t.lTMin < lTNormal && lTNormal < t.lTMax)) {
    lTNormal = 0.5 * (t.lTMin + t.lTMax);
    t.TNormal = sp_T(t, lTNormal);
  }
  // reference-state density: the file's normalDensity (:559-561), or the
  // middle of the log-density range when that lies off the table (:665-670)
  double rhoNormal = 0.0;
  attr("normalDensity", rhoNormal);
  rhoNormal = std::fabs(rhoNormal);
  double lRhoNormal = sp_lRho(t, rhoNormal);
  if (!(t.lRhoMin < lRhoNormal && lRhoNormal < t.lRhoMax)) {
    lRhoNormal = 0.5 * (t.lRhoMin + t.lRhoMax);
    rhoNormal = sp_rho(t, lRhoNormal);
  }
  t.rhoNormal = rhoNormal;
  const int nR = h.nRho, nT = h.nT;
  // fixBulkModulus_ (:689-714)
  for (int j = 0; j < nR; j++) {
    const double lRho = t.gRho.x(j);
    const double rho = sp_rho(t, lRho);
    for (int i = 0; i < nT; i++) {
      const double lT = t.gT.x(i);
      const double press = interp2(t, t.f2[F_P], lRho, lT);
      const double DPDR_E = interp2(t, t.f2[F_DPDRHO], lRho, lT);
      const double DPDE_R = interp2(t, t.f2[F_DPDE], lRho, lT);
      const double DEDR_T = interp2(t, t.f2[F_DEDRHO], lRho, lT);
      const double DPDR_T = DPDR_E + DPDE_R * DEDR_T;
      double bMod;
      if (DPDE_R > 0.0 && rho > 0.0)
        bMod = rho * DPDR_E + DPDE_R * (press / rho);
      else if (rho > 0.0)
        bMod = smax(rho * DPDR_T, 0.0);
      else
        bMod = 0.0;
      h.f2[F_BMOD][j * nT + i] = smax(bMod, std::fabs(lim<double>::eps));
    }
  }
  // setlTColdCrit_ (:716-775)
  for (int j = 0; j < nR; j++)
    h.f1[F_LTCOLDCRIT][j] = cold_crit(h, j, t.gCold);
  // SetRhoPMin without vapor-dome exclusion (eos_spiner_common.hpp:59-109)
  double PMin = DBL_MAX;
  for (int i = 0; i < nT; ++i) {
    double PMin_at_T = DBL_MAX;
    int jmax = 0;
    for (int j = 0; j < nR; ++j) {
      if (h.f2[F_P][j * nT + i] < PMin_at_T) {
        PMin_at_T = h.f2[F_P][j * nT + i];
        jmax = j;
      }
    }
    if (PMin_at_T > 0) {
      h.f1[F_RHO_AT_PMIN][i] = 0;
      PMin_at_T = 0;
    } else {
      h.f1[F_RHO_AT_PMIN][i] = from_log(t.gRho.x(jmax), t.lRhoOffset);
    }
    PMin = smin(PMin_at_T, PMin);
  }
  (void)VAPOR_DPDR_THRESH;
  t.PMin = PMin;
  // cold-curve derived tables (:629-643)
  for (int j = 0; j < nR; j++) {
    const double lRho = t.gCold.x(j);
    const double lT = h.f1[F_LTCOLDCRIT][j];
    h.f1[F_BMODCOLD][j] = interp2(t, t.f2[F_BMOD], lRho, lT);
    h.f1[F_DPDECOLD][j] = interp2(t, t.f2[F_DPDE], lRho, lT);
    h.f1[F_DTDRHOCOLD][j] = interp2(t, t.f2[F_DTDRHO], lRho, lT);
    h.f1[F_DTDECOLD][j] = interp2(t, t.f2[F_DTDE], lRho, lT);
    h.f1[F_DEDTCOLD][j] = interp2(t, t.f2[F_DEDT], lRho, lT);
  }
  // maximum-temperature 1-D tables (:645-656)
  for (int j = 0; j < nR; j++) {
    const double lRho = t.gRho.x(j);
    const double rho = sp_rho(t, lRho);
    h.f1[F_PMAX][j] = h.f2[F_P][j * nT + nT - 1];
    h.f1[F_DEDTMAX][j] = h.f2[F_DEDT][j * nT + nT - 1];
    h.f1[F_GM1MAX][j] = ratio(h.f2[F_DPDE][j * nT + nT - 1], rho);
    h.f1[F_SIELTMAX][j] = h.f2[F_SIE][j * nT + nT - 1];
  }

  // reference-state pressure and (fixed) bulk modulus (:679-681)
  t.PNormal = interp2(t, t.f2[F_P], lRhoNormal, lTNormal);
  t.bModNormal = interp2(t, t.f2[F_BMOD], lRhoNormal, lTNormal);

  // ---- device image ----
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  const size_t ncell = static_cast<size_t>(nR - 1) * (nT - 1);
  size_t off = align(sizeof(SpinerTable));
  size_t off2[NF2D], off1[NF1D], offq[3], offf;
  for (int k = 0; k < NF2D; ++k) {
    off2[k] = off;
    off = align(off + h.f2[k].size() * 8);
  }
  for (int k = 0; k < NF1D; ++k) {
    off1[k] = off;
    off = align(off + h.f1[k].size() * 8);
  }
  for (int k = 0; k < 3; ++k) {
    offq[k] = off;
    off = align(off + ncell * sizeof(dq4));
  }
  offf = off;
  off = align(off + ncell * sizeof(fq4));
  const size_t offsr = off;
  off = align(off + ncell * sizeof(SieRec));
  const size_t offpr = off;
  off = align(off + ncell * sizeof(FfRec));
  const size_t offbr = off;
  off = align(off + ncell * sizeof(FfRec));
  const size_t offxl = off;
  off = align(off + static_cast<size_t>(nR) * sizeof(double));
  const size_t offco = off;
  off = align(off + static_cast<size_t>(nR - 1) * SP_COARSE_ROW * sizeof(float2));
  const size_t offc32 = off;
  off = align(off + static_cast<size_t>(nR) * sizeof(float));
  const size_t offm32 = off;
  off = align(off + static_cast<size_t>(nR) * sizeof(float));
  // the thermal-energy bin index (see SpinerTable::therm_idx)
  std::vector<uint16_t> therm;
  build_thermal_index(h.f2[F_SIE], h.f1[F_SIECOLD], nR, nT, t, therm);
  const size_t offth = off;
  off = align(off + therm.size() * sizeof(uint16_t));
  const size_t bytes = off;
  std::vector<unsigned char> img(bytes, 0);
  for (int k = 0; k < NF2D; ++k)
    std::memcpy(img.data() + off2[k], h.f2[k].data(), h.f2[k].size() * 8);
  for (int k = 0; k < NF1D; ++k)
    std::memcpy(img.data() + off1[k], h.f1[k].data(), h.f1[k].size() * 8);
  const int qsrc[3] = {F_SIE, F_P, F_BMOD};
  for (int k = 0; k < 3; ++k) {
    unsigned char *q = img.data() + offq[k];
    const std::vector<double> &f = h.f2[qsrc[k]];
    for (int j = 0; j < nR - 1; ++j)
      for (int i = 0; i < nT - 1; ++i) {
        const double c[4] = {f[j * nT + i], f[j * nT + i + 1], f[(j + 1) * nT + i],
                             f[(j + 1) * nT + i + 1]};
        std::memcpy(q + (static_cast<size_t>(j) * (nT - 1) + i) * sizeof(dq4), c, sizeof(c));
      }
  }
  {
    unsigned char *q = img.data() + offf;
    const std::vector<double> &f = h.f2[F_SIE];
    for (int j = 0; j < nR - 1; ++j)
      for (int i = 0; i < nT - 1; ++i) {
        const float c[4] = {static_cast<float>(f[j * nT + i]), static_cast<float>(f[j * nT + i + 1]),
                            static_cast<float>(f[(j + 1) * nT + i]),
                            static_cast<float>(f[(j + 1) * nT + i + 1])};
        std::memcpy(q + (static_cast<size_t>(j) * (nT - 1) + i) * sizeof(fq4), c, sizeof(c));
      }
  }
  {
    // difference-form records; values beyond the float range disable them
    bool ok = true;
    auto split = [&ok](const double v, float out[2]) {
      if (!(std::fabs(v) <= 1e37)) ok = false;
      const double w = std::fabs(v) < 1e-30 ? 0.0 : v;
      out[0] = static_cast<float>(w);
      out[1] = static_cast<float>(w - static_cast<double>(out[0]));
    };
    const std::vector<double> &fs = h.f2[F_SIE], &fp = h.f2[F_P], &fb = h.f2[F_BMOD];
    for (int j = 0; j < nR - 1; ++j)
      for (int i = 0; i < nT - 1; ++i) {
        const size_t c = static_cast<size_t>(j) * (nT - 1) + i;
        const size_t k00 = static_cast<size_t>(j) * nT + i, k01 = k00 + 1, k10 = k00 + nT,
                     k11 = k10 + 1;
        SieRec sr;
        sr.x = fs[k00];
        sr.dT = fs[k01] - fs[k00];
        sr.dR = fs[k10] - fs[k00];
        sr.dRT = (fs[k11] - fs[k10]) - (fs[k01] - fs[k00]);
        std::memcpy(img.data() + offsr + c * sizeof(SieRec), &sr, sizeof(sr));
        const std::vector<double> *pf[2] = {&fp, &fb};
        const size_t offr[2] = {offpr, offbr};
        for (int q = 0; q < 2; ++q) {
          const std::vector<double> &f = *pf[q];
          FfRec r;
          split(f[k00], r.x);
          split(f[k01] - f[k00], r.dT);
          split(f[k10] - f[k00], r.dR);
          split((f[k11] - f[k10]) - (f[k01] - f[k00]), r.dRT);
          std::memcpy(img.data() + offr[q] + c * sizeof(FfRec), &r, sizeof(r));
        }
      }
    t.ff_ok = ok ? 1 : 0;
    for (int j = 0; j < nR; ++j) {
      const double xl = t.gRho.min + j * t.gRho.dx; // as Grid1D::weights (no contraction)
      std::memcpy(img.data() + offxl + j * sizeof(double), &xl, sizeof(double));
    }
    const int nc = nT - 1;
    t.coarse_stride = (nc + SP_COARSE - 1) / SP_COARSE;
    // entries 0..SP_COARSE-1: nodes k * coarse_stride; entry SP_COARSE: the
    // last node (the end of the last stretch); the rest +inf
    for (int j = 0; j < nR - 1; ++j)
      for (int k = 0; k < SP_COARSE_ROW; ++k) {
        const int i = k < SP_COARSE ? k * t.coarse_stride : nc;
        float2 v;
        if (k <= SP_COARSE && i <= nc && (k == SP_COARSE || i < nc)) {
          v.x = static_cast<float>(fs[static_cast<size_t>(j) * nT + i]);
          v.y = static_cast<float>(fs[static_cast<size_t>(j + 1) * nT + i]);
        } else {
          v.x = v.y = INFINITY;
        }
        std::memcpy(img.data() + offco +
                        (static_cast<size_t>(j) * SP_COARSE_ROW + k) * sizeof(float2),
                    &v, sizeof(v));
      }
  }
  for (int j = 0; j < nR; ++j) {
    const float c = static_cast<float>(h.f1[F_SIECOLD][j]);
    const float m = static_cast<float>(h.f1[F_SIELTMAX][j]);
    std::memcpy(img.data() + offc32 + j * sizeof(float), &c, sizeof(float));
    std::memcpy(img.data() + offm32 + j * sizeof(float), &m, sizeof(float));
  }
  if (!therm.empty())
    std::memcpy(img.data() + offth, therm.data(), therm.size() * sizeof(uint16_t));
  void *dev = nullptr;
  cudaError_t e = cudaMalloc(&dev, bytes);
  if (e != cudaSuccess) {
    msg = std::string("cudaMalloc of table: ") + cudaGetErrorString(e);
    return SGX_ERR_CUDA;
  }
  unsigned char *d = static_cast<unsigned char *>(dev);
  SpinerTable td = t;
  for (int k = 0; k < NF2D; ++k)
    td.f2[k] = reinterpret_cast<const double *>(d + off2[k]);
  for (int k = 0; k < NF1D; ++k)
    td.f1[k] = reinterpret_cast<const double *>(d + off1[k]);
  td.sie4 = reinterpret_cast<const dq4 *>(d + offq[0]);
  td.P4 = reinterpret_cast<const dq4 *>(d + offq[1]);
  td.bmod4 = reinterpret_cast<const dq4 *>(d + offq[2]);
  td.sie4f = reinterpret_cast<const fq4 *>(d + offf);
  td.sieCold32 = reinterpret_cast<const float *>(d + offc32);
  td.sielTMax32 = reinterpret_cast<const float *>(d + offm32);
  td.sieR = reinterpret_cast<const SieRec *>(d + offsr);
  td.PR = reinterpret_cast<const FfRec *>(d + offpr);
  td.bmodR = reinterpret_cast<const FfRec *>(d + offbr);
  td.rhoNodes = reinterpret_cast<const double *>(d + offxl);
  td.sieCoarse = reinterpret_cast<const float2 *>(d + offco);
  td.therm_idx = therm.empty() ? nullptr : reinterpret_cast<const uint16_t *>(d + offth);
  std::memcpy(img.data(), &td, sizeof(td));
  e = cudaMemcpy(dev, img.data(), bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(dev);
    msg = std::string("cudaMemcpy of table: ") + cudaGetErrorString(e);
    return SGX_ERR_CUDA;
  }
  Resident r;
  r.dev = dev;
  r.bytes = bytes;
  cudaGetDevice(&r.device);
  r.host = std::move(h);
  r.host.bind();
  const uint64_t key = reinterpret_cast<uint64_t>(dev);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_tables[key] = std::move(r);
    g_tables[key].host.bind();
  }
  *handle = key;
  return SGX_OK;
}

// SpinerEOSDependsRhoSie::loadDataboxes_ (eos/eos_spiner_rho_sie.hpp:433-552)
// and calcBMod_ (:554-578): both groups' tables, the bulk moduli recomputed
// from P, dP/drho|e, dP/de|rho and de/drho|T at the nodes, the slices of P
// and dP/drho at the densest row, SetRhoPMin (eos_spiner_common.hpp:59-109,
// without vapor-dome exclusion) and the reference state. The reference's
// DataBox dump order (DBLIST, :329-336) is kept for parity checks.
int table_load_spiner_sie(const char *path, int matid, bool reproducible, uint64_t *handle,
                          std::string &msg) {
  Sp5 s;
  if (!read_sp5(path, s, msg)) return SGX_ERR_IO;
  const int lt = s.i32.count("/@log_type") ? s.i32["/@log_type"] : 1;
  if (lt != 2) {
    msg = "sp5-lite image was written with a log type other than NQT order 2";
    return SGX_ERR_IO;
  }
  const std::string mat = "/" + std::to_string(matid);
  // one group's tables, all of one shape; names in the order loadDataboxes_
  // reads them (the first is sie_ / T_)
  struct Group {
    std::vector<std::vector<double>> f;
    Grid1D gx, gr;
    int nx = 0, nr = 0;
  };
  auto load_group = [&](const std::string &g, const char *const *names, int count, Group &out) {
    out.f.resize(count);
    for (int k = 0; k < count; ++k) {
      auto it = s.ds.find(g + names[k]);
      if (it == s.ds.end() || it->second.n.size() != 2) {
        msg = "missing 2-D field " + g + names[k];
        return false;
      }
      const Dataset &d = it->second;
      if (k == 0) {
        out.nx = d.n[0];
        out.nr = d.n[1];
        out.gx = make_grid(d.mn[0], d.mx[0], out.nx);
        out.gr = make_grid(d.mn[1], d.mx[1], out.nr);
      } else if (d.n[0] != out.nx || d.n[1] != out.nr || d.mn[0] != out.gx.min ||
                 d.mx[0] != out.gx.max || d.mn[1] != out.gr.min || d.mx[1] != out.gr.max) {
        msg = "inconsistent 2-D field grids in " + g;
        return false;
      }
      out.f[k] = d.data;
    }
    return true;
  };
  // 0 sie or T, then P, bMod, dPdRho, dPdE, dTdRho, dTdE, dEdRho
  enum { G_X = 0, G_P, G_BMOD, G_DPDRHO, G_DPDE, G_DTDRHO, G_DTDE, G_DEDRHO, G_N };
  const char *namesT[G_N] = {"specific internal energy", "pressure", "bulk modulus", "dPdRho",
                             "dPdE", "dTdRho", "dTdE", "dEdRho"};
  const char *namesE[G_N] = {"temperature", "pressure", "bulk modulus", "dPdRho",
                             "dPdE", "dTdRho", "dTdE", "dEdRho"};
  Group gt, ge;
  if (!load_group(mat + "/dependsLogRhoLogT/", namesT, G_N, gt) ||
      !load_group(mat + "/dependsLogRhoLogSie/", namesE, G_N, ge))
    return SGX_ERR_IO;
  const std::string cg = mat + "/coldCurve/";
  const char *namesc[4] = {"pressure", "specific internal energy", "bulk modulus", "dPdRho"};
  std::vector<double> cold[4];
  Grid1D gCold{};
  for (int k = 0; k < 4; ++k) {
    auto it = s.ds.find(cg + namesc[k]);
    if (it == s.ds.end() || it->second.n.size() != 1) {
      msg = "missing cold-curve field " + cg + namesc[k];
      return SGX_ERR_IO;
    }
    if (k == 1) gCold = make_grid(it->second.mn[0], it->second.mx[0], it->second.n[0]);
    cold[k] = it->second.data;
  }
  auto attr = [&](const char *name, double &v) {
    auto it = s.f64.find(mat + "@" + name);
    if (it == s.f64.end()) return false;
    v = it->second;
    return true;
  };
  double rOff = 0, tOff = 0, eOff = 0, rhoNormal = 0, abar = 0, zbar = 0;
  if (!attr("rhoOffset", rOff) || !attr("TOffset", tOff) || !attr("sieOffset", eOff) ||
      !attr("normalDensity", rhoNormal) || !attr("meanAtomicMass", abar) ||
      !attr("meanAtomicNumber", zbar)) {
    msg = "missing offsets or material attributes on " + mat;
    return SGX_ERR_IO;
  }
  SieTable t;
  std::memset(&t, 0, sizeof(t));
  t.lRhoOffset = std::fabs(rOff);
  t.lTOffset = std::fabs(tOff);
  t.lEOffset = std::fabs(eOff);
  t.gT = gt.gx;
  t.gRhoT = gt.gr;
  t.gE = ge.gx;
  t.gRhoE = ge.gr;
  t.gCold = gCold;
  t.nT = gt.nx;
  t.nRhoT = gt.nr;
  t.nE = ge.nx;
  t.nRhoE = ge.nr;
  t.reproducible = reproducible ? 1 : 0;
  // calcBMod_ on each group
  for (Group *g : {&gt, &ge}) {
    for (int j = 0; j < g->nr; j++) {
      const double lRho = g->gr.x(j);
      const double rho = from_log(lRho, t.lRhoOffset);
      for (int i = 0; i < g->nx; i++) {
        const size_t k = static_cast<size_t>(j) * g->nx + i;
        const double press = g->f[G_P][k];
        const double DPDR_E = g->f[G_DPDRHO][k];
        const double DPDE_R = g->f[G_DPDE][k];
        const double DEDR_T = g->f[G_DEDRHO][k];
        const double DPDR_T = DPDR_E + DPDE_R * DEDR_T;
        double bMod;
        if (DPDE_R > 0.0 && rho > 0.0)
          bMod = rho * DPDR_E + DPDE_R * (press / rho);
        else if (rho > 0.0)
          bMod = smax(rho * DPDR_T, 0.0);
        else
          bMod = 0.0;
        g->f[G_BMOD][k] = smax(bMod, lim<double>::eps);
      }
    }
  }
  const int nR = gt.nr, nT = gt.nx;
  t.lRhoMin = gt.gr.min;
  t.lRhoMax = gt.gr.max;
  t.rhoMax = from_log(t.lRhoMax, t.lRhoOffset);
  // the densest row of P and dP/drho|e on the rho-T grid
  std::vector<double> PlRhoMax(gt.f[G_P].begin() + static_cast<size_t>(nR - 1) * nT,
                               gt.f[G_P].begin() + static_cast<size_t>(nR) * nT);
  std::vector<double> dPdRhoMax(gt.f[G_DPDRHO].begin() + static_cast<size_t>(nR - 1) * nT,
                                gt.f[G_DPDRHO].begin() + static_cast<size_t>(nR) * nT);
  // SetRhoPMin without vapor-dome exclusion
  std::vector<double> rho_at_pmin(nT, 0.0);
  double PMin = DBL_MAX;
  for (int i = 0; i < nT; ++i) {
    double PMin_at_T = DBL_MAX;
    int jmax = 0;
    for (int j = 0; j < nR; ++j) {
      const double p = gt.f[G_P][static_cast<size_t>(j) * nT + i];
      if (p < PMin_at_T) {
        PMin_at_T = p;
        jmax = j;
      }
    }
    if (PMin_at_T > 0) {
      rho_at_pmin[i] = 0;
      PMin_at_T = 0;
    } else {
      rho_at_pmin[i] = from_log(gt.gr.x(jmax), t.lRhoOffset);
    }
    PMin = smin(PMin_at_T, PMin);
  }
  t.PMin = PMin;
  // reference state (:526-548)
  rhoNormal = std::fabs(rhoNormal);
  double lRhoNormal = to_log(rhoNormal, t.lRhoOffset);
  if (!(t.lRhoMin < lRhoNormal && lRhoNormal < t.lRhoMax)) {
    lRhoNormal = 0.5 * (t.lRhoMin + t.lRhoMax);
    rhoNormal = from_log(lRhoNormal, t.lRhoOffset);
  }
  double TNormal = ROOM_TEMPERATURE;
  double lTNormal = to_log(TNormal, t.lTOffset);
  const double lTMin = gt.gx.min, lTMax = gt.gx.max;
  if (!(lTMin < lTNormal && lTNormal < lTMax)) {
    lTNormal = 0.5 * (lTMin + lTMax);
    TNormal = from_log(lTNormal, t.lTOffset);
  }
  auto at = [&](const std::vector<double> &f) {
    return sie_interp2(gt.gx, gt.gr, nT, f.data(), lRhoNormal, lTNormal);
  };
  t.rhoNormal = rhoNormal;
  t.TNormal = TNormal;
  t.sieNormal = at(gt.f[G_X]);
  t.PNormal = at(gt.f[G_P]);
  t.CvNormal = 1. / at(gt.f[G_DTDE]);
  t.bModNormal = at(gt.f[G_BMOD]);
  t.dPdENormal = at(gt.f[G_DPDE]);
  const double dPdR = at(gt.f[G_DPDRHO]);
  t.dVdTNormal = t.dPdENormal * t.CvNormal / (t.rhoNormal * t.rhoNormal * dPdR);

  // ---- device image ----
  auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
  const int srcT[NST2D] = {G_X, G_P, G_BMOD, G_DPDE, G_DTDE};
  const int srcE[NSE2D] = {G_X, G_P, G_BMOD, G_DPDE, G_DTDE};
  size_t off = align(sizeof(SieTable));
  size_t offT[NST2D], offE[NSE2D];
  for (int k = 0; k < NST2D; ++k) {
    offT[k] = off;
    off = align(off + gt.f[srcT[k]].size() * 8);
  }
  for (int k = 0; k < NSE2D; ++k) {
    offE[k] = off;
    off = align(off + ge.f[srcE[k]].size() * 8);
  }
  const std::vector<double> *one[4] = {&cold[1], &PlRhoMax, &dPdRhoMax, &rho_at_pmin};
  size_t off1[4];
  for (int k = 0; k < 4; ++k) {
    off1[k] = off;
    off = align(off + one[k]->size() * 8);
  }
  // the float-float cells of the rho-sie group (see SieCellFF); values
  // beyond the float range leave the mixed path off for this table
  const int nE = ge.nx, nRE = ge.nr;
  std::vector<SieCellFF> cells(static_cast<size_t>(nRE - 1) * (nE - 1));
  bool ff_ok = true;
  {
    auto split = [&ff_ok](const double v, float out[2]) {
      if (!(std::fabs(v) <= 1e37)) ff_ok = false;
      const double w = std::fabs(v) < 1e-30 ? 0.0 : v;
      out[0] = static_cast<float>(w);
      out[1] = static_cast<float>(w - static_cast<double>(out[0]));
    };
    auto rec = [&](const std::vector<double> &f, const int j, const int i, FfRec &r) {
      const size_t k00 = static_cast<size_t>(j) * nE + i, k01 = k00 + 1, k10 = k00 + nE,
                   k11 = k10 + 1;
      split(f[k00], r.x);
      split(f[k01] - f[k00], r.dT);
      split(f[k10] - f[k00], r.dR);
      split((f[k11] - f[k10]) - (f[k01] - f[k00]), r.dRT);
    };
    for (int j = 0; j < nRE - 1; ++j)
      for (int i = 0; i < nE - 1; ++i) {
        SieCellFF &c = cells[static_cast<size_t>(j) * (nE - 1) + i];
        rec(ge.f[G_X], j, i, c.T);
        rec(ge.f[G_P], j, i, c.P);
        rec(ge.f[G_DTDE], j, i, c.dTdE);
        rec(ge.f[G_BMOD], j, i, c.bMod);
      }
    // per axis: u = lX inv - min inv with lX = v K, K = scale_down
    // log10(2); in fixed point with F fractional bits, u 2^F =
    // floor(v M / 2^64) - Off, M = K inv 2^(64+F) in [2^60, 2^61) and
    // |u 2^F| < 2^60 for |v| < 2^62. The products are formed in double-double
    // (fma gives each rounding error exactly).
    const Grid1D *ax[2] = {&t.gRhoE, &t.gE};
    for (int k = 0; k < 2; ++k) {
      const double a = nqt::scale_down, b = nqt::log2_over_log10, inv = ax[k]->inv_dx;
      const double k1 = a * b, k1e = std::fma(a, b, -k1); // K = k1 + k1e
      const double c1 = k1 * inv;
      const double c1e = std::fma(k1, inv, -c1) + k1e * inv; // K inv = c1 + c1e
      const int F = static_cast<int>(std::floor(-std::log2(c1))) - 3;
      const double mh = std::ldexp(c1, 64 + F), ml = std::ldexp(c1e, 64 + F);
      t.fxM[k] = std::llround(mh) + std::llround(ml);
      const double o = ax[k]->min * inv, oe = std::fma(ax[k]->min, inv, -o);
      t.fxOff[k] = std::llround(std::ldexp(o, F)) + std::llround(std::ldexp(oe, F));
      t.fxF[k] = F;
    }
  }
  const size_t offc = off;
  if (ff_ok) off = align(off + cells.size() * sizeof(SieCellFF));
  const size_t bytes = off;
  std::vector<unsigned char> img(bytes, 0);
  for (int k = 0; k < NST2D; ++k)
    std::memcpy(img.data() + offT[k], gt.f[srcT[k]].data(), gt.f[srcT[k]].size() * 8);
  for (int k = 0; k < NSE2D; ++k)
    std::memcpy(img.data() + offE[k], ge.f[srcE[k]].data(), ge.f[srcE[k]].size() * 8);
  for (int k = 0; k < 4; ++k)
    std::memcpy(img.data() + off1[k], one[k]->data(), one[k]->size() * 8);
  if (ff_ok) std::memcpy(img.data() + offc, cells.data(), cells.size() * sizeof(SieCellFF));
  void *dev = nullptr;
  cudaError_t e = cudaMalloc(&dev, bytes);
  if (e != cudaSuccess) {
    msg = std::string("cudaMalloc of table: ") + cudaGetErrorString(e);
    return SGX_ERR_CUDA;
  }
  unsigned char *d = static_cast<unsigned char *>(dev);
  SieTable td = t;
  for (int k = 0; k < NST2D; ++k)
    td.fT[k] = reinterpret_cast<const double *>(d + offT[k]);
  for (int k = 0; k < NSE2D; ++k)
    td.fE[k] = reinterpret_cast<const double *>(d + offE[k]);
  td.sieCold = reinterpret_cast<const double *>(d + off1[0]);
  td.PlRhoMax = reinterpret_cast<const double *>(d + off1[1]);
  td.dPdRhoMax = reinterpret_cast<const double *>(d + off1[2]);
  td.rho_at_pmin = reinterpret_cast<const double *>(d + off1[3]);
  td.cellsE = ff_ok ? reinterpret_cast<const SieCellFF *>(d + offc) : nullptr;
  std::memcpy(img.data(), &td, sizeof(td));
  e = cudaMemcpy(dev, img.data(), bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(dev);
    msg = std::string("cudaMemcpy of table: ") + cudaGetErrorString(e);
    return SGX_ERR_CUDA;
  }
  Resident r;
  r.dev = dev;
  r.bytes = bytes;
  r.sie_cells = ff_ok;
  cudaGetDevice(&r.device);
  // DBLIST: sie_, T_, rho_at_pmin_, the rho-T tables, the rho-sie tables,
  // mF_ (none), PlRhoMax_, dPdRhoMax_, PCold_, sieCold_, bModCold_, dPdRhoCold_
  std::vector<const std::vector<double> *> order = {&gt.f[G_X], &ge.f[G_X], &rho_at_pmin};
  for (Group *g : {&gt, &ge})
    for (int k = G_P; k < G_N; ++k)
      order.push_back(&g->f[k]);
  for (const std::vector<double> *v : {&PlRhoMax, &dPdRhoMax, &cold[0], &cold[1], &cold[2],
                                       &cold[3]})
    order.push_back(v);
  for (const std::vector<double> *v : order)
    r.dump.insert(r.dump.end(), v->begin(), v->end());
  const uint64_t key = reinterpret_cast<uint64_t>(dev);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_tables[key] = std::move(r);
  }
  *handle = key;
  return SGX_OK;
}

// HelmElectrons::InitDataFile_ (eos/eos_helmholtz.hpp:962-989): four blocks
// of whitespace-separated values, each over j (temperature) then i (electron
// density, fastest); then the node values 10^x of both grids, computed on
// the host as math_utils::pow10 does (exp(ln10 * x)).
int table_load_helm(const char *path, uint64_t *handle, std::string &msg) {
  std::ifstream file(path, std::ios::binary);
  if (!file.is_open()) {
    msg = std::string("HelmElectrons file ") + path + " not found!";
    return SGX_ERR_IO;
  }
  std::stringstream ss;
  ss << file.rdbuf();
  const std::string text = ss.str();
  const char *cur = text.c_str();
  constexpr int NT = HELM_NT, NR = HELM_NRHO;
  const int nper[4] = {9, 4, 4, 4};
  // fields[b][k][j * NR + i]
  std::vector<std::vector<double>> fields[4];
  for (int b = 0; b < 4; ++b) {
    fields[b].assign(nper[b], std::vector<double>(static_cast<size_t>(NT) * NR));
    for (int j = 0; j < NT; ++j)
      for (int i = 0; i < NR; ++i)
        for (int k = 0; k < nper[b]; ++k) {
          char *end = nullptr;
          const double v = std::strtod(cur, &end);
          if (end == cur) {
            msg = "Error reading the Helmholtz free energy table at j = " + std::to_string(j) +
                  ", i = " + std::to_string(i);
            return SGX_ERR_IO;
          }
          fields[b][k][static_cast<size_t>(j) * NR + i] = v;
          cur = end;
        }
  }
  HelmTable t{};
  t.lRhoMin = -12.0;
  t.lRhoMax = 15.0;
  t.dlRho = (t.lRhoMax - t.lRhoMin) / static_cast<double>(NR - 1);
  t.inv_dlRho = 1 / t.dlRho;
  t.lTMin = 3.0;
  t.lTMax = 13.0;
  t.dlT = (t.lTMax - t.lTMin) / static_cast<double>(NT - 1);
  t.inv_dlT = 1 / t.dlT;
  t.rhoMin = 1e-12; // ipow10<-12>(): 1 / 10^12, correctly rounded
  t.rhoMax = 1e15;
  std::vector<double> rho(NR), T(NT);
  for (int i = 0; i < NR; ++i)
    rho[i] = std::exp(helm::LN10 * (t.lRhoMin + i * t.dlRho));
  for (int j = 0; j < NT; ++j)
    T[j] = std::exp(helm::LN10 * (t.lTMin + j * t.dlT));
  // per-cell records in the order the kernels read them
  const std::vector<double> *f5[9] = {&fields[0][0], &fields[0][2], &fields[0][4],
                                      &fields[0][1], &fields[0][3], &fields[0][5],
                                      &fields[0][6], &fields[0][7], &fields[0][8]};
  // block 1 columns: f fd ft fdd ftt fdt fddt fdtt fddtt -> record order
  // f, ft, ftt, fd, fdd, fdt, fddt, fdtt, fddtt
  const int cub[4] = {0, 2, 1, 3}; // dpdf dpdfd dpdft dpdfdt -> val, dT, dD, dDdT
  const size_t ncell = static_cast<size_t>(NT - 1) * (NR - 1);
  std::vector<double> cells(ncell * HELM_REC);
  for (int j = 0; j < NT - 1; ++j)
    for (int i = 0; i < NR - 1; ++i) {
      double *r = cells.data() + (static_cast<size_t>(j) * (NR - 1) + i) * HELM_REC;
      const size_t c[4] = {static_cast<size_t>(j) * NR + i, static_cast<size_t>(j) * NR + i + 1,
                           static_cast<size_t>(j + 1) * NR + i,
                           static_cast<size_t>(j + 1) * NR + i + 1};
      int o = 0;
      for (int f = 0; f < 9; ++f)
        for (int q = 0; q < 4; ++q)
          r[o++] = (*f5[f])[c[q]];
      for (int b = 1; b < 4; ++b)
        for (int f = 0; f < 4; ++f)
          for (int q = 0; q < 4; ++q)
            r[o++] = fields[b][cub[f]][c[q]];
    }
  // FP32 normalised biquintic coefficients (HelmTable::cells32): term k's
  // coefficient times the powers of the cell widths its weights carry, laid
  // out [T weight][density weight]
  std::vector<float> cells32(ncell * 36);
  bool f32_ok = true;
  for (int j = 0; j < NT - 1 && f32_ok; ++j)
    for (int i = 0; i < NR - 1; ++i) {
      const double *r = cells.data() + (static_cast<size_t>(j) * (NR - 1) + i) * HELM_REC;
      float *o = cells32.data() + (static_cast<size_t>(j) * (NR - 1) + i) * 36;
      const double dth = T[j + 1] - T[j], dd = rho[i + 1] - rho[i];
      const double ts[6] = {1.0, 1.0, dth, -dth, dth * dth, dth * dth};
      const double ds[6] = {1.0, 1.0, dd, -dd, dd * dd, dd * dd};
      for (int k = 0; k < 36; ++k) {
        const double v = r[k] * ts[helm::H5_TI[k]] * ds[helm::H5_DI[k]];
        if (!(std::fabs(v) < 1e37)) f32_ok = false;
        o[helm::H5_TI[k] * 6 + helm::H5_DI[k]] = static_cast<float>(v);
      }
    }
  const size_t off_cells = 256;
  const size_t off_rho = off_cells + cells.size() * 8;
  const size_t off_T = off_rho + NR * 8;
  const size_t off_c32 = (off_T + NT * 8 + 255) / 256 * 256;
  const size_t off_rho32 = off_c32 + cells32.size() * sizeof(float);
  const size_t off_T32 = off_rho32 + NR * sizeof(float);
  const size_t bytes = f32_ok ? off_T32 + NT * sizeof(float) : off_c32;
  // the FP32 phase's float copies of the nodes and grid constants
  std::vector<float> rho32(NR), T32(NT);
  for (int i = 0; i < NR; ++i)
    rho32[i] = static_cast<float>(rho[i]);
  for (int j = 0; j < NT; ++j)
    T32[j] = static_cast<float>(T[j]);
  t.f_lRhoMin = static_cast<float>(t.lRhoMin);
  t.f_lRhoMax = static_cast<float>(t.lRhoMax);
  t.f_inv_dlRho = static_cast<float>(t.inv_dlRho);
  t.f_lTMin = static_cast<float>(t.lTMin);
  t.f_inv_dlT = static_cast<float>(t.inv_dlT);
  t.f_rhoMin = static_cast<float>(t.rhoMin);
  t.f_rhoMax = static_cast<float>(t.rhoMax);
  void *dev = nullptr;
  cudaError_t e = cudaMalloc(&dev, bytes);
  if (e != cudaSuccess) {
    msg = std::string("cudaMalloc of table: ") + cudaGetErrorString(e);
    return SGX_ERR_CUDA;
  }
  unsigned char *d = static_cast<unsigned char *>(dev);
  t.cells = reinterpret_cast<const double *>(d + off_cells);
  t.rho = reinterpret_cast<const double *>(d + off_rho);
  t.T = reinterpret_cast<const double *>(d + off_T);
  t.cells32 = f32_ok ? reinterpret_cast<const float *>(d + off_c32) : nullptr;
  t.rho32 = f32_ok ? reinterpret_cast<const float *>(d + off_rho32) : nullptr;
  t.T32 = f32_ok ? reinterpret_cast<const float *>(d + off_T32) : nullptr;
  std::vector<unsigned char> img(bytes, 0);
  std::memcpy(img.data(), &t, sizeof(t));
  std::memcpy(img.data() + off_cells, cells.data(), cells.size() * 8);
  std::memcpy(img.data() + off_rho, rho.data(), NR * 8);
  std::memcpy(img.data() + off_T, T.data(), NT * 8);
  if (f32_ok) {
    std::memcpy(img.data() + off_c32, cells32.data(), cells32.size() * sizeof(float));
    std::memcpy(img.data() + off_rho32, rho32.data(), NR * sizeof(float));
    std::memcpy(img.data() + off_T32, T32.data(), NT * sizeof(float));
  }
  e = cudaMemcpy(dev, img.data(), bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(dev);
    msg = std::string("cudaMemcpy of table: ") + cudaGetErrorString(e);
    return SGX_ERR_CUDA;
  }
  Resident r;
  r.dev = dev;
  r.bytes = bytes;
  cudaGetDevice(&r.device);
  // dump: the node values and the fields in the reference's DBLIST order
  // (rho_, T_, f_ .. fddtt_, dpdf_ .., ef_ .., xf_ ..; eos_helmholtz.hpp:281-292)
  r.dump = rho;
  r.dump.insert(r.dump.end(), T.begin(), T.end());
  for (int b = 0; b < 4; ++b)
    for (auto &v : fields[b])
      r.dump.insert(r.dump.end(), v.begin(), v.end());
  const uint64_t key = reinterpret_cast<uint64_t>(dev);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_tables[key] = std::move(r);
  }
  *handle = key;
  return SGX_OK;
}

int table_free(uint64_t handle, std::string &msg) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(handle);
  if (it == g_tables.end()) {
    msg = "sgx_eos_finalize: unknown table (already finalized?)";
    return SGX_ERR_INVALID;
  }
  cudaFree(it->second.dev);
  g_tables.erase(it);
  return SGX_OK;
}

int table_nrho(uint64_t handle) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(handle);
  return (it == g_tables.end() || !it->second.dump.empty()) ? 0 : it->second.host.t.nRho;
}

bool table_has_thermal_index(uint64_t handle) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(handle);
  return it != g_tables.end() && it->second.dump.empty() && it->second.host.t.therm_bins > 0;
}

bool table_has_sie_cells(uint64_t handle) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(handle);
  return it != g_tables.end() && it->second.sie_cells;
}

size_t table_bytes(uint64_t handle) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(handle);
  return it == g_tables.end() ? 0 : it->second.bytes;
}

long table_dump(uint64_t handle, double *out, long cap) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_tables.find(handle);
  if (it == g_tables.end()) return -1;
  if (!it->second.dump.empty()) {
    const long total = static_cast<long>(it->second.dump.size());
    if (out && cap >= total) std::memcpy(out, it->second.dump.data(), total * 8);
    return total;
  }
  const HostTable &h = it->second.host;
  // DBLIST order (eos_spiner_rho_temp.hpp:253-257); mF_ is empty.
  std::vector<const std::vector<double> *> order;
  for (int k = 0; k < NF2D; ++k)
    order.push_back(&h.f2[k]);
  const int o1[] = {F_PMAX,     F_SIELTMAX,   F_DEDTMAX,   F_GM1MAX,    F_LTCOLDCRIT,
                    F_PCOLD,    F_SIECOLD,    F_BMODCOLD,  F_DPDRHOCOLD, F_DPDECOLD,
                    F_DTDRHOCOLD, F_DTDECOLD, F_DEDTCOLD,  F_RHO_AT_PMIN};
  for (int k : o1)
    order.push_back(&h.f1[k]);
  long total = 0;
  for (auto *v : order)
    total += static_cast<long>(v->size());
  if (out && cap >= total) {
    long o = 0;
    for (auto *v : order) {
      std::memcpy(out + o, v->data(), v->size() * 8);
      o += static_cast<long>(v->size());
    }
  }
  return total;
}

} // namespace sgx
