// get_sg_eos (singularity-eos eos/get_sg_eos.cpp:35-280) in all its input
// modes: per cell, the mass fractions are normalised, the materials above
// the mass-fraction cutoff take part in a PTE solve (or, alone, in direct
// lookups), and the cell's pressure, temperature, energy, bulk modulus, heat
// capacity and dP/de are formed from the material states
// (get_sg_eos_functors.hpp).
//
//   input_int 0, 1  (rho, sie)  PTESolverRhoT    get_sg_eos_rho_e.cpp:30-88
//   input_int -3    (rho, T)    PTESolverFixedT  get_sg_eos_rho_t.cpp:21-110
//   input_int -2    (rho, P)    PTESolverFixedP  get_sg_eos_rho_p.cpp:21-118
//   input_int -1    (P, T)      no solve         get_sg_eos_p_t.cpp:23-102
//
// Three stages on one stream: sgeos_init packs each cell's participating
// materials into the [slot][cell] arrays of the PTE kernels (init_functor,
// :28-118; the whole (P, T) mode), the PTE kernels of sgx_pte_solve run on
// them (cells with fewer than two participating materials carry no
// material and are skipped), and sgeos_final does the pure-cell lookups and
// the averages (final_functor, :185-300). Per-cell arrays are [cell_dim];
// per-material arrays are LayoutLeft [nmat][cell_dim] (element (i, m) at
// i + m * cell_dim); offsets are the reference's 1-based cell indices.
//
// The reference places each cell's lambda cache inside the solver scratch,
// where it overlaps solver arrays (get_sg_eos_rho_e.cpp:50-52,
// get_sg_eos_rho_t.cpp:50-54); here it has its own array. The two agree for
// every EOS that does not write its lambda (all but the tabulated ones).
#include <cstring>
#include <string>

#include <cuda_runtime.h>

#include "sgx_dispatch.cuh"
#include "sgx_internal.h"

namespace sgx {

namespace {

constexpr double EV2K = 1.160451930280894026e4; // get_sg_eos.hpp:68
constexpr int SG_BLOCK = 128;

struct SgArgs {
  int nmat, ncell, cell_dim, neos;
  int mode; // input_int
  sgx_eos eos[MAX_EOS];
  int eos_of[MAX_NMAT]; // eos_offsets - 1
  const int *offsets;
  double *press, *pmax, *vol, *spvol, *sie, *temp, *bmod, *dpde, *cv;
  double *frac_mass, *frac_vol, *frac_ie, *frac_bmod, *frac_dpde, *frac_cv;
  double cutoff;
  // PTE inputs and outputs, [slot][ncell]; lambda [slot][3][ncell]
  int32_t *eos_idx;
  double *vfrac_tot, *sie_tot, *rho, *vfrac, *psie, *ptemp, *ppress, *lambda;
  // per cell: mass sum, participating count, participating materials [slot][ncell]
  double *mass_sum;
  int *npte, *mats;
};

// (P, T) input (get_sg_eos_p_t.cpp:33-86): every material at the cell's
// P and T, volumes from the resulting densities; no solve.
__device__ void sgeos_init_pt(const SgArgs &a, const sgx_eos *eos, const int iloop, const int i) {
  const long long nc = a.ncell, cd = a.cell_dim;
  double mass_sum = 0.0;
  for (int m = 0; m < a.nmat; ++m) {
    const long long k = m * nc + iloop;
    mass_sum += a.frac_mass[i + m * cd];
    a.mats[k] = m;
    a.eos_idx[k] = -1;
    a.ptemp[k] = a.temp[i] * EV2K;
    a.ppress[k] = a.press[i];
  }
  for (int m = 0; m < a.nmat; ++m)
    a.frac_mass[i + m * cd] /= mass_sum;
  double vfrac_tot = 0.0, sie_tot = 0.0;
  for (int m = 0; m < a.nmat; ++m) {
    const long long k = m * nc + iloop;
    double cache[3] = {0.0, 0.0, 0.0};
    double r = 0.0, e = 0.0;
    int err = 0;
    ev_rho_sie_from_PT(eos[a.eos_of[m]], a.ppress[k], a.ptemp[k], r, e, cache, &err);
    for (int l = 0; l < 3; ++l)
      a.lambda[(m * 3LL + l) * nc + iloop] = cache[l];
    a.rho[k] = r;
    a.psie[k] = e;
    const double fm = a.frac_mass[i + m * cd];
    a.vfrac[k] = fm / r * mass_sum;
    vfrac_tot += a.vfrac[k];
    sie_tot += e * fm;
  }
  a.sie[i] = sie_tot;
  a.vol[i] = vfrac_tot;
  a.spvol[i] = a.vol[i] / mass_sum;
  for (int m = 0; m < a.nmat; ++m)
    a.vfrac[m * nc + iloop] /= vfrac_tot;
  a.mass_sum[iloop] = mass_sum;
  a.npte[iloop] = a.nmat;
  a.vfrac_tot[iloop] = vfrac_tot;
  a.sie_tot[iloop] = 0.0;
}

__global__ void __launch_bounds__(SG_BLOCK) sgeos_init(const SgArgs a) {
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  const int iloop = blockIdx.x * blockDim.x + threadIdx.x;
  if (iloop >= a.ncell) return;
  const long long nc = a.ncell, cd = a.cell_dim;
  const int i = a.offsets[iloop] - 1;
  if (a.mode == -1) {
    sgeos_init_pt(a, s_eos, iloop, i);
    return;
  }
  // init_functor's multipliers: (rho, sie) t 0 s 1 p 0; (rho, T) t 1 s 0 p 0;
  // (rho, P) t 0 s 0 p 1
  const double t_mult = a.mode == -3 ? 1.0 : 0.0;
  const double s_mult = a.mode >= 0 ? 1.0 : 0.0;
  const double p_mult = a.mode == -2 ? 1.0 : 0.0;
  double mass_sum = 0.0;
  for (int m = 0; m < a.nmat; ++m) {
    const double fm = a.frac_mass[i + m * cd];
    mass_sum += fm;
    a.frac_vol[i + m * cd] = fm;
    a.frac_ie[i + m * cd] = a.sie[i] * fm * s_mult;
  }
  for (int m = 0; m < a.nmat; ++m)
    a.frac_mass[i + m * cd] /= mass_sum;
  int npte = 0;
  int mats[MAX_NMAT];
  for (int m = 0; m < a.nmat; ++m)
    if (a.frac_mass[i + m * cd] > a.cutoff) mats[npte++] = m;
  double vfrac_sum = 0.0;
  for (int mp = 0; mp < a.nmat; ++mp) {
    const long long k = mp * nc + iloop;
    if (mp < npte) {
      const int m = mats[mp];
      const double fm = a.frac_mass[i + m * cd];
      a.vfrac[k] = fm;
      vfrac_sum += fm;
      a.rho[k] = fm / a.spvol[i] / fm;
      a.ptemp[k] = a.temp[i] * EV2K * t_mult;
      a.ppress[k] = a.press[i] * p_mult;
      a.psie[k] = a.sie[i] * fm * s_mult;
      a.eos_idx[k] = npte > 1 ? a.eos_of[m] : -1;
      a.mats[k] = m;
    } else {
      a.vfrac[k] = a.rho[k] = a.ptemp[k] = a.ppress[k] = a.psie[k] = 0.0;
      a.eos_idx[k] = -1;
      a.mats[k] = -1;
    }
    for (int l = 0; l < 3; ++l)
      a.lambda[(mp * 3LL + l) * nc + iloop] = 0.0;
  }
  a.vfrac_tot[iloop] = vfrac_sum;
  // the solver's scalar argument: sie (RhoT), T_true = temp_pte(0)
  // (FixedT), P = press_pte(0) (FixedP)
  a.sie_tot[iloop] = a.mode == -3 ? a.ptemp[iloop] : a.mode == -2 ? a.ppress[iloop] : a.sie[i];
  a.mass_sum[iloop] = mass_sum;
  a.npte[iloop] = npte;
}

__global__ void __launch_bounds__(SG_BLOCK) sgeos_final(const SgArgs a) {
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  const int iloop = blockIdx.x * blockDim.x + threadIdx.x;
  if (iloop >= a.ncell) return;
  const long long nc = a.ncell, cd = a.cell_dim;
  const int i = a.offsets[iloop] - 1;
  const int npte = a.npte[iloop];
  const double mass_sum = a.mass_sum[iloop];
  auto lam = [&](int mp) { return a.lambda + mp * 3LL * nc + iloop; };
  // the lambda cache is [slot][3][cell]: gather one material's row
  double cache[MAX_NMAT][3];
  for (int mp = 0; mp < npte; ++mp)
    for (int l = 0; l < 3; ++l)
      cache[mp][l] = lam(mp)[l * nc];
  // final_functor's multipliers per mode
  double t_mult = 0.0, p_mult = 0.0;
  if (a.mode >= 0) {
    // (rho, sie) pure cell (get_sg_eos_rho_e.cpp:76-83)
    if (npte == 1) {
      const sgx_eos &e = s_eos[a.eos_of[a.mats[iloop]]];
      const double r = a.rho[iloop];
      const double t = ev_T_from_rho_sie<double>(e, r, a.psie[iloop], cache[0]);
      a.ptemp[iloop] = t;
      a.ppress[iloop] = ev_P_from_rho_T<double>(e, r, t, cache[0]);
    }
    t_mult = 1.0, p_mult = 1.0;
  } else if (a.mode == -3 || a.mode == -2) {
    double sie_tot_true = 0.0;
    if (npte > 1) {
      for (int mp = 0; mp < npte; ++mp) {
        const long long k = mp * nc + iloop;
        sie_tot_true += a.psie[k] * a.frac_mass[i + a.mats[k] * cd];
      }
    } else {
      const sgx_eos &e = s_eos[a.eos_of[a.mats[iloop]]];
      const double r = a.rho[iloop];
      if (a.mode == -3) {
        // get_sg_eos_rho_t.cpp:78-90
        const double t = a.ptemp[iloop];
        a.psie[iloop] = ev_sie_from_rho_T<double>(e, r, t, cache[0]);
        sie_tot_true = a.psie[iloop];
        a.ppress[iloop] = ev_P_from_rho_T<double>(e, r, t, cache[0]);
      } else {
        // get_sg_eos_rho_p.cpp:76-96: T from P(rho, T) = P by findRoot
        // between 1e-10 and 1e10 times the reference temperature
        double *c0 = cache[0];
        auto p_from_t = [&](const double t) { return ev_P_from_rho_T<double>(e, r, t, c0); };
        const double r_temp = ev_reference_T(e);
        double temp_i = 0.0;
        find_root(p_from_t, a.press[i], r_temp, 1.e-10 * r_temp, 1.e10 * r_temp, 1.e-12,
                  1.e-12, temp_i);
        a.psie[iloop] = ev_sie_from_rho_T<double>(e, r, temp_i, cache[0]);
        sie_tot_true = a.psie[iloop];
        a.ptemp[iloop] = temp_i;
      }
    }
    a.sie[i] = sie_tot_true;
    if (a.mode == -3)
      p_mult = 1.0;
    else
      t_mult = 1.0;
  }
  const bool do_t = t_mult == 1.0, do_p = p_mult == 1.0;
  double press = do_p ? 0.0 : a.press[i], temp = do_t ? 0.0 : a.temp[i];
  double bmod = 0.0, cv = 0.0, dpde = 0.0, sie = a.sie[i];
  for (int mp = 0; mp < npte; ++mp) {
    const long long k = mp * nc + iloop;
    const int m = a.mats[k];
    const double vf = a.vfrac[k], r = a.rho[k], t = a.ptemp[k];
    const double fm = a.frac_mass[i + m * cd];
    press += a.ppress[k] * vf * p_mult;
    temp += t * vf * t_mult;
    const double ie_m = a.psie[k] * fm * mass_sum;
    sie += ie_m * 0.0;
    a.frac_ie[i + m * cd] = ie_m;
    a.frac_vol[i + m * cd] = vf * a.vol[i];
    const sgx_eos &e = s_eos[a.eos_of[m]];
    const double bmod_m = ev_B_from_rho_T<double>(e, r, t, cache[mp]);
    bmod += bmod_m * vf;
    const double cv_m = EV2K * ev_cv_from_rho_T<double>(e, r, t, cache[mp]);
    cv += cv_m * fm;
    const double dpde_m = ev_gamma_from_rho_T<double>(e, r, t, cache[mp]);
    dpde += dpde_m * vf;
    if (a.frac_bmod) a.frac_bmod[i + m * cd] = bmod_m;
    if (a.frac_cv) a.frac_cv[i + m * cd] = cv_m;
    if (a.frac_dpde) a.frac_dpde[i + m * cd] = dpde_m;
  }
  a.press[i] = press;
  a.temp[i] = do_t ? temp / EV2K : temp;
  a.sie[i] = sie;
  a.bmod[i] = bmod;
  a.cv[i] = cv;
  a.dpde[i] = dpde;
  for (int m = 0; m < a.nmat; ++m)
    a.frac_mass[i + m * cd] *= mass_sum;
  a.pmax[i] = press > a.pmax[i] ? press : a.pmax[i];
}

// The argument checks shared by the host-array and device-array calls,
// before any array is touched.
int sgeos_check(const char *who, int nmat, int ncell, int cell_dim, int input_int,
                const int *eos_offsets, const sgx_eos *eos, int neos, int precision) {
  const std::string w(who);
  if (input_int < -3 || input_int > 1) return set_error(SGX_ERR_INVALID, w + ": bad input_int");
  if (nmat < 1 || nmat > PTE_MAX_N)
    return set_error(SGX_ERR_UNSUPPORTED, w + ": nmat must be in 1..6");
  if (ncell < 0 || cell_dim < ncell)
    return set_error(SGX_ERR_INVALID, w + ": need 0 <= ncell <= cell_dim");
  if (ncell == 0) return SGX_OK;
  if (!eos || neos < 1 || neos > MAX_EOS || !eos_offsets)
    return set_error(SGX_ERR_INVALID, w + ": eos list / offsets");
  if (precision != SGX_PREC_FP64 && precision != SGX_PREC_MIXED)
    return set_error(SGX_ERR_INVALID, w + ": bad precision");
  if (precision == SGX_PREC_MIXED && (input_int == -3 || input_int == -2))
    return set_error(SGX_ERR_UNSUPPORTED,
                     w + ": SGX_PREC_MIXED is for the (rho, sie) and (P, T) modes");
  return SGX_OK;
}

} // namespace

} // namespace sgx

extern "C" int sgx_get_sg_eos_device(int nmat, int ncell, int cell_dim, int input_int,
                                     const int *eos_offsets, const sgx_eos *eos, int neos,
                                     const int *offsets, double *press, double *pmax,
                                     double *vol, double *spvol, double *sie, double *temp,
                                     double *bmod, double *dpde, double *cv, double *frac_mass,
                                     double *frac_vol, double *frac_ie, double *frac_bmod,
                                     double *frac_dpde, double *frac_cv, double mass_frac_cutoff,
                                     int precision, sgx_stream_t stream) {
  using namespace sgx;
  const int ck = sgeos_check("sgx_get_sg_eos_device", nmat, ncell, cell_dim, input_int,
                             eos_offsets, eos, neos, precision);
  if (ck != SGX_OK || ncell == 0) return ck;
  if (!offsets || !press || !pmax || !vol || !spvol || !sie || !temp || !bmod || !dpde || !cv ||
      !frac_mass || !frac_vol || !frac_ie)
    return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos_device: null array");
  SgArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nmat = nmat;
  a.ncell = ncell;
  a.cell_dim = cell_dim;
  a.neos = neos;
  a.mode = input_int;
  for (int k = 0; k < neos; ++k) {
    if (!pte_model(eos[k].type))
      return set_error(SGX_ERR_UNSUPPORTED, "sgx_get_sg_eos_device: EOS not available in PTE");
    if (const int rc = check_eos_mods(eos[k], precision == SGX_PREC_MIXED, "sgx_get_sg_eos_device"))
      return rc;
    a.eos[k] = eos[k];
  }
  for (int m = 0; m < nmat; ++m) {
    if (eos_offsets[m] < 1 || eos_offsets[m] > neos)
      return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos_device: eos_offsets out of range");
    a.eos_of[m] = eos_offsets[m] - 1;
  }
  a.offsets = offsets;
  a.press = press, a.pmax = pmax, a.vol = vol, a.spvol = spvol, a.sie = sie, a.temp = temp;
  a.bmod = bmod, a.dpde = dpde, a.cv = cv;
  a.frac_mass = frac_mass, a.frac_vol = frac_vol, a.frac_ie = frac_ie;
  a.frac_bmod = frac_bmod, a.frac_dpde = frac_dpde, a.frac_cv = frac_cv;
  a.cutoff = mass_frac_cutoff;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // scratch: PTE arrays and per-cell bookkeeping
  const size_t n = static_cast<size_t>(ncell), nm = n * nmat;
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t bytes = up(4 * nm) * 2 + up(8 * n) * 3 + up(8 * nm) * 5 + up(24 * nm) + up(4 * n);
  void *scratch = nullptr;
  cudaError_t e = scratch_alloc(&scratch, bytes, s);
  if (e != cudaSuccess) return set_error(SGX_ERR_CUDA, "sgx_get_sg_eos_device: scratch allocation");
  char *p = static_cast<char *>(scratch);
  auto take = [&](size_t b) {
    char *q = p;
    p += up(b);
    return q;
  };
  a.eos_idx = reinterpret_cast<int32_t *>(take(4 * nm));
  a.mats = reinterpret_cast<int *>(take(4 * nm));
  a.vfrac_tot = reinterpret_cast<double *>(take(8 * n));
  a.sie_tot = reinterpret_cast<double *>(take(8 * n));
  a.mass_sum = reinterpret_cast<double *>(take(8 * n));
  a.rho = reinterpret_cast<double *>(take(8 * nm));
  a.vfrac = reinterpret_cast<double *>(take(8 * nm));
  a.psie = reinterpret_cast<double *>(take(8 * nm));
  a.ptemp = reinterpret_cast<double *>(take(8 * nm));
  a.ppress = reinterpret_cast<double *>(take(8 * nm));
  a.lambda = reinterpret_cast<double *>(take(24 * nm));
  a.npte = reinterpret_cast<int *>(take(4 * n));
  const int grid = (ncell + SG_BLOCK - 1) / SG_BLOCK;
  sgeos_init<<<grid, SG_BLOCK, 0, s>>>(a);
  e = cudaGetLastError();
  if (e == cudaSuccess && input_int != -1) {
    PteArgs pa;
    std::memset(&pa, 0, sizeof(pa));
    pa.solver = input_int == -3 ? SGX_PTE_FIXED_T
                : input_int == -2 ? SGX_PTE_FIXED_P
                                  : SGX_PTE_RHOT;
    pa.nmat = nmat;
    pa.ncell = ncell;
    pa.neos = neos;
    for (int k = 0; k < neos; ++k)
      pa.eos[k] = eos[k];
    pa.eos_idx = a.eos_idx;
    pa.vfrac_tot = a.vfrac_tot;
    pa.sie_tot = a.sie_tot;
    pa.rho = a.rho, pa.vfrac = a.vfrac, pa.sie = a.psie, pa.temp = a.ptemp;
    pa.press = a.ppress, pa.lambda = a.lambda;
    pa.status = nullptr;
    sgx_mix_params_default(&pa.params);
    e = precision == SGX_PREC_MIXED ? launch_pte_mixed(pa, s) : launch_pte_fp64(pa, s);
  }
  if (e == cudaSuccess) {
    sgeos_final<<<grid, SG_BLOCK, 0, s>>>(a);
    e = cudaGetLastError();
  }
  const cudaError_t f = scratch_free(scratch, s);
  if (e == cudaSuccess) e = f;
  if (e != cudaSuccess)
    return set_error(SGX_ERR_CUDA, std::string("sgx_get_sg_eos_device: ") + cudaGetErrorString(e));
  return SGX_OK;
}

// get_sg_eos over host arrays, as the reference takes them: every array is
// copied to device memory, the device call runs, and every array is copied
// back before the call returns (get_sg_eos.cpp:99-120 and the deep copies at
// its end do the same through Kokkos views). Arguments are checked by the
// device call; the copies use the library's stream-ordered pool.
extern "C" int sgx_get_sg_eos(int nmat, int ncell, int cell_dim, int input_int,
                              const int *eos_offsets, const sgx_eos *eos, int neos,
                              const int *offsets, double *press, double *pmax, double *vol,
                              double *spvol, double *sie, double *temp, double *bmod,
                              double *dpde, double *cv, double *frac_mass, double *frac_vol,
                              double *frac_ie, double *frac_bmod, double *frac_dpde,
                              double *frac_cv, double mass_frac_cutoff, int precision,
                              sgx_stream_t stream) {
  using namespace sgx;
  static const char *who = "sgx_get_sg_eos";
  const int ck = sgeos_check(who, nmat, ncell, cell_dim, input_int, eos_offsets, eos, neos,
                             precision);
  if (ck != SGX_OK || ncell == 0) return ck;
  if (!offsets || !press || !pmax || !vol || !spvol || !sie || !temp || !bmod || !dpde || !cv ||
      !frac_mass || !frac_vol || !frac_ie)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": null array");
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  double *cells[9] = {press, pmax, vol, spvol, sie, temp, bmod, dpde, cv};
  double *fracs[6] = {frac_mass, frac_vol, frac_ie, frac_bmod, frac_dpde, frac_cv};
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  const size_t cb = static_cast<size_t>(cell_dim) * sizeof(double);
  const size_t fb = cb * static_cast<size_t>(nmat);
  const size_t ob = static_cast<size_t>(ncell) * sizeof(int);
  const size_t bytes = up(ob) + 9 * up(cb) + 6 * up(fb);
  void *scratch = nullptr;
  cudaError_t e = scratch_alloc(&scratch, bytes, s);
  if (e != cudaSuccess) return set_error(SGX_ERR_CUDA, std::string(who) + ": device buffers");
  char *p = static_cast<char *>(scratch);
  int *d_off = reinterpret_cast<int *>(p);
  p += up(ob);
  double *d_cells[9], *d_fracs[6];
  for (int k = 0; k < 9; ++k, p += up(cb))
    d_cells[k] = reinterpret_cast<double *>(p);
  for (int k = 0; k < 6; ++k, p += up(fb))
    d_fracs[k] = fracs[k] ? reinterpret_cast<double *>(p) : nullptr;
  e = cudaMemcpyAsync(d_off, offsets, ob, cudaMemcpyHostToDevice, s);
  for (int k = 0; k < 9 && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(d_cells[k], cells[k], cb, cudaMemcpyHostToDevice, s);
  for (int k = 0; k < 6 && e == cudaSuccess; ++k)
    if (fracs[k]) e = cudaMemcpyAsync(d_fracs[k], fracs[k], fb, cudaMemcpyHostToDevice, s);
  int rc = SGX_OK;
  if (e == cudaSuccess) {
    rc = sgx_get_sg_eos_device(nmat, ncell, cell_dim, input_int, eos_offsets, eos, neos, d_off,
                               d_cells[0], d_cells[1], d_cells[2], d_cells[3], d_cells[4],
                               d_cells[5], d_cells[6], d_cells[7], d_cells[8], d_fracs[0],
                               d_fracs[1], d_fracs[2], d_fracs[3], d_fracs[4], d_fracs[5],
                               mass_frac_cutoff, precision, stream);
    for (int k = 0; k < 9 && rc == SGX_OK && e == cudaSuccess; ++k)
      e = cudaMemcpyAsync(cells[k], d_cells[k], cb, cudaMemcpyDeviceToHost, s);
    for (int k = 0; k < 6 && rc == SGX_OK && e == cudaSuccess; ++k)
      if (fracs[k]) e = cudaMemcpyAsync(fracs[k], d_fracs[k], fb, cudaMemcpyDeviceToHost, s);
  }
  const cudaError_t f = scratch_free(scratch, s);
  if (e == cudaSuccess) e = f;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (rc != SGX_OK) return rc;
  if (e != cudaSuccess)
    return set_error(SGX_ERR_CUDA, std::string(who) + ": " + cudaGetErrorString(e));
  return SGX_OK;
}
