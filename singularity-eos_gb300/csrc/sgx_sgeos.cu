// get_sg_eos in its (rho, sie) input modes (singularity-eos
// eos/get_sg_eos.cpp:35-280, get_sg_eos_rho_e.cpp:30-88): per cell, the mass
// fractions are normalised, the materials above the mass-fraction cutoff take
// part in a PTESolverRhoT solve (or, alone, a T(rho, sie) and P(rho, T)
// lookup), and the cell's pressure, temperature, bulk modulus, heat capacity
// and dP/de are formed from the material states (get_sg_eos_functors.hpp).
//
// Three stages on one stream: sgeos_init packs each cell's participating
// materials into the [slot][cell] arrays of the PTE kernels (init_functor,
// :28-118), the PTE kernels of sgx_pte_solve run on them (cells with fewer
// than two participating materials carry no material and are skipped), and
// sgeos_final does the pure-cell lookups and the averages (final_functor,
// :185-300). Per-cell arrays are [cell_dim]; per-material arrays are
// LayoutLeft [nmat][cell_dim] (element (i, m) at i + m * cell_dim); offsets
// are the reference's 1-based cell indices.
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

__global__ void __launch_bounds__(SG_BLOCK) sgeos_init(const SgArgs a) {
  const int iloop = blockIdx.x * blockDim.x + threadIdx.x;
  if (iloop >= a.ncell) return;
  const long long nc = a.ncell, cd = a.cell_dim;
  const int i = a.offsets[iloop] - 1;
  double mass_sum = 0.0;
  for (int m = 0; m < a.nmat; ++m) {
    const double fm = a.frac_mass[i + m * cd];
    mass_sum += fm;
    a.frac_vol[i + m * cd] = fm;
    a.frac_ie[i + m * cd] = a.sie[i] * fm * 1.0;
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
      a.ptemp[k] = a.temp[i] * EV2K * 0.0;
      a.ppress[k] = a.press[i] * 0.0;
      a.psie[k] = a.sie[i] * fm * 1.0;
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
  a.sie_tot[iloop] = a.sie[i];
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
  if (npte == 1) {
    // pure cell (get_sg_eos_rho_e.cpp:76-83)
    const sgx_eos &e = s_eos[a.eos_of[a.mats[iloop]]];
    const double r = a.rho[iloop];
    const double t = ev_T_from_rho_sie<double>(e, r, a.psie[iloop], cache[0]);
    a.ptemp[iloop] = t;
    a.ppress[iloop] = ev_P_from_rho_T<double>(e, r, t, cache[0]);
  }
  double press = 0.0, temp = 0.0, bmod = 0.0, cv = 0.0, dpde = 0.0, sie = a.sie[i];
  for (int mp = 0; mp < npte; ++mp) {
    const long long k = mp * nc + iloop;
    const int m = a.mats[k];
    const double vf = a.vfrac[k], r = a.rho[k], t = a.ptemp[k];
    const double fm = a.frac_mass[i + m * cd];
    press += a.ppress[k] * vf * 1.0;
    temp += t * vf * 1.0;
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
  a.temp[i] = temp / EV2K;
  a.sie[i] = sie;
  a.bmod[i] = bmod;
  a.cv[i] = cv;
  a.dpde[i] = dpde;
  for (int m = 0; m < a.nmat; ++m)
    a.frac_mass[i + m * cd] *= mass_sum;
  a.pmax[i] = press > a.pmax[i] ? press : a.pmax[i];
}

} // namespace

} // namespace sgx

extern "C" int sgx_get_sg_eos(int nmat, int ncell, int cell_dim, int input_int,
                              const int *eos_offsets, const sgx_eos *eos, int neos,
                              const int *offsets, double *press, double *pmax, double *vol,
                              double *spvol, double *sie, double *temp, double *bmod,
                              double *dpde, double *cv, double *frac_mass, double *frac_vol,
                              double *frac_ie, double *frac_bmod, double *frac_dpde,
                              double *frac_cv, double mass_frac_cutoff, int precision,
                              sgx_stream_t stream) {
  using namespace sgx;
  if (input_int == -3 || input_int == -2 || input_int == -1)
    return set_error(SGX_ERR_UNSUPPORTED, "sgx_get_sg_eos: only the (rho, sie) input modes "
                                          "0 and 1 are available");
  if (input_int != 0 && input_int != 1)
    return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos: bad input_int");
  if (nmat < 1 || nmat > PTE_MAX_N)
    return set_error(SGX_ERR_UNSUPPORTED, "sgx_get_sg_eos: nmat must be in 1..6");
  if (ncell < 0 || cell_dim < ncell)
    return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos: need 0 <= ncell <= cell_dim");
  if (ncell == 0) return SGX_OK;
  if (!eos || neos < 1 || neos > MAX_EOS || !eos_offsets)
    return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos: eos list / offsets");
  if (precision != SGX_PREC_FP64 && precision != SGX_PREC_MIXED)
    return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos: bad precision");
  if (!offsets || !press || !pmax || !vol || !spvol || !sie || !temp || !bmod || !dpde || !cv ||
      !frac_mass || !frac_vol || !frac_ie)
    return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos: null array");
  SgArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nmat = nmat;
  a.ncell = ncell;
  a.cell_dim = cell_dim;
  a.neos = neos;
  for (int k = 0; k < neos; ++k) {
    if (eos[k].type < SGX_IDEAL_GAS || eos[k].type > SGX_SPINER_RHOT)
      return set_error(SGX_ERR_UNSUPPORTED, "sgx_get_sg_eos: EOS not available in PTE");
    a.eos[k] = eos[k];
  }
  for (int m = 0; m < nmat; ++m) {
    if (eos_offsets[m] < 1 || eos_offsets[m] > neos)
      return set_error(SGX_ERR_INVALID, "sgx_get_sg_eos: eos_offsets out of range");
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
  cudaError_t e = cudaMallocAsync(&scratch, bytes, s);
  if (e != cudaSuccess) return set_error(SGX_ERR_CUDA, "sgx_get_sg_eos: scratch allocation");
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
  if (e == cudaSuccess) {
    PteArgs pa;
    std::memset(&pa, 0, sizeof(pa));
    pa.solver = SGX_PTE_RHOT;
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
  const cudaError_t f = cudaFreeAsync(scratch, s);
  if (e == cudaSuccess) e = f;
  if (e != cudaSuccess)
    return set_error(SGX_ERR_CUDA, std::string("sgx_get_sg_eos: ") + cudaGetErrorString(e));
  return SGX_OK;
}
