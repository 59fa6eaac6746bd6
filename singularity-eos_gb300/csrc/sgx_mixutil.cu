// Per-cell utilities of the closure layer, one thread per cell:
//
//   approx_temperature_kernel   ApproxTemperatureFromRhoMatU
//                               (closure/mixed_cell_models.hpp:790-847)
//   enforce_volumes_kernel      MixUtils::EnforceMassVolumesSum (:93-117)
//   enforce_energies_kernel     MixUtils::EnforceEnergiesSum (:119-150)
//
// Materials are the cell's present slots in slot order (eos_idx >= 0, or
// every slot when there is no index map), which is the material list the
// reference functions receive. Compiled with --fmad=false: the same
// roundings as the reference built without contraction.
#include <cstring>

#include <cuda_runtime.h>

#include "sgx_dispatch.cuh"
#include "sgx_internal.h"

namespace sgx {

namespace {

constexpr int MU_BLOCK = 128;

struct MixUtilArgs {
  int nmat;
  long long ncell;
  int neos;
  sgx_eos eos[MAX_EOS];
  const int32_t *eos_idx;
  const double *u_tot, *Tguess, *tot_vol, *tot_rho, *tot_sie;
  double *rho, *vfrac, *sie, *lambda, *temp_out;
};

// present material slots of cell i and their EOS indices
__device__ int mu_gather(const MixUtilArgs &a, long long i, int (&slot)[MAX_NMAT],
                         int (&eidx)[MAX_NMAT]) {
  int n = 0;
  for (int m = 0; m < a.nmat; ++m) {
    const int ie = a.eos_idx ? a.eos_idx[m * a.ncell + i] : m;
    if (ie < 0 || ie >= a.neos) continue;
    slot[n] = m;
    eidx[n] = ie;
    ++n;
  }
  return n;
}

__global__ void __launch_bounds__(MU_BLOCK) approx_temperature_kernel(const MixUtilArgs a) {
  __shared__ sgx_eos s_eos[MAX_EOS];
  for (int k = threadIdx.x; k < a.neos; k += blockDim.x)
    s_eos[k] = a.eos[k];
  __syncthreads();
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.ncell) return;
  int slot[MAX_NMAT], eidx[MAX_NMAT];
  const int n = mu_gather(a, i, slot, eidx);
  const long long nc = a.ncell;
  double rho[MAX_NMAT], vfrac[MAX_NMAT], cache[MAX_NMAT][3];
  for (int q = 0; q < n; ++q) {
    const long long k = slot[q] * nc + i;
    rho[q] = a.rho[k];
    vfrac[q] = a.vfrac[k];
    for (int l = 0; l < 3; ++l)
      cache[q][l] = a.lambda ? a.lambda[(slot[q] * 3LL + l) * nc + i] : 0.0;
  }
  const double u_tot = a.u_tot[i];
  const double Tguess = a.Tguess ? a.Tguess[i] : 0.0;
  auto ufunc = [&](const double T) {
    double usum = 0.0;
    for (int q = 0; q < n; q++)
      usum += rho[q] * vfrac[q] * ev_sie_from_rho_T<double>(s_eos[eidx[q]], rho[q], T, cache[q]);
    return usum;
  };
  constexpr double minimum_temperature = 1.e-9;
  constexpr double maximum_temperature = 1.e9;
  double T;
  double ulo = ufunc(minimum_temperature);
  if (u_tot < ulo) {
    T = minimum_temperature;
  } else {
    double uhi = ufunc(maximum_temperature);
    if (u_tot > uhi) {
      T = maximum_temperature;
    } else {
      double lTlo = lg_nqt(minimum_temperature);
      double lThi = lg_nqt(maximum_temperature);
      if (Tguess > minimum_temperature && Tguess < maximum_temperature) {
        const double ug = ufunc(Tguess);
        if (ug < u_tot) {
          lTlo = lg_nqt(Tguess);
          ulo = ug;
        } else {
          lThi = lg_nqt(Tguess);
          uhi = ug;
        }
      }
      int iter = 0;
      constexpr int max_iter = 10;
      while (lThi - lTlo > 0.01 && iter < max_iter) {
        const double lT = 0.5 * (lTlo + lThi);
        const double uT = ufunc(pow2_nqt(lT));
        if (uT < u_tot) {
          lTlo = lT;
          ulo = uT;
        } else {
          lThi = lT;
          uhi = uT;
        }
        iter++;
      }
      const double alpha = ratio((u_tot - ulo), (uhi - ulo));
      T = pow2_nqt((1.0 - alpha) * lTlo + alpha * lThi);
    }
  }
  a.temp_out[i] = T;
  if (a.lambda)
    for (int q = 0; q < n; ++q)
      for (int l = 0; l < 3; ++l)
        a.lambda[(slot[q] * 3LL + l) * nc + i] = cache[q][l];
}

__global__ void __launch_bounds__(MU_BLOCK) enforce_volumes_kernel(const MixUtilArgs a) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.ncell) return;
  int slot[MAX_NMAT], eidx[MAX_NMAT];
  const int n = mu_gather(a, i, slot, eidx);
  if (n == 0) return;
  const long long nc = a.ncell;
  int imax = 0;
  double fmax = -1;
  for (int q = 0; q < n; ++q) {
    const double v = a.vfrac[slot[q] * nc + i];
    if (v > fmax) {
      fmax = v;
      imax = q;
    }
  }
  double vfrac_new = a.tot_vol[i];
  for (int q = 0; q < n; ++q) {
    if (q == imax) continue;
    vfrac_new -= a.vfrac[slot[q] * nc + i];
  }
  const long long k = slot[imax] * nc + i;
  a.rho[k] *= ratio(a.vfrac[k], vfrac_new);
  a.vfrac[k] = vfrac_new;
}

__global__ void __launch_bounds__(MU_BLOCK) enforce_energies_kernel(const MixUtilArgs a) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.ncell) return;
  int slot[MAX_NMAT], eidx[MAX_NMAT];
  const int n = mu_gather(a, i, slot, eidx);
  if (n == 0) return;
  const long long nc = a.ncell;
  const double tot_u = a.tot_sie[i] * a.tot_rho[i];
  int imax = 0;
  double max_contribution = 0;
  for (int q = 0; q < n; ++q) {
    const long long k = slot[q] * nc + i;
    const double um = a.rho[k] * a.vfrac[k] * a.sie[k];
    if (sabs(um) > max_contribution) {
      imax = q;
      max_contribution = sabs(um);
    }
  }
  double unew = tot_u;
  for (int q = 0; q < n; ++q) {
    if (q == imax) continue;
    const long long k = slot[q] * nc + i;
    unew -= a.rho[k] * a.vfrac[k] * a.sie[k];
  }
  const long long k = slot[imax] * nc + i;
  a.sie[k] = ratio(unew, a.rho[k] * a.vfrac[k]);
}

int check_common(const char *who, int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                 const int32_t *eos_idx, bool need_eos) {
  if (nmat < 1 || nmat > MAX_NMAT)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": nmat must be in 1..8");
  if (ncell < 0) return set_error(SGX_ERR_INVALID, std::string(who) + ": ncell < 0");
  if (need_eos) {
    if (!eos_list || neos < 1 || neos > MAX_EOS)
      return set_error(SGX_ERR_INVALID, std::string(who) + ": neos must be in 1..16");
    if (!eos_idx && neos < nmat)
      return set_error(SGX_ERR_INVALID, std::string(who) + ": eos_idx NULL needs neos >= nmat");
    for (int k = 0; k < neos; ++k)
      if (!pte_model(eos_list[k].type))
        return set_error(SGX_ERR_UNSUPPORTED, std::string(who) + ": EOS type not available");
  }
  return SGX_OK;
}

int launch(const char *who, void (*kern)(MixUtilArgs), const MixUtilArgs &a,
           sgx_stream_t stream) {
  const long long blocks = (a.ncell + MU_BLOCK - 1) / MU_BLOCK;
  kern<<<static_cast<unsigned>(blocks), MU_BLOCK, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_error(SGX_ERR_CUDA, std::string(who) + ": " + cudaGetErrorString(e));
  return SGX_OK;
}

} // namespace

} // namespace sgx

extern "C" int sgx_pte_approx_temperature(int nmat, int64_t ncell, const sgx_eos *eos_list,
                                          int neos, const int32_t *eos_idx,
                                          const double *u_tot, const double *rho,
                                          const double *vfrac, const double *Tguess,
                                          double *lambda, double *temp_out,
                                          sgx_stream_t stream) {
  using namespace sgx;
  const char *who = "sgx_pte_approx_temperature";
  int rc = check_common(who, nmat, ncell, eos_list, neos, eos_idx, true);
  if (rc != SGX_OK) return rc;
  if (ncell == 0) return SGX_OK;
  if (!u_tot || !rho || !vfrac || !temp_out)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": null array");
  MixUtilArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nmat = nmat, a.ncell = ncell, a.neos = neos;
  for (int k = 0; k < neos; ++k)
    a.eos[k] = eos_list[k];
  a.eos_idx = eos_idx, a.u_tot = u_tot, a.Tguess = Tguess;
  a.rho = const_cast<double *>(rho), a.vfrac = const_cast<double *>(vfrac);
  a.lambda = lambda, a.temp_out = temp_out;
  return launch(who, approx_temperature_kernel, a, stream);
}

extern "C" int sgx_mix_enforce_mass_volumes_sum(int nmat, int64_t ncell, const int32_t *eos_idx,
                                                const double *tot_vol, double *rho,
                                                double *vfrac, sgx_stream_t stream) {
  using namespace sgx;
  const char *who = "sgx_mix_enforce_mass_volumes_sum";
  int rc = check_common(who, nmat, ncell, nullptr, 0, eos_idx, false);
  if (rc != SGX_OK) return rc;
  if (ncell == 0) return SGX_OK;
  if (!tot_vol || !rho || !vfrac)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": null array");
  MixUtilArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nmat = nmat, a.ncell = ncell, a.neos = 1 << 30; // presence only
  a.eos_idx = eos_idx, a.tot_vol = tot_vol, a.rho = rho, a.vfrac = vfrac;
  return launch(who, enforce_volumes_kernel, a, stream);
}

extern "C" int sgx_mix_enforce_energies_sum(int nmat, int64_t ncell, const int32_t *eos_idx,
                                            const double *tot_rho, const double *tot_sie,
                                            const double *rho, const double *vfrac, double *sie,
                                            sgx_stream_t stream) {
  using namespace sgx;
  const char *who = "sgx_mix_enforce_energies_sum";
  int rc = check_common(who, nmat, ncell, nullptr, 0, eos_idx, false);
  if (rc != SGX_OK) return rc;
  if (ncell == 0) return SGX_OK;
  if (!tot_rho || !tot_sie || !rho || !vfrac || !sie)
    return set_error(SGX_ERR_INVALID, std::string(who) + ": null array");
  MixUtilArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nmat = nmat, a.ncell = ncell, a.neos = 1 << 30; // presence only
  a.eos_idx = eos_idx, a.tot_rho = tot_rho, a.tot_sie = tot_sie;
  a.rho = const_cast<double *>(rho), a.vfrac = const_cast<double *>(vfrac), a.sie = sie;
  return launch(who, enforce_energies_kernel, a, stream);
}
