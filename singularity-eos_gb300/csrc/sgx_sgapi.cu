// The reference's C interface (eos/singularity_eos.hpp:25-134,
// eos/singularity_eos.cpp) over sgx_eos values: init_sg_eos, the
// init_sg_<model> constructors with their modifier step, the get_sg_*
// vector lookups with a (stride, lambda_data) lambda indexer, and
// finalize_sg_eos. Each keeps the reference's argument list, with an sgx_
// prefix; arrays passed to get_sg_* are device arrays, and the lookups are
// ordered on the legacy default stream as the reference's portableFor runs
// on the default execution space.
#include <cstring>
#include <new>
#include <string>

#include "sgx_internal.h"

namespace {

// init_sg_<model>: the bare model, then the init_sg_* modifier step
// (singularity_eos.cpp:67-79); enabled / vals NULL mean none (def_en, def_v).
int finish_init(const int rc, const int matindex, sgx_eos *eos, sgx_eos &e,
                const int *enabled, double *vals) {
  if (rc != SGX_OK) return rc;
  if (enabled && vals) {
    if (const int r = sgx_eos_apply_modifiers(&e, enabled, vals)) {
      sgx_eos_finalize(&e);
      return r;
    }
  }
  eos[matindex] = e;
  return SGX_OK;
}

int check_slot(const int matindex, const sgx_eos *eos, const char *who) {
  if (!eos) return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": null eos array");
  // the reference asserts matindex >= 0 (singularity_eos.cpp:69)
  if (matindex < 0) return sgx::set_error(SGX_ERR_INVALID, std::string(who) + ": matindex < 0");
  return SGX_OK;
}

// lambdaIndexer2D (singularity_eos.cpp:39-49): rows of `stride` doubles,
// used when stride != -1 and lambda_data is given.
int get_sg(const int fn, const int matindex, const sgx_eos *eos, const double *in1,
           const double *in2, double *out, const int len, const int stride,
           double *lambda_data, const char *who) {
  if (const int rc = check_slot(matindex, eos, who)) return rc;
  const bool lam = stride != -1 && lambda_data != nullptr;
  return sgx_eos_eval(&eos[matindex], fn, len, in1, in2, out, lam ? lambda_data : nullptr,
                      lam ? stride : 0, nullptr);
}

} // namespace

extern "C" {

int sgx_init_sg_eos(int nmat, sgx_eos **eos) {
  if (!eos || nmat < 0) return sgx::set_error(SGX_ERR_INVALID, "sgx_init_sg_eos: bad arguments");
  // init_sg_eos (singularity_eos.cpp:58-65): a host array of nmat EOS
  sgx_eos *p = new (std::nothrow) sgx_eos[nmat > 0 ? nmat : 1];
  if (!p) return sgx::set_error(SGX_ERR_INVALID, "sgx_init_sg_eos: out of host memory");
  std::memset(p, 0, sizeof(sgx_eos) * (nmat > 0 ? nmat : 1));
  *eos = p;
  return SGX_OK;
}

int sgx_init_sg_IdealGas(int matindex, sgx_eos *eos, double gm1, double Cv, const int *enabled,
                         double *vals) {
  if (const int rc = check_slot(matindex, eos, "sgx_init_sg_IdealGas")) return rc;
  sgx_eos e;
  return finish_init(sgx_eos_ideal_gas(&e, gm1, Cv), matindex, eos, e, enabled, vals);
}

int sgx_init_sg_StiffGas(int matindex, sgx_eos *eos, double gm1, double Cv, double Pinf,
                         double qq, const int *enabled, double *vals) {
  if (const int rc = check_slot(matindex, eos, "sgx_init_sg_StiffGas")) return rc;
  sgx_eos e;
  return finish_init(sgx_eos_stiff_gas(&e, gm1, Cv, Pinf, qq), matindex, eos, e, enabled, vals);
}

int sgx_init_sg_NobleAbel(int matindex, sgx_eos *eos, double gm1, double Cv, double bb,
                          double qq, const int *enabled, double *vals) {
  if (const int rc = check_slot(matindex, eos, "sgx_init_sg_NobleAbel")) return rc;
  sgx_eos e;
  return finish_init(sgx_eos_noble_abel(&e, gm1, Cv, bb, qq), matindex, eos, e, enabled, vals);
}

int sgx_init_sg_Gruneisen(int matindex, sgx_eos *eos, double C0, double s1, double s2,
                          double s3, double G0, double b, double rho0, double T0, double P0,
                          double Cv, const int *enabled, double *vals) {
  if (const int rc = check_slot(matindex, eos, "sgx_init_sg_Gruneisen")) return rc;
  sgx_eos e;
  // rho_max from ComputeRhoMax, as Gruneisen's ten-parameter constructor
  return finish_init(sgx_eos_gruneisen(&e, C0, s1, s2, s3, G0, b, rho0, T0, P0, Cv, 0.0),
                     matindex, eos, e, enabled, vals);
}

int sgx_init_sg_SpinerDependsRhoT(int matindex, sgx_eos *eos, const char *filename, int id,
                                  int split, const int *enabled, double *vals) {
  static const char *who = "sgx_init_sg_SpinerDependsRhoT";
  if (const int rc = check_slot(matindex, eos, who)) return rc;
  // TableSplit::Total only (the sp5-lite tables hold the total EOS)
  if (split != 0)
    return sgx::set_error(SGX_ERR_UNSUPPORTED, std::string(who) + ": only TableSplit::Total");
  sgx_eos e;
  return finish_init(sgx_eos_spiner_rhot(&e, filename, id, 0), matindex, eos, e, enabled, vals);
}

int sgx_init_sg_SpinerDependsRhoSie(int matindex, sgx_eos *eos, const char *filename, int id,
                                    int split, const int *enabled, double *vals) {
  static const char *who = "sgx_init_sg_SpinerDependsRhoSie";
  if (const int rc = check_slot(matindex, eos, who)) return rc;
  if (split != 0)
    return sgx::set_error(SGX_ERR_UNSUPPORTED, std::string(who) + ": only TableSplit::Total");
  sgx_eos e;
  return finish_init(sgx_eos_spiner_rhosie(&e, filename, id, 0), matindex, eos, e, enabled,
                     vals);
}

int sgx_init_sg_Helmholtz(int matindex, sgx_eos *eos, const char *filename, int rad, int gas,
                          int coul, int ion, int ele, int verbose, const int *enabled,
                          double *vals) {
  static const char *who = "sgx_init_sg_Helmholtz";
  if (const int rc = check_slot(matindex, eos, who)) return rc;
  (void)verbose;
  const int opts = (rad ? SGX_HELM_RAD : 0) | (gas ? SGX_HELM_GAS : 0) |
                   (coul ? SGX_HELM_COUL : 0) | (ion ? SGX_HELM_ION : 0) |
                   (ele ? SGX_HELM_ELE : 0);
  sgx_eos e;
  return finish_init(sgx_eos_helmholtz(&e, filename, opts), matindex, eos, e, enabled, vals);
}

int sgx_get_sg_EntropyFromDensityInternalEnergy(int matindex, const sgx_eos *eos,
                                                const double *rhos, const double *sies,
                                                double *entropies, int len, int stride,
                                                double *lambda_data) {
  return get_sg(SGX_FN_S_FROM_RHO_SIE, matindex, eos, rhos, sies, entropies, len, stride,
                lambda_data, "sgx_get_sg_EntropyFromDensityInternalEnergy");
}

int sgx_get_sg_PressureFromDensityInternalEnergy(int matindex, const sgx_eos *eos,
                                                 const double *rhos, const double *sies,
                                                 double *pressures, int len, int stride,
                                                 double *lambda_data) {
  return get_sg(SGX_FN_P_FROM_RHO_SIE, matindex, eos, rhos, sies, pressures, len, stride,
                lambda_data, "sgx_get_sg_PressureFromDensityInternalEnergy");
}

int sgx_get_sg_MinInternalEnergyFromDensity(int matindex, const sgx_eos *eos,
                                            const double *rhos, double *sies, int len) {
  return get_sg(SGX_FN_MIN_SIE_FROM_RHO, matindex, eos, rhos, nullptr, sies, len, -1, nullptr,
                "sgx_get_sg_MinInternalEnergyFromDensity");
}

int sgx_get_sg_BulkModulusFromDensityInternalEnergy(int matindex, const sgx_eos *eos,
                                                    const double *rhos, const double *sies,
                                                    double *bmods, int len, int stride,
                                                    double *lambda_data) {
  return get_sg(SGX_FN_B_FROM_RHO_SIE, matindex, eos, rhos, sies, bmods, len, stride,
                lambda_data, "sgx_get_sg_BulkModulusFromDensityInternalEnergy");
}

int sgx_finalize_sg_eos(int nmat, sgx_eos **eos) {
  if (!eos) return sgx::set_error(SGX_ERR_INVALID, "sgx_finalize_sg_eos: null");
  // finalize_sg_eos (singularity_eos.cpp:430-444): release every EOS's
  // device memory, then the array
  if (*eos) {
    for (int k = 0; k < nmat; ++k)
      sgx_eos_finalize(&(*eos)[k]);
    delete[] * eos;
    *eos = nullptr;
  }
  return SGX_OK;
}

} // extern "C"
