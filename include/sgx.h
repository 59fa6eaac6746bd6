/*
 * sgx.h -- C ABI of the GB300 closure library (libsgx.so).
 *
 * A drop-in for singularity-eos's data-parallel closure path: the vector EOS
 * lookups and the per-cell pressure-temperature-equilibrium (PTE) solve.
 * Every entry point takes plain pointers and sizes. Arrays passed to the
 * sgx_* compute calls live in device memory unless the name says _host; the
 * call is stream-ordered on the given CUDA stream (NULL = legacy default
 * stream) and returns an sgx_status code. Nothing here aborts the process.
 *
 * Reference interfaces replaced (paths inside lanl/singularity-eos):
 *   sgx_eos_*            constructors of IdealGas/StiffGas/NobleAbel/
 *                        Gruneisen/SpinerEOSDependsRhoT/Helmholtz
 *                        (eos/eos_ideal.hpp:41, eos_stiff.hpp:40,
 *                        eos_noble_abel.hpp:40, eos_gruneisen.hpp:62,
 *                        eos_spiner_rho_temp.hpp:85, eos_helmholtz.hpp:446)
 *                        plus GetOnDevice()/Finalize() (eos_variant.hpp:183-186,
 *                        865-867)
 *   sgx_eos_eval         the vector overloads generated by SG_EOS_VEC_2IN_1OUT
 *                        (eos/eos_base.hpp:169-230) and forwarded by Variant
 *                        (eos/eos_variant.hpp:56-143), including
 *                        MinInternalEnergyFromDensity (eos_base.hpp:428-494)
 *   sgx_eos_fill         vector FillEos (eos/eos_base.hpp:503-531)
 *   sgx_pte_solve        a per-cell loop of PTESolverRhoT / PTESolverPT driven
 *                        by PTESolver() (closure/mixed_cell_models.hpp:884-1193,
 *                        1207-1446, 2188-2291), as get_sg_eos_rho_e.cpp:30-88
 *                        runs it
 *   sgx_mix_params_default  MixParams defaults (mixed_cell_models.hpp:43-78)
 *   sgx_pte_rhot_required_scratch  PTESolverRhoTRequiredScratch (:873-881)
 *   sgx_pte_pt_required_scratch    PTESolverPTRequiredScratch (:1198-1206)
 *   sgx_eos_modify_*     ShiftedEOS / ScaledEOS / BilinearRampEOS around a
 *                        model (eos/modifiers/), as Variant::Modify builds them
 *   sgx_eos_apply_modifiers  the modifier step of init_sg_*
 *                        (eos/singularity_eos.cpp:67-79)
 */
#ifndef SGX_H_
#define SGX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* cudaStream_t without including the CUDA runtime headers. */
typedef struct CUstream_st *sgx_stream_t;

typedef enum sgx_status {
  SGX_OK = 0,
  SGX_ERR_INVALID = 1,   /* bad argument (null pointer, bad size, bad type) */
  SGX_ERR_CUDA = 2,      /* a CUDA runtime call failed; see sgx_last_error() */
  SGX_ERR_NO_DEVICE = 3, /* no CUDA device visible */
  SGX_ERR_IO = 4,        /* a table file could not be read */
  SGX_ERR_UNSUPPORTED = 5, /* combination not implemented (e.g. nmat > 8) */
  SGX_ERR_TIMEOUT = 6    /* a bounded device wait ran out */
} sgx_status;

/* EOS model codes. */
enum {
  SGX_IDEAL_GAS = 1,
  SGX_STIFF_GAS = 2,
  SGX_NOBLE_ABEL = 3,
  SGX_GRUNEISEN = 4,
  SGX_SPINER_RHOT = 5,
  SGX_HELMHOLTZ = 6,
  SGX_SPINER_RHOSIE = 7
};

/* thermalqs bits (singularity-eos/base/constants.hpp:22-34). */
enum {
  SGX_Q_DENSITY = 1,
  SGX_Q_SIE = 2,
  SGX_Q_PRESSURE = 4,
  SGX_Q_TEMPERATURE = 8,
  SGX_Q_SPECIFIC_HEAT = 16,
  SGX_Q_BULK_MODULUS = 32
};

/* Vector lookup selectors for sgx_eos_eval (the EosBase vector members). */
enum {
  SGX_FN_T_FROM_RHO_SIE = 0,  /* TemperatureFromDensityInternalEnergy */
  SGX_FN_SIE_FROM_RHO_T = 1,  /* InternalEnergyFromDensityTemperature */
  SGX_FN_P_FROM_RHO_T = 2,    /* PressureFromDensityTemperature */
  SGX_FN_P_FROM_RHO_SIE = 3,  /* PressureFromDensityInternalEnergy */
  SGX_FN_CV_FROM_RHO_T = 4,   /* SpecificHeatFromDensityTemperature */
  SGX_FN_CV_FROM_RHO_SIE = 5, /* SpecificHeatFromDensityInternalEnergy */
  SGX_FN_B_FROM_RHO_T = 6,    /* BulkModulusFromDensityTemperature */
  SGX_FN_B_FROM_RHO_SIE = 7,  /* BulkModulusFromDensityInternalEnergy */
  SGX_FN_G_FROM_RHO_T = 8,    /* GruneisenParamFromDensityTemperature */
  SGX_FN_G_FROM_RHO_SIE = 9,  /* GruneisenParamFromDensityInternalEnergy */
  SGX_FN_MIN_SIE_FROM_RHO = 10, /* MinInternalEnergyFromDensity (in2 unused) */
  SGX_FN_S_FROM_RHO_T = 11,     /* EntropyFromDensityTemperature */
  SGX_FN_S_FROM_RHO_SIE = 12,   /* EntropyFromDensityInternalEnergy */
  SGX_FN_SIE_FROM_RHO_P = 13    /* InternalEnergyFromDensityPressure (in2 = P) */
};
/* Entropy exists for IdealGas, StiffGas and NobleAbel (and their modified
 * forms); Gruneisen and the tabulated model abort in the reference
 * (EntropyIsNotEnabled) and return SGX_ERR_UNSUPPORTED here. Helmholtz takes
 * functions 0..9. */

/* Modifier bits of sgx_eos.mods (eos/modifiers/). The reference's EOS
 * variant holds a model, Shifted<model>, Scaled<model>,
 * Scaled<Shifted<model>> and BilinearRamp<any of these>
 * (eos/eos_type_lists.hpp:80-96), so the wrappers always nest as
 * BilinearRamp(Scaled(Shifted(model))), outermost first. */
enum {
  SGX_MOD_SHIFTED = 1, /* ShiftedEOS (eos/modifiers/shifted_eos.hpp) */
  SGX_MOD_SCALED = 2,  /* ScaledEOS (eos/modifiers/scaled_eos.hpp) */
  SGX_MOD_RAMP = 4     /* BilinearRampEOS (eos/modifiers/ramps_eos.hpp) */
};

/* One EOS instance: a 208-byte trivially copyable value (the analogue of the
 * reference's GetOnDevice() copy). Analytic models keep their parameters in
 * p[]; tabulated models also hold a device table owned by the library, freed
 * by sgx_eos_finalize. Modifiers are set by sgx_eos_modify_* and
 * sgx_eos_apply_modifiers. */
typedef struct sgx_eos {
  int32_t type;  /* SGX_* model code */
  int32_t flags; /* model options (Spiner: bit0 reproducibility mode;
                    Helmholtz: bits 0-4 rad, gas, coul, ion, ele) */
  uint64_t table; /* device address of the table image, 0 if analytic */
  double p[14];  /* parameters, per model:
                    IdealGas:  gm1, Cv
                    StiffGas:  gm1, Cv, Pinf, qq
                    NobleAbel: gm1, Cv, bb, qq
                    Gruneisen: C0, s1, s2, s3, G0, b, rho0, T0, P0, Cv, rho_max */
  uint32_t mods;     /* SGX_MOD_* bits; 0 for a bare model */
  uint32_t mods_reserved;
  double shift;      /* ShiftedEOS shift_ */
  double scale;      /* ScaledEOS scale_ */
  double inv_scale;  /* ScaledEOS inv_scale_ = 1 / scale_ */
  double ramp[6];    /* BilinearRampEOS r0_, a_, b_, c_, rmid_, Pmid_ */
} sgx_eos;

/* Field-for-field singularity::MixParams (mixed_cell_models.hpp:43-78). */
typedef struct sgx_mix_params {
  int32_t verbose;
  int32_t iterate_t_guess;
  double derivative_eps;
  double pte_rel_tolerance_p, pte_rel_tolerance_t, pte_rel_tolerance_e;
  double pte_rel_tolerance_v, pte_abs_tolerance_p, pte_abs_tolerance_t;
  double pte_slow_convergence_thresh;
  double pte_rel_tolerance_p_sufficient, pte_rel_tolerance_t_sufficient;
  double pte_rel_tolerance_e_sufficient, pte_rel_tolerance_v_sufficient;
  double pte_abs_tolerance_p_sufficient, pte_abs_tolerance_t_sufficient;
  int64_t pte_max_iter_per_mat;
  double line_search_alpha;
  int64_t line_search_max_iter;
  double line_search_fac;
  double vfrac_safety_fac;
  double temperature_limit;
  double default_tguess;
  double min_dtde;
  int64_t pte_small_step_tries;
  double pte_small_step_thresh;
  double pte_max_dpdv;
  int64_t pte_reduced_system_exclude_idx;
} sgx_mix_params;

/* Per-cell result of a PTE solve (the reference's SolverStatus,
 * mixed_cell_models.hpp:80-87, plus the iteration count). small_step_iters
 * holds the count in bits 0-5; bit 6 is set when the mixed-precision path
 * re-solved the cell with the FP64 iteration; bit 7 when a path that aborts
 * in the reference (e.g. a failed Gruneisen root find) was taken. */
typedef struct sgx_pte_status {
  double residual;
  int32_t niter;
  uint8_t converged;
  uint8_t slow_convergence_detected;
  uint8_t max_line_niter;
  uint8_t small_step_iters;
} sgx_pte_status;

/* PTE solvers (closure/mixed_cell_models.hpp):
 *  SGX_PTE_RHOT     PTESolverRhoT   :884-1193, unknowns T and n-1 volume fractions
 *  SGX_PTE_PT       PTESolverPT     :1207-1446, unknowns T and P
 *  SGX_PTE_RHOU     PTESolverRhoU   :1934-2183, unknowns n volume fractions and
 *                                   n energy densities
 *  SGX_PTE_FIXED_T  PTESolverFixedT :1462-1660, volume fractions at a given T
 *  SGX_PTE_FIXED_P  PTESolverFixedP :1676-1919, volume fractions and T at a given P */
enum {
  SGX_PTE_RHOT = 0,
  SGX_PTE_PT = 1,
  SGX_PTE_RHOU = 2,
  SGX_PTE_FIXED_T = 3,
  SGX_PTE_FIXED_P = 4
};

/* Precision of the PTE / lookup arithmetic.
 * SGX_PREC_FP64: the plain path; follows the reference's iteration exactly.
 * SGX_PREC_MIXED: the PTE's Newton iteration in FP32 followed by FP64
 *   residual correction to 1e-12 (cells it cannot finish take the FP64
 *   iteration); the tabulated lookups in float-float; the Helmholtz
 *   inversion from an FP32 phase (sgx_eos_fill_ex). */
enum { SGX_PREC_FP64 = 0, SGX_PREC_MIXED = 1 };

const char *sgx_version(void);
/* Message of the last failing call on this host thread. */
const char *sgx_last_error(void);

/* ---- EOS construction ---- */
int sgx_eos_ideal_gas(sgx_eos *out, double gm1, double Cv);
int sgx_eos_stiff_gas(sgx_eos *out, double gm1, double Cv, double Pinf, double qq);
int sgx_eos_noble_abel(sgx_eos *out, double gm1, double Cv, double bb, double qq);
/* The constructors with a reference state: IdealGas(gm1, Cv, EntropyT0,
 * EntropyRho0) (eos_ideal.hpp:49-56) and StiffGas / NobleAbel(..., qp, T0,
 * P0) (eos_stiff.hpp:52-59, eos_noble_abel.hpp:52-60). The reference state
 * enters the entropy and ValuesAtReferenceState only; the short forms above
 * use STP (293 K, 1e6) and qp = 0, as the reference's do. */
int sgx_eos_ideal_gas_entropy(sgx_eos *out, double gm1, double Cv, double EntropyT0,
                              double EntropyRho0);
int sgx_eos_stiff_gas_ref(sgx_eos *out, double gm1, double Cv, double Pinf, double qq,
                          double qp, double T0, double P0);
int sgx_eos_noble_abel_ref(sgx_eos *out, double gm1, double Cv, double bb, double qq,
                           double qp, double T0, double P0);
/* rho_max <= 0 computes it from the Us-up polynomial
 * (Gruneisen::ComputeRhoMax, eos_gruneisen.hpp:231-329). */
int sgx_eos_gruneisen(sgx_eos *out, double C0, double s1, double s2, double s3,
                      double G0, double b, double rho0, double T0, double P0, double Cv,
                      double rho_max);
/* Loads a tabulated rho-T EOS from an sp5-lite image, derives the load-time
 * tables (SpinerEOSDependsRhoT::loadDataboxes_, eos_spiner_rho_temp.hpp:545-687)
 * and makes the table resident on the current device. */
int sgx_eos_spiner_rhot(sgx_eos *out, const char *path, int matid, int reproducible);
/* Loads a tabulated EOS on rho-T and rho-sie grids (SpinerEOSDependsRhoSie
 * with the default NullTransform, eos_spiner_rho_sie.hpp:80-1052) from an
 * sp5-lite image: /<matid>/dependsLogRhoLogT, /<matid>/dependsLogRhoLogSie
 * and /<matid>/coldCurve, with the bulk moduli recomputed and the
 * minimum-pressure tables derived as loadDataboxes_ (:433-552) does, and
 * makes the table resident on the current device. Functions of (rho, sie)
 * interpolate the rho-sie grid directly (no root find); lambda rows carry
 * one entry, log10(rho). TableSplit::Total only; no mass fractions. */
int sgx_eos_spiner_rhosie(sgx_eos *out, const char *path, int matid, int reproducible);
/* Option bits of sgx_eos_helmholtz (Helmholtz::Options, eos_helmholtz.hpp:420-441). */
enum {
  SGX_HELM_RAD = 1,            /* ENABLE_RAD */
  SGX_HELM_GAS = 2,            /* ENABLE_GAS */
  SGX_HELM_COUL = 4,           /* ENABLE_COULOMB_CORRECTIONS */
  SGX_HELM_ION = 8,            /* GAS_IONIZED */
  SGX_HELM_ELE = 16,           /* GAS_DEGENERATE */
  SGX_HELM_DEFAULT = 31,       /* the reference's defaults: all of the above */
  SGX_HELM_REGULA_FALSI = 32,  /* USE_NEWTON_RAPHSON = false */
  SGX_HELM_CACHE_READBACK = 64 /* reproduce the reference's lT cache read-back (below) */
};
/* Loads the electron free-energy table of the Helmholtz EOS from a file in
 * the reference's helm_table.dat layout (HelmElectrons::InitDataFile_,
 * eos_helmholtz.hpp:962-989) and makes it resident on the current device;
 * replaces Helmholtz(filename, options) + GetOnDevice(). Abar, Zbar and the
 * log10 T cache come in per element through lambda rows [Abar, Zbar, lT]
 * (Helmholtz::Lambda, :409-416), so every lookup needs lambda (stride >= 3).
 * T(rho, sie) stores the root in the lT cache. The reference ends
 * lTFromRhoSie_ (:957) by reading the cache back over the root, which with a
 * plain array lambda returns the guess instead of the root;
 * SGX_HELM_CACHE_READBACK reproduces that. */
int sgx_eos_helmholtz(sgx_eos *out, const char *path, int options);
/* Node values and fields of a Helmholtz table in the reference's DBLIST order
 * (rho_, T_, f_ .. xfdt_; eos_helmholtz.hpp:281-292); returns the count or -1. */
long sgx_eos_helmholtz_dump(const sgx_eos *eos, double *out, long cap);
/* ---- Modifiers (eos/modifiers/) ----
 * Each wraps *eos in place, as eos.Modify<W>(args) does in the reference
 * (eos_variant.hpp:213-223), and checks the wrapper's CheckParams. Only the nestings
 * the reference's variant holds are accepted: Shifted of a bare model,
 * Scaled of a bare or shifted model, BilinearRamp of any of those
 * (SGX_ERR_UNSUPPORTED otherwise, and for Helmholtz). Modified EOS run on
 * the FP64 paths; the mixed-precision paths return SGX_ERR_UNSUPPORTED. */
/* ShiftedEOS(t, shift) (shifted_eos.hpp:53-61): shift must be a number. */
int sgx_eos_modify_shifted(sgx_eos *eos, double shift);
/* ScaledEOS(t, scale) (scaled_eos.hpp:53-66): scale and 1/scale nonzero
 * and numbers. */
int sgx_eos_modify_scaled(sgx_eos *eos, double scale);
/* BilinearRampEOS(t, r0, a, b, c) (ramps_eos.hpp:86-104): r0 > 0, a > 0,
 * b >= 0, a != b; rmid = r0 (a - b c) / (a - b) and Pmid = a (rmid/r0 - 1)
 * must be numbers. */
int sgx_eos_modify_bilinear_ramp(sgx_eos *eos, double r0, double a, double b, double c);
/* pAlpha2BilinearRampParams (ramps_eos.hpp:43-77): the ramp through the
 * p-alpha crush curve of *eos (alpha0 > 1, elastic limit Pe, full
 * compaction Pc) from its reference state and two root finds of
 * P(alpha0 rho, T0) = Pe and P(rho, T0) = Pc. The root finds run on the
 * current device (tabulated models need their table there). */
int sgx_eos_p_alpha_ramp_params(const sgx_eos *eos, double alpha0, double Pe, double Pc,
                                double *r0, double *a, double *b, double *c);
/* The modifier step of the reference's init_sg_* functions
 * (singularity_eos.cpp:67-79 and the SGAPPLYMOD macros of
 * singularity_eos_init_utils.hpp): enabled[0] scaled by vals[0],
 * enabled[1] shifted by vals[1], enabled[2] a bilinear ramp with
 * (r0, a, b, c) = vals[2..5], enabled[3] a ramp whose parameters come from
 * sgx_eos_p_alpha_ramp_params(alpha0, Pe, Pc = vals[2..4]) of the shifted
 * and scaled EOS and are written back into vals[2..5], as the reference
 * does. Entries equal to 1 enable; *eos must be a bare model. */
int sgx_eos_apply_modifiers(sgx_eos *eos, const int enabled[4], double vals[6]);

/* Releases a tabulated EOS's device table (no-op for analytic models). */
int sgx_eos_finalize(sgx_eos *eos);
/* Size in bytes of the device table behind a tabulated EOS (0 if analytic). */
size_t sgx_eos_table_bytes(const sgx_eos *eos);
/* Copies out a tabulated EOS's derived tables in the reference's DBLIST order
 * (for parity checks). Returns the double count, or -1. */
long sgx_eos_spiner_dump(const sgx_eos *eos, double *out, long cap);

/* ---- Vector lookups (device arrays) ---- */
/* out[i] = F(in1[i], in2[i], lambda row i). lambda may be NULL; otherwise
 * row i starts at lambda + i*lambda_stride. */
int sgx_eos_eval(const sgx_eos *eos, int fn, int64_t n, const double *in1,
                 const double *in2, double *out, double *lambda, int lambda_stride,
                 sgx_stream_t stream);
/* The bounds a model reports (eos_base.hpp:533-560 and the overrides of
 * each model, through the modifiers as eos_base.hpp:134-153 and
 * scaled_eos.hpp:254-275 forward them), one per element: out[i] =
 * MinimumDensity(), MinimumTemperature(), MaximumDensity(),
 * MinimumPressure(), MaximumPressureAtTemperature(temp[i]) or
 * RhoPmin(temp[i]). temp may be NULL for the first four. Device arrays. */
enum {
  SGX_BOUND_MIN_DENSITY = 0,
  SGX_BOUND_MIN_TEMPERATURE = 1,
  SGX_BOUND_MAX_DENSITY = 2,
  SGX_BOUND_MIN_PRESSURE = 3,
  SGX_BOUND_MAX_PRESSURE_AT_T = 4,
  SGX_BOUND_RHO_PMIN = 5
};
int sgx_eos_bounds(const sgx_eos *eos, int what, int64_t n, const double *temp, double *out,
                   sgx_stream_t stream);
/* PTDerivativesFromPreferred (eos/eos_base.hpp:410-419, eos_variant.hpp:
 * 386-398) at n states (rho, sie, press, temp): dedP_T = (dsie/dP)_T,
 * drdP_T = (drho/dP)_T, dedT_P = (dsie/dT)_P, drdT_P = (drho/dT)_P.
 * IdealGas answers in closed form (eos_ideal.hpp:152-168); the other models
 * by the reference's one-sided differences of
 * DensityEnergyFromPressureTemperature (PTDerivativesByFiniteDifferences,
 * eos_base.hpp:299-320); modifiers as theirs do. The reference has only the
 * scalar member; this is its per-element loop. lambda as in sgx_eos_eval.
 * Helmholtz returns SGX_ERR_UNSUPPORTED. */
int sgx_eos_pt_derivatives(const sgx_eos *eos, int64_t n, const double *rho, const double *sie,
                           const double *press, const double *temp, double *dedP_T,
                           double *drdP_T, double *dedT_P, double *drdT_P, double *lambda,
                           int lambda_stride, sgx_stream_t stream);
/* Vector FillEos: output is a bit set of SGX_Q_*; arrays not in output are
 * inputs. Any array that is neither read nor written may be NULL. */
int sgx_eos_fill(const sgx_eos *eos, int64_t n, double *rho, double *temp, double *sie,
                 double *press, double *cv, double *bmod, uint32_t output, double *lambda,
                 int lambda_stride, sgx_stream_t stream);
/* FillEos with two extensions: cs (nullable) receives the sound speed
 * sqrt(bmod / rho), and precision selects the arithmetic. SGX_PREC_MIXED
 * takes (rho, sie) inputs with T among the outputs, for three models:
 *  - SpinerEOSDependsRhoT: the root and the outputs in float-float on the
 *    FP32 pipe, the roundings the root is sensitive to (log10 rho, the
 *    density weight) in FP64 as the reference takes them. Against
 *    SGX_PREC_FP64: T within 1e-11 relative; P, bmod, cs within 1e-10, or,
 *    where P is a small difference of large table entries, within how far
 *    the FP64 value moves under a 1e-14 relative change of sie. Elements it
 *    cannot answer (off the table's top, roots within 1e-8 of either end of
 *    the T range) take the reference's FP64 iteration in the same call.
 *  - SpinerEOSDependsRhoSie: the interpolations in float-float, within
 *    about 1e-11 of the interpolant's magnitude.
 *  - Helmholtz: the inversion's Newton iteration starts from an FP32 phase;
 *    every output is the FP64 evaluation at the temperature found.
 * The analytic models, and the tabulated ones with other inputs or outputs,
 * return SGX_ERR_UNSUPPORTED; Helmholtz without T among the outputs runs its
 * FP64 path. No reference counterpart beyond FillEos
 * (eos/eos_base.hpp:503-531). */
int sgx_eos_fill_ex(const sgx_eos *eos, int64_t n, double *rho, double *temp, double *sie,
                    double *press, double *cv, double *bmod, double *cs, uint32_t output,
                    double *lambda, int lambda_stride, int precision, sgx_stream_t stream);

/* FillEos over HOST arrays (the arguments of sgx_eos_fill_ex with host
 * pointers and no stream). Blocks until the outputs are in the host arrays.
 * When every array is page-locked (sgx_host_alloc, cudaHostAlloc) and the
 * GPU uses the host's page tables (a coherent CPU-GPU system such as Grace
 * over NVLink-C2C), the kernel reads and writes the host arrays in place.
 * Otherwise the library streams the arrays through the device in chunks of
 * 2^21 elements on three streams, so the copies of one chunk overlap the
 * kernel of the next; inputs are the non-null arrays whose bit is not in
 * output (rho always, lambda both ways), outputs the arrays whose bit is in
 * output, cs and lambda. No reference counterpart beyond FillEos on host
 * data. */
int sgx_eos_fill_host(const sgx_eos *eos, int64_t n, double *rho, double *temp, double *sie,
                      double *press, double *cv, double *bmod, double *cs, uint32_t output,
                      double *lambda, int lambda_stride, int precision);

/* ---- PTE ---- */
int sgx_mix_params_default(sgx_mix_params *p);
/* Scratch doubles the reference's solver of that kind takes per cell
 * (PTESolverRhoTRequiredScratch :873-881, PTESolverPTRequiredScratch
 * :1198-1206, PTESolverFixedTRequiredScratch :1451-1457,
 * PTESolverFixedPRequiredScratch :1665-1671, PTESolverRhoURequiredScratch
 * :1924-1929). The GPU solvers keep this state in registers. */
int sgx_pte_rhot_required_scratch(int nmat);
int sgx_pte_pt_required_scratch(int nmat);
int sgx_pte_fixed_t_required_scratch(int nmat);
int sgx_pte_fixed_p_required_scratch(int nmat);
int sgx_pte_rhou_required_scratch(int nmat);
/* The ...RequiredScratchInBytes companions (mixed_cell_models.hpp:879-881,
 * 1204-1206 and the other solvers'): the count above times sizeof(double)
 * for solver SGX_PTE_*; 0 for a bad solver. */
size_t sgx_pte_required_scratch_bytes(int solver, int nmat);

/* Solves PTE in every cell.
 *  solver     SGX_PTE_RHOT, SGX_PTE_PT, SGX_PTE_RHOU, SGX_PTE_FIXED_T or
 *             SGX_PTE_FIXED_P (the last three with SGX_PREC_FP64 only)
 *  nmat       material slots per cell (1..6, the Jacobian is at most 6x6);
 *             [nmat][ncell], cell index fastest
 *  eos_list   host array of neos EOS values (neos <= 16)
 *  eos_idx    device [nmat][ncell] index into eos_list, -1 = material absent;
 *             NULL = material m uses eos_list[m] in every cell
 *  vfrac_tot, sie_tot   device [ncell]; sie_tot carries the solver's scalar
 *             constructor argument: the cell's specific internal energy for
 *             RHOT, PT and RHOU, the temperature T_true for FIXED_T, the
 *             pressure P for FIXED_P
 *  rho, vfrac, sie, temp, press   device [nmat][ncell], in/out (the reference's
 *             initial guesses in, equilibrium state out)
 *  lambda     device [nmat][3][ncell] per-material cache, or NULL
 *  params     NULL = defaults
 *  status     device [ncell] or NULL
 *  precision  SGX_PREC_FP64 or SGX_PREC_MIXED */
int sgx_pte_solve(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                  const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
                  double *rho, double *vfrac, double *sie, double *temp, double *press,
                  double *lambda, const sgx_mix_params *params, sgx_pte_status *status,
                  int precision, sgx_stream_t stream);

/* ApproxTemperatureFromRhoMatU (closure/mixed_cell_models.hpp:790-847) per
 * cell: the temperature at which the materials' energy densities
 * rho_m vfrac_m e_m(rho_m, T) add up to u_tot, by bisection in NQT log2 T
 * (at most 10 steps, then one linear interpolation), clamped to
 * [1e-9, 1e9] K. A rough initial guess, as the reference intends.
 *  eos_list, neos, eos_idx   as for sgx_pte_solve
 *  u_tot      device [ncell], total internal energy density (rho * sie)
 *  rho, vfrac device [nmat][ncell] (read only)
 *  Tguess     device [ncell] or NULL (no guess)
 *  lambda     device [nmat][3][ncell] or NULL
 *  temp_out   device [ncell] */
int sgx_pte_approx_temperature(int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                               const int32_t *eos_idx, const double *u_tot, const double *rho,
                               const double *vfrac, const double *Tguess, double *lambda,
                               double *temp_out, sgx_stream_t stream);

/* MixUtils::EnforceMassVolumesSum (mixed_cell_models.hpp:93-117) per cell:
 * the present material with the largest volume fraction takes
 * tot_vol - sum(others), its density rescaled so its mass is kept.
 * eos_idx (device [nmat][ncell], -1 = absent) or NULL = all slots present;
 * tot_vol device [ncell]; rho, vfrac device [nmat][ncell], in/out. */
int sgx_mix_enforce_mass_volumes_sum(int nmat, int64_t ncell, const int32_t *eos_idx,
                                     const double *tot_vol, double *rho, double *vfrac,
                                     sgx_stream_t stream);

/* MixUtils::EnforceEnergiesSum (mixed_cell_models.hpp:119-150) per cell: the
 * present material with the largest |rho vfrac sie| takes the energy that
 * makes sum(rho_m vfrac_m sie_m) = tot_rho * tot_sie. tot_rho, tot_sie
 * device [ncell]; rho, vfrac device [nmat][ncell]; sie in/out. */
int sgx_mix_enforce_energies_sum(int nmat, int64_t ncell, const int32_t *eos_idx,
                                 const double *tot_rho, const double *tot_sie, const double *rho,
                                 const double *vfrac, double *sie, sgx_stream_t stream);

/* Launch-shape and iteration knobs, process-wide.
 *  SGX_TUNE_LOOKUP_BLOCKS_PER_SM  4..6 (default 5): resident blocks per SM
 *      of the mixed-precision tabulated lookup (register budget 64/48/40).
 *  SGX_TUNE_LOOKUP_STAGE  0..2 (default 2): how that lookup stages the
 *      table's coarse search index in shared memory: 0 not at all, 1 by
 *      vector loads, 2 by one bulk copy (TMA). Tables with the thermal bin
 *      index (monotone thermal energy) do not use the coarse index.
 *  SGX_TUNE_L2_PERSIST  0/1 (default 0): mark the table's lines persisting
 *      in L2 (an access-policy window on the lookup's launch; sets aside
 *      L2 for persisting lines in this process's context).
 *  SGX_TUNE_HOST_FILL_STAGED  0/1 (default 0): sgx_eos_fill_host copies
 *      through device buffers even where the kernel could work on the host
 *      arrays in place.
 *  SGX_TUNE_PTE_FP32_ITERS  2..64 (default 8): FP32 Newton iterations per
 *      material in pass 1 of the mixed PTE path.
 *  SGX_TUNE_PTE_RETRY_ITERS  4..128 (default 8): iterations per material of
 *      the FP64 re-solve (pass 2) of the mixed PTE path; a cell that has not
 *      converged by then is reported unconverged. These two change which
 *      cells converge (never their converged values beyond the stated
 *      tolerance); the others change nothing but speed.
 *  SGX_TUNE_PTE_COUNT_ORDER  0/1 (default 0): the mixed path takes the
 *      material counts from the smallest (0) or from the largest (1); pass 2
 *      of one count overlaps pass 1 of the next, so the order decides
 *      which pass 2 is left without overlap. Results do not change.
 *  SGX_TUNE_PTE_MIXED_BLOCK  32..128 (default 128): threads per block of
 *      the mixed path's pass 1 (rounded down to 32, 64 or 128). Results do
 *      not change.
 *  SGX_TUNE_PTE_GROUP_MIN_N  2..7 (default 3): pass 1 of the mixed path
 *      solves cells with at least this many materials with a group of 2, 4
 *      or 8 lanes per cell (one material per lane), and smaller cells with
 *      one thread each; 7 keeps one thread per cell everywhere. Both forms
 *      meet the same tolerance; their results differ in rounding.
 *  SGX_TUNE_PTE_FP32_TOL  3..6 (default 4): the FP32 Newton phase of the
 *      mixed path iterates to relative residuals of 10^-value before the
 *      FP64 residual correction (which ends at 1e-12 either way).
 *  SGX_TUNE_HELM_PASS1_STEPS  0..100: Newton steps of the Helmholtz
 *      T(rho, sie) inversion in its first pass (FP64 steps after the FP32
 *      phase on the mixed path); the elements still iterating are resumed
 *      from their saved state over a compacted queue.
 *  SGX_TUNE_HELM_MID_STEPS, SGX_TUNE_HELM_MID2_STEPS  0..100: each one
 *      above the cap before it adds a middle pass that resumes the elements
 *      still iterating up to that many steps, before the last pass takes the
 *      rest to the reference's 100 (100: no such pass).
 *      Left at 0, the three take their precision's defaults: 10, 20, 40 for
 *      FP64 and 3, 12, 40 for the mixed path. Results do not change.
 */
enum {
  SGX_TUNE_LOOKUP_BLOCKS_PER_SM = 1,
  SGX_TUNE_LOOKUP_STAGE = 2,
  SGX_TUNE_L2_PERSIST = 3,
  SGX_TUNE_HOST_FILL_STAGED = 4,
  SGX_TUNE_PTE_FP32_ITERS = 5,
  SGX_TUNE_PTE_RETRY_ITERS = 6,
  SGX_TUNE_PTE_COUNT_ORDER = 7,
  SGX_TUNE_PTE_MIXED_BLOCK = 8,
  SGX_TUNE_PTE_GROUP_MIN_N = 9,
  SGX_TUNE_PTE_FP32_TOL = 10,
  SGX_TUNE_HELM_PASS1_STEPS = 11,
  SGX_TUNE_HELM_MID_STEPS = 12,
  SGX_TUNE_HELM_MID2_STEPS = 13
};
int sgx_tune_set(int knob, int value);
int sgx_tune_get(int knob, int *value);
/* The autotuner of the lookup's launch shape: times every
 * (SGX_TUNE_LOOKUP_BLOCKS_PER_SM, SGX_TUNE_LOOKUP_STAGE) pair on the
 * caller's own mixed-precision FillEos batch (the arguments of
 * sgx_eos_fill_ex), 1 + reps calls per pair with CUDA events on `stream`,
 * and keeps the fastest pair set; blocks_per_sm / stage (nullable) receive
 * it. These knobs never change a lookup's result. Each trial is an ordinary
 * call, so outputs (and a lambda cache) are written. */
int sgx_tune_autotune_fill(const sgx_eos *eos, int64_t n, double *rho, double *temp,
                           double *sie, double *press, double *cv, double *bmod, double *cs,
                           uint32_t output, double *lambda, int lambda_stride, int reps,
                           int *blocks_per_sm, int *stage, sgx_stream_t stream);

/* The autotuner of the mixed-precision PTE launch: times every combination
 * of SGX_TUNE_PTE_MIXED_BLOCK (32, 64, 128) and SGX_TUNE_PTE_COUNT_ORDER (0,
 * 1) -- and, with tune_group non-zero, SGX_TUNE_PTE_GROUP_MIN_N (the current
 * value, 3, 4, 7) -- on the caller's own RhoT batch (the arguments of
 * sgx_pte_solve), 1 + reps solves per setting with CUDA events on `stream`,
 * and keeps the fastest set; chosen (nullable, 3 ints) receives (block,
 * order, group_min_n). The starting state is copied aside and restored
 * before every trial (stream-ordered pool memory, five arrays' worth); on
 * return the arrays hold the solve of the winning setting. The first two
 * knobs never change a result; the lane-group threshold changes results
 * within the mixed path's stated tolerance only. No reference counterpart. */
int sgx_tune_autotune_pte(int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                          const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
                          double *rho, double *vfrac, double *sie, double *temp, double *press,
                          double *lambda, const sgx_mix_params *params, sgx_pte_status *status,
                          int reps, int tune_group, int *chosen, sgx_stream_t stream);

/* Largest ncell sgx_pte_solve_noalloc accepts. */
#define SGX_PTE_NOALLOC_MAX_CELLS 1048576

/* sgx_pte_solve with precision SGX_PREC_MIXED and solver SGX_PTE_RHOT, for
 * callers that must not allocate device memory at solve time (host codes
 * that hand all device memory to their own allocator at start-up). It has
 * no reference counterpart. Arguments and results are those of
 * sgx_pte_solve; the solver's scratch (8 bytes per cell plus 153 KiB) is a
 * static device array of the library sized for SGX_PTE_NOALLOC_MAX_CELLS
 * cells, so nothing is allocated.
 *  - ncell > SGX_PTE_NOALLOC_MAX_CELLS returns SGX_ERR_INVALID before any
 *    device work; split the batch or call sgx_pte_solve.
 *  - solver other than SGX_PTE_RHOT returns SGX_ERR_UNSUPPORTED.
 *  - The first call in a CUDA context looks up the array's device address
 *    (with that device current) and caches it for that context; make that
 *    first call before any stream capture begins. After cudaDeviceReset, or
 *    with another driver context current, the next call is again a first
 *    call (the cache is keyed on the context's id, not the device).
 *  - There is one array per device: calls that overlap in time on the same
 *    device (other streams, other host threads) race on it and give wrong
 *    results. Order them on one stream or serialise them. */
int sgx_pte_solve_noalloc(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list,
                          int neos, const int32_t *eos_idx, const double *vfrac_tot,
                          const double *sie_tot, double *rho, double *vfrac, double *sie,
                          double *temp, double *press, double *lambda,
                          const sgx_mix_params *params, sgx_pte_status *status,
                          sgx_stream_t stream);

/* get_sg_eos (singularity_eos.hpp:114-132; eos/get_sg_eos.cpp:35-280) over
 * HOST arrays, as the reference takes them: every array is copied to the
 * device, solved there, and copied back before the call returns (the
 * reference deep-copies its host arrays to and from Kokkos views the same
 * way, get_sg_eos.cpp:99-120). Per cell offsets[k]-1 (1-based, as the
 * Fortran interface passes them), k < ncell: the mass fractions are
 * normalised, materials above mass_frac_cutoff take part in the closure
 * solve of the input mode, and press, temp, bmod, cv, dpde, frac_vol,
 * frac_ie and the optional frac_bmod / frac_dpde / frac_cv (NULL to skip)
 * are written; pmax becomes max(pmax, press). input_int as the reference's
 * input_condition (get_sg_eos.cpp:65-71): 1 (rho, sie), 0 (rho, sie) with
 * normalised mass fractions, -1 (P, T), -2 (rho, P), -3 (rho, T)
 * (get_sg_eos_p_t.cpp, _rho_p.cpp, _rho_t.cpp). Per-cell arrays
 * [cell_dim], per-material LayoutLeft [nmat][cell_dim]. eos_offsets (host,
 * [nmat], 1-based) picks each material's entry of the host list eos (neos
 * entries). Cells with no material above the cutoff get zero pressure and
 * temperature. precision: SGX_PREC_FP64 (the reference iteration) or
 * SGX_PREC_MIXED ((rho, sie) and (P, T) modes). The copies and the solve
 * run on `stream`, which is synchronised before the return. */
int sgx_get_sg_eos(int nmat, int ncell, int cell_dim, int input_int, const int *eos_offsets,
                   const sgx_eos *eos, int neos, const int *offsets, double *press,
                   double *pmax, double *vol, double *spvol, double *sie, double *temp,
                   double *bmod, double *dpde, double *cv, double *frac_mass, double *frac_vol,
                   double *frac_ie, double *frac_bmod, double *frac_dpde, double *frac_cv,
                   double mass_frac_cutoff, int precision, sgx_stream_t stream);
/* The same over DEVICE arrays (offsets and every per-cell and per-material
 * array in device memory; eos_offsets and eos stay host arrays), stream-
 * ordered and without copies or synchronisation. No reference counterpart:
 * it is get_sg_eos without its host copies, for callers whose fields already
 * live on the device. */
int sgx_get_sg_eos_device(int nmat, int ncell, int cell_dim, int input_int,
                          const int *eos_offsets, const sgx_eos *eos, int neos,
                          const int *offsets, double *press, double *pmax, double *vol,
                          double *spvol, double *sie, double *temp, double *bmod, double *dpde,
                          double *cv, double *frac_mass, double *frac_vol, double *frac_ie,
                          double *frac_bmod, double *frac_dpde, double *frac_cv,
                          double mass_frac_cutoff, int precision, sgx_stream_t stream);

/* ---- PTE plans: one solve bound to fixed arrays, replayed as a CUDA graph ----
 * sgx_pte_plan_create checks its arguments as sgx_pte_solve does, allocates
 * the solve's scratch and captures the whole launch sequence (binning, both
 * passes, the side-stream fork and join) into a graph. Each
 * sgx_pte_plan_run is one graph launch on `stream` and solves whatever the
 * bound arrays hold at that time, with the result sgx_pte_solve would give.
 * Iteration knobs (sgx_tune_set) are read at creation. A plan belongs to the
 * device current at creation; runs of one plan must not overlap (they share
 * its scratch). No reference counterpart: the reference's closure is a
 * per-cell loop the caller runs each cycle. */
typedef struct sgx_pte_plan sgx_pte_plan;
int sgx_pte_plan_create(int solver, int nmat, int64_t ncell, const sgx_eos *eos_list, int neos,
                        const int32_t *eos_idx, const double *vfrac_tot, const double *sie_tot,
                        double *rho, double *vfrac, double *sie, double *temp, double *press,
                        double *lambda, const sgx_mix_params *params, sgx_pte_status *status,
                        int precision, sgx_pte_plan **out);
int sgx_pte_plan_run(sgx_pte_plan *plan, sgx_stream_t stream);
int sgx_pte_plan_destroy(sgx_pte_plan *plan);

/* ---- The reference's C interface (eos/singularity_eos.hpp:25-134) ----
 * Same argument lists with an sgx_ prefix, over sgx_eos values. enabled /
 * vals NULL take the reference's defaults (no modifiers); otherwise they
 * are applied as sgx_eos_apply_modifiers does. get_sg_* arrays are device
 * arrays; the lookups are ordered on the legacy default stream; stride -1
 * or lambda_data NULL means no lambda (lambdaIndexer2D otherwise). */
int sgx_init_sg_eos(int nmat, sgx_eos **eos);
int sgx_init_sg_IdealGas(int matindex, sgx_eos *eos, double gm1, double Cv, const int *enabled,
                         double *vals);
int sgx_init_sg_StiffGas(int matindex, sgx_eos *eos, double gm1, double Cv, double Pinf,
                         double qq, const int *enabled, double *vals);
int sgx_init_sg_NobleAbel(int matindex, sgx_eos *eos, double gm1, double Cv, double bb,
                          double qq, const int *enabled, double *vals);
int sgx_init_sg_Gruneisen(int matindex, sgx_eos *eos, double C0, double s1, double s2,
                          double s3, double G0, double b, double rho0, double T0, double P0,
                          double Cv, const int *enabled, double *vals);
/* split: TableSplit::Total (0) only. */
int sgx_init_sg_SpinerDependsRhoT(int matindex, sgx_eos *eos, const char *filename, int id,
                                  int split, const int *enabled, double *vals);
int sgx_init_sg_SpinerDependsRhoSie(int matindex, sgx_eos *eos, const char *filename, int id,
                                    int split, const int *enabled, double *vals);
int sgx_init_sg_Helmholtz(int matindex, sgx_eos *eos, const char *filename, int rad, int gas,
                          int coul, int ion, int ele, int verbose, const int *enabled,
                          double *vals);
int sgx_get_sg_EntropyFromDensityInternalEnergy(int matindex, const sgx_eos *eos,
                                                const double *rhos, const double *sies,
                                                double *entropies, int len, int stride,
                                                double *lambda_data);
int sgx_get_sg_PressureFromDensityInternalEnergy(int matindex, const sgx_eos *eos,
                                                 const double *rhos, const double *sies,
                                                 double *pressures, int len, int stride,
                                                 double *lambda_data);
int sgx_get_sg_MinInternalEnergyFromDensity(int matindex, const sgx_eos *eos,
                                            const double *rhos, double *sies, int len);
int sgx_get_sg_BulkModulusFromDensityInternalEnergy(int matindex, const sgx_eos *eos,
                                                    const double *rhos, const double *sies,
                                                    double *bmods, int len, int stride,
                                                    double *lambda_data);
/* Releases every EOS's device table, then the array; *eos becomes NULL. */
int sgx_finalize_sg_eos(int nmat, sgx_eos **eos);

/* ---- Serving: a device-resident request loop for PTE closure batches ----
 * No reference counterpart: the reference is a library called once per
 * batch (get_sg_eos, singularity_eos.hpp:114-132). The server keeps the EOS
 * tables and a device arena of hbm_budget_bytes resident. Whenever one of
 * its max_inflight batch slots (each a CUDA stream) is free, it folds the
 * requests waiting at that moment, in arrival order and as many as fit the
 * arena (up to 2^22 cells), into ONE merged batch: their cells laid end to
 * end, one binned PTE solve over all of them, each request's rows copied
 * back to its own arrays. Requests that arrive while batches are on the GPU
 * form the next batch, which overlaps with them. A request's result is the
 * one sgx_pte_solve gives for the same inputs alone, bit for bit (every cell
 * is solved independently). Requests larger than the whole arena are
 * rejected at submission; a request that does not fit waits at the head of
 * the queue until memory frees up (no overtaking). */
typedef struct sgx_server sgx_server;

typedef struct sgx_server_config {
  size_t hbm_budget_bytes; /* device arena for request arrays and scratch */
  int max_inflight;        /* merged batches on the device at once (1..64) */
  int solver;              /* SGX_PTE_RHOT (SGX_PTE_PT with SGX_PREC_FP64 only) */
  int precision;           /* SGX_PREC_FP64 or SGX_PREC_MIXED */
  const sgx_eos *eos_list; /* host array, copied; tables must stay resident */
  int neos;                /* 1..16 */
  const sgx_mix_params *params; /* NULL = defaults */
} sgx_server_config;

/* One closure request: host arrays in the layout of sgx_pte_solve
 * ([nmat][ncell], cell fastest). Inputs are read when the request is
 * admitted and outputs written when it completes; the caller keeps every
 * array alive and unmodified until sgx_server_wait reports completion.
 * Host arrays from sgx_host_alloc (page-locked) let the copies overlap with
 * other requests' kernels. eos_idx may be NULL (material m uses eos_list[m]);
 * status may be NULL. */
typedef struct sgx_pte_request {
  int nmat;
  int64_t ncell;
  const int32_t *eos_idx;
  const double *vfrac_tot, *sie_tot;
  const double *rho_in, *vfrac_in, *sie_in, *temp_in, *press_in;
  double *rho_out, *vfrac_out, *sie_out, *temp_out, *press_out;
  sgx_pte_status *status;
} sgx_pte_request;

typedef struct sgx_server_stats {
  uint64_t submitted, completed, failed;
  uint64_t cells_completed;
  int inflight, queued; /* requests on the device, requests waiting */
  size_t arena_used, arena_peak;
  uint64_t batches;     /* merged solves issued */
} sgx_server_stats;

int sgx_server_create(const sgx_server_config *cfg, sgx_server **out);
/* Queues a request; *ticket identifies it. Never blocks on the device. */
int sgx_server_submit(sgx_server *s, const sgx_pte_request *req, uint64_t *ticket);
/* Waits up to timeout_s seconds (< 0: forever) for a request. Returns SGX_OK
 * when it completed (latency_s, if not NULL, receives submit-to-completion
 * seconds), SGX_ERR_TIMEOUT when it is still pending, or the request's error.
 * A completed ticket can be waited on once. */
int sgx_server_wait(sgx_server *s, uint64_t ticket, double timeout_s, double *latency_s);
int sgx_server_stats_get(sgx_server *s, sgx_server_stats *out);
/* Waits for every request, then releases the arena, the streams and the
 * worker thread. */
int sgx_server_destroy(sgx_server *s);
/* Page-locked host memory for request arrays (cudaHostAlloc / cudaFreeHost). */
void *sgx_host_alloc(size_t bytes);
void sgx_host_free(void *p);

#ifdef __cplusplus
}
#endif

#endif /* SGX_H_ */
