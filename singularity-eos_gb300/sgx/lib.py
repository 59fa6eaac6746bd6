"""ctypes binding of libsgx.so (include/sgx.h).

Device arrays are passed as torch CUDA tensors (torch is used for device
memory and streams only); every call goes through the C ABI. Loading fails
loudly when the library has not been built -- there is no fallback.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(HERE), "lib", "libsgx.so")

IDEAL_GAS, STIFF_GAS, NOBLE_ABEL, GRUNEISEN, SPINER_RHOT, HELMHOLTZ, SPINER_RHOSIE = 1, 2, 3, 4, 5, 6, 7
(BOUND_MIN_DENSITY, BOUND_MIN_TEMPERATURE, BOUND_MAX_DENSITY, BOUND_MIN_PRESSURE,
 BOUND_MAX_PRESSURE_AT_T, BOUND_RHO_PMIN) = range(6)
Q_DENSITY, Q_SIE, Q_PRESSURE, Q_TEMPERATURE, Q_SPECIFIC_HEAT, Q_BULK_MODULUS = 1, 2, 4, 8, 16, 32
(FN_T_FROM_RHO_SIE, FN_SIE_FROM_RHO_T, FN_P_FROM_RHO_T, FN_P_FROM_RHO_SIE, FN_CV_FROM_RHO_T,
 FN_CV_FROM_RHO_SIE, FN_B_FROM_RHO_T, FN_B_FROM_RHO_SIE, FN_G_FROM_RHO_T, FN_G_FROM_RHO_SIE,
 FN_MIN_SIE_FROM_RHO) = range(11)
PTE_RHOT, PTE_PT, PTE_RHOU, PTE_FIXED_T, PTE_FIXED_P = 0, 1, 2, 3, 4
TUNE_LOOKUP_BLOCKS_PER_SM, TUNE_LOOKUP_STAGE, TUNE_L2_PERSIST, TUNE_HOST_FILL_STAGED = 1, 2, 3, 4
TUNE_PTE_FP32_ITERS, TUNE_PTE_RETRY_ITERS, TUNE_PTE_COUNT_ORDER = 5, 6, 7
TUNE_PTE_MIXED_BLOCK, TUNE_PTE_GROUP_MIN_N, TUNE_PTE_FP32_TOL = 8, 9, 10
TUNE_HELM_PASS1_STEPS, TUNE_HELM_MID_STEPS, TUNE_HELM_MID2_STEPS = 11, 12, 13
PREC_FP64, PREC_MIXED = 0, 1

EXPORTED = [
    "sgx_version", "sgx_last_error", "sgx_eos_ideal_gas", "sgx_eos_stiff_gas",
    "sgx_eos_noble_abel", "sgx_eos_gruneisen", "sgx_eos_spiner_rhot", "sgx_eos_spiner_rhosie",
    "sgx_eos_finalize",
    "sgx_eos_table_bytes", "sgx_eos_spiner_dump", "sgx_eos_eval", "sgx_eos_fill",
    "sgx_eos_fill_ex", "sgx_eos_bounds",
    "sgx_mix_params_default", "sgx_pte_rhot_required_scratch", "sgx_pte_pt_required_scratch",
    "sgx_pte_fixed_t_required_scratch", "sgx_pte_fixed_p_required_scratch",
    "sgx_pte_rhou_required_scratch", "sgx_pte_approx_temperature",
    "sgx_mix_enforce_mass_volumes_sum", "sgx_mix_enforce_energies_sum", "sgx_tune_set",
    "sgx_tune_get",
    "sgx_pte_solve", "sgx_pte_solve_noalloc", "sgx_eos_helmholtz", "sgx_eos_helmholtz_dump",
    "sgx_server_create", "sgx_server_submit", "sgx_server_wait", "sgx_server_stats_get",
    "sgx_server_destroy", "sgx_host_alloc", "sgx_host_free", "sgx_eos_fill_host",
    "sgx_get_sg_eos", "sgx_get_sg_eos_device", "sgx_tune_autotune_pte", "sgx_eos_modify_shifted", "sgx_eos_modify_scaled",
    "sgx_eos_modify_bilinear_ramp", "sgx_eos_p_alpha_ramp_params", "sgx_eos_apply_modifiers",
    "sgx_eos_pt_derivatives", "sgx_eos_ideal_gas_entropy", "sgx_eos_stiff_gas_ref",
    "sgx_eos_noble_abel_ref", "sgx_init_sg_eos", "sgx_init_sg_IdealGas", "sgx_init_sg_StiffGas",
    "sgx_init_sg_NobleAbel", "sgx_init_sg_Gruneisen", "sgx_init_sg_SpinerDependsRhoT",
    "sgx_init_sg_SpinerDependsRhoSie",
    "sgx_init_sg_Helmholtz", "sgx_get_sg_EntropyFromDensityInternalEnergy",
    "sgx_get_sg_PressureFromDensityInternalEnergy", "sgx_get_sg_MinInternalEnergyFromDensity",
    "sgx_get_sg_BulkModulusFromDensityInternalEnergy", "sgx_finalize_sg_eos",
    "sgx_pte_plan_create", "sgx_pte_plan_run", "sgx_pte_plan_destroy", "sgx_tune_autotune_fill",
    "sgx_pte_required_scratch_bytes",
]
MOD_SHIFTED, MOD_SCALED, MOD_RAMP = 1, 2, 4
HELM_DEFAULT, HELM_REGULA_FALSI, HELM_CACHE_READBACK = 31, 32, 64
PTE_NOALLOC_MAX_CELLS = 1 << 20  # SGX_PTE_NOALLOC_MAX_CELLS


class SgxEos(C.Structure):
    _fields_ = [("type", C.c_int32), ("flags", C.c_int32), ("table", C.c_uint64),
                ("p", C.c_double * 14), ("mods", C.c_uint32), ("mods_reserved", C.c_uint32),
                ("shift", C.c_double), ("scale", C.c_double), ("inv_scale", C.c_double),
                ("ramp", C.c_double * 6)]


class MixParams(C.Structure):
    _fields_ = [
        ("verbose", C.c_int32), ("iterate_t_guess", C.c_int32),
        ("derivative_eps", C.c_double), ("pte_rel_tolerance_p", C.c_double),
        ("pte_rel_tolerance_t", C.c_double), ("pte_rel_tolerance_e", C.c_double),
        ("pte_rel_tolerance_v", C.c_double), ("pte_abs_tolerance_p", C.c_double),
        ("pte_abs_tolerance_t", C.c_double), ("pte_slow_convergence_thresh", C.c_double),
        ("pte_rel_tolerance_p_sufficient", C.c_double),
        ("pte_rel_tolerance_t_sufficient", C.c_double),
        ("pte_rel_tolerance_e_sufficient", C.c_double),
        ("pte_rel_tolerance_v_sufficient", C.c_double),
        ("pte_abs_tolerance_p_sufficient", C.c_double),
        ("pte_abs_tolerance_t_sufficient", C.c_double),
        ("pte_max_iter_per_mat", C.c_int64), ("line_search_alpha", C.c_double),
        ("line_search_max_iter", C.c_int64), ("line_search_fac", C.c_double),
        ("vfrac_safety_fac", C.c_double), ("temperature_limit", C.c_double),
        ("default_tguess", C.c_double), ("min_dtde", C.c_double),
        ("pte_small_step_tries", C.c_int64), ("pte_small_step_thresh", C.c_double),
        ("pte_max_dpdv", C.c_double), ("pte_reduced_system_exclude_idx", C.c_int64),
    ]


class PteStatus(C.Structure):
    _fields_ = [("residual", C.c_double), ("niter", C.c_int32), ("converged", C.c_uint8),
                ("slow_convergence_detected", C.c_uint8), ("max_line_niter", C.c_uint8),
                ("small_step_iters", C.c_uint8)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_inflight", C.c_int),
                ("solver", C.c_int), ("precision", C.c_int), ("eos_list", C.c_void_p),
                ("neos", C.c_int), ("params", C.c_void_p)]


class PteRequest(C.Structure):
    _fields_ = [("nmat", C.c_int), ("ncell", C.c_int64), ("eos_idx", C.c_void_p),
                ("vfrac_tot", C.c_void_p), ("sie_tot", C.c_void_p),
                ("rho_in", C.c_void_p), ("vfrac_in", C.c_void_p), ("sie_in", C.c_void_p),
                ("temp_in", C.c_void_p), ("press_in", C.c_void_p),
                ("rho_out", C.c_void_p), ("vfrac_out", C.c_void_p), ("sie_out", C.c_void_p),
                ("temp_out", C.c_void_p), ("press_out", C.c_void_p), ("status", C.c_void_p)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("cells_completed", C.c_uint64), ("inflight", C.c_int), ("queued", C.c_int),
                ("arena_used", C.c_size_t), ("arena_peak", C.c_size_t),
                ("batches", C.c_uint64)]


_lib = None


def load():
    """Loads libsgx.so (built by singularity-eos_gb300/build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libsgx.so not built ({LIB_PATH}); run __graft_entry__.build()")
    lib = C.CDLL(LIB_PATH)
    P, I, D, V, U64 = C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_uint64
    lib.sgx_version.restype = C.c_char_p
    lib.sgx_last_error.restype = C.c_char_p
    lib.sgx_eos_ideal_gas.argtypes = [C.POINTER(SgxEos), D, D]
    lib.sgx_eos_stiff_gas.argtypes = [C.POINTER(SgxEos), D, D, D, D]
    lib.sgx_eos_noble_abel.argtypes = [C.POINTER(SgxEos), D, D, D, D]
    lib.sgx_eos_ideal_gas_entropy.argtypes = [C.POINTER(SgxEos), D, D, D, D]
    lib.sgx_eos_stiff_gas_ref.argtypes = [C.POINTER(SgxEos)] + [D] * 7
    lib.sgx_eos_noble_abel_ref.argtypes = [C.POINTER(SgxEos)] + [D] * 7
    lib.sgx_eos_gruneisen.argtypes = [C.POINTER(SgxEos)] + [D] * 11
    lib.sgx_eos_spiner_rhot.argtypes = [C.POINTER(SgxEos), C.c_char_p, I, I]
    lib.sgx_eos_spiner_rhosie.argtypes = [C.POINTER(SgxEos), C.c_char_p, I, I]
    lib.sgx_eos_bounds.argtypes = [C.POINTER(SgxEos), I, C.c_int64, P, P, P]
    lib.sgx_eos_finalize.argtypes = [C.POINTER(SgxEos)]
    lib.sgx_eos_table_bytes.argtypes = [C.POINTER(SgxEos)]
    lib.sgx_eos_table_bytes.restype = C.c_size_t
    lib.sgx_eos_spiner_dump.argtypes = [C.POINTER(SgxEos), P, C.c_long]
    lib.sgx_eos_spiner_dump.restype = C.c_long
    lib.sgx_eos_eval.argtypes = [C.POINTER(SgxEos), I, C.c_int64, P, P, P, P, I, P]
    lib.sgx_eos_fill.argtypes = [C.POINTER(SgxEos), C.c_int64, P, P, P, P, P, P, C.c_uint32,
                                 P, I, P]
    lib.sgx_eos_fill_ex.argtypes = [C.POINTER(SgxEos), C.c_int64, P, P, P, P, P, P, P,
                                    C.c_uint32, P, I, I, P]
    lib.sgx_mix_params_default.argtypes = [C.POINTER(MixParams)]
    lib.sgx_pte_solve.argtypes = [I, I, C.c_int64, P, I, P, P, P, P, P, P, P, P, P,
                                  C.POINTER(MixParams), P, I, P]
    lib.sgx_eos_helmholtz.argtypes = [C.POINTER(SgxEos), C.c_char_p, I]
    lib.sgx_eos_helmholtz_dump.argtypes = [C.POINTER(SgxEos), P, C.c_long]
    lib.sgx_eos_helmholtz_dump.restype = C.c_long
    lib.sgx_eos_fill_host.argtypes = [C.POINTER(SgxEos), C.c_int64, P, P, P, P, P, P, P,
                                      C.c_uint32, P, I, I]
    lib.sgx_get_sg_eos.argtypes = [I, I, I, I, P, P, I, P] + [P] * 15 + [D, I, P]
    lib.sgx_get_sg_eos_device.argtypes = [I, I, I, I, P, P, I, P] + [P] * 15 + [D, I, P]
    lib.sgx_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]
    lib.sgx_server_submit.argtypes = [C.c_void_p, C.POINTER(PteRequest),
                                      C.POINTER(C.c_uint64)]
    lib.sgx_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_double,
                                    C.POINTER(C.c_double)]
    lib.sgx_server_stats_get.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    lib.sgx_server_destroy.argtypes = [C.c_void_p]
    lib.sgx_host_alloc.argtypes = [C.c_size_t]
    lib.sgx_host_alloc.restype = C.c_void_p
    lib.sgx_host_free.argtypes = [C.c_void_p]
    lib.sgx_pte_solve_noalloc.argtypes = [I, I, C.c_int64, P, I, P, P, P, P, P, P, P, P, P,
                                          C.POINTER(MixParams), P, P]
    lib.sgx_tune_set.argtypes = [I, I]
    lib.sgx_tune_get.argtypes = [I, C.POINTER(C.c_int)]
    lib.sgx_pte_approx_temperature.argtypes = [I, C.c_int64, P, I, P, P, P, P, P, P, P, P]
    lib.sgx_mix_enforce_mass_volumes_sum.argtypes = [I, C.c_int64, P, P, P, P, P]
    lib.sgx_mix_enforce_energies_sum.argtypes = [I, C.c_int64, P, P, P, P, P, P, P]
    lib.sgx_eos_modify_shifted.argtypes = [C.POINTER(SgxEos), D]
    lib.sgx_eos_modify_scaled.argtypes = [C.POINTER(SgxEos), D]
    lib.sgx_eos_modify_bilinear_ramp.argtypes = [C.POINTER(SgxEos), D, D, D, D]
    lib.sgx_eos_p_alpha_ramp_params.argtypes = [C.POINTER(SgxEos), D, D, D] + [
        C.POINTER(C.c_double)] * 4
    lib.sgx_eos_apply_modifiers.argtypes = [C.POINTER(SgxEos), C.POINTER(C.c_int),
                                            C.POINTER(C.c_double)]
    lib.sgx_eos_pt_derivatives.argtypes = [C.POINTER(SgxEos), C.c_int64] + [P] * 9 + [I, P]
    PE = C.POINTER(SgxEos)
    lib.sgx_init_sg_eos.argtypes = [I, C.POINTER(PE)]
    lib.sgx_init_sg_IdealGas.argtypes = [I, PE, D, D, P, P]
    lib.sgx_init_sg_StiffGas.argtypes = [I, PE, D, D, D, D, P, P]
    lib.sgx_init_sg_NobleAbel.argtypes = [I, PE, D, D, D, D, P, P]
    lib.sgx_init_sg_Gruneisen.argtypes = [I, PE] + [D] * 10 + [P, P]
    lib.sgx_init_sg_SpinerDependsRhoT.argtypes = [I, PE, C.c_char_p, I, I, P, P]
    lib.sgx_init_sg_SpinerDependsRhoSie.argtypes = [I, PE, C.c_char_p, I, I, P, P]
    lib.sgx_init_sg_Helmholtz.argtypes = [I, PE, C.c_char_p, I, I, I, I, I, I, P, P]
    for name in ("Entropy", "Pressure", "BulkModulus"):
        getattr(lib, f"sgx_get_sg_{name}FromDensityInternalEnergy").argtypes = [
            I, PE, P, P, P, I, I, P]
    lib.sgx_get_sg_MinInternalEnergyFromDensity.argtypes = [I, PE, P, P, I]
    lib.sgx_finalize_sg_eos.argtypes = [I, C.POINTER(PE)]
    lib.sgx_pte_plan_create.argtypes = [I, I, C.c_int64, P, I, P, P, P, P, P, P, P, P, P,
                                        C.POINTER(MixParams), P, I, C.POINTER(C.c_void_p)]
    lib.sgx_pte_plan_run.argtypes = [C.c_void_p, P]
    lib.sgx_pte_plan_destroy.argtypes = [C.c_void_p]
    lib.sgx_pte_required_scratch_bytes.argtypes = [I, I]
    lib.sgx_pte_required_scratch_bytes.restype = C.c_size_t
    lib.sgx_tune_autotune_fill.argtypes = [C.POINTER(SgxEos), C.c_int64] + [P] * 7 + [
        C.c_uint32, P, I, I, C.POINTER(C.c_int), C.POINTER(C.c_int), P]
    lib.sgx_tune_autotune_pte.argtypes = [I, C.c_int64, P, I] + [P] * 9 + [
        C.POINTER(MixParams), P, I, I, P, P]
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        raise RuntimeError(f"sgx error {rc}: {load().sgx_last_error().decode()}")


def ptr(t):
    """Device address of a torch tensor (or None)."""
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def make_eos(kind, params):
    """An sgx_eos value from (model code, parameters) as in sgx.workloads."""
    lib = load()
    e = SgxEos()
    p = list(params)
    if kind == IDEAL_GAS and len(p) >= 4:  # (gm1, Cv, EntropyT0, EntropyRho0)
        check(lib.sgx_eos_ideal_gas_entropy(C.byref(e), *p[:4]))
    elif kind == IDEAL_GAS:
        check(lib.sgx_eos_ideal_gas(C.byref(e), *p[:2]))
    elif kind == STIFF_GAS and len(p) >= 7:  # (..., qp, T0, P0)
        check(lib.sgx_eos_stiff_gas_ref(C.byref(e), *p[:7]))
    elif kind == STIFF_GAS:
        check(lib.sgx_eos_stiff_gas(C.byref(e), *p[:4]))
    elif kind == NOBLE_ABEL and len(p) >= 7:
        check(lib.sgx_eos_noble_abel_ref(C.byref(e), *p[:7]))
    elif kind == NOBLE_ABEL:
        check(lib.sgx_eos_noble_abel(C.byref(e), *p[:4]))
    elif kind == GRUNEISEN:
        rho_max = p[10] if len(p) > 10 else 0.0
        check(lib.sgx_eos_gruneisen(C.byref(e), *p[:10], rho_max))
    else:
        raise ValueError(f"use spiner_eos() for model {kind}")
    return e


def spiner_eos(path, matid, reproducible=False):
    lib = load()
    e = SgxEos()
    check(lib.sgx_eos_spiner_rhot(C.byref(e), path.encode(), int(matid), int(reproducible)))
    return e


def spiner_rhosie_eos(path, matid, reproducible=False):
    """SpinerEOSDependsRhoSie from an sp5-lite image with rho-T and rho-sie
    groups (sp5lite.rhosie_table writes one)."""
    lib = load()
    e = SgxEos()
    check(lib.sgx_eos_spiner_rhosie(C.byref(e), path.encode(), int(matid), int(reproducible)))
    return e


def helmholtz_eos(path, options=HELM_DEFAULT):
    lib = load()
    e = SgxEos()
    check(lib.sgx_eos_helmholtz(C.byref(e), path.encode(), int(options)))
    return e


def modify(eos, shift=None, scale=None, ramp=None):
    """A copy of eos wrapped as the reference's modifiers nest:
    BilinearRamp(Scaled(Shifted(model))); ramp = (r0, a, b, c)."""
    lib = load()
    e = SgxEos.from_buffer_copy(eos)
    if shift is not None:
        check(lib.sgx_eos_modify_shifted(C.byref(e), float(shift)))
    if scale is not None:
        check(lib.sgx_eos_modify_scaled(C.byref(e), float(scale)))
    if ramp is not None:
        check(lib.sgx_eos_modify_bilinear_ramp(C.byref(e), *[float(v) for v in ramp]))
    return e


def p_alpha_ramp_params(eos, alpha0, Pe, Pc):
    """pAlpha2BilinearRampParams: (r0, a, b, c) of the ramp through the
    p-alpha crush curve of eos."""
    out = [C.c_double() for _ in range(4)]
    check(load().sgx_eos_p_alpha_ramp_params(C.byref(eos), float(alpha0), float(Pe), float(Pc),
                                             *[C.byref(o) for o in out]))
    return tuple(o.value for o in out)


def apply_modifiers(eos, enabled, vals):
    """The modifier step of the reference's init_sg_* on a bare model:
    returns (modified copy, vals as the call leaves them)."""
    e = SgxEos.from_buffer_copy(eos)
    en = (C.c_int * 4)(*[int(v) for v in enabled])
    vv = (C.c_double * 6)(*[float(v) for v in vals])
    check(load().sgx_eos_apply_modifiers(C.byref(e), en, vv))
    return e, list(vv)


def pt_derivatives(eos, rho, sie, press, temp, lam=None, lam_stride=0, stream=None):
    """PTDerivativesFromPreferred per element of device tensors: returns
    (dedP_T, drdP_T, dedT_P, drdT_P)."""
    import torch
    out = [torch.empty_like(rho) for _ in range(4)]
    check(load().sgx_eos_pt_derivatives(C.byref(eos), rho.numel(), ptr(rho), ptr(sie),
                                        ptr(press), ptr(temp), *[ptr(o) for o in out],
                                        ptr(lam), lam_stride, stream_ptr(stream)))
    return tuple(out)


def mix_params(**kw):
    m = MixParams()
    check(load().sgx_mix_params_default(C.byref(m)))
    for k, v in kw.items():
        setattr(m, k, v)
    return m


def eval_eos(eos, fn, in1, in2, out, lam=None, lam_stride=0, stream=None):
    n = in1.numel()
    check(load().sgx_eos_eval(C.byref(eos), fn, n, ptr(in1), ptr(in2), ptr(out), ptr(lam),
                              lam_stride, stream_ptr(stream)))


def eos_bounds(eos, what, out, temp=None, stream=None):
    """out[i] = the model's bound `what` (BOUND_*), at temp[i] for the
    temperature-dependent two."""
    check(load().sgx_eos_bounds(C.byref(eos), int(what), out.numel(), ptr(temp), ptr(out),
                                stream_ptr(stream)))


def fill_eos(eos, rho, temp, sie, press, cv, bmod, output, lam=None, lam_stride=0, stream=None,
             cs=None, precision=PREC_FP64):
    n = rho.numel()
    if cs is None and precision == PREC_FP64:
        check(load().sgx_eos_fill(C.byref(eos), n, ptr(rho), ptr(temp), ptr(sie), ptr(press),
                                  ptr(cv), ptr(bmod), output, ptr(lam), lam_stride,
                                  stream_ptr(stream)))
    else:
        check(load().sgx_eos_fill_ex(C.byref(eos), n, ptr(rho), ptr(temp), ptr(sie),
                                     ptr(press), ptr(cv), ptr(bmod), ptr(cs), output, ptr(lam),
                                     lam_stride, precision, stream_ptr(stream)))


def fill_eos_host(eos, rho, temp, sie, press, cv, bmod, output, lam=None, lam_stride=0,
                  cs=None, precision=PREC_FP64):
    """FillEos over host numpy arrays (float64, contiguous), streamed through
    the device by the library."""
    def p(a):
        return None if a is None else C.c_void_p(a.ctypes.data)
    check(load().sgx_eos_fill_host(C.byref(eos), rho.size, p(rho), p(temp), p(sie), p(press),
                                   p(cv), p(bmod), p(cs), output, p(lam), lam_stride,
                                   precision))


def pte_solve(solver, eos_list, eos_idx, vfrac_tot, sie_tot, rho, vfrac, sie, temp, press,
              lam=None, params=None, status=None, precision=PREC_FP64, stream=None):
    """Per-cell PTE on device tensors; per-material tensors are [nmat, ncell]
    float64 (updated in place); status is a uint8 tensor of ncell*16 bytes."""
    nmat, ncell = rho.shape
    arr = (SgxEos * len(eos_list))(*eos_list)
    check(load().sgx_pte_solve(
        solver, nmat, ncell, C.cast(arr, C.c_void_p), len(eos_list), ptr(eos_idx),
        ptr(vfrac_tot), ptr(sie_tot), ptr(rho), ptr(vfrac), ptr(sie), ptr(temp), ptr(press),
        ptr(lam), C.byref(params) if params is not None else None, ptr(status), precision,
        stream_ptr(stream)))


def tune_set(knob, value):
    """sgx_tune_set: a process-wide launch or iteration knob (TUNE_*);
    raises on a value outside the knob's range."""
    check(load().sgx_tune_set(int(knob), int(value)))


def tune_get(knob):
    """sgx_tune_get: the knob's current value."""
    v = C.c_int()
    check(load().sgx_tune_get(int(knob), C.byref(v)))
    return v.value


def autotune_fill(eos, rho, temp, sie, press, cv, bmod, output, cs=None, lam=None,
                  lam_stride=0, reps=3, stream=None):
    """sgx_tune_autotune_fill on device tensors: returns the (blocks per SM,
    staging) pair it kept."""
    b, st = C.c_int(), C.c_int()
    check(load().sgx_tune_autotune_fill(
        C.byref(eos), rho.numel(), ptr(rho), ptr(temp), ptr(sie), ptr(press), ptr(cv), ptr(bmod),
        ptr(cs), output, ptr(lam), lam_stride, reps, C.byref(b), C.byref(st),
        stream_ptr(stream)))
    return b.value, st.value


def autotune_pte(eos_list, eos_idx, vfrac_tot, sie_tot, rho, vfrac, sie, temp, press,
                 lam=None, params=None, status=None, reps=2, tune_group=True, stream=None):
    """sgx_tune_autotune_pte on device tensors: returns the (block, count
    order, group_min_n) it kept; the arrays end holding that setting's solve."""
    nmat, ncell = rho.shape
    arr = (SgxEos * len(eos_list))(*eos_list)
    chosen = (C.c_int * 3)()
    check(load().sgx_tune_autotune_pte(
        nmat, ncell, C.cast(arr, C.c_void_p), len(eos_list), ptr(eos_idx), ptr(vfrac_tot),
        ptr(sie_tot), ptr(rho), ptr(vfrac), ptr(sie), ptr(temp), ptr(press), ptr(lam),
        C.byref(params) if params is not None else None, ptr(status), reps,
        1 if tune_group else 0, chosen, stream_ptr(stream)))
    return tuple(chosen)


class PtePlan:
    """sgx_pte_plan over device tensors (kept alive with the plan): one
    solve captured as a CUDA graph; run() replays it on the tensors'
    current contents."""

    def __init__(self, solver, eos_list, eos_idx, vfrac_tot, sie_tot, rho, vfrac, sie, temp,
                 press, lam=None, params=None, status=None, precision=PREC_FP64):
        nmat, ncell = rho.shape
        self._keep = (eos_idx, vfrac_tot, sie_tot, rho, vfrac, sie, temp, press, lam, status)
        arr = (SgxEos * len(eos_list))(*eos_list)
        self._h = C.c_void_p()
        check(load().sgx_pte_plan_create(
            solver, nmat, ncell, C.cast(arr, C.c_void_p), len(eos_list), ptr(eos_idx),
            ptr(vfrac_tot), ptr(sie_tot), ptr(rho), ptr(vfrac), ptr(sie), ptr(temp), ptr(press),
            ptr(lam), C.byref(params) if params is not None else None, ptr(status), precision,
            C.byref(self._h)))

    def run(self, stream=None):
        check(load().sgx_pte_plan_run(self._h, stream_ptr(stream)))

    def close(self):
        if self._h:
            load().sgx_pte_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def approx_temperature(eos_list, eos_idx, u_tot, rho, vfrac, temp_out, Tguess=None, lam=None,
                       stream=None):
    """ApproxTemperatureFromRhoMatU per cell on device tensors."""
    nmat, ncell = rho.shape
    arr = (SgxEos * len(eos_list))(*eos_list)
    check(load().sgx_pte_approx_temperature(
        nmat, ncell, C.cast(arr, C.c_void_p), len(eos_list), ptr(eos_idx), ptr(u_tot), ptr(rho),
        ptr(vfrac), ptr(Tguess), ptr(lam), ptr(temp_out), stream_ptr(stream)))


def enforce_mass_volumes_sum(eos_idx, tot_vol, rho, vfrac, stream=None):
    """MixUtils::EnforceMassVolumesSum per cell on device tensors."""
    nmat, ncell = rho.shape
    check(load().sgx_mix_enforce_mass_volumes_sum(nmat, ncell, ptr(eos_idx), ptr(tot_vol),
                                                  ptr(rho), ptr(vfrac), stream_ptr(stream)))


def enforce_energies_sum(eos_idx, tot_rho, tot_sie, rho, vfrac, sie, stream=None):
    """MixUtils::EnforceEnergiesSum per cell on device tensors."""
    nmat, ncell = rho.shape
    check(load().sgx_mix_enforce_energies_sum(nmat, ncell, ptr(eos_idx), ptr(tot_rho),
                                              ptr(tot_sie), ptr(rho), ptr(vfrac), ptr(sie),
                                              stream_ptr(stream)))


def pte_solve_noalloc(eos_list, eos_idx, vfrac_tot, sie_tot, rho, vfrac, sie, temp, press,
                      lam=None, params=None, status=None, stream=None):
    """pte_solve(PTE_RHOT, ..., precision=PREC_MIXED) through the entry point
    whose scratch is a static device array (at most PTE_NOALLOC_MAX_CELLS
    cells; calls must not overlap in time on one device)."""
    nmat, ncell = rho.shape
    arr = (SgxEos * len(eos_list))(*eos_list)
    check(load().sgx_pte_solve_noalloc(
        PTE_RHOT, nmat, ncell, C.cast(arr, C.c_void_p), len(eos_list), ptr(eos_idx),
        ptr(vfrac_tot), ptr(sie_tot), ptr(rho), ptr(vfrac), ptr(sie), ptr(temp), ptr(press),
        ptr(lam), C.byref(params) if params is not None else None, ptr(status),
        stream_ptr(stream)))


class Server:
    """The serving loop (sgx_server_*). Request arrays are host numpy arrays
    (page-locked ones, e.g. from torch pin_memory, let copies overlap);
    they must stay alive until wait() returns for the ticket."""

    def __init__(self, eos_list, hbm_budget_bytes=1 << 30, max_inflight=8,
                 precision=PREC_MIXED, solver=PTE_RHOT, params=None):
        self.h = None  # set once sgx_server_create succeeds; close() checks it
        lib = load()
        self._eos = (SgxEos * len(eos_list))(*eos_list)
        self._params = params
        cfg = ServerConfig(hbm_budget_bytes, max_inflight, solver, precision,
                           C.cast(self._eos, C.c_void_p), len(eos_list),
                           C.cast(C.byref(params), C.c_void_p) if params is not None else None)
        h = C.c_void_p()
        check(lib.sgx_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, req):
        """req: dict with nmat, ncell, eos_idx (or None), vfrac_tot, sie_tot,
        the five *_in and five *_out arrays and status (or None)."""
        def p(a):
            return None if a is None else C.c_void_p(a.ctypes.data)
        r = PteRequest(req["nmat"], req["ncell"], p(req.get("eos_idx")), p(req["vfrac_tot"]),
                       p(req["sie_tot"]), *(p(req[k + "_in"]) for k in
                                            ("rho", "vfrac", "sie", "temp", "press")),
                       *(p(req[k + "_out"]) for k in ("rho", "vfrac", "sie", "temp", "press")),
                       p(req.get("status")))
        t = C.c_uint64()
        check(load().sgx_server_submit(self.h, C.byref(r), C.byref(t)))
        self._keep[t.value] = req
        return t.value

    def wait(self, ticket, timeout=-1.0):
        """Returns the submit-to-completion latency in seconds, or None on
        timeout."""
        lat = C.c_double()
        rc = load().sgx_server_wait(self.h, ticket, timeout, C.byref(lat))
        if rc == 6:
            return None
        self._keep.pop(ticket, None)
        check(rc)
        return lat.value

    def stats(self):
        st = ServerStats()
        check(load().sgx_server_stats_get(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self):
        if self.h:
            load().sgx_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def get_sg_eos(eos_list, eos_offsets, offsets, cells, fracs, mass_frac_cutoff,
               precision=PREC_FP64, input_int=1, stream=None):
    """get_sg_eos over device tensors. cells: dict of the nine [cell_dim]
    arrays (press, pmax, vol, spvol, sie, temp, bmod, dpde, cv); fracs: dict
    of [nmat, cell_dim] arrays (frac_mass, frac_vol, frac_ie and optionally
    frac_bmod, frac_dpde, frac_cv); eos_offsets: 1-based host ints."""
    nmat, cell_dim = fracs["frac_mass"].shape
    arr = (SgxEos * len(eos_list))(*eos_list)
    eo = (C.c_int * nmat)(*[int(x) for x in eos_offsets])
    check(load().sgx_get_sg_eos_device(
        nmat, offsets.numel(), cell_dim, input_int, C.cast(eo, C.c_void_p),
        C.cast(arr, C.c_void_p), len(eos_list), ptr(offsets),
        *(ptr(cells[k]) for k in ("press", "pmax", "vol", "spvol", "sie", "temp", "bmod",
                                  "dpde", "cv")),
        *(ptr(fracs.get(k)) for k in ("frac_mass", "frac_vol", "frac_ie", "frac_bmod",
                                      "frac_dpde", "frac_cv")),
        mass_frac_cutoff, precision, stream_ptr(stream)))


def get_sg_eos_host(eos_list, eos_offsets, offsets, cells, fracs, mass_frac_cutoff,
                    precision=PREC_FP64, input_int=1):
    """get_sg_eos over host numpy arrays (contiguous; int32 offsets, float64
    fields), updated in place, as the reference's interface takes them."""
    nmat, cell_dim = fracs["frac_mass"].shape
    arr = (SgxEos * len(eos_list))(*eos_list)
    eo = (C.c_int * nmat)(*[int(x) for x in eos_offsets])

    def p(a):
        return None if a is None else C.c_void_p(a.ctypes.data)
    check(load().sgx_get_sg_eos(
        nmat, offsets.size, cell_dim, input_int, C.cast(eo, C.c_void_p),
        C.cast(arr, C.c_void_p), len(eos_list), p(offsets),
        *(p(cells[k]) for k in ("press", "pmax", "vol", "spvol", "sie", "temp", "bmod",
                                "dpde", "cv")),
        *(p(fracs.get(k)) for k in ("frac_mass", "frac_vol", "frac_ie", "frac_bmod",
                                    "frac_dpde", "frac_cv")),
        mass_frac_cutoff, precision, None))


def status_view(status_u8):
    """Splits a [ncell*16] uint8 status tensor (on host) into numpy fields."""
    import numpy as np
    raw = status_u8.cpu().numpy().view(np.uint8).reshape(-1, 16)
    residual = raw[:, 0:8].copy().view(np.float64).ravel()
    niter = raw[:, 8:12].copy().view(np.int32).ravel()
    return dict(residual=residual, niter=niter, converged=raw[:, 12].astype(bool),
                slow=raw[:, 13].astype(bool), max_line_niter=raw[:, 14],
                small_step_iters=raw[:, 15] & 0x3F, resolved_fp64=(raw[:, 15] & 0x40) != 0,
                error=(raw[:, 15] & 0x80) != 0)
