"""CPU-side checks: the C-ABI library builds, loads and exports every symbol
include/sgx.h declares; host-side argument validation returns error codes
without touching a GPU; the table writer and NQT transforms are bit-exact."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from sgx import lib as L
from sgx import sp5lite

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "sgx.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(sgx_[A-Za-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(L.LIB_PATH):
        pytest.skip("libsgx.so not built")
    try:
        return L.load()
    except OSError as e:  # e.g. no libcudart on a CPU-only machine
        pytest.skip(f"cannot load libsgx.so here: {e}")


def test_header_declares_the_binding_list():
    assert set(L.EXPORTED) <= set(declared_symbols())


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_constructors_and_validation_need_no_gpu(lib):
    e = L.SgxEos()
    assert lib.sgx_eos_ideal_gas(C.byref(e), 0.4, 0.718e7) == 0
    assert e.type == L.IDEAL_GAS and e.p[0] == 0.4
    assert lib.sgx_eos_ideal_gas(C.byref(e), -1.0, 1.0) == 1  # CheckParams
    assert lib.sgx_eos_gruneisen(C.byref(e), 3.94e5, 1.489, 0, 0, 2.02, 0.47, 8.93, 298.0,
                                 0.0, 3.9e6, 0.0) == 0
    # rho_max = 0.99 * rho0 / ((1 - 1/s1) + eps)  (eos_gruneisen.hpp:235-236, 321-322)
    assert e.p[10] == 0.99 * (8.93 / ((1 - 1 / 1.489) + 10 * np.finfo(float).eps))
    # bad solver / sizes fail before any device work
    arr = (L.SgxEos * 1)(e)
    rc = lib.sgx_pte_solve(7, 1, 10, C.cast(arr, C.c_void_p), 1, *([None] * 10), None, 0, None)
    assert rc == 1
    rc = lib.sgx_pte_solve(0, 7, 10, C.cast(arr, C.c_void_p), 1, *([None] * 10), None, 0, None)
    assert rc == 5
    assert lib.sgx_pte_solve(0, 1, 0, C.cast(arr, C.c_void_p), 1, *([None] * 10), None, 0,
                             None) == 0  # empty batch
    assert lib.sgx_eos_eval(C.byref(e), 99, 4, None, None, None, None, 0, None) == 1
    assert b"bad fn" in lib.sgx_last_error()
    m = L.MixParams()
    assert lib.sgx_mix_params_default(C.byref(m)) == 0
    assert m.pte_max_iter_per_mat == 128 and m.line_search_max_iter == 6
    assert lib.sgx_pte_rhot_required_scratch(5) == 25 + 20 + 30
    assert lib.sgx_pte_pt_required_scratch(3) == 4 + 8 + 6
    # PTESolverFixedT/FixedP/RhoURequiredScratch (mixed_cell_models.hpp:1451-1457,
    # 1665-1671, 1924-1929)
    assert lib.sgx_pte_fixed_t_required_scratch(3) == 9 + 12 + 6 + 6
    assert lib.sgx_pte_fixed_p_required_scratch(3) == 16 + 16 + 6 + 9
    assert lib.sgx_pte_rhou_required_scratch(3) == 36 + 24 + 24
    # the ...InBytes companions
    assert lib.sgx_pte_required_scratch_bytes(0, 5) == 8 * (25 + 20 + 30)
    assert lib.sgx_pte_required_scratch_bytes(2, 3) == 8 * (36 + 24 + 24)
    assert lib.sgx_pte_required_scratch_bytes(9, 3) == 0
    # mixed precision is for PTESolverRhoT only
    rc = lib.sgx_pte_solve(3, 1, 10, C.cast(arr, C.c_void_p), 1, *([None] * 10), None, 1, None)
    assert rc == 5


def test_missing_table_reports_io_error(lib, tmp_path):
    e = L.SgxEos()
    rc = lib.sgx_eos_spiner_rhot(C.byref(e), str(tmp_path / "nope.sp5").encode(), 1, 0)
    assert rc in (3, 4)  # no device here, or unreadable file


def test_nqt_transforms_are_near_inverses():
    x = np.exp(np.random.default_rng(0).uniform(-30, 30, 10000))
    # pow10(log10(x)) returns x up to the rounding of the log2/log10 factors
    # (logs.hpp:188-214, 282-292)
    y = sp5lite.pow10_nqt(sp5lite.log10_nqt(x))
    assert np.max(np.abs(y - x) / x) < 1e-13


def test_table_image_is_deterministic(tmp_path):
    a, b = tmp_path / "a.sp5", tmp_path / "b.sp5"
    sp5lite.stiffgas_table(str(a))
    sp5lite.stiffgas_table(str(b))
    assert a.read_bytes() == b.read_bytes()


def test_helm_table_is_reproducible(tmp_path):
    """The synthetic Helmholtz table is bit-identical to the one the golden
    fixture was made with (decimal arithmetic for the node transcendentals,
    only + - * / on arrays)."""
    from common import golden
    from sgx import helmtable
    sha = helmtable.helm_table(str(tmp_path / "helm_table.dat"))
    assert sha == str(golden("helmholtz")["table_sha256"])


def test_helm_table_derivatives_are_exact():
    """Every tabulated derivative is the derivative of the free energy (the
    Hermite interpolation relies on it), checked symbolically."""
    sp = pytest.importorskip("sympy")
    import mpmath
    from sgx import helmtable as H
    d, T = sp.symbols("d T", positive=True)
    a23 = sp.Rational(2, 3)
    F = (-H.A_GAS * T * (sp.Rational(3, 2) * sp.log(T) - sp.log(d) + H.C0)
         + H.K_DEG * d**a23 - H.B_TH * T**2 / (d**a23 + H.D0))
    P = d**2 * sp.diff(F, d)
    eta = sp.log(d) - sp.Rational(3, 2) * sp.log(T) + H.C1 + H.K2 * d**a23 / T
    X = H.NA * d + H.X0 * T**3
    want = [[F, sp.diff(F, d), sp.diff(F, T), sp.diff(F, d, 2), sp.diff(F, T, 2),
             sp.diff(F, d, T), sp.diff(F, d, 2, T), sp.diff(F, d, T, 2), sp.diff(F, d, 2, T, 2)],
            [sp.diff(P, d), sp.diff(P, d, 2), sp.diff(P, d, T), sp.diff(P, d, 2, T)],
            [eta, sp.diff(eta, d), sp.diff(eta, T), sp.diff(eta, d, T)],
            [X, sp.diff(X, d), sp.diff(X, T), sp.diff(X, d, T)]]
    blocks = H._fields()
    mpmath.mp.dps = 40
    for j, i in ((0, 0), (40, 100), (70, 200), (100, 270), (13, 137)):
        (dv, _, _, _, _, _), (tv, _) = H._node_values()
        dd, tt = float(dv.ravel()[i]), float(tv.ravel()[j])
        for exprs, blk in zip(want, blocks):
            for e, v in zip(exprs, blk):
                ref = float(sp.lambdify((d, T), e, "mpmath")(mpmath.mpf(dd), mpmath.mpf(tt)))
                assert abs(v[j, i] - ref) <= 1e-11 * max(abs(ref), 1e-300) + 1e-300, (j, i)


def test_modifier_checks_without_gpu():
    # the modifier calls are host-side value edits with the wrappers'
    # CheckParams; no device is touched
    from sgx import lib as L
    L.load()
    e = L.make_eos(L.IDEAL_GAS, (0.5, 2.0))
    m = L.modify(e, shift=0.1, scale=2.0)
    assert (m.mods, m.shift, m.scale, m.inv_scale) == (3, 0.1, 2.0, 0.5)
    r = L.modify(m, ramp=(1.0, 3.0, 1.0, 0.5))
    assert r.mods == 7
    # rmid = r0 (a - b c) / (a - b), Pmid = a (rmid / r0 - 1)
    assert list(r.ramp) == [1.0, 3.0, 1.0, 0.5, 1.0 * (3.0 - 1.0 * 0.5) / (3.0 - 1.0),
                            3.0 * (1.0 * (3.0 - 1.0 * 0.5) / (3.0 - 1.0) / 1.0 - 1.0)]
    with pytest.raises(RuntimeError, match="sgx error 5"):
        L.modify(m, shift=1.0)  # Shifted<Scaled<...>> is not in the variant
    with pytest.raises(RuntimeError, match="sgx error 5"):
        L.modify(r, scale=2.0)
    with pytest.raises(RuntimeError, match="sgx error 1"):
        L.modify(e, scale=0.0)
    with pytest.raises(RuntimeError, match="sgx error 1"):
        L.modify(e, shift=float("nan"))
    with pytest.raises(RuntimeError, match="sgx error 1"):
        L.modify(e, ramp=(1.0, 2.0, 2.0, 0.0))  # a == b
    with pytest.raises(RuntimeError, match="sgx error 1"):
        L.modify(e, ramp=(0.0, 2.0, 1.0, 0.0))  # r0 > 0
    # nothing enabled: the value comes back unchanged; a modified value is
    # not accepted
    same, vals = L.apply_modifiers(e, [0, 0, 0, 0], [0.0] * 6)
    assert same.mods == 0 and vals == [0.0] * 6
    with pytest.raises(RuntimeError, match="sgx error 1"):
        L.apply_modifiers(m, [1, 0, 0, 0], [2.0, 0, 0, 0, 0, 0])
    # shift and scale without a ramp need no device
    sc, _ = L.apply_modifiers(e, [1, 1, 0, 0], [2.0, 0.1, 0, 0, 0, 0])
    assert (sc.mods, sc.scale, sc.shift) == (3, 2.0, 0.1)


def test_init_sg_interface_without_gpu():
    # init_sg_eos / init_sg_<model> / finalize_sg_eos (singularity_eos.cpp)
    # over sgx_eos values; shift and scale need no device
    from sgx import lib as L
    lib = L.load()
    arr = C.POINTER(L.SgxEos)()
    assert lib.sgx_init_sg_eos(3, C.byref(arr)) == 0
    assert lib.sgx_init_sg_IdealGas(0, arr, 0.4, 0.718e7, None, None) == 0
    en = (C.c_int * 4)(1, 1, 0, 0)
    vals = (C.c_double * 6)(2.0, 0.1, 0, 0, 0, 0)
    assert lib.sgx_init_sg_StiffGas(1, arr, 3.4, 1.816e7, 6e9, 0.0, en, vals) == 0
    assert lib.sgx_init_sg_NobleAbel(2, arr, 0.4, 0.718e7, 1e-3, 0.0, None, None) == 0
    assert (arr[0].type, arr[0].mods) == (L.IDEAL_GAS, 0)
    assert (arr[1].type, arr[1].mods, arr[1].scale, arr[1].shift) == (L.STIFF_GAS, 3, 2.0, 0.1)
    assert arr[2].type == L.NOBLE_ABEL
    assert lib.sgx_init_sg_IdealGas(-1, arr, 0.4, 1.0, None, None) == 1  # matindex < 0
    assert lib.sgx_init_sg_SpinerDependsRhoT(0, arr, b"x.sp5", 1, 1, None, None) == 5
    assert lib.sgx_finalize_sg_eos(3, C.byref(arr)) == 0
    assert not arr


def test_plan_and_derivative_argument_checks_without_gpu():
    # argument errors come back before any CUDA call
    from sgx import lib as L
    lib = L.load()
    e = L.make_eos(L.IDEAL_GAS, (0.4, 0.718e7))
    arr = (L.SgxEos * 1)(e)
    out = C.c_void_p()
    # bad solver, bad precision, null arrays
    assert lib.sgx_pte_plan_create(9, 1, 8, C.cast(arr, C.c_void_p), 1, None, None, None, None,
                                   None, None, None, None, None, None, None, 0,
                                   C.byref(out)) == 1
    assert lib.sgx_pte_plan_create(0, 1, 8, C.cast(arr, C.c_void_p), 1, None, None, None, None,
                                   None, None, None, None, None, None, None, 7,
                                   C.byref(out)) == 1
    assert lib.sgx_pte_plan_create(0, 1, 8, C.cast(arr, C.c_void_p), 1, None, None, None, None,
                                   None, None, None, None, None, None, None, 0,
                                   C.byref(out)) == 1
    assert not out.value
    assert lib.sgx_pte_plan_run(None, None) == 1
    assert lib.sgx_pte_plan_destroy(None) == 0
    # PT derivatives: Helmholtz unsupported, null arrays invalid, n = 0 a no-op
    h = L.SgxEos()
    h.type = L.HELMHOLTZ if hasattr(L, "HELMHOLTZ") else 6
    assert lib.sgx_eos_pt_derivatives(C.byref(h), 4, *([None] * 9), 0, None) == 5
    assert lib.sgx_eos_pt_derivatives(C.byref(e), 4, *([None] * 9), 0, None) == 1
    assert lib.sgx_eos_pt_derivatives(C.byref(e), 0, *([None] * 9), 0, None) == 0
    # entropy of a model without one
    g = L.make_eos(L.GRUNEISEN, (3.94e5, 1.489, 0.0, 0.0, 2.02, 0.47, 8.93, 298.0, 0.0, 3.9e6))
    assert lib.sgx_eos_eval(C.byref(g), 11, 4, C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                            None, 0, None) == 5



def test_tuning_knobs_hold_their_documented_ranges(lib):
    """sgx_tune_set / sgx_tune_get (host only): every knob of sgx.h takes
    the values of its documented range and refuses the ones outside it,
    leaving the value unchanged; unknown knobs are refused."""
    ranges = {L.TUNE_LOOKUP_BLOCKS_PER_SM: (4, 6), L.TUNE_LOOKUP_STAGE: (0, 2),
              L.TUNE_L2_PERSIST: (0, 1), L.TUNE_HOST_FILL_STAGED: (0, 1),
              L.TUNE_PTE_FP32_ITERS: (2, 64), L.TUNE_PTE_RETRY_ITERS: (4, 128),
              L.TUNE_PTE_COUNT_ORDER: (0, 1), L.TUNE_PTE_MIXED_BLOCK: (32, 128),
              L.TUNE_PTE_GROUP_MIN_N: (2, 7), L.TUNE_PTE_FP32_TOL: (3, 6),
              L.TUNE_HELM_PASS1_STEPS: (0, 100), L.TUNE_HELM_MID_STEPS: (0, 100),
              L.TUNE_HELM_MID2_STEPS: (0, 100)}
    for knob, (lo, hi) in ranges.items():
        v = C.c_int()
        assert lib.sgx_tune_get(knob, C.byref(v)) == 0
        keep = v.value
        try:
            for x in (lo, hi):
                assert lib.sgx_tune_set(knob, x) == 0, (knob, x)
                assert lib.sgx_tune_get(knob, C.byref(v)) == 0 and v.value == x
            for x in (lo - 1, hi + 1):
                assert lib.sgx_tune_set(knob, x) != 0, (knob, x)
                assert lib.sgx_tune_get(knob, C.byref(v)) == 0 and v.value == hi
        finally:
            lib.sgx_tune_set(knob, keep)
    for knob in (0, max(ranges) + 1, -1):
        assert lib.sgx_tune_set(knob, 1) != 0
        assert lib.sgx_tune_get(knob, C.byref(C.c_int())) != 0


def test_python_tune_wrappers(lib):
    """sgx.lib.tune_set / tune_get over the C calls: a value in range is
    kept, one outside raises and leaves it."""
    keep = L.tune_get(L.TUNE_HELM_MID_STEPS)
    try:
        L.tune_set(L.TUNE_HELM_MID_STEPS, 30)
        assert L.tune_get(L.TUNE_HELM_MID_STEPS) == 30
        with pytest.raises(RuntimeError):
            L.tune_set(L.TUNE_HELM_MID_STEPS, 101)
        assert L.tune_get(L.TUNE_HELM_MID_STEPS) == 30
    finally:
        L.tune_set(L.TUNE_HELM_MID_STEPS, keep)
