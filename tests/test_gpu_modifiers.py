"""ShiftedEOS, ScaledEOS and BilinearRampEOS on the device, through the C
ABI, against golden fixtures made from the compiled reference
(tests/golden/make_golden.py: modifiers, pte_rhot_modified, pte_pt_modified).

The wrapped evaluations are plain FP64 arithmetic on both sides, without
contraction, so vector lookups, FillEos and the PTE solves are expected bit
for bit (checked within 1e-12 relative, the plain path's bar, with the
bitwise fraction reported). pAlpha2BilinearRampParams takes the exp and log
of its bracket from the host's C library, which may round differently on
another machine: its parameters are checked within 1e-12 relative, the
tolerance of the reference's own test."""
import ctypes as C

import numpy as np
import pytest

from common import PARITY_RTOL, bitwise_frac, golden, materials_from_rows, rel_err
from common import stiffgas_table_path

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

ALL_FN = list(range(11))
Q_DENSITY, Q_SIE, Q_PRESSURE, Q_TEMPERATURE, Q_CV, Q_BMOD = 1, 2, 4, 8, 16, 32
Q_TPB = Q_TEMPERATURE | Q_PRESSURE | Q_BMOD | Q_CV
PALPHA_RTOL = 1e-12


@pytest.fixture(scope="module")
def sgx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sgx import lib
    lib.load()
    return lib


@pytest.fixture(scope="module")
def table(sgx):
    path, sha = stiffgas_table_path()
    assert sha == str(golden("modifiers")["table_sha256"]), "table generation is not reproducible"
    t = sgx.spiner_eos(path, 1)
    yield t
    sgx.load().sgx_eos_finalize(C.byref(t))


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def wrap(sgx, base, row):
    bits = int(row[0])
    return sgx.modify(base, shift=row[1] if bits & 1 else None,
                      scale=row[2] if bits & 2 else None,
                      ramp=row[3:7] if bits & 4 else None)


def case_eos(sgx, table, mat, row):
    base = table if mat[0] == 5 else sgx.make_eos(*mat)
    return wrap(sgx, base, row)


def close(a, b, label):
    err = rel_err(a, b)
    assert err.max() <= PARITY_RTOL, f"{label}: max rel err {err.max():.3e}"
    return bitwise_frac(a, b)


def test_modified_vector_lookups(sgx, table):
    fx = golden("modifiers")
    mats = materials_from_rows(fx["materials"])
    worst = 1.0
    for k, (mat, row) in enumerate(zip(mats, fx["mods"])):
        e = case_eos(sgx, table, mat, row)
        rho, sie, T = (dev(fx[f"c{k}_{q}"]) for q in ("rho", "sie", "T"))
        for fn in ALL_FN:
            out = torch.empty_like(rho)
            sgx.eval_eos(e, fn, rho, T if fn in (1, 2, 4, 6, 8) else sie, out)
            torch.cuda.synchronize()
            worst = min(worst, close(out.cpu().numpy(), fx[f"c{k}_fn{fn}"], f"case {k} fn {fn}"))
    # the reference's own value: shifted by 0.1 then scaled by 2, P(2, 0.5) = 0.3
    assert fx["c0_fn3"][0] == 0.3
    print(f"modified lookups: worst bitwise fraction {worst:.4f}")


def test_modified_fill(sgx, table):
    fx = golden("modifiers")
    mats = materials_from_rows(fx["materials"])
    for k, (mat, row) in enumerate(zip(mats, fx["mods"])):
        e = case_eos(sgx, table, mat, row)
        for tag, output in (("fill", Q_TPB), ("fillrho", Q_DENSITY | Q_SIE)):
            if f"c{k}_{tag}_rho" not in fx:
                continue
            n = fx[f"c{k}_rho"].size
            if tag == "fill":
                a = dict(rho=fx[f"c{k}_rho"], temp=np.zeros(n), sie=fx[f"c{k}_sie"],
                         press=np.zeros(n), cv=np.zeros(n), bmod=np.zeros(n))
            else:
                a = dict(rho=np.zeros(n), temp=fx[f"c{k}_T"], sie=np.zeros(n),
                         press=fx[f"c{k}_fillrho_P"], cv=np.zeros(n), bmod=np.zeros(n))
            t = {q: dev(v) for q, v in a.items()}
            sgx.fill_eos(e, t["rho"], t["temp"], t["sie"], t["press"], t["cv"], t["bmod"], output)
            torch.cuda.synchronize()
            # a modified EOS writes back every array (the reference's FillEos
            # takes them all by reference): compare all six
            for q in a:
                close(t[q].cpu().numpy(), fx[f"c{k}_{tag}_{q}"], f"case {k} {tag} {q}")


def test_shifted_ideal_gas_fill_leaves_arrays(sgx):
    # ShiftedEOS::FillEos aborts in the reference for IdealGas, whose
    # PreferredInput has all four bits; the element is left as it was
    e = sgx.modify(sgx.make_eos(1, (0.5, 2.0)), shift=0.1)
    n = 64
    rho, sie = dev(np.linspace(0.5, 2.0, n)), dev(np.linspace(0.1, 1.0, n))
    temp, press, cv, bmod = (dev(np.full(n, 7.0)) for _ in range(4))
    sgx.fill_eos(e, rho, temp, sie, press, cv, bmod, Q_TPB)
    torch.cuda.synchronize()
    for t in (temp, press, cv, bmod):
        assert torch.all(t == 7.0)


def test_p_alpha_ramp_params(sgx, table):
    fx = golden("modifiers")
    mats = materials_from_rows(fx["materials"])
    n = 0
    for k, (mat, row) in enumerate(zip(mats, fx["mods"])):
        if f"c{k}_palpha" not in fx:
            continue
        e = case_eos(sgx, table, mat, np.concatenate([[int(row[0]) & 3], row[1:3], np.zeros(4)]))
        got = sgx.p_alpha_ramp_params(e, *fx[f"c{k}_palpha_in"])
        np.testing.assert_allclose(got, fx[f"c{k}_palpha"], rtol=PALPHA_RTOL)
        n += 1
    assert n == 5
    # a bracket end root: infinite slope, as in the reference
    got = sgx.p_alpha_ramp_params(table, *fx["palpha_edge_in"])
    np.testing.assert_allclose(got, fx["palpha_edge"], rtol=PALPHA_RTOL)


def test_apply_modifiers_matches_init_sg(sgx):
    fx = golden("modifiers")
    mats = materials_from_rows(fx["init_materials"])
    rng = np.random.default_rng(9)
    for mat, en, vin, vout in zip(mats, fx["init_enabled"], fx["init_vals_in"],
                                  fx["init_vals_out"]):
        e, vals = sgx.apply_modifiers(sgx.make_eos(*mat), en, vin)
        np.testing.assert_allclose(vals, vout, rtol=PALPHA_RTOL, atol=0)
        bits = (2 if en[0] == 1 else 0) | (1 if en[1] == 1 else 0) | \
            (4 if (en[2] == 1 or en[3] == 1) else 0)
        assert e.mods == bits
        if bits & 4:
            assert list(e.ramp)[:4] == list(vals[2:6])
        # the modified value evaluates as modify() of the same parameters
        ref = sgx.modify(sgx.make_eos(*mat), shift=vals[1] if bits & 1 else None,
                         scale=vals[0] if bits & 2 else None,
                         ramp=vals[2:6] if bits & 4 else None)
        rho = dev(np.exp(rng.uniform(-8, 3, 256)))
        T = dev(np.exp(rng.uniform(np.log(50.0), np.log(1e5), 256)))
        for fn in (1, 2, 6):
            a, b = torch.empty_like(rho), torch.empty_like(rho)
            sgx.eval_eos(e, fn, rho, T, a)
            sgx.eval_eos(ref, fn, rho, T, b)
            torch.cuda.synchronize()
            assert torch.equal(a, b)


@pytest.mark.parametrize("name", ["pte_rhot_modified", "pte_pt_modified"])
@pytest.mark.parametrize("shape", ["2mat", "batched"])
def test_pte_with_modified_materials(sgx, name, shape):
    fx = golden(name)
    solver = int(fx["solver"])
    mats = materials_from_rows(fx[f"{shape}_materials"])
    eos_list = [wrap(sgx, sgx.make_eos(*m), r) for m, r in zip(mats, fx[f"{shape}_mods"])]
    t = {k: dev(fx[f"{shape}_in_" + k]) for k in ("rho", "vfrac", "sie", "temp", "press")}
    idx = dev(fx[f"{shape}_eos_idx"], torch.int32) if f"{shape}_eos_idx" in fx else None
    ncell = fx[f"{shape}_sie_tot"].shape[0]
    status = torch.zeros(ncell * 16, dtype=torch.uint8, device="cuda")
    sgx.pte_solve(solver, eos_list, idx, dev(fx[f"{shape}_vfrac_tot"]),
                  dev(fx[f"{shape}_sie_tot"]), t["rho"], t["vfrac"], t["sie"], t["temp"],
                  t["press"], status=status)
    torch.cuda.synchronize()
    st = sgx.status_view(status)
    present = fx[f"{shape}_in_rho"] > 0
    for k in ("press", "temp", "sie", "vfrac", "rho"):
        a = t[k].cpu().numpy()[present]
        b = fx[f"{shape}_out_" + k][present]
        f = close(a, b, f"{name} {shape} {k}")
        print(f"{name} {shape} {k}: bitwise {f:.4f}")
    np.testing.assert_array_equal(st["converged"], fx[f"{shape}_converged"].astype(bool))
    np.testing.assert_array_equal(st["niter"], fx[f"{shape}_niter"])


def test_mixed_precision_rejects_modified_eos(sgx, table):
    # the mixed-precision lookup and PTE take bare models only
    e = sgx.modify(table, scale=1.5)
    rho = dev(np.ones(8))
    z = [dev(np.zeros(8)) for _ in range(5)]
    with pytest.raises(RuntimeError, match="unmodified EOS only"):
        sgx.fill_eos(e, rho, z[0], z[1], z[2], z[3], z[4], Q_TPB, precision=1)
    g = sgx.modify(sgx.make_eos(1, (0.4, 0.718e7)), shift=1e8)
    m = [dev(np.full((2, 8), 0.5)) for _ in range(5)]
    with pytest.raises(RuntimeError, match="unmodified EOS only"):
        sgx.pte_solve(0, [g, sgx.make_eos(1, (0.4, 0.718e7))], None, dev(np.ones(8)),
                      dev(np.full(8, 1e10)), *m, precision=1)


def test_pt_derivatives(sgx, table):
    # PTDerivativesFromPreferred for every model, bare and modified, at
    # consistent states (tests/golden/make_golden.py pt_derivs)
    fx = golden("pt_derivs")
    assert str(fx["table_sha256"]) == str(golden("modifiers")["table_sha256"])
    mats = materials_from_rows(fx["materials"])
    worst = 1.0
    for k, (mat, row) in enumerate(zip(mats, fx["mods"])):
        e = case_eos(sgx, table, mat, row)
        t = [dev(fx[f"c{k}_{q}"]) for q in ("rho", "sie", "P", "T")]
        lam = dev(np.full(2 * t[0].numel(), np.nan))
        got = sgx.pt_derivatives(e, *t, lam=lam, lam_stride=2)
        torch.cuda.synchronize()
        for j, name in enumerate(("dedP_T", "drdP_T", "dedT_P", "drdT_P")):
            worst = min(worst, close(got[j].cpu().numpy(), fx[f"c{k}_d"][j], f"case {k} {name}"))
        close(lam.cpu().numpy(), fx[f"c{k}_lambda"], f"case {k} lambda")
    # the ideal gas in closed form at the reference test's state
    # (test_eos_modifiers.cpp:160-167): shifted by 0.1, scaled by 2
    np.testing.assert_allclose(fx["c5_d"][:, 0], [0.0, 0.25, 4.0, -0.75], rtol=1e-15)
    print(f"PT derivatives: worst bitwise fraction {worst:.4f}")


def test_entropy_and_sie_from_rho_P(sgx, table):
    # EntropyFromDensityTemperature / EntropyFromDensityInternalEnergy
    # (fn 11, 12) and InternalEnergyFromDensityPressure (fn 13), bare and
    # modified (tests/golden/make_golden.py eos_vector_ext). Entropy goes
    # through log, whose CUDA and glibc results may differ in the last bit:
    # it is held to 1e-12 of the largest magnitude in the batch.
    fx = golden("eos_vector_ext")
    assert str(fx["table_sha256"]) == str(golden("modifiers")["table_sha256"])
    mats = materials_from_rows(fx["materials"])
    for k, (mat, row) in enumerate(zip(mats, fx["mods"])):
        e = case_eos(sgx, table, mat, row)
        rho = dev(fx[f"c{k}_rho"])
        for fn, second in ((11, "T"), (12, "sie"), (13, "P")):
            key = f"c{k}_fn{fn}"
            out = torch.empty_like(rho)
            if key not in fx:
                # Gruneisen and the table have no entropy
                with pytest.raises(RuntimeError, match="sgx error 5"):
                    sgx.eval_eos(e, fn, rho, dev(fx[f"c{k}_{second}"]), out)
                continue
            sgx.eval_eos(e, fn, rho, dev(fx[f"c{k}_{second}"]), out)
            torch.cuda.synchronize()
            got, ref = out.cpu().numpy(), fx[key]
            if fn == 13:
                close(got, ref, f"case {k} fn {fn}")
            else:
                np.testing.assert_allclose(got, ref, rtol=1e-12,
                                           atol=1e-12 * np.abs(ref).max(),
                                           err_msg=f"case {k} fn {fn}")


def test_entropy_with_reference_states(sgx):
    # the constructors with a reference state, at the reference's own test
    # states (the first rows) and at random ones
    fx = golden("eos_vector_ext")
    for j in range(3):
        e = sgx.make_eos(int(fx[f"r{j}_kind"]), tuple(fx[f"r{j}_params"]))
        rho = dev(fx[f"r{j}_rho"])
        for fn, second in ((11, "T"), (12, "sie")):
            out = torch.empty_like(rho)
            sgx.eval_eos(e, fn, rho, dev(fx[f"r{j}_{second}"]), out)
            torch.cuda.synchronize()
            ref = fx[f"r{j}_fn{fn}"]
            np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12,
                                       atol=1e-12 * np.abs(ref).max(),
                                       err_msg=f"ref case {j} fn {fn}")
    assert fx["r0_fn11"][0] == 0.0 and fx["r1_fn12"][0] == -2.0044437857420778e+08


def test_init_sg_and_get_sg_interface(sgx, table):
    # the reference's C interface: init_sg_<model> with the modifier step,
    # get_sg_* with and without a lambda indexer, finalize_sg_eos
    lib = sgx.load()
    fx = golden("modifiers")
    arr = C.POINTER(sgx.SgxEos)()
    assert lib.sgx_init_sg_eos(2, C.byref(arr)) == 0
    en = (C.c_int * 4)(*[int(v) for v in fx["init_enabled"][0]])
    vals = (C.c_double * 6)(*fx["init_vals_in"][0])
    assert lib.sgx_init_sg_IdealGas(0, arr, 0.5, 2.0, en, vals) == 0  # the p-alpha ramp
    np.testing.assert_allclose(list(vals), fx["init_vals_out"][0], rtol=PALPHA_RTOL)
    assert lib.sgx_init_sg_StiffGas(1, arr, 3.4, 1.816e7, 6e9, 0.0, None, None) == 0
    vec = golden("eos_vector")
    rho, sie = dev(vec["m1_rho"]), dev(vec["m1_sie"])
    out = torch.empty_like(rho)
    P = C.c_void_p
    n = rho.numel()
    for name, fn in (("Pressure", 3), ("BulkModulus", 7)):
        f = getattr(lib, f"sgx_get_sg_{name}FromDensityInternalEnergy")
        assert f(1, arr, P(rho.data_ptr()), P(sie.data_ptr()), P(out.data_ptr()), n, -1, None) == 0
        torch.cuda.synchronize()
        np.testing.assert_array_equal(out.cpu().numpy(), vec[f"m1_fn{fn}"])
    assert lib.sgx_get_sg_MinInternalEnergyFromDensity(1, arr, P(rho.data_ptr()),
                                                       P(out.data_ptr()), n) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), vec["m1_fn10"])
    assert lib.sgx_get_sg_EntropyFromDensityInternalEnergy(
        1, arr, P(rho.data_ptr()), P(sie.data_ptr()), P(out.data_ptr()), n, -1, None) == 0
    # the tabulated model through a lambda indexer (stride 2)
    assert lib.sgx_finalize_sg_eos(2, C.byref(arr)) == 0 and not arr
    spl = golden("spiner_lookup")
    arr2 = (sgx.SgxEos * 1)(table)
    r, s = dev(spl["rho"]), dev(spl["sie"])
    lam = dev(np.full(2 * r.numel(), np.nan))
    out = torch.empty_like(r)
    assert lib.sgx_get_sg_PressureFromDensityInternalEnergy(
        0, arr2, P(r.data_ptr()), P(s.data_ptr()), P(out.data_ptr()), r.numel(), 2,
        P(lam.data_ptr())) == 0
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy(), spl["fn3"])


def test_modified_fill_from_host_arrays(sgx, table):
    # the host-array FillEos with a modified EOS moves every array both ways
    # (a modifier may write a quantity that is not an output) and matches
    # the reference like the device-array call
    fx = golden("modifiers")
    mats = materials_from_rows(fx["materials"])
    for k in (5, 6):  # shifted+scaled+ramped stiff gas; shifted+scaled table
        e = case_eos(sgx, table, mats[k], fx["mods"][k])
        n = fx[f"c{k}_rho"].size
        a = dict(rho=fx[f"c{k}_rho"].copy(), temp=np.zeros(n), sie=fx[f"c{k}_sie"].copy(),
                 press=np.zeros(n), cv=np.zeros(n), bmod=np.zeros(n))
        sgx.fill_eos_host(e, a["rho"], a["temp"], a["sie"], a["press"], a["cv"], a["bmod"], Q_TPB)
        for q in a:
            close(a[q], fx[f"c{k}_fill_{q}"], f"case {k} host fill {q}")


def test_plan_with_modified_materials(sgx):
    # a plan over a list with modified EOS runs the build with modifier code
    fx = golden("pte_rhot_modified")
    mats = materials_from_rows(fx["batched_materials"])
    eos_list = [wrap(sgx, sgx.make_eos(*m), r) for m, r in zip(mats, fx["batched_mods"])]
    t = {k: dev(fx["batched_in_" + k]) for k in ("rho", "vfrac", "sie", "temp", "press")}
    idx = dev(fx["batched_eos_idx"], torch.int32)
    ncell = fx["batched_sie_tot"].shape[0]
    status = torch.zeros(ncell * 16, dtype=torch.uint8, device="cuda")
    plan = sgx.PtePlan(0, eos_list, idx, dev(fx["batched_vfrac_tot"]), dev(fx["batched_sie_tot"]),
                       t["rho"], t["vfrac"], t["sie"], t["temp"], t["press"], status=status)
    plan.run()
    torch.cuda.synchronize()
    plan.close()
    present = fx["batched_in_rho"] > 0
    for k in ("press", "temp", "sie", "vfrac", "rho"):
        close(t[k].cpu().numpy()[present], fx["batched_out_" + k][present], f"plan {k}")
    st = sgx.status_view(status)
    np.testing.assert_array_equal(st["converged"], fx["batched_converged"].astype(bool))
