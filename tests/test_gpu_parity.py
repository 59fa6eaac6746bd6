"""Parity of the CUDA library (through its C ABI) with the reference's own
CPU implementation, on the committed golden fixtures
(tests/golden/make_golden.py). The plain FP64 path must agree within 1e-12
relative on P, T, sie_i and alpha_i with the same per-cell convergence flag;
it is in fact expected to be bit-identical (same operation order, no FMA
contraction on either side), and the tests report that fraction."""
import numpy as np
import pytest

from common import PARITY_RTOL, bitwise_frac, golden, materials_from_rows, rel_err
from common import stiffgas_table_path

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sgx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sgx import lib
    lib.load()
    return lib


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def run_pte(sgx, fx, eos_list, params=None, precision=0):
    solver = int(fx.get("solver", 0))
    t = {k: dev(fx["in_" + k]) for k in ("rho", "vfrac", "sie", "temp", "press")}
    idx = dev(fx["eos_idx"], torch.int32) if "eos_idx" in fx else None
    ncell = fx["sie_tot"].shape[0]
    status = torch.zeros(ncell * 16, dtype=torch.uint8, device="cuda")
    sgx.pte_solve(solver, eos_list, idx, dev(fx["vfrac_tot"]), dev(fx["sie_tot"]), t["rho"],
                  t["vfrac"], t["sie"], t["temp"], t["press"], params=params, status=status,
                  precision=precision)
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in t.items()}
    return out, sgx.status_view(status)


def check_pte(fx, out, st, label):
    present = fx["in_rho"] > 0
    for k in ("press", "temp", "sie", "vfrac", "rho"):
        a, b = out[k][present], fx["out_" + k][present]
        err = rel_err(a, b)
        assert err.max() <= PARITY_RTOL, f"{label} {k}: max rel err {err.max():.3e}"
        print(f"{label} {k}: bitwise {bitwise_frac(a, b):.4f}")
    np.testing.assert_array_equal(st["converged"], fx["converged"].astype(bool))
    np.testing.assert_array_equal(st["niter"], fx["niter"])


@pytest.mark.parametrize("name", ["pte_rhot_2mat", "pte_rhot_batched", "pte_pt_2mat",
                                  "pte_pt_batched", "pte_rhou_2mat", "pte_rhou_batched",
                                  "pte_fixedt_2mat", "pte_fixedt_batched", "pte_fixedp_2mat",
                                  "pte_fixedp_batched"])
def test_pte_matches_reference(sgx, name):
    fx = golden(name)
    eos_list = [sgx.make_eos(k, p) for k, p in materials_from_rows(fx["materials"])]
    out, st = run_pte(sgx, fx, eos_list)
    check_pte(fx, out, st, name)


def test_pte_tight_tolerances_match_reference(sgx):
    fx = golden("pte_rhot_2mat_tight")
    params = sgx.mix_params(**{k[6:]: float(v) for k, v in fx.items() if k.startswith("param_")})
    eos_list = [sgx.make_eos(k, p) for k, p in materials_from_rows(fx["materials"])]
    out, st = run_pte(sgx, fx, eos_list, params=params)
    check_pte(fx, out, st, "tight")


def test_pte_with_tabulated_material(sgx):
    fx = golden("pte_rhot_spiner")
    path, sha = stiffgas_table_path()
    assert sha == str(fx["table_sha256"]), "table generation is not reproducible"
    import ctypes as C
    tab = sgx.spiner_eos(path, 1)
    try:
        out, st = run_pte(sgx, fx, [sgx.make_eos(1, (0.4, 0.718e7)), tab])
        check_pte(fx, out, st, "spiner-pte")
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


def test_analytic_vector_lookups(sgx):
    fx = golden("eos_vector")
    for k, (kind, params) in enumerate(materials_from_rows(fx["materials"])):
        eos = sgx.make_eos(kind, params)
        rho, sie, T = (dev(fx[f"m{k}_{n}"]) for n in ("rho", "sie", "T"))
        for fn in range(11):
            out = torch.empty_like(rho)
            second = T if fn in (1, 2, 4, 6, 8) else sie
            sgx.eval_eos(eos, fn, rho, second, out)
            got = out.cpu().numpy()
            err = rel_err(got, fx[f"m{k}_fn{fn}"])
            assert err.max() <= PARITY_RTOL, f"model {kind} fn {fn}: {err.max():.3e}"
            assert bitwise_frac(got, fx[f"m{k}_fn{fn}"]) == 1.0, f"model {kind} fn {fn}"


def test_tabulated_lookups(sgx):
    fx = golden("spiner_lookup")
    path, sha = stiffgas_table_path()
    assert sha == str(fx["table_sha256"])
    import ctypes as C
    tab = sgx.spiner_eos(path, 1)
    try:
        n = int(fx["dump_len"])
        buf = np.zeros(n)
        got_n = sgx.load().sgx_eos_spiner_dump(C.byref(tab), buf.ctypes.data_as(C.c_void_p), n)
        assert got_n == n
        import hashlib
        assert hashlib.sha256(buf.tobytes()).hexdigest() == str(fx["dump_sha256"]), \
            "derived tables differ from the reference's"
        rho, sie, Tq = dev(fx["rho"]), dev(fx["sie"]), dev(fx["Tq"])
        T, P, cv, bm = (torch.zeros_like(rho) for _ in range(4))
        lam = torch.full((2 * rho.numel(),), float("nan"), dtype=torch.float64, device="cuda")
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS | sgx.Q_SPECIFIC_HEAT
        sgx.fill_eos(tab, rho, T, sie, P, cv, bm, q, lam=lam, lam_stride=2)
        for name, t in (("T", T), ("P", P), ("cv", cv), ("bmod", bm), ("lambda", lam)):
            a, b = t.cpu().numpy(), fx["fill_" + name]
            assert rel_err(a, b).max() <= PARITY_RTOL, name
            assert bitwise_frac(a, b) == 1.0, name
        for fn in range(11):
            out = torch.empty_like(rho)
            second = Tq if fn in (1, 2, 4, 6, 8) else sie
            sgx.eval_eos(tab, fn, rho, second, out)
            got = out.cpu().numpy()
            assert rel_err(got, fx[f"fn{fn}"]).max() <= PARITY_RTOL, f"fn {fn}"
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


@pytest.mark.parametrize("name", ["pte_rhot_2mat", "pte_rhot_batched"])
@pytest.mark.parametrize("precision", [0, 1])
def test_pte_plan_replays_the_solve(sgx, name, precision):
    # a plan (the solve captured as a CUDA graph) gives what sgx_pte_solve
    # gives, run after run, on whatever the bound arrays hold
    fx = golden(name)
    eos_list = [sgx.make_eos(k, p) for k, p in materials_from_rows(fx["materials"])]
    ref, st_ref = run_pte(sgx, fx, eos_list, precision=precision)
    t = {k: dev(fx["in_" + k]) for k in ("rho", "vfrac", "sie", "temp", "press")}
    idx = dev(fx["eos_idx"], torch.int32) if "eos_idx" in fx else None
    ncell = fx["sie_tot"].shape[0]
    status = torch.zeros(ncell * 16, dtype=torch.uint8, device="cuda")
    plan = sgx.PtePlan(0, eos_list, idx, dev(fx["vfrac_tot"]), dev(fx["sie_tot"]), t["rho"],
                       t["vfrac"], t["sie"], t["temp"], t["press"], status=status,
                       precision=precision)
    for _ in range(2):
        for k in t:
            t[k].copy_(dev(fx["in_" + k]))
        status.zero_()
        plan.run()
        torch.cuda.synchronize()
        for k in t:
            np.testing.assert_array_equal(t[k].cpu().numpy(), ref[k], err_msg=k)
        st = sgx.status_view(status)
        np.testing.assert_array_equal(st["converged"], st_ref["converged"])
        np.testing.assert_array_equal(st["niter"], st_ref["niter"])
    plan.close()
    if precision == 0:
        check_pte(fx, ref, st_ref, name + " (plan)")
