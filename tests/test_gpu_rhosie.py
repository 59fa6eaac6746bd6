"""SpinerEOSDependsRhoSie (eos/eos_spiner_rho_sie.hpp) through the C ABI
against the compiled reference's outputs (tests/golden/spiner_rhosie.npz,
pte_rhot_rhosie.npz, pte_pt_rhosie.npz):

  * the load-time tables (bulk moduli recomputed by calcBMod_, the densest
    row's slices, rho_at_pmin) bit for bit, by SHA-256 of the DBLIST dump;
  * the eleven vector functions and e(rho, P), with the lambda rows of one
    entry (log10 rho) they write;
  * FillEos from (rho, sie), from (rho, T) and from (P, T);
  * the bounds (MinimumDensity ... RhoPmin);
  * PTE with the model beside an ideal gas, RhoT and PT solvers: within
    1e-12 with identical flags and iteration counts.
"""
import ctypes as C
import hashlib

import numpy as np
import pytest

from common import PARITY_RTOL, bitwise_frac, golden, rel_err, rhosie_table_path

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sgx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sgx import lib
    lib.load()
    return lib


@pytest.fixture(scope="module")
def table(sgx):
    fx = golden("spiner_rhosie")
    path, sha = rhosie_table_path()
    assert sha == str(fx["table_sha256"]), "the generated table differs from the fixture's"
    tab = sgx.spiner_rhosie_eos(path, 3)
    yield tab, fx
    sgx.load().sgx_eos_finalize(C.byref(tab))


def dev(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def same(got, want, name):
    assert rel_err(got, want).max() <= PARITY_RTOL, name
    assert bitwise_frac(got, want) == 1.0, name


def test_load_time_tables(sgx, table):
    tab, fx = table
    n = int(fx["dump_len"])
    buf = np.zeros(n)
    got_n = sgx.load().sgx_eos_spiner_dump(C.byref(tab), buf.ctypes.data_as(C.c_void_p), n)
    assert got_n == n
    assert np.array_equal(buf[::97], fx["dump_sample"])
    assert hashlib.sha256(buf.tobytes()).hexdigest() == str(fx["dump_sha256"])


@pytest.mark.parametrize("fn", list(range(11)) + [13])
def test_vector_functions(sgx, table, fn):
    tab, fx = table
    rho = dev(fx["rho"])
    second = dev(fx["P_target"] if fn == 13 else
                 (fx["T"] if fn in (1, 2, 4, 6, 8) else fx["sie"]))
    out = torch.empty_like(rho)
    lam = torch.full_like(rho, float("nan"))
    sgx.eval_eos(tab, fn, rho, second, out, lam=lam, lam_stride=1)
    torch.cuda.synchronize()
    same(out.cpu().numpy(), fx[f"fn{fn}"], f"fn {fn}")
    same(lam.cpu().numpy(), fx[f"fn{fn}_lambda"], f"fn {fn} lambda")


@pytest.mark.parametrize("tag", ["e", "t", "pt"])
def test_fill_eos(sgx, table, tag):
    tab, fx = table
    q = int(fx[f"fill_{tag}_output"])
    rho, T, sie, P = dev(fx["rho"]), dev(fx["T"]), dev(fx["sie"]), dev(fx["P_in"])
    cv, bm = torch.zeros_like(rho), torch.zeros_like(rho)
    lam = torch.full_like(rho, float("nan"))
    sgx.fill_eos(tab, rho, T, sie, P, cv, bm, q, lam=lam, lam_stride=1)
    torch.cuda.synchronize()
    for name, t in (("rho", rho), ("T", T), ("sie", sie), ("P", P), ("cv", cv), ("bmod", bm),
                    ("lambda", lam)):
        same(t.cpu().numpy(), fx[f"fill_{tag}_{name}"], f"{tag} {name}")


def test_bounds(sgx, table):
    tab, fx = table
    Tb = dev(fx["bounds_T"])
    for what in range(6):
        out = torch.empty_like(Tb)
        sgx.eos_bounds(tab, what, out, temp=Tb)
        torch.cuda.synchronize()
        same(out.cpu().numpy(), fx[f"bound{what}"], f"bound {what}")


@pytest.mark.parametrize("name", ["pte_rhot_rhosie", "pte_pt_rhosie"])
def test_pte_with_rhosie_material(sgx, table, name):
    from sgx import workloads as W
    tab, _ = table
    fx = golden(name)
    eos_list = [sgx.make_eos(*W.IDEAL_AIR), tab]
    t = {k: dev(fx["in_" + k]) for k in ("rho", "vfrac", "sie", "temp", "press")}
    ncell = fx["sie_tot"].shape[0]
    status = torch.zeros(ncell * 16, dtype=torch.uint8, device="cuda")
    sgx.pte_solve(int(fx["solver"]), eos_list, None, dev(fx["vfrac_tot"]), dev(fx["sie_tot"]),
                  t["rho"], t["vfrac"], t["sie"], t["temp"], t["press"], status=status)
    torch.cuda.synchronize()
    st = sgx.status_view(status)
    np.testing.assert_array_equal(st["converged"], fx["converged"].astype(bool))
    np.testing.assert_array_equal(st["niter"], fx["niter"])
    for k in ("press", "temp", "sie", "vfrac", "rho"):
        got, want = t[k].cpu().numpy(), fx["out_" + k]
        e = rel_err(got, want)
        print(f"{name} {k}: max rel {e.max():.3e}, bitwise {bitwise_frac(got, want):.4f}")
        assert e.max() <= PARITY_RTOL, k


def test_rejects(sgx, table):
    tab, fx = table
    rho = dev(fx["rho"][:8])
    out = torch.empty_like(rho)
    # entropy is not enabled for this model (EntropyIsNotEnabled)
    with pytest.raises(RuntimeError):
        sgx.eval_eos(tab, 11, rho, rho, out)
    # FillEos with both T and sie among the outputs (UNDEFINED_ERROR) leaves
    # the elements as they are
    T = torch.zeros_like(rho)
    sie = torch.zeros_like(rho)
    q = sgx.Q_TEMPERATURE | sgx.Q_SIE
    try:
        sgx.fill_eos(tab, rho, T, sie, None, None, None, q)
    except RuntimeError:
        pass
    torch.cuda.synchronize()
    assert float(T.abs().sum()) == 0.0 and float(sie.abs().sum()) == 0.0
