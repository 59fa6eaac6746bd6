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


def interp_scale(path, field, rho, sie):
    """sum_k |w_k| |f_k| over the four corners of each query's cell on the
    rho-sie grid: the magnitude the bilinear form's roundings scale with."""
    from sgx import sp5lite
    img = sp5lite.read(path)
    a = img["attrs"]
    g = "/3/dependsLogRhoLogSie/"
    data, ranges = img["datasets"][g + field]
    (ne, emin, emax), (nr, rmin, rmax) = ranges
    if field == "bulk modulus":
        # the values calcBMod_ (eos_spiner_rho_sie.hpp:554-578) leaves
        r = (sp5lite.pow10_nqt(np.linspace(rmin, rmax, nr)) - a["/3@rhoOffset"])[:, None]
        P, dPdR, dPdE, dEdR = (img["datasets"][g + k][0] for k in
                               ("pressure", "dPdRho", "dPdE", "dEdRho"))
        b = np.where(dPdE > 0, r * dPdR + dPdE * (P / r), np.maximum(r * (dPdR + dPdE * dEdR), 0))
        data = np.maximum(b, 10 * np.finfo(float).eps)
    lr = sp5lite.to_log(rho, a["/3@rhoOffset"])
    le = sp5lite.to_log(sie, a["/3@sieOffset"])

    def weights(x, n, mn, mx):
        dx = (mx - mn) / (n - 1)
        u = (x - mn) / dx
        i = np.clip(np.where(u >= 0, np.floor(u), 0), 0, n - 2).astype(int)
        w1 = u - i
        return i, 1.0 - w1, w1
    j, b0, b1 = weights(lr, nr, rmin, rmax)
    i, a0, a1 = weights(le, ne, emin, emax)
    f = np.abs(data)
    return (np.abs(b0) * (np.abs(a0) * f[j, i] + np.abs(a1) * f[j, i + 1]) +
            np.abs(b1) * (np.abs(a0) * f[j + 1, i] + np.abs(a1) * f[j + 1, i + 1]))


def test_mixed_fill_against_fp64(sgx, table):
    """The float-float FillEos (sgx_lookup_sie.cu) against the FP64 path (bit
    for bit the reference's, test_fill_eos): every output within 1e-11 of
    the interpolant's own magnitude scale sum_k |w_k f_k| (that is, within
    1e-11 relative wherever the cell's corners share a sign), the lambda
    entry log10(rho) within 1e-13, the sound speed within 1e-10 relative."""
    tab, fx = table
    path, _ = rhosie_table_path()
    # the fixture's queries (5 % off the table) plus a denser on-table set
    from sgx import sp5lite
    r2, e2, _ = sp5lite.rhosie_queries(1 << 16, seed=11, off_table=0.0)
    rho_h = np.concatenate([fx["rho"], r2])
    sie_h = np.concatenate([fx["sie"], e2])
    rho, sie = dev(rho_h), dev(sie_h)
    q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_SPECIFIC_HEAT | sgx.Q_BULK_MODULUS
    res = {}
    for prec in (sgx.PREC_FP64, sgx.PREC_MIXED):
        T, P, cv, bm, cs = (torch.zeros_like(rho) for _ in range(5))
        lam = torch.full_like(rho, float("nan"))
        sgx.fill_eos(tab, rho, T, sie, P, cv, bm, q, lam=lam, lam_stride=1, cs=cs,
                     precision=prec)
        torch.cuda.synchronize()
        res[prec] = {k: v.cpu().numpy() for k, v in
                     (("T", T), ("P", P), ("cv", cv), ("bmod", bm), ("cs", cs), ("lam", lam))}
    ref, got = res[sgx.PREC_FP64], res[sgx.PREC_MIXED]
    for name, field in (("T", "temperature"), ("P", "pressure"), ("bmod", "bulk modulus")):
        S = interp_scale(path, field, rho_h, sie_h)
        e = np.abs(got[name] - ref[name]) / S
        print(f"mixed {name}: max |err| / scale {e.max():.2e}, max rel "
              f"{rel_err(got[name], ref[name]).max():.2e}")
        assert e.max() <= 1e-11, name
    # cv = 1 / dT/de: relative error of the reciprocal is that of dT/de
    S = interp_scale(path, "dTdE", rho_h, sie_h)
    e = np.abs(1.0 / got["cv"] - 1.0 / ref["cv"]) / S
    assert e.max() <= 1e-11, "cv"
    assert np.abs(got["lam"] - ref["lam"]).max() <= 1e-13
    ok = ref["bmod"] > 0
    assert rel_err(got["cs"][ok], ref["cs"][ok]).max() <= 1e-10
