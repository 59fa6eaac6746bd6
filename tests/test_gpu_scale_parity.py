"""The plain FP64 path against the oracle at the benchmark workloads' full
sizes, on the GPU host's own cores (oracle/port, all threads).

The contract is the reference's: agreement within 1e-12 relative on P, T,
sie_i, alpha_i (and rho_i), with the same per-cell convergence flag and
iteration count. Each test also reports the fraction of values that agree
bit for bit (the path is built to match bitwise: no FMA contraction on either
side, the reference's operation order).

  * two-material closure, 65,536 cells (IdealGas + StiffGas);
  * uneven closure, a 2^20-cell slice of the 2^22-cell batch's distribution
    (2-5 materials from the 8-EOS pool; the same generator and seed as the
    benchmark);
  * tabulated lookup, all 2^24 queries: T, P, bmod and the sound speed.
"""
import numpy as np
import pytest

from common import PARITY_RTOL, bitwise_frac, rel_err, stiffgas_table_path

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
def port():
    import refbind as rb
    return rb.port()


def gpu_pte(sgx, wl):
    eos_list = [sgx.make_eos(k, p) for k, p in wl["materials"]]
    t = {k: torch.as_tensor(wl[k], device="cuda") for k in ("rho", "vfrac", "sie", "temp",
                                                             "press")}
    idx = torch.as_tensor(wl["eos_idx"], device="cuda") if wl["eos_idx"] is not None else None
    n = wl["sie_tot"].shape[0]
    status = torch.zeros(n * 16, dtype=torch.uint8, device="cuda")
    sgx.pte_solve(sgx.PTE_RHOT, eos_list, idx, torch.as_tensor(wl["vfrac_tot"], device="cuda"),
                  torch.as_tensor(wl["sie_tot"], device="cuda"), t["rho"], t["vfrac"], t["sie"],
                  t["temp"], t["press"], status=status, precision=sgx.PREC_FP64)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in t.items()}, sgx.status_view(status)


def port_pte(port, wl):
    import refbind as rb
    r = {k: wl[k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
    conv, nit, _ = port.pte(0, [rb.eos_desc(k, p) for k, p in wl["materials"]], wl["eos_idx"],
                            wl["vfrac_tot"], wl["sie_tot"], r["rho"], r["vfrac"], r["sie"],
                            r["temp"], r["press"], params=port.mix_params(), nthreads=0)
    return r, conv.astype(bool), nit


@pytest.mark.parametrize("case", ["two_material_65536", "uneven_2e20"])
def test_plain_pte_matches_oracle_at_scale(sgx, port, case):
    from sgx import workloads as W
    wl = W.pte_two_material(65536, seed=77) if case == "two_material_65536" else \
        W.pte_batched(1 << 20, seed=77)
    present = wl["eos_idx"] >= 0 if wl["eos_idx"] is not None else np.ones_like(wl["rho"], bool)
    got, st = gpu_pte(sgx, wl)
    want, conv, nit = port_pte(port, wl)
    assert np.array_equal(st["converged"], conv), int((st["converged"] != conv).sum())
    assert np.array_equal(st["niter"], nit), int((st["niter"] != nit).sum())
    for k in ("press", "temp", "sie", "vfrac", "rho"):
        e = rel_err(got[k][present], want[k][present])
        bw = bitwise_frac(got[k][present], want[k][present])
        print(f"{case} {k}: max rel {e.max():.3e}, bitwise {bw:.6f}")
        assert e.max() <= PARITY_RTOL, (k, e.max())


def test_plain_lookup_matches_oracle_at_scale(sgx, port):
    """All 2^24 queries of the lookup workload, FillEos T|P|bmod plus the
    sound speed sqrt(bmod / rho)."""
    import ctypes as C
    import refbind as rb
    from sgx import sp5lite
    path, _ = stiffgas_table_path()
    n = 1 << 24
    rho_h, sie_h = sp5lite.stiffgas_queries(n, seed=2024)
    tab = sgx.spiner_eos(path, 1)
    try:
        rho = torch.as_tensor(rho_h, device="cuda")
        sie = torch.as_tensor(sie_h, device="cuda")
        T, P, B, CS = (torch.zeros_like(rho) for _ in range(4))
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS
        sgx.fill_eos(tab, rho, T, sie, P, None, B, q, cs=CS, precision=sgx.PREC_FP64)
        torch.cuda.synchronize()
        got = [x.cpu().numpy() for x in (T, P, B, CS)]
        del rho, sie, T, P, B, CS
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))
    d = rb.eos_desc(rb.SPINER_RHOT, [], path=path, matid=1)
    Tp, Pp, cvp, Bp = (np.zeros(n) for _ in range(4))
    port.fill_eos(d, rho_h.copy(), Tp, sie_h.copy(), Pp, cvp, Bp, q)
    for name, g, w in zip(("T", "P", "bmod", "cs"), got, (Tp, Pp, Bp, np.sqrt(Bp / rho_h))):
        e = rel_err(g, w)
        print(f"lookup {name}: max rel {e.max():.3e}, bitwise {bitwise_frac(g, w):.6f}")
        assert e.max() <= PARITY_RTOL, (name, e.max())
