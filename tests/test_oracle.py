"""The oracle, pinned (CPU only).

1. The compiled reference (oracle/_ref, only where the reference sources are
   present) reproduces the known-answer values hard-coded in the reference's
   own unit tests.
2. This project's restatement (oracle/port) reproduces every golden fixture
   made from the compiled reference, bit for bit.
"""
import hashlib

import numpy as np
import pytest

import refbind as rb
from common import PARITY_RTOL, bitwise_frac, golden, materials_from_rows, rel_err
from common import stiffgas_table_path


def oracles():
    out = [("port", rb.port)]
    if rb.have_reference():
        out.append(("reference", rb.reference))
    return out


@pytest.fixture(scope="module", params=[o[0] for o in oracles()])
def oracle(request):
    return dict(oracles())[request.param]()


# ---- known-answer values from the reference's unit tests -------------------

def test_stiffgas_known_answers(oracle):
    # test/test_eos_stiff.cpp:35-90 (liquid-water parameters, 4 states)
    d = rb.eos_desc(rb.STIFF, [1.35, 1816.00e+04, 1.00e+10, -1167.00e+07])
    rho = np.array([1.3682314734849790e+00, 2.6715104028907288e-01,
                    1.4846658731195411e-01, 1.0300747471039322e-01])
    sie = np.array([1.0531088454815292e+09, 5.3584944459257431e+10,
                    1.0591669035038826e+11, 1.5805033352060248e+11])
    P = oracle.eos_vec(d, 3, rho, sie)
    B = oracle.eos_vec(d, 7, rho, sie)
    T = oracle.eos_vec(d, 0, rho, sie)
    G = oracle.eos_vec(d, 9, rho, sie)
    np.testing.assert_allclose(P, [1.01324999999964016e+06, 3.44504999999983162e+07,
                                   6.78877500000010729e+07, 1.01324999999999583e+08], rtol=1e-12)
    np.testing.assert_allclose(B, [2.35023811375000000e+10, 2.35809586749999962e+10,
                                   2.36595362125000038e+10, 2.37381137500000000e+10], rtol=1e-12)
    np.testing.assert_allclose(T, [2.98149999999999920e+02, 1.53209999999999968e+03,
                                   2.76605000000000064e+03, 3.99999999999999955e+03], rtol=1e-12)
    np.testing.assert_allclose(G, 1.35, rtol=1e-12)


def test_ideal_gas_known_answers(oracle):
    # IdealGas(gm1 = 0.4, Cv = 0.718e7): P = gm1 rho sie, T = sie / Cv
    # (test/test_eos_ideal.cpp:44-90 uses the same closed forms)
    d = rb.eos_desc(rb.IDEAL, [0.4, 0.718e7])
    rho = np.array([1.0, 2.0, 0.5])
    sie = np.array([2.0e10, 1.0e9, 3.5e10])
    np.testing.assert_allclose(oracle.eos_vec(d, 3, rho, sie), 0.4 * rho * sie, rtol=1e-15)
    np.testing.assert_allclose(oracle.eos_vec(d, 0, rho, sie), sie / 0.718e7, rtol=1e-15)


def test_gruneisen_max_density(oracle):
    # rho_max = 0.99 rho0 / (1 - 1/s1 + eps) for a linear Us-up fit
    # (eos_gruneisen.hpp:62-67, 231-245, 321-322)
    d = rb.eos_desc(rb.GRUNEISEN, [3.94e5, 1.489, 0, 0, 2.02, 0.47, 8.93, 298.0, 0.0, 3.9e6])
    got = oracle.eos_bounds(d, 2, np.zeros(1))[0]
    assert got == 0.99 * (8.93 / ((1 - 1 / 1.489) + 10 * np.finfo(float).eps))


def test_pte_reaches_equilibrium(oracle):
    # Property the reference's PTE tests assert (test_pte_ideal.cpp:98-231):
    # converged cells share one temperature, volume fractions sum to the
    # total, and the material energies add up to the cell energy.
    fx = golden("pte_rhot_2mat")
    conv = fx["converged"].astype(bool)
    T, P, v, r, e = (fx["out_" + k] for k in ("temp", "press", "vfrac", "rho", "sie"))
    assert conv.mean() > 0.99
    assert np.all(T[0, conv] == T[1, conv])
    np.testing.assert_allclose(v.sum(axis=0)[conv], fx["vfrac_tot"][conv], rtol=1e-12)
    u = (r * v * e).sum(axis=0)
    rho_tot = (fx["in_rho"] * fx["in_vfrac"]).sum(axis=0)
    np.testing.assert_allclose(u[conv], (rho_tot * fx["sie_tot"])[conv], rtol=1e-5)
    # pressures agree to the solver's "sufficient" tolerances: 100 x 1e-6 of
    # the mean pressure, or 100 x 1e-6 absolute in units of the energy scale
    # rho_tot * sie_tot (mixed_cell_models.hpp:55-60, 634, 1032-1039)
    mean_p = np.abs((v * P).sum(axis=0))
    uscale = rho_tot * fx["sie_tot"]
    tol = np.maximum(2e-4 * mean_p, 1e-4 * uscale)
    assert np.all(np.abs(P[0, conv] - P[1, conv]) <= tol[conv])


# ---- the restatement reproduces the compiled reference -----------------------

def _port_pte(fx, descs, params=None):
    port = rb.port()
    r = {k: fx["in_" + k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
    conv, nit, res = port.pte(int(fx.get("solver", 0)), descs, fx.get("eos_idx"),
                              fx["vfrac_tot"], fx["sie_tot"], r["rho"], r["vfrac"], r["sie"],
                              r["temp"], r["press"], params=params or port.mix_params())
    return r, conv, nit


@pytest.mark.parametrize("name", ["pte_rhot_2mat", "pte_rhot_batched", "pte_pt_2mat",
                                  "pte_pt_batched", "pte_rhot_2mat_tight"])
def test_port_pte_matches_golden(name):
    fx = golden(name)
    descs = [rb.eos_desc(k, p) for k, p in materials_from_rows(fx["materials"])]
    params = rb.port().mix_params(
        **{k[6:]: float(v) for k, v in fx.items() if k.startswith("param_")})
    r, conv, nit = _port_pte(fx, descs, params)
    np.testing.assert_array_equal(conv, fx["converged"])
    np.testing.assert_array_equal(nit, fx["niter"])
    for k in r:
        assert bitwise_frac(r[k], fx["out_" + k]) == 1.0, k


def test_port_spiner_matches_golden():
    fx = golden("spiner_lookup")
    path, sha = stiffgas_table_path()
    assert sha == str(fx["table_sha256"])
    port = rb.port()
    dump, scal = port.spiner_dump(path, 1)
    assert dump.size == int(fx["dump_len"])
    assert hashlib.sha256(dump.tobytes()).hexdigest() == str(fx["dump_sha256"])
    np.testing.assert_array_equal(scal[:7], fx["scal"][:7])
    d = rb.eos_desc(rb.SPINER_RHOT, [], path=path, matid=1)
    n = fx["rho"].size
    T, P, cv, bm = (np.zeros(n) for _ in range(4))
    lam = np.full(2 * n, np.nan)
    port.fill_eos(d, fx["rho"].copy(), T, fx["sie"].copy(), P, cv, bm,
                  rb.Q_TEMPERATURE | rb.Q_PRESSURE | rb.Q_BULK_MODULUS | rb.Q_SPECIFIC_HEAT,
                  lam=lam, lam_stride=2)
    for name, a in (("T", T), ("P", P), ("cv", cv), ("bmod", bm), ("lambda", lam)):
        assert bitwise_frac(a, fx["fill_" + name]) == 1.0, name
    for fn in range(11):
        second = fx["Tq"] if fn in (1, 2, 4, 6, 8) else fx["sie"]
        got = port.eos_vec(d, fn, fx["rho"], second)
        assert rel_err(got, fx[f"fn{fn}"]).max() <= PARITY_RTOL, fn
    # PTE with the tabulated material
    fx = golden("pte_rhot_spiner")
    descs = [rb.eos_desc(rb.IDEAL, [0.4, 0.718e7]), d]
    r, conv, nit = _port_pte(fx, descs)
    np.testing.assert_array_equal(conv, fx["converged"])
    for k in r:
        assert bitwise_frac(r[k], fx["out_" + k]) == 1.0, k


def test_port_vector_lookups_match_golden():
    fx = golden("eos_vector")
    port = rb.port()
    for k, (kind, params) in enumerate(materials_from_rows(fx["materials"])):
        d = rb.eos_desc(kind, params)
        for fn in range(11):
            second = fx[f"m{k}_T"] if fn in (1, 2, 4, 6, 8) else fx[f"m{k}_sie"]
            got = port.eos_vec(d, fn, fx[f"m{k}_rho"], second)
            assert bitwise_frac(got, fx[f"m{k}_fn{fn}"]) == 1.0, (kind, fn)
