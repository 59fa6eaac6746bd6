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


# ---- modifiers: known answers of test/test_eos_modifiers.cpp ----------------

needs_reference = pytest.mark.skipif(not rb.have_reference(),
                                     reason="the compiled reference (oracle/_ref) is absent")


@needs_reference
def test_modifiers_known_answers():
    ref = rb.reference()
    # shifted by 0.1, then scaled by 2: P(rho = 2, sie = 0.5) == 0.3 exactly
    # (test_eos_modifiers.cpp:125-139)
    d = rb.eos_desc(rb.IDEAL, [0.5, 2.0], shift=0.1, scale=2.0)
    assert ref.eos_vec(d, 3, np.array([2.0]), np.array([0.5]))[0] == 0.3
    # a non-modifying modifier matches the bare model (:219-230)
    rng = np.random.default_rng(3)
    rho, sie = np.exp(rng.uniform(-3, 3, 64)), rng.uniform(0.1, 10, 64)
    bare = rb.eos_desc(rb.IDEAL, [0.5, 2.0])
    for kw in (dict(scale=1.0), dict(shift=0.0), dict(ramp=[1e9, 1.0, 2.0, 1.0])):
        for fn in (0, 3, 5, 7, 9):
            np.testing.assert_array_equal(ref.eos_vec(rb.eos_desc(rb.IDEAL, [0.5, 2.0], **kw),
                                                      fn, rho, sie),
                                          ref.eos_vec(bare, fn, rho, sie))


@needs_reference
def test_p_alpha_ramp_known_answers():
    # the ramp from a p-alpha model through init_sg_IdealGas
    # (test_eos_modifiers.cpp:231-314): parameters, pressures on both slopes
    # and beyond, bulk moduli on both slopes
    ref = rb.reference()
    gm1, Cv = 0.5, 2.0
    Pe, Pc, alpha0, T0 = 5.e7, 1.e8, 1.5, 293.0
    vals = ref.init_mods(rb.eos_desc(rb.IDEAL, [gm1, Cv]), [0, 0, 0, 1],
                         [0.0, 0.0, alpha0, Pe, Pc, 0.0])
    rho0 = 1.e6 / (gm1 * Cv * T0)
    r0 = rho0 / alpha0
    r1 = Pc / (gm1 * Cv * T0)
    rmid = Pe / (gm1 * Cv * T0 * alpha0)
    a = r0 * Pe / (rmid - r0)
    b = r0 * (Pc - Pe) / (r1 - rmid)
    c = (Pc * rmid - Pe * r1) / (r0 * (Pc - Pe))
    np.testing.assert_allclose(vals[2:], [r0, a, b, c], rtol=1e-12)
    d = rb.eos_desc(rb.IDEAL, [gm1, Cv], ramp=vals[2:])
    rho_t1, rho_t2 = 0.5 * (r0 + rmid), 0.5 * (rmid + r1)
    rho = np.array([rmid, rho_t1, rho_t2, 0.8 * r0, 1.2 * r0])
    P = ref.eos_vec(d, 2, rho, np.full(5, T0))
    np.testing.assert_allclose(P, [alpha0 * gm1 * Cv * rmid * T0, a * (rho_t1 / r0 - 1.0),
                                   b * (rho_t2 / r0 - c), 0.8 * r0 * gm1 * Cv * T0,
                                   1.2 * r0 * gm1 * Cv * T0], rtol=1e-12)
    B = ref.eos_vec(d, 6, np.array([rho_t1, rho_t2, 0.8 * r0, 1.2 * r1]), np.full(4, T0))
    np.testing.assert_allclose(B, [rho_t1 * a / r0, rho_t2 * b / r0,
                                   0.8 * r0 * gm1 * (gm1 + 1.0) * Cv * T0,
                                   1.2 * r1 * gm1 * (gm1 + 1.0) * Cv * T0], rtol=1e-12)


@needs_reference
def test_modifier_fixture_is_current():
    # the committed fixture is what the compiled reference gives today
    ref = rb.reference()
    fx = golden("modifiers")
    mats = materials_from_rows(fx["materials"])
    for k, (mat, row) in enumerate(zip(mats, fx["mods"])):
        if mat[0] == rb.SPINER_RHOT:
            continue
        bits = int(row[0])
        d = rb.eos_desc(mat[0], mat[1], shift=row[1] if bits & 1 else None,
                        scale=row[2] if bits & 2 else None, ramp=row[3:7] if bits & 4 else None)
        for fn in (2, 3, 6, 7):
            second = fx[f"c{k}_T"] if fn in (2, 6) else fx[f"c{k}_sie"]
            np.testing.assert_array_equal(ref.eos_vec(d, fn, fx[f"c{k}_rho"], second),
                                          fx[f"c{k}_fn{fn}"])


def test_port_rejects_modified_eos():
    # the port restates bare models only and says so
    d = rb.eos_desc(rb.IDEAL, [0.4, 0.718e7], shift=1.0)
    with pytest.raises(RuntimeError):
        rb.port().eos_vec(d, 3, np.array([1.0]), np.array([1.0]))


@needs_reference
def test_pt_derivatives_known_answers():
    # IdealGas answers in closed form (eos_ideal.hpp:152-168); StiffGas takes
    # the base class's one-sided differences (eos_base.hpp:299-320), which
    # must approach rho = (P + Pinf) / (gm1 Cv T), e = Cv T + Pinf / rho + q
    ref = rb.reference()
    gm1, Cv = 0.4, 0.718e7
    rho, T = np.array([1e-3, 0.2, 3.0]), np.array([300.0, 2e3, 5e4])
    d = rb.eos_desc(rb.IDEAL, [gm1, Cv])
    sie, P = Cv * T, gm1 * rho * Cv * T
    dedP, drdP, dedT, drdT = ref.pt_derivs(d, rho, sie, P, T)
    np.testing.assert_array_equal(dedP, 0.0)
    np.testing.assert_array_equal(dedT, Cv)
    np.testing.assert_allclose(drdP, 1.0 / (gm1 * sie), rtol=1e-15)
    np.testing.assert_allclose(drdT, -P / (gm1 * Cv * T * T), rtol=1e-15)
    gm1, Cv, Pinf, q = 3.4, 1.816e7, 6e9, 0.0
    d = rb.eos_desc(rb.STIFF, [gm1, Cv, Pinf, q])
    rho, T = np.array([0.8, 1.0, 1.5]), np.array([300.0, 600.0, 1200.0])
    sie = ref.eos_vec(d, 1, rho, T)
    P = ref.eos_vec(d, 2, rho, T)
    dedP, drdP, dedT, drdT = ref.pt_derivs(d, rho, sie, P, T)
    drdP_exact = 1.0 / (gm1 * Cv * T)
    np.testing.assert_allclose(drdP, drdP_exact, rtol=1e-4)
    np.testing.assert_allclose(drdT, -(P + Pinf) / (gm1 * Cv * T * T), rtol=1e-4)
    np.testing.assert_allclose(dedP, -Pinf / rho**2 * drdP_exact, rtol=1e-4)


@needs_reference
def test_entropy_known_answers():
    ref = rb.reference()
    # test_eos_ideal.cpp:44-90: zero at the reference state, and the two
    # closed forms when rho^3 or T^2 equals its reference
    gm1, Cv, T0, rho0 = 0.4, 5.0, 100.0, 1e-3
    d = rb.eos_desc(rb.IDEAL, [gm1, Cv, T0, rho0], flags=2)
    S = ref.eos_vec(d, 11, np.array([rho0, 0.1, rho0]), np.array([T0, T0, 10.0]))
    assert S[0] == 0.0
    np.testing.assert_allclose(S[1:], [2. / 3. * gm1 * Cv * np.log(rho0),
                                       -1. / 2. * Cv * np.log(T0)], rtol=1e-12)
    # test_eos_stiff.cpp:495-580: S(rho, e) of the seven-parameter stiff gas
    d = rb.eos_desc(rb.STIFF, [1.35, 1816.e4, 1.0e9, 2030.00e+07, -23.0e+7, 200.0, 1e6],
                    flags=2)
    S = ref.eos_vec(d, 12, np.array([1.0218087167564040e-01]),
                    np.array([3.7350567520918861e+10]))
    np.testing.assert_allclose(S, [-2.0044437857420778e+08], rtol=1e-12)


def test_port_helmholtz_matches_golden(tmp_path):
    """The port's Helmholtz restatement (sgport_helm_fill) against the
    fixture the compiled reference made on the synthetic table: the forward
    FillEos (rho, T -> sie, P, cv, bmod) within 1e-12, and the inversion as
    it is meant (the root kept, as sgref_helm_T_from_rho_sie finds it) within
    the reference's own stopping band where the reference recovers T."""
    import refbind as rb
    from common import golden, rel_err
    from sgx import helmtable
    fx = golden("helmholtz")
    path = str(tmp_path / "helm_table.dat")
    assert helmtable.helm_table(path) == str(fx["table_sha256"])
    port = rb.port()
    n = fx["rho"].size

    def lam_rows():
        lam = np.zeros(3 * n)
        lam[0::3], lam[1::3], lam[2::3] = fx["abar"], fx["zbar"], np.nan
        return lam

    sie, P, cv, bm = (np.zeros(n) for _ in range(4))
    port.helm_fill(path, 31, fx["rho"].copy(), fx["T"].copy(), sie, P, cv, bm,
                   rb.Q_SIE | rb.Q_PRESSURE | rb.Q_SPECIFIC_HEAT | rb.Q_BULK_MODULUS,
                   lam_rows())
    for k, got in (("sie", sie), ("P", P), ("cv", cv), ("bmod", bm)):
        e = rel_err(got, fx["fwd_" + k])
        assert e.max() <= 1e-12, (k, e.max())
    T = np.zeros(n)
    port.helm_fill(path, 31, fx["rho"].copy(), T, fx["fwd_sie"].copy(), np.zeros(n),
                   np.zeros(n), np.zeros(n), rb.Q_TEMPERATURE | rb.Q_PRESSURE, lam_rows())
    # where the reference recovers T, both stop within 1e-10 |e| of the
    # target: |dT| <= 2e-10 |e| / cv
    fix, Tin = fx["fix_T"], fx["T"]
    good = np.abs(fix - Tin) <= 1e-8 * Tin
    assert good.mean() > 0.75
    bound = 2e-10 * np.abs(fx["fwd_sie"][good]) / np.abs(fx["fwd_cv"][good]) + 1e-12 * fix[good]
    assert (np.abs(T[good] - fix[good]) <= bound).all()


# ---- SpinerEOSDependsRhoSie: fixture provenance --------------------------

def test_rhosie_table_generator_is_stable():
    # the table the fixture was made on is what sp5lite writes today
    from common import rhosie_table_path
    _, sha = rhosie_table_path()
    assert sha == str(golden("spiner_rhosie")["table_sha256"])


@needs_reference
def test_rhosie_fixture_is_current():
    # the committed fixture is what the compiled reference gives today
    from common import rhosie_table_path
    ref = rb.reference()
    fx = golden("spiner_rhosie")
    path, _ = rhosie_table_path()
    d = rb.eos_desc(rb.SPINER_RHOSIE, [], path=path, matid=3)
    for fn in (0, 1, 3, 5, 7, 10):
        second = fx["T"] if fn in (1, 2, 4, 6, 8) else fx["sie"]
        np.testing.assert_array_equal(ref.eos_vec(d, fn, fx["rho"], second), fx[f"fn{fn}"])
    dump, scal = ref.spiner_sie_dump(path, 3)
    import hashlib
    assert hashlib.sha256(dump.tobytes()).hexdigest() == str(fx["dump_sha256"])
    np.testing.assert_array_equal(scal, fx["scal"])


def test_port_rhosie_matches_golden():
    # the port's SpinerEOSDependsRhoSie reproduces the compiled reference's
    # fixture bit for bit: load-time tables, vector functions with their
    # lambda rows, the three FillEos forms and the bounds
    import hashlib
    from common import rhosie_table_path
    port = rb.port()
    fx = golden("spiner_rhosie")
    path, _ = rhosie_table_path()
    dump, scal = port.spiner_sie_dump(path, 3)
    assert hashlib.sha256(dump.tobytes()).hexdigest() == str(fx["dump_sha256"])
    np.testing.assert_array_equal(scal, fx["scal"])
    d = rb.eos_desc(rb.SPINER_RHOSIE, [], path=path, matid=3)
    for fn in list(range(11)) + [13]:
        second = fx["P_target"] if fn == 13 else (fx["T"] if fn in (1, 2, 4, 6, 8) else fx["sie"])
        lam = np.full(fx["rho"].size, np.nan)
        np.testing.assert_array_equal(port.eos_vec(d, fn, fx["rho"], second, lam=lam,
                                                   lam_stride=1), fx[f"fn{fn}"])
        np.testing.assert_array_equal(lam, fx[f"fn{fn}_lambda"])
    for tag in ("e", "t", "pt"):
        a = {k: fx[k].copy() for k in ("rho", "T", "sie", "P_in")}
        cv, bm, lam = np.zeros(a["rho"].size), np.zeros(a["rho"].size), np.full(a["rho"].size,
                                                                              np.nan)
        port.fill_eos(d, a["rho"], a["T"], a["sie"], a["P_in"], cv, bm,
                      int(fx[f"fill_{tag}_output"]), lam=lam, lam_stride=1)
        for name, v in (("rho", a["rho"]), ("T", a["T"]), ("sie", a["sie"]), ("P", a["P_in"]),
                        ("cv", cv), ("bmod", bm), ("lambda", lam)):
            np.testing.assert_array_equal(v, fx[f"fill_{tag}_{name}"])
    for w in range(6):
        np.testing.assert_array_equal(port.eos_bounds(d, w, fx["bounds_T"]), fx[f"bound{w}"])


def test_bench_reference_arm_line():
    """bench.py --impl reference (the CPU arm the benchmark's ratio is
    taken against) on a small workload: exactly the requested steps, one
    JSON line with the headline metric's keys, impl = reference, no host
    copies."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--queries", "65536", "--steps", "2", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 3
    for k in ("metric", "value", "unit", "n_gpus", "ms_per_step", "higher_is_better",
              "scaling", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["unit"] == "lookups/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert abs(line["ms_per_step"] * 1e-3 * line["value"] - 65536) <= 1e-6 * 65536
