"""Generates the golden fixtures in this folder from the compiled reference.

TEST INFRASTRUCTURE. Runs the reference's own hot-path code
(oracle/_ref/libsgref.so, built by oracle/build_ref.sh from the reference
sources with the shims in oracle/shims) on small seeded inputs and stores
inputs and outputs as .npz. The GPU parity tests compare the CUDA library
against these files on machines where the reference sources are absent.

Usage: python tests/golden/make_golden.py [name ...]   (default: all)
"""
import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "singularity-eos_gb300"))

import refbind as rb  # noqa: E402
from sgx import sp5lite, workloads as W  # noqa: E402

ALL_FN = list(range(11))
Q_TPB = rb.Q_TEMPERATURE | rb.Q_PRESSURE | rb.Q_BULK_MODULUS | rb.Q_SPECIFIC_HEAT


def desc(mat):
    kind, params = mat
    return rb.eos_desc(kind, params)


def mats_array(materials):
    """[n, 16] parameter rows with the model code in column 15."""
    out = np.zeros((len(materials), 16))
    for k, (kind, params) in enumerate(materials):
        out[k, : len(params)] = params
        out[k, 15] = kind
    return out


def pte_fixture(ref, wl, solver, params=None):
    r = {k: wl[k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
    mp = ref.mix_params(**(params or {}))
    conv, nit, res = ref.pte(solver, [desc(m) for m in wl["materials"]], wl["eos_idx"],
                             wl["vfrac_tot"], wl["sie_tot"], r["rho"], r["vfrac"], r["sie"],
                             r["temp"], r["press"], params=mp)
    out = dict(materials=mats_array(wl["materials"]), vfrac_tot=wl["vfrac_tot"],
               sie_tot=wl["sie_tot"], converged=conv, niter=nit, residual=res,
               solver=np.int32(solver))
    if wl["eos_idx"] is not None:
        out["eos_idx"] = wl["eos_idx"]
    for k in ("rho", "vfrac", "sie", "temp", "press"):
        out["in_" + k] = wl[k]
        out["out_" + k] = r[k]
    for k, v in (params or {}).items():
        out["param_" + k] = np.float64(v)
    return out


def vector_fixture(ref, materials, n=512, seed=11):
    rng = np.random.default_rng(seed)
    out = dict(materials=mats_array(materials))
    for k, mat in enumerate(materials):
        rho = np.exp(rng.uniform(np.log(1e-3), np.log(20.0), n))
        sie = rng.uniform(1e8, 1e11, n)
        T = np.exp(rng.uniform(np.log(50.0), np.log(1e5), n))
        out[f"m{k}_rho"], out[f"m{k}_sie"], out[f"m{k}_T"] = rho, sie, T
        d = desc(mat)
        for fn in ALL_FN:
            second = T if fn in (1, 2, 4, 6, 8) else sie
            out[f"m{k}_fn{fn}"] = ref.eos_vec(d, fn, rho, second)
    return out


def spiner_fixture(ref, path, nq=4096, seed=5):
    rho, sie = sp5lite.stiffgas_queries(nq, seed=seed)
    d = rb.eos_desc(rb.SPINER_RHOT, [], path=path, matid=1)
    out = dict(rho=rho, sie=sie)
    T, P, cv, bm = (np.zeros(nq) for _ in range(4))
    lam = np.full(2 * nq, np.nan)
    ref.fill_eos(d, rho.copy(), T, sie.copy(), P, cv, bm, Q_TPB, lam=lam, lam_stride=2)
    out.update(fill_T=T, fill_P=P, fill_cv=cv, fill_bmod=bm, fill_lambda=lam)
    Tq = np.exp(np.random.default_rng(seed + 1).uniform(np.log(50.0), np.log(3e6), nq))
    out["Tq"] = Tq
    for fn in ALL_FN:
        second = Tq if fn in (1, 2, 4, 6, 8) else sie
        out[f"fn{fn}"] = ref.eos_vec(d, fn, rho, second)
    dump, scal = ref.spiner_dump(path, 1)
    # the full derived-table image is 4.7 MB: keep its hash and a strided sample
    out["dump_sha256"] = np.array(hashlib.sha256(dump.tobytes()).hexdigest())
    out["dump_len"] = np.int64(dump.size)
    out["dump_sample"] = dump[::97].copy()
    out["scal"] = scal
    return out


def spiner_rhosie_fixture(ref, path, n=2048, seed=7):
    """SpinerEOSDependsRhoSie on the StiffGas-sampled rho-T / rho-sie table:
    the eleven vector functions and e(rho, P) with lambda rows of one entry,
    FillEos from (rho, sie), from (rho, T) and from (P, T), the load-time
    tables (DBLIST order), the scalars and the bounds."""
    rho, sie, T = sp5lite.rhosie_queries(n, seed=seed)
    d = rb.eos_desc(rb.SPINER_RHOSIE, [], path=path, matid=3)
    out = dict(rho=rho, sie=sie, T=T)
    for fn in ALL_FN + [13]:
        second = T if fn in (1, 2, 4, 6, 8) else sie
        if fn == 13:
            second = ref.eos_vec(d, 3, rho, sie)  # P(rho, sie) as the target pressure
            out["P_target"] = second
        lam = np.full(n, np.nan)
        out[f"fn{fn}"] = ref.eos_vec(d, fn, rho, second, lam=lam, lam_stride=1)
        out[f"fn{fn}_lambda"] = lam
    # FillEos: (rho, sie) -> T, P, cv, bmod; (rho, T) -> sie, P, cv, bmod;
    # (P, T) -> rho, sie
    fills = {"e": (Q_TPB, rb.Q_SIE), "t": (rb.Q_SIE | rb.Q_PRESSURE | rb.Q_SPECIFIC_HEAT |
                                             rb.Q_BULK_MODULUS, rb.Q_TEMPERATURE),
             "pt": (rb.Q_DENSITY | rb.Q_SIE, rb.Q_PRESSURE | rb.Q_TEMPERATURE)}
    P_in = ref.eos_vec(d, 2, rho, T)
    for tag, (q, _) in fills.items():
        r, t, e, p, cv, bm = rho.copy(), T.copy(), sie.copy(), P_in.copy(), np.zeros(n), np.zeros(n)
        lam = np.full(n, np.nan)
        ref.fill_eos(d, r, t, e, p, cv, bm, q, lam=lam, lam_stride=1)
        out.update({f"fill_{tag}_rho": r, f"fill_{tag}_T": t, f"fill_{tag}_sie": e,
                    f"fill_{tag}_P": p, f"fill_{tag}_cv": cv, f"fill_{tag}_bmod": bm,
                    f"fill_{tag}_lambda": lam, f"fill_{tag}_output": np.int64(q)})
    out["P_in"] = P_in
    dump, scal = ref.spiner_sie_dump(path, 3)
    out["dump_sha256"] = np.array(hashlib.sha256(dump.tobytes()).hexdigest())
    out["dump_len"] = np.int64(dump.size)
    out["dump_sample"] = dump[::97].copy()
    out["scal"] = scal
    Tb = np.array([50.0, 300.0, 1e4, 1e6])
    out["bounds_T"] = Tb
    for w in range(6):
        out[f"bound{w}"] = ref.eos_bounds(d, w, Tb)
    return out


def helm_fixture(ref, path, n=2048, seed=31):
    """Helmholtz EOS on the synthetic table, default options (all on): the
    forward FillEos, the vector member functions, the inversion as the
    reference performs it (reading the lT cache back over the root) and as
    it is meant (sgref_helm_T_from_rho_sie), and the loaded table."""
    from sgx import helmtable
    rho, T, abar, zbar = helmtable.helm_queries(n, seed=seed)
    out = dict(rho=rho, T=T, abar=abar, zbar=zbar)
    d = rb.eos_desc(rb.HELMHOLTZ, [], path=path, flags=31)

    def lam_fresh(lT=np.nan):
        lam = np.zeros(3 * n)
        lam[0::3], lam[1::3], lam[2::3] = abar, zbar, lT
        return lam

    sie, P, cv, bm = (np.zeros(n) for _ in range(4))
    lam = lam_fresh()
    ref.fill_eos(d, rho.copy(), T.copy(), sie, P, cv, bm,
                 rb.Q_SIE | rb.Q_PRESSURE | rb.Q_SPECIFIC_HEAT | rb.Q_BULK_MODULUS,
                 lam=lam, lam_stride=3)
    out.update(fwd_sie=sie, fwd_P=P, fwd_cv=cv, fwd_bmod=bm, fwd_lam=lam.copy())
    for fn in (1, 2, 4, 6, 8):
        out[f"fn{fn}"] = ref.eos_vec(d, fn, rho, T, lam=lam_fresh(), lam_stride=3)
    # the reference's inversion: with the cache from the forward call the
    # root is replaced by the cached log10 T
    Tr, Pr, cvr, bmr = (np.zeros(n) for _ in range(4))
    lam_rb = lam.copy()
    ref.fill_eos(d, rho.copy(), Tr, sie.copy(), Pr, cvr, bmr,
                 rb.Q_TEMPERATURE | rb.Q_PRESSURE | rb.Q_SPECIFIC_HEAT | rb.Q_BULK_MODULUS,
                 lam=lam_rb, lam_stride=3)
    out.update(rb_T=Tr, rb_P=Pr, rb_cv=cvr, rb_bmod=bmr)
    for fn in (3, 5, 7, 9):
        out[f"rb_fn{fn}"] = ref.eos_vec(d, fn, rho, sie, lam=lam.copy(), lam_stride=3)
    # ... and with an out-of-table cache value
    out["rb_invalid_T"] = ref.eos_vec(d, 0, rho, sie, lam=lam_fresh(-1.0), lam_stride=3)
    out["fix_T"] = ref.helm_T_from_rho_sie(path, rho, sie, abar, zbar)
    dump = ref.helm_dump(path)
    nodes = helmtable.NRHO + helmtable.NTEMP
    out["dump_nodes"] = dump[:nodes].copy()
    out["dump_fields_sha256"] = np.array(hashlib.sha256(dump[nodes:].tobytes()).hexdigest())
    out["dump_len"] = np.int64(dump.size)
    return out


def mixutil_fixture(ref, ncell=2048, seed=121):
    """ApproxTemperatureFromRhoMatU, EnforceMassVolumesSum and
    EnforceEnergiesSum on the batched workload's cells after a PTESolverRhoT
    solve, with the volume fractions and energies perturbed by 1e-6 so that
    the sums need fixing, and a temperature guess in half the cells."""
    wl = W.pte_batched(ncell, seed=seed)
    descs = [desc(m) for m in wl["materials"]]
    r = {k: wl[k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
    ref.pte(0, descs, wl["eos_idx"], wl["vfrac_tot"], wl["sie_tot"], r["rho"], r["vfrac"],
            r["sie"], r["temp"], r["press"], params=ref.mix_params())
    rng = np.random.default_rng(seed + 1)
    present = wl["eos_idx"] >= 0
    rho = np.where(present, r["rho"], 0.0)
    vfrac = np.where(present, r["vfrac"] * (1 + 1e-6 * rng.standard_normal(rho.shape)), 0.0)
    sie = np.where(present, r["sie"] * (1 + 1e-6 * rng.standard_normal(rho.shape)), 0.0)
    rho_tot = (wl["rho"] * wl["vfrac"]).sum(axis=0)
    u_tot = rho_tot * wl["sie_tot"]
    tguess = np.where(rng.random(ncell) < 0.5, 0.0,
                      np.abs(r["temp"][0]) * rng.uniform(0.5, 2.0, ncell))
    out = dict(materials=mats_array(wl["materials"]), eos_idx=wl["eos_idx"], rho=rho,
               vfrac=vfrac, sie=sie, rho_tot=rho_tot, sie_tot=wl["sie_tot"], u_tot=u_tot,
               tguess=tguess, vfrac_tot=wl["vfrac_tot"])
    out["approx_T"] = ref.approx_temperature(descs, wl["eos_idx"], u_tot, rho, vfrac)
    out["approx_T_guess"] = ref.approx_temperature(descs, wl["eos_idx"], u_tot, rho, vfrac,
                                                   Tguess=tguess)
    r1, v1 = rho.copy(), vfrac.copy()
    ref.enforce_sums(0, wl["eos_idx"], wl["vfrac_tot"], r1, v1)
    out["vol_rho"], out["vol_vfrac"] = r1, v1
    e2 = sie.copy()
    ref.enforce_sums(1, wl["eos_idx"], wl["sie_tot"], rho.copy(), vfrac.copy(), tot_rho=rho_tot,
                     sie=e2)
    out["energy_sie"] = e2
    return out


SGEOS_CELLS = ("press", "pmax", "vol", "spvol", "sie", "temp", "bmod", "dpde", "cv")
SGEOS_FRACS = ("frac_mass", "frac_vol", "frac_ie", "frac_bmod", "frac_dpde", "frac_cv")


def sgeos_fixture(ref, cell_dim=700, ncell=512, seed=41, cutoff=1e-8, mode=1, rows=None):
    """get_sg_eos on four materials (IdealGas, StiffGas, NobleAbel, copper
    Gruneisen) in input mode `mode` (1 rho-sie, -1 P-T, -2 rho-P, -3 rho-T):
    mass fractions with some materials absent or below the cutoff, pure
    cells among them, cells addressed through a 1-based offset list. The
    (rho, sie) mode keeps its original inputs; the others draw T from
    [0.01, 10] eV and P from [1e8, 1e10] microbar."""
    rng = np.random.default_rng(seed)
    mats = [W.IDEAL_AIR, W.STIFF_WATER, W.NOBLE_ABEL_GAS, W.GRUNEISEN_CU]
    nmat = len(mats)
    fm = rng.exponential(1.0, (nmat, cell_dim))
    kind = rng.random(cell_dim)
    fm[:, kind < 0.2] *= (rng.random((nmat, (kind < 0.2).sum())) < 0.3)  # some absent
    pure = kind > 0.9
    fm[:, pure] = 0.0
    fm[rng.integers(0, nmat, pure.sum()), np.flatnonzero(pure)] = 1.0
    tiny = rng.random((nmat, cell_dim)) < 0.05
    fm[tiny] = 1e-12  # below the cutoff
    fm[0, fm.sum(axis=0) == 0] = 1.0
    fm *= rng.uniform(0.5, 2.0, cell_dim)  # not normalised
    rho = np.exp(rng.uniform(np.log(1e-3), np.log(10.0), cell_dim))
    cells = dict(press=rng.uniform(0, 1e10, cell_dim), pmax=rng.uniform(0, 1e12, cell_dim),
                 vol=rng.uniform(0.5, 2.0, cell_dim), spvol=1.0 / rho,
                 sie=rng.uniform(1e9, 1e11, cell_dim), temp=rng.uniform(0, 1e3, cell_dim),
                 bmod=np.zeros(cell_dim), dpde=np.zeros(cell_dim), cv=np.zeros(cell_dim))
    if mode != 1:
        cells["press"] = rng.uniform(1e8, 1e10, cell_dim)
        cells["temp"] = rng.uniform(0.01, 10.0, cell_dim)
    fracs = dict(frac_mass=np.ascontiguousarray(fm), frac_vol=np.zeros((nmat, cell_dim)),
                 frac_ie=np.zeros((nmat, cell_dim)), frac_bmod=np.zeros((nmat, cell_dim)),
                 frac_dpde=np.zeros((nmat, cell_dim)), frac_cv=np.zeros((nmat, cell_dim)))
    offsets = (rng.permutation(cell_dim)[:ncell] + 1).astype(np.int32)
    eos_offsets = np.array([1, 2, 3, 4], np.int32)
    out = {"in_" + k: v.copy() for k, v in {**cells, **fracs}.items()}
    descs = [desc(m) for m in mats] if rows is None else \
        [mdesc(m, r) for m, r in zip(mats, rows)]
    conv = ref.get_sg_eos(mode, descs, eos_offsets, offsets, cells, fracs, cutoff)
    out.update({"out_" + k: v for k, v in {**cells, **fracs}.items()})
    if rows is not None:  # modifiers per material (mods_row layout)
        out["mods"] = np.array(rows)
    out.update(materials=mats_array(mats), offsets=offsets, eos_offsets=eos_offsets,
               cutoff=np.float64(cutoff), converged=conv, mode=np.int32(mode))
    return out


def mods_row(shift=None, scale=None, ramp=None):
    """[bits, shift, scale, r0, a, b, c]: bit 0 shifted, 1 scaled, 2 ramped."""
    row = np.zeros(7)
    if shift is not None:
        row[0] += 1
        row[1] = shift
    if scale is not None:
        row[0] += 2
        row[2] = scale
    if ramp is not None:
        row[0] += 4
        row[3:7] = ramp
    return row


def mdesc(mat, row, path=None):
    """desc() of a model (or, with path, the tabulated one) with the
    modifiers of a mods_row."""
    bits = int(row[0])
    kw = dict(shift=row[1] if bits & 1 else None, scale=row[2] if bits & 2 else None,
              ramp=row[3:7] if bits & 4 else None)
    if path is not None:
        return rb.eos_desc(rb.SPINER_RHOT, [], path=path, matid=1, **kw)
    return rb.eos_desc(mat[0], mat[1], **kw)


# (model, shift, scale, p-alpha (alpha0, Pe, Pc) or None); model None = the
# tabulated StiffGas table
MOD_CASES = [
    ((rb.IDEAL, (0.5, 2.0)), 0.1, 2.0, None),  # test_eos_modifiers.cpp:125-139
    (W.STIFF_WATER, None, 1.5, None),
    (W.NOBLE_ABEL_GAS, 1e8, None, None),
    (W.GRUNEISEN_CU, 1e8, 1.5, (1.2, 1e9, 1e10)),
    (W.IDEAL_AIR, None, None, (1.5, 5e6, 1e7)),
    (W.STIFF_WATER, 1e8, 1.02, (1.3, 1e9, 5e9)),
    (None, 1e8, 1.5, None),
    (None, None, None, (1.5, 1e11, 1e12)),
    (None, 1e8, 1.5, (1.5, 1e11, 1e12)),
]


def modifiers_fixture(ref, path, n=512, seed=61):
    """ShiftedEOS / ScaledEOS / BilinearRampEOS around each model: vector
    lookups, FillEos, pAlpha2BilinearRampParams and the init_sg_* modifier
    step."""
    rng = np.random.default_rng(seed)
    out = {}
    mats, rows = [], []
    for k, (mat, shift, scale, pa) in enumerate(MOD_CASES):
        base = mods_row(shift, scale)
        d0 = mdesc(mat, base, path if mat is None else None)
        ramp = None
        if pa is not None:
            ramp = ref.p_alpha(d0, *pa)
            out[f"c{k}_palpha_in"] = np.array(pa)
            out[f"c{k}_palpha"] = ramp
        row = mods_row(shift, scale, ramp)
        mats.append(mat if mat is not None else (rb.SPINER_RHOT, ()))
        rows.append(row)
        d = mdesc(mat, row, path if mat is None else None)
        if mat is None:
            rho, sie = sp5lite.stiffgas_queries(n, seed=seed + k)
            T = np.exp(rng.uniform(np.log(50.0), np.log(3e6), n))
        else:
            lo, hi = (1e-3, 20.0) if ramp is None else (0.3 * ramp[0], 30 * ramp[0])
            rho = np.exp(rng.uniform(np.log(lo), np.log(hi), n))
            T = np.exp(rng.uniform(np.log(50.0), np.log(1e5), n))
            if k == 0:  # the unit-scale gas of the reference's test, and its point
                sie = rng.uniform(0.05, 5.0, n)
                rho[0], sie[0] = 2.0, 0.5
            else:
                sie = rng.uniform(1e8, 1e11, n)
        out[f"c{k}_rho"], out[f"c{k}_sie"], out[f"c{k}_T"] = rho, sie, T
        for fn in ALL_FN:
            second = T if fn in (1, 2, 4, 6, 8) else sie
            out[f"c{k}_fn{fn}"] = ref.eos_vec(d, fn, rho, second)
        # FillEos with (rho, sie) in; IdealGas under ShiftedEOS / ScaledEOS
        # aborts in the reference (PreferredInput has all four bits) and is
        # left out
        if not (mat is not None and mat[0] == rb.IDEAL and row[0] % 4):
            a = dict(rho=rho.copy(), temp=np.zeros(n), sie=sie.copy(), press=np.zeros(n),
                     cv=np.zeros(n), bmod=np.zeros(n))
            ref.fill_eos(d, a["rho"], a["temp"], a["sie"], a["press"], a["cv"], a["bmod"], Q_TPB)
            for q, v in a.items():
                out[f"c{k}_fill_{q}"] = v
        # FillEos of a density under a ramp: (P, T) in, (rho, sie) out
        if ramp is not None and mat is not None:
            P = np.exp(rng.uniform(np.log(1e5), np.log(5e10), n))
            a = dict(rho=np.zeros(n), temp=T.copy(), sie=np.zeros(n), press=P.copy(),
                     cv=np.zeros(n), bmod=np.zeros(n))
            ref.fill_eos(d, a["rho"], a["temp"], a["sie"], a["press"], a["cv"], a["bmod"],
                         rb.Q_DENSITY | rb.Q_SIE)
            for q, v in a.items():
                out[f"c{k}_fillrho_{q}"] = v
            out[f"c{k}_fillrho_P"] = P
    out["materials"] = mats_array(mats)
    out["mods"] = np.array(rows)
    # the tabulated p-alpha whose first root sits on the bracket's end: a and
    # the ramp are infinite (no ramp can be built from them)
    out["palpha_edge_in"] = np.array([1.3, 1e9, 5e9])
    out["palpha_edge"] = ref.p_alpha(mdesc(None, mods_row(), path), 1.3, 1e9, 5e9)
    # the init_sg_* modifier step (test_eos_modifiers.cpp:225-247 and others)
    inits = [((rb.IDEAL, (0.5, 2.0)), [0, 0, 0, 1], [0.0, 0.0, 1.5, 5e7, 1e8, 0.0]),
             ((rb.IDEAL, (0.5, 2.0)), [0, 0, 1, 0], [0.0, 0.0, 1e9, 1.0, 2.0, 1.0]),
             (W.STIFF_WATER, [1, 1, 0, 1], [1.02, 1e8, 1.3, 1e9, 5e9, 0.0]),
             (W.GRUNEISEN_CU, [1, 0, 0, 1], [1.5, 0.0, 1.2, 1e9, 1e10, 0.0]),
             (W.NOBLE_ABEL_GAS, [0, 1, 0, 0], [0.0, 1e8, 0.0, 0.0, 0.0, 0.0])]
    out["init_materials"] = mats_array([m for m, _, _ in inits])
    out["init_enabled"] = np.array([e for _, e, _ in inits], np.int32)
    out["init_vals_in"] = np.array([v for _, _, v in inits])
    out["init_vals_out"] = np.array([ref.init_mods(desc(m), e, v) for m, e, v in inits])
    return out


def pt_derivs_fixture(ref, path, n=256, seed=71):
    """PTDerivativesFromPreferred at consistent states (sie and P from
    (rho, T) of the same EOS): every model, bare and modified."""
    rng = np.random.default_rng(seed)
    air_ramp = ref.p_alpha(desc(W.IDEAL_AIR), 1.5, 5e6, 1e7)
    cases = [  # (model or None for the table, mods row, rho range, T range)
        (W.IDEAL_AIR, mods_row(), (1e-4, 1.0), (50.0, 1e5)),
        (W.STIFF_WATER, mods_row(), (0.5, 3.0), (200.0, 5e3)),
        (W.NOBLE_ABEL_GAS, mods_row(), (1e-4, 1.0), (50.0, 1e5)),
        (W.GRUNEISEN_CU, mods_row(), (8.0, 11.0), (300.0, 3e3)),
        (None, mods_row(), (0.5, 20.0), (300.0, 1e5)),
        ((rb.IDEAL, (0.5, 2.0)), mods_row(0.1, 2.0), (0.5, 3.0), (1.0, 10.0)),
        (W.IDEAL_AIR, mods_row(ramp=air_ramp), (0.3 * air_ramp[0], 30 * air_ramp[0]),
         (50.0, 3e3)),
        (W.STIFF_WATER, mods_row(1e8, 1.02), (0.5, 3.0), (200.0, 5e3)),
        (None, mods_row(1e8, 1.5), (0.5, 10.0), (300.0, 1e5)),
    ]
    out = {}
    mats, rows = [], []
    for k, (mat, row, (rlo, rhi), (tlo, thi)) in enumerate(cases):
        d = mdesc(mat, row, path if mat is None else None)
        rho = np.exp(rng.uniform(np.log(rlo), np.log(rhi), n))
        T = np.exp(rng.uniform(np.log(tlo), np.log(thi), n))
        if k == 5:  # test_eos_modifiers.cpp:160-167
            rho[0], T[0] = 1.5, 2.0
        sie = ref.eos_vec(d, 1, rho, T)
        P = ref.eos_vec(d, 2, rho, T)
        out[f"c{k}_rho"], out[f"c{k}_sie"], out[f"c{k}_P"], out[f"c{k}_T"] = rho, sie, P, T
        # lambda rows of NaN: with none, the tabulated model's
        # DensityEnergyFromPressureTemperature starts its root find from an
        # uninitialised cache (eos_spiner_rho_temp.hpp:1147-1151)
        lam = np.full(2 * n, np.nan)
        out[f"c{k}_d"] = np.array(ref.pt_derivs(d, rho, sie, P, T, lam=lam, lam_stride=2))
        out[f"c{k}_lambda"] = lam
        mats.append(mat if mat is not None else (rb.SPINER_RHOT, ()))
        rows.append(row)
    out["materials"] = mats_array(mats)
    out["mods"] = np.array(rows)
    return out


def vector_ext_fixture(ref, path, n=384, seed=81):
    """EntropyFromDensityTemperature / EntropyFromDensityInternalEnergy
    (fn 11, 12) and InternalEnergyFromDensityPressure (fn 13), bare and
    modified; P inputs are P(rho, T) of the same EOS, so roots exist."""
    rng = np.random.default_rng(seed)
    air_ramp = ref.p_alpha(desc(W.IDEAL_AIR), 1.5, 5e6, 1e7)
    cases = [  # (model or None, mods row, rho range, T range, entropy?)
        (W.IDEAL_AIR, mods_row(), (1e-4, 1.0), (50.0, 1e5), True),
        (W.STIFF_WATER, mods_row(), (0.5, 3.0), (200.0, 5e3), True),
        (W.NOBLE_ABEL_GAS, mods_row(), (1e-4, 1.0), (50.0, 1e5), True),
        (W.GRUNEISEN_CU, mods_row(), (8.0, 11.0), (300.0, 3e3), False),
        (None, mods_row(), (0.5, 20.0), (300.0, 1e5), False),
        ((rb.IDEAL, (0.5, 2.0)), mods_row(0.1, 2.0), (0.5, 3.0), (1.0, 10.0), True),
        (W.IDEAL_AIR, mods_row(ramp=air_ramp), (0.3 * air_ramp[0], 30 * air_ramp[0]),
         (50.0, 3e3), True),
        (W.STIFF_WATER, mods_row(1e8, 1.02), (0.5, 3.0), (200.0, 5e3), True),
        (None, mods_row(1e8, 1.5), (0.5, 10.0), (300.0, 1e5), False),
    ]
    out = {}
    mats, rows = [], []
    for k, (mat, row, (rlo, rhi), (tlo, thi), ent) in enumerate(cases):
        d = mdesc(mat, row, path if mat is None else None)
        rho = np.exp(rng.uniform(np.log(rlo), np.log(rhi), n))
        T = np.exp(rng.uniform(np.log(tlo), np.log(thi), n))
        sie = ref.eos_vec(d, 1, rho, T)
        P = ref.eos_vec(d, 2, rho, T)
        out[f"c{k}_rho"], out[f"c{k}_sie"], out[f"c{k}_P"], out[f"c{k}_T"] = rho, sie, P, T
        if ent:
            out[f"c{k}_fn11"] = ref.eos_vec(d, 11, rho, T)
            out[f"c{k}_fn12"] = ref.eos_vec(d, 12, rho, sie)
        out[f"c{k}_fn13"] = ref.eos_vec(d, 13, rho, P)
        mats.append(mat if mat is not None else (rb.SPINER_RHOT, ()))
        rows.append(row)
    out["materials"] = mats_array(mats)
    out["mods"] = np.array(rows)
    # the constructors with a reference state (flags bit 1), at the states
    # of the reference's own entropy tests (test_eos_ideal.cpp:44-90,
    # test_eos_stiff.cpp:495-580) and at random ones
    refs = [(rb.IDEAL, [0.4, 5.0, 100.0, 1e-3]),
            (rb.STIFF, [1.35, 1816.e4, 1.0e9, 2030.00e+07, -23.0e+7, 200.0, 1e6]),
            (rb.NOBLE_ABEL, [0.4, 0.718e7, 1e-3, 1e8, -2e7, 250.0, 2e6])]
    for j, (kind, params) in enumerate(refs):
        d = rb.eos_desc(kind, params, flags=2)
        rho = np.exp(rng.uniform(np.log(1e-3), np.log(1.0), n))
        T = np.exp(rng.uniform(np.log(50.0), np.log(1e4), n))
        if j == 0:
            rho[:3], T[:3] = [1e-3, 0.1, 1e-3], [100.0, 100.0, 10.0]
        sie = ref.eos_vec(d, 1, rho, T)
        if j == 1:
            rho[0], sie[0] = 1.0218087167564040e-01, 3.7350567520918861e+10
        out[f"r{j}_kind"], out[f"r{j}_params"] = np.int32(kind), np.array(params)
        out[f"r{j}_rho"], out[f"r{j}_T"], out[f"r{j}_sie"] = rho, T, sie
        out[f"r{j}_fn11"] = ref.eos_vec(d, 11, rho, T)
        out[f"r{j}_fn12"] = ref.eos_vec(d, 12, rho, sie)
    return out


def modified_pte_fixture(ref, solver, seed):
    """PTE over materials with modifiers: an ideal gas under a p-alpha ramp
    next to a shifted and scaled stiff gas (two materials), and the batched
    workload with three of its materials modified."""
    out = {}
    air_ramp = ref.p_alpha(desc(W.IDEAL_AIR), 1.5, 5e6, 1e7)
    wl = W.pte_two_material(512, seed=seed)
    rows = [mods_row(ramp=air_ramp), mods_row(1e8, 1.02)]
    wl2 = W.pte_batched(1024, seed=seed + 1)
    if solver == 1:  # as pte_pt_batched: ideal, stiff and Noble-Abel only
        wl2["materials"] = wl2["materials"][:7]
        wl2["eos_idx"] = np.where(wl2["eos_idx"] == 7, 6, wl2["eos_idx"]).astype(np.int32)
    rows2 = [mods_row() for _ in wl2["materials"]]
    rows2[0] = mods_row(ramp=air_ramp)
    rows2[1] = mods_row(None, 1.02)
    rows2[2] = mods_row(1e7, None)
    rows2[5] = mods_row(1e8, 1.02)
    for tag, w, rr in (("2mat", wl, rows), ("batched", wl2, rows2)):
        mats = list(w["materials"])
        descs = [mdesc(m, r) for m, r in zip(mats, rr)]
        r = {k: w[k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
        conv, nit, res = ref.pte(solver, descs, w["eos_idx"], w["vfrac_tot"], w["sie_tot"],
                                 r["rho"], r["vfrac"], r["sie"], r["temp"], r["press"],
                                 params=ref.mix_params())
        out[f"{tag}_materials"] = mats_array(mats)
        out[f"{tag}_mods"] = np.array(rr)
        out[f"{tag}_vfrac_tot"], out[f"{tag}_sie_tot"] = w["vfrac_tot"], w["sie_tot"]
        if w["eos_idx"] is not None:
            out[f"{tag}_eos_idx"] = w["eos_idx"]
        out[f"{tag}_converged"], out[f"{tag}_niter"] = conv, nit
        for k in ("rho", "vfrac", "sie", "temp", "press"):
            out[f"{tag}_in_" + k] = w[k]
            out[f"{tag}_out_" + k] = r[k]
    out["solver"] = np.int32(solver)
    return out


def main():
    if not rb.have_reference():
        sys.exit("oracle/_ref/libsgref.so not built; run oracle/build_ref.sh")
    ref = rb.reference()
    fx = {}
    fx["pte_rhot_2mat"] = pte_fixture(ref, W.pte_two_material(2048, seed=101), 0)
    fx["pte_rhot_2mat_tight"] = pte_fixture(
        ref, W.pte_two_material(512, seed=102), 0,
        dict(pte_rel_tolerance_p=1e-12, pte_rel_tolerance_e=1e-12,
             pte_abs_tolerance_p=0.0, pte_rel_tolerance_p_sufficient=1e-10,
             pte_rel_tolerance_e_sufficient=1e-10, pte_abs_tolerance_p_sufficient=0.0))
    fx["pte_rhot_batched"] = pte_fixture(ref, W.pte_batched(2048, seed=103), 0)
    fx["pte_pt_2mat"] = pte_fixture(ref, W.pte_two_material(1024, seed=104), 1)
    wl = W.pte_batched(1024, seed=105)
    wl["materials"] = wl["materials"][:7]  # ideal, stiff and Noble-Abel only
    wl["eos_idx"] = np.where(wl["eos_idx"] == 7, 6, wl["eos_idx"]).astype(np.int32)
    fx["pte_pt_batched"] = pte_fixture(ref, wl, 1)
    # PTESolverRhoU, PTESolverFixedT (target T), PTESolverFixedP (target P)
    for solver, tag, seed in ((2, "rhou", 107), (3, "fixedt", 109), (4, "fixedp", 111)):
        for shape, make in (("2mat", W.pte_two_material), ("batched", W.pte_batched)):
            wl = make(1024, seed=seed + (shape == "batched"))
            n = wl["sie_tot"].size
            trng = np.random.default_rng(seed + 50)
            if solver == 3:
                wl["sie_tot"] = np.exp(trng.uniform(np.log(300.0), np.log(3e4), n))
            elif solver == 4:
                wl["sie_tot"] = np.exp(trng.uniform(np.log(1e8), np.log(1e11), n))
            fx[f"pte_{tag}_{shape}"] = pte_fixture(ref, wl, solver)
    fx["eos_vector"] = vector_fixture(
        ref, [W.IDEAL_AIR, W.STIFF_WATER, W.NOBLE_ABEL_GAS, W.GRUNEISEN_CU])
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "stiffgas.sp5")
        sp5lite.stiffgas_table(path)
        sha = hashlib.sha256(open(path, "rb").read()).hexdigest()
        fx["spiner_lookup"] = spiner_fixture(ref, path)
        fx["spiner_lookup"]["table_sha256"] = np.array(sha)
        # PTE with the tabulated material next to an ideal gas
        wl = W.pte_two_material(512, seed=106)
        wl["materials"] = [W.IDEAL_AIR, (rb.SPINER_RHOT, ())]
        descs = [desc(W.IDEAL_AIR), rb.eos_desc(rb.SPINER_RHOT, [], path=path, matid=1)]
        r = {k: wl[k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
        conv, nit, res = ref.pte(0, descs, None, wl["vfrac_tot"], wl["sie_tot"], r["rho"],
                                 r["vfrac"], r["sie"], r["temp"], r["press"],
                                 params=ref.mix_params())
        o = dict(vfrac_tot=wl["vfrac_tot"], sie_tot=wl["sie_tot"], converged=conv, niter=nit,
                 residual=res, table_sha256=np.array(sha))
        for k in ("rho", "vfrac", "sie", "temp", "press"):
            o["in_" + k] = wl[k]
            o["out_" + k] = r[k]
        fx["pte_rhot_spiner"] = o
        fx["modifiers"] = modifiers_fixture(ref, path)
        fx["modifiers"]["table_sha256"] = np.array(sha)
        fx["pt_derivs"] = pt_derivs_fixture(ref, path)
        fx["pt_derivs"]["table_sha256"] = np.array(sha)
        fx["eos_vector_ext"] = vector_ext_fixture(ref, path)
        fx["eos_vector_ext"]["table_sha256"] = np.array(sha)
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "rhosie.sp5")
        sp5lite.rhosie_table(path)
        sha = hashlib.sha256(open(path, "rb").read()).hexdigest()
        fx["spiner_rhosie"] = spiner_rhosie_fixture(ref, path)
        fx["spiner_rhosie"]["table_sha256"] = np.array(sha)
        # PTE with the rho-sie tabulated material beside an ideal gas, both
        # solvers that take it (RhoT and PT)
        for solver, tag, seed in ((0, "rhot", 141), (1, "pt", 143)):
            wl = W.pte_two_material(512, seed=seed)
            wl["materials"] = [W.IDEAL_AIR, (rb.SPINER_RHOSIE, ())]
            descs = [desc(W.IDEAL_AIR), rb.eos_desc(rb.SPINER_RHOSIE, [], path=path, matid=3)]
            r = {k: wl[k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
            conv, nit, res = ref.pte(solver, descs, None, wl["vfrac_tot"], wl["sie_tot"],
                                     r["rho"], r["vfrac"], r["sie"], r["temp"], r["press"],
                                     params=ref.mix_params())
            o = dict(vfrac_tot=wl["vfrac_tot"], sie_tot=wl["sie_tot"], converged=conv,
                     niter=nit, residual=res, table_sha256=np.array(sha),
                     solver=np.int32(solver))
            for k in ("rho", "vfrac", "sie", "temp", "press"):
                o["in_" + k] = wl[k]
                o["out_" + k] = r[k]
            fx[f"pte_{tag}_rhosie"] = o
    air_ramp = ref.p_alpha(desc(W.IDEAL_AIR), 1.5, 5e6, 1e7)
    sg_rows = [mods_row(ramp=air_ramp), mods_row(1e8, 1.02), mods_row(1e7, None),
               mods_row(None, 1.01)]
    fx["get_sg_eos_modified"] = sgeos_fixture(ref, seed=47, rows=sg_rows)
    fx["get_sg_eos_p_t_modified"] = sgeos_fixture(ref, seed=48, mode=-1, rows=sg_rows)
    fx["pte_rhot_modified"] = modified_pte_fixture(ref, 0, 131)
    fx["pte_pt_modified"] = modified_pte_fixture(ref, 1, 133)
    fx["get_sg_eos"] = sgeos_fixture(ref)
    fx["mix_utils"] = mixutil_fixture(ref)
    for mode, tag in ((-3, "rho_t"), (-2, "rho_p"), (-1, "p_t")):
        fx[f"get_sg_eos_{tag}"] = sgeos_fixture(ref, seed=42 - mode, mode=mode)
    with tempfile.TemporaryDirectory() as td:
        from sgx import helmtable
        path = os.path.join(td, "helm_table.dat")
        sha = helmtable.helm_table(path)
        fx["helmholtz"] = helm_fixture(ref, path)
        fx["helmholtz"]["table_sha256"] = np.array(sha)
    only = set(sys.argv[1:])
    for name, d in fx.items():
        if only and name not in only:
            continue
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: getattr(v, "shape", None) for k, v in list(d.items())[:4]})


if __name__ == "__main__":
    main()
