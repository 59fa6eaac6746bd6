"""The mixed-precision lookup path (FP32 bracket search + FP64 root and
outputs) and the mixed-precision PTE path against the reference fixtures
and against the plain FP64 path.

Error bars, per output and per element (plain relative error, no batch-wide
floor):
  * T: the reference stops regula falsi within 1e-14 in log10 T, the mixed
    path solves the bracketing cell in closed form. Where sie is dominated by
    its cold (T-independent) part, rounding of sie itself limits the root to
    about eps * sie / (d sie / d log10 T): for this table up to ~5e-12
    relative at 100 K and low density. T must be within 1e-11 relative
    everywhere and within 1e-12 for 99.9% of queries.
  * P, bmod, cv, cs: within 1e-10 relative of the FP64 value, or, where the
    value is a small difference of large table entries (P crosses zero
    inside the table), closer to the FP64 value than the FP64 value itself
    moves when the input sie changes by 1e-14 relative (a backward-error
    bound: the mixed answer is the FP64 answer of an input within ~50 ulp).
  * PTE: T of every cell both solvers converge within 1e-10 relative of a
    tight-tolerance FP64 solve (tolerances 1e-13); P within 1e-10 relative,
    widened by that solve's own disagreement between the materials'
    pressures and by the change of P_m(rho_m, T) when T moves by 1e-12
    relative (a stiffened gas near P = 0 turns the solves' ~1e-13 in T into
    ~1e-10 in P)."""
import numpy as np
import pytest

from common import golden, rel_err, stiffgas_table_path

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sgx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sgx import lib
    lib.load()
    return lib


def within(got, want, moved, rtol=1e-10):
    """Per element: |got - want| <= rtol |want| + |moved - want|, where
    moved is the FP64 value at an input perturbed by 1e-14 relative. Returns
    the largest ratio of the error to that bound (<= 1 passes) and prints the
    plain relative error."""
    got, want, moved = (np.asarray(x, np.float64) for x in (got, want, moved))
    err = np.abs(got - want)
    bound = rtol * np.abs(want) + np.abs(moved - want)
    e = rel_err(got, want)
    print(f"  plain rel err: max {e.max():.2e} p99.9 {np.quantile(e, 0.999):.2e}; "
          f"{int((e > rtol).sum())} above {rtol:g}")
    r = np.where(err == 0, 0.0, err / np.maximum(bound, 1e-300))
    return float(r.max())


def fp64_moved(sgx, tab, rho, sie, q, lam=None, lam_stride=0):
    """The FP64 path's T, P, bmod, cs at sie (1 + 1e-14)."""
    sie_p = sie * (1.0 + 1e-14)
    T, P, bm, cs = (torch.zeros_like(rho) for _ in range(4))
    sgx.fill_eos(tab, rho, T, sie_p, P, None, bm, q, cs=cs, precision=sgx.PREC_FP64,
                 lam=lam, lam_stride=lam_stride)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in (T, P, bm, cs)]


def check_T(got, want, bulk=True):
    """bulk: the queries are the table's usual population, for which 99.9%
    must also be within 1e-12; a batch made only of cold-dominated states
    (the worst conditioned) is held to the 1e-11 bound alone."""
    e = rel_err(got, want)
    print(f"T rel err: max {e.max():.2e} p99.9 {np.quantile(e, 0.999):.2e} "
          f"median {np.median(e):.2e}")
    assert e.max() <= 1e-11, e.max()
    if bulk:
        assert np.quantile(e, 0.999) <= 1e-12


def test_mixed_lookup_matches_reference(sgx):
    import ctypes as C
    fx = golden("spiner_lookup")
    path, sha = stiffgas_table_path()
    assert sha == str(fx["table_sha256"])
    tab = sgx.spiner_eos(path, 1)
    try:
        rho = torch.as_tensor(fx["rho"], device="cuda")
        sie = torch.as_tensor(fx["sie"], device="cuda")
        T, P, cv, bm, cs = (torch.zeros_like(rho) for _ in range(5))
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS | sgx.Q_SPECIFIC_HEAT
        sgx.fill_eos(tab, rho, T, sie, P, cv, bm, q, cs=cs, precision=sgx.PREC_MIXED)
        torch.cuda.synchronize()
        check_T(T.cpu().numpy(), fx["fill_T"])
        # the FP64 path reproduces the fixture bit for bit (test_gpu_parity),
        # so its perturbed run gives the fixture's sensitivity
        Tm, Pm, bmm, csm = fp64_moved(sgx, tab, rho, sie, sgx.Q_TEMPERATURE | sgx.Q_PRESSURE |
                                      sgx.Q_BULK_MODULUS)
        cvm = torch.zeros_like(rho)
        sgx.fill_eos(tab, rho, torch.zeros_like(rho), sie * (1.0 + 1e-14), torch.zeros_like(rho),
                     cvm, torch.zeros_like(rho), q)
        torch.cuda.synchronize()
        for name, t, m in (("P", P, Pm), ("bmod", bm, bmm), ("cv", cv, cvm.cpu().numpy())):
            r = within(t.cpu().numpy(), fx["fill_" + name], m)
            assert r <= 1.0, (name, r)
        want_cs = np.sqrt(fx["fill_bmod"] / fx["rho"])
        assert within(cs.cpu().numpy(), want_cs, csm) <= 1.0
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


def test_mixed_lookup_full_size_against_fp64(sgx):
    """2^22 queries: mixed vs plain FP64 on device, size-independent bounds."""
    import ctypes as C
    from sgx import sp5lite
    path, _ = stiffgas_table_path()
    tab = sgx.spiner_eos(path, 1)
    try:
        n = 1 << 22
        rho_h, sie_h = sp5lite.stiffgas_queries(n, seed=99)
        rho = torch.as_tensor(rho_h, device="cuda")
        sie = torch.as_tensor(sie_h, device="cuda")
        out = {}
        for prec in (sgx.PREC_FP64, sgx.PREC_MIXED):
            T, P, bm, cs = (torch.zeros_like(rho) for _ in range(4))
            q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS
            sgx.fill_eos(tab, rho, T, sie, P, None, bm, q, cs=cs, precision=prec)
            torch.cuda.synchronize()
            out[prec] = [x.cpu().numpy() for x in (T, P, bm, cs)]
        a, b = out[sgx.PREC_MIXED], out[sgx.PREC_FP64]
        assert np.all(np.isfinite(a[0]))
        check_T(a[0], b[0])
        moved = fp64_moved(sgx, tab, rho, sie, sgx.Q_TEMPERATURE | sgx.Q_PRESSURE |
                           sgx.Q_BULK_MODULUS)
        for k, name in ((1, "P"), (2, "bmod"), (3, "cs")):
            r = within(a[k], b[k], moved[k])
            assert r <= 1.0, (name, r)
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


def test_mixed_lookup_launch_knobs_keep_results(sgx):
    """Blocks per SM, the staging of the coarse index (none, vector loads,
    bulk copy) and the L2 persistence window change the launch, not the
    numbers: every combination returns the default's bits. The batch mixes
    on-table queries with states the float-float pass leaves to the FP64
    pass (off the table in density and energy, zero and NaN inputs), which
    then match the plain FP64 path bit for bit."""
    import ctypes as C
    from sgx import sp5lite
    L = sgx.load()
    path, _ = stiffgas_table_path()
    tab = sgx.spiner_eos(path, 1)
    knobs = (sgx.TUNE_LOOKUP_BLOCKS_PER_SM, sgx.TUNE_LOOKUP_STAGE, sgx.TUNE_L2_PERSIST)
    saved = []
    for k in knobs:
        v = C.c_int()
        assert L.sgx_tune_get(k, C.byref(v)) == 0
        saved.append(v.value)
    try:
        n = (1 << 18) + 77  # a partial last mask word
        rho_h, sie_h = sp5lite.stiffgas_queries(n, seed=7)
        rng = np.random.default_rng(8)
        odd = rng.choice(n, 4000, replace=False)
        # the table spans rho in [1e-4, 1e2]
        rho_h[odd[:1000]] = 1e3 * (1.0 + rng.random(1000))      # above it
        rho_h[odd[1000:2000]] = 1e-6 * (1.0 + rng.random(1000))  # below it
        sie_h[odd[2000:3000]] = -np.abs(sie_h[odd[2000:3000]])  # negative energies
        rho_h[odd[3000:3500]] = 0.0
        sie_h[odd[3500:]] = np.nan
        off = np.concatenate([odd[:2000], odd[3000:]])  # surely off the fast path
        rho = torch.as_tensor(rho_h, device="cuda")
        sie = torch.as_tensor(sie_h, device="cuda")
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS

        def run(prec):
            T, P, bm, cs = (torch.zeros_like(rho) for _ in range(4))
            sgx.fill_eos(tab, rho, T, sie, P, None, bm, q, cs=cs, precision=prec)
            torch.cuda.synchronize()
            return np.stack([x.cpu().numpy() for x in (T, P, bm, cs)])

        base = run(sgx.PREC_MIXED)
        for minb in (4, 5, 6):
            for stage in (0, 1, 2):
                for l2 in (0, 1):
                    for k, v in zip(knobs, (minb, stage, l2)):
                        assert L.sgx_tune_set(k, v) == 0
                    got = run(sgx.PREC_MIXED)
                    assert np.array_equal(got, base, equal_nan=True), (minb, stage, l2)
        fp64 = run(sgx.PREC_FP64)
        assert np.array_equal(base[:, off], fp64[:, off], equal_nan=True)
        check_T(base[0], fp64[0])
        assert L.sgx_tune_set(knobs[0], 9) != 0  # out of range
    finally:
        for k, v in zip(knobs, saved):
            L.sgx_tune_set(k, v)
        L.sgx_eos_finalize(C.byref(tab))


def test_mixed_lookup_between_coarse_density_nodes(sgx):
    """Low density, low temperature, midway between density nodes: the
    table's bilinear interpolant of Pinf/rho overshoots there, so the query
    lies under the interpolated cold curve (off the table's bottom) or under
    the interpolant at the lowest temperature, where the reference's regula
    falsi finds no bracket and returns its guess (the middle of the log T
    range, or the lambda cache). The mixed path reproduces both outcomes,
    with and without a lambda cache."""
    import ctypes as C
    path, _ = stiffgas_table_path()
    tab = sgx.spiner_eos(path, 1)
    try:
        rng = np.random.default_rng(12)
        n = 1 << 16
        lrho = np.log10(1e-4) + 6.0 / 255 * (rng.integers(0, 60, n) + rng.uniform(0.3, 0.7, n))
        rho_h = 10.0 ** lrho
        T = rng.uniform(100.0, 2000.0, n)
        sie_h = 1.816e7 * T + 6e9 / rho_h
        rho = torch.as_tensor(rho_h, device="cuda")
        sie = torch.as_tensor(sie_h, device="cuda")
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS
        # a lambda cache of log10 T: in range for most elements, out of it for some
        lam_init = np.zeros(2 * n)
        lam_init[1::2] = rng.uniform(1.5, 6.5, n)
        for cached in (False, True):
            out = {}
            for prec in (sgx.PREC_FP64, sgx.PREC_MIXED):
                Tt, P, bm, cs = (torch.zeros_like(rho) for _ in range(4))
                lam = torch.as_tensor(lam_init, device="cuda").clone() if cached else None
                sgx.fill_eos(tab, rho, Tt, sie, P, None, bm, q, cs=cs, precision=prec, lam=lam,
                             lam_stride=2 if cached else 0)
                torch.cuda.synchronize()
                out[prec] = [x.cpu().numpy() for x in (Tt, P, bm, cs)]
                if cached:
                    out[prec].append(lam.cpu().numpy())
            a, b = out[sgx.PREC_MIXED], out[sgx.PREC_FP64]
            check_T(a[0], b[0], bulk=False)
            lam_m = torch.as_tensor(lam_init, device="cuda").clone() if cached else None
            moved = fp64_moved(sgx, tab, rho, sie, q, lam=lam_m, lam_stride=2 if cached else 0)
            for k in (1, 2, 3):
                assert within(a[k], b[k], moved[k]) <= 1.0, k
            if cached:
                # the cache holds log10 rho (the reference's rounding, exactly)
                # and log10 T (the root, within T's error / ln 10)
                assert np.array_equal(a[4][0::2], b[4][0::2])
                assert np.abs(a[4][1::2] - b[4][1::2]).max() <= 1e-11 / np.log(10.0)
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


def test_mixed_lookup_roots_just_above_T_nodes(sgx):
    """Roots a hair above a T node: the lower cell's weight 1 + 1e-10 ..
    5e-8 has a float leading part of exactly 1, yet the root is the next
    cell's (the lower cell's form extended past the node misses it by up to
    ~1e-10 relative in T on this table). T within the same bounds as
    everywhere else."""
    import ctypes as C
    import refbind as rb
    from sgx import sp5lite
    path, _ = stiffgas_table_path()
    grid = sp5lite.read(path)["datasets"]["/1/dependsLogRhoLogT/specific internal energy"][1]
    nT, lTmin, lTmax = grid[0]
    dlT = (lTmax - lTmin) / (nT - 1)
    tab = sgx.spiner_eos(path, 1)
    try:
        rng = np.random.default_rng(33)
        n = 1 << 14
        k = rng.integers(1, nT - 2, n)
        lT = lTmin + k * dlT + dlT * 10.0 ** rng.uniform(-10.0, np.log10(5e-8), n)
        T_in = rb.port().nqt(1, lT)  # the reference's 10^lT (NQT)
        rho_h = 10.0 ** rng.uniform(-3.5, 2.0, n)
        rho = torch.as_tensor(rho_h, device="cuda")
        sie = torch.zeros_like(rho)
        sgx.fill_eos(tab, rho, torch.as_tensor(T_in, device="cuda"), sie, None, None, None,
                     sgx.Q_SIE)
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS
        out = {}
        for prec in (sgx.PREC_FP64, sgx.PREC_MIXED):
            Tt, P, bm, cs = (torch.zeros_like(rho) for _ in range(4))
            sgx.fill_eos(tab, rho, Tt, sie, P, None, bm, q, cs=cs, precision=prec)
            torch.cuda.synchronize()
            out[prec] = [x.cpu().numpy() for x in (Tt, P, bm, cs)]
        a, b = out[sgx.PREC_MIXED], out[sgx.PREC_FP64]
        check_T(a[0], b[0], bulk=False)
        moved = fp64_moved(sgx, tab, rho, sie, q)
        for j in (1, 2, 3):
            assert within(a[j], b[j], moved[j]) <= 1.0, j
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


def test_mixed_lookup_top_band(sgx):
    """Roots in the band within 1e-8 of lTMax, below the table's top in sie:
    the reference's regula falsi finds lT there, and its outputs take the
    off-top forms (e0 + Cv (T - TMax) from the lTMax curves). The mixed path
    leaves these to its FP64 pass; T, P, bmod and cs within the same bounds
    as everywhere else."""
    import ctypes as C
    path, _ = stiffgas_table_path()
    tab = sgx.spiner_eos(path, 1)
    try:
        rng = np.random.default_rng(21)
        n = 1 << 14
        rho_h = 10.0 ** rng.uniform(-3.0, 2.0, n)
        # T within 1.1e-7 of TMax = 1e6: lT inside (1 - 1e-8) lTMax .. lTMax
        T_in = 1e6 * (1.0 - rng.uniform(0.5, 0.9, n) * 1.2e-7)
        rho = torch.as_tensor(rho_h, device="cuda")
        sie = torch.zeros_like(rho)
        sgx.fill_eos(tab, rho, torch.as_tensor(T_in, device="cuda"), sie, None, None, None,
                     sgx.Q_SIE)
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS
        out = {}
        for prec in (sgx.PREC_FP64, sgx.PREC_MIXED):
            Tt, P, bm, cs = (torch.zeros_like(rho) for _ in range(4))
            sgx.fill_eos(tab, rho, Tt, sie, P, None, bm, q, cs=cs, precision=prec)
            torch.cuda.synchronize()
            out[prec] = [x.cpu().numpy() for x in (Tt, P, bm, cs)]
        a, b = out[sgx.PREC_MIXED], out[sgx.PREC_FP64]
        # the reference's roots lie in the band (T within 1.4e-7 of TMax)
        assert (b[0] >= 1e6 * (1 - 1.4e-7)).all() and (b[0] <= 1e6 * (1 + 1e-12)).all()
        check_T(a[0], b[0], bulk=False)
        moved = fp64_moved(sgx, tab, rho, sie, q)
        for k in (1, 2, 3):
            assert within(a[k], b[k], moved[k]) <= 1.0, k
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


def test_mixed_rejects_unsupported_calls(sgx):
    e = sgx.make_eos(1, (0.4, 0.718e7))
    x = torch.ones(4, dtype=torch.float64, device="cuda")
    with pytest.raises(RuntimeError, match="mixed precision"):
        sgx.fill_eos(e, x, x.clone(), x.clone(), x.clone(), None, x.clone(),
                     sgx.Q_TEMPERATURE, precision=sgx.PREC_MIXED)


TIGHT = dict(pte_rel_tolerance_p=1e-13, pte_rel_tolerance_e=1e-13, pte_abs_tolerance_p=0.0,
             pte_rel_tolerance_p_sufficient=1e-12, pte_rel_tolerance_e_sufficient=1e-12,
             pte_abs_tolerance_p_sufficient=0.0)


def run_pte(sgx, wl, precision, params=None):
    eos_list = [sgx.make_eos(k, p) for k, p in wl["materials"]]
    t = {k: torch.as_tensor(wl[k], device="cuda") for k in ("rho", "vfrac", "sie", "temp",
                                                             "press")}
    idx = torch.as_tensor(wl["eos_idx"], device="cuda") if wl["eos_idx"] is not None else None
    n = wl["sie_tot"].shape[0]
    status = torch.zeros(n * 16, dtype=torch.uint8, device="cuda")
    sgx.pte_solve(sgx.PTE_RHOT, eos_list, idx, torch.as_tensor(wl["vfrac_tot"], device="cuda"),
                  torch.as_tensor(wl["sie_tot"], device="cuda"), t["rho"], t["vfrac"], t["sie"],
                  t["temp"], t["press"], params=params, status=status, precision=precision)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in t.items()}, sgx.status_view(status)


@pytest.fixture
def group_min_n(sgx, request):
    """Sets SGX_TUNE_PTE_GROUP_MIN_N for one test, restoring it after."""
    import ctypes as C
    L = sgx.load()
    v = C.c_int()
    assert L.sgx_tune_get(sgx.TUNE_PTE_GROUP_MIN_N, C.byref(v)) == 0
    assert L.sgx_tune_set(sgx.TUNE_PTE_GROUP_MIN_N, request.param) == 0
    yield request.param
    L.sgx_tune_set(sgx.TUNE_PTE_GROUP_MIN_N, v.value)


@pytest.mark.parametrize("group_min_n", [3, 7], indirect=True,
                         ids=["lane_groups_from_3", "thread_per_cell"])
@pytest.mark.parametrize("kind", ["two_material", "batched"])
def test_mixed_pte_accuracy(sgx, kind, group_min_n):
    """Against a tight FP64 solve, every cell both converge: P and T within
    1e-10 relative (P widened by the tight solve's own spread of the
    materials' pressures); converged flags as the reference's default solve
    within 1e-5 of the cells (pass 2 caps the FP64 re-solve at 8 iterations
    per material, the reference at 128)."""
    from sgx import workloads as W
    wl = W.pte_two_material(65536, seed=5) if kind == "two_material" else \
        W.pte_batched(1 << 18, seed=6)
    ref, st_ref = run_pte(sgx, wl, sgx.PREC_FP64, params=sgx.mix_params(**TIGHT))
    dflt, st_d = run_pte(sgx, wl, sgx.PREC_FP64)
    got, st = run_pte(sgx, wl, sgx.PREC_MIXED)
    present = wl["eos_idx"] >= 0 if wl["eos_idx"] is not None else np.ones_like(wl["rho"], bool)
    both = st["converged"] & st_ref["converged"]
    ncell = both.size
    flag_diff = int((st["converged"] != st_d["converged"]).sum())
    print(f"{kind}: converged mixed {st['converged'].mean():.5f} default {st_d['converged'].mean():.5f}"
          f" tight {st_ref['converged'].mean():.5f}; fp64 re-solve {st['resolved_fp64'].mean():.4f};"
          f" flags differing from the default solve: {flag_diff}")
    assert flag_diff <= 1e-5 * ncell + 1
    P_t = np.where(present, ref["press"], np.nan)
    spread = np.nanmax(P_t, axis=0) - np.nanmin(P_t, axis=0)
    # |P_m(rho_m, T (1 + 1e-12)) - P_m(rho_m, T)| per material slot
    eos = [sgx.make_eos(kk, pp) for kk, pp in wl["materials"]]
    idx = wl["eos_idx"] if wl["eos_idx"] is not None else \
        np.repeat(np.arange(len(eos), dtype=np.int32)[:, None], ncell, axis=1)
    moved = np.zeros_like(ref["press"])
    for m in range(ref["press"].shape[0]):
        r = torch.as_tensor(ref["rho"][m], device="cuda")
        T0 = torch.as_tensor(ref["temp"][m], device="cuda")
        for k, e in enumerate(eos):
            sel = idx[m] == k
            if not sel.any():
                continue
            p0, p1 = torch.zeros_like(r), torch.zeros_like(r)
            sgx.eval_eos(e, sgx.FN_P_FROM_RHO_T, r, T0, p0)
            sgx.eval_eos(e, sgx.FN_P_FROM_RHO_T, r, T0 * (1.0 + 1e-12), p1)
            torch.cuda.synchronize()
            moved[m, sel] = np.abs((p1 - p0).cpu().numpy())[sel]
    dP = np.where(present, moved, 0.0).max(axis=0)
    for k in ("temp", "press"):
        e = rel_err(got[k], ref[k])
        e[~present] = 0.0
        e = e.max(axis=0)[both]
        print(f"  {k}: max {e.max():.2e} p99.9 {np.quantile(e, 0.999):.2e}")
        if k == "temp":
            assert e.max() <= 1e-10, e.max()
        else:
            err = np.where(present, np.abs(got[k] - ref[k]), 0.0).max(axis=0)
            bound = 1e-10 * np.where(present, np.abs(ref[k]), np.inf).min(axis=0) + spread + dP
            assert np.all(err[both] <= bound[both]), float((err / bound)[both].max())
    # closure constraints hold exactly in FP64 for polished cells
    pol = st["converged"] & ~st["resolved_fp64"]
    vsum = np.where(present, got["vfrac"], 0).sum(axis=0)
    assert np.abs(vsum[pol] - wl["vfrac_tot"][pol]).max() <= 1e-13


@pytest.mark.parametrize("precision", [0, 1])
def test_host_array_fill_matches_device_fill(sgx, precision):
    """sgx_eos_fill_host (chunks streamed through three streams) gives
    exactly the device call's results, across chunk boundaries."""
    import ctypes as C
    from sgx import sp5lite
    path, _ = stiffgas_table_path()
    tab = sgx.spiner_eos(path, 1)
    try:
        n = (1 << 22) + 12345  # three chunks, the last partial
        rho_h, sie_h = sp5lite.stiffgas_queries(n, seed=5)
        host = [torch.empty(n, dtype=torch.float64).pin_memory().numpy() for _ in range(4)]
        lam_h = torch.full((2 * n,), float("nan"), dtype=torch.float64).pin_memory().numpy()
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS
        sgx.fill_eos_host(tab, rho_h, host[0], sie_h, host[1], None, host[2], q, lam=lam_h,
                          lam_stride=2, cs=host[3], precision=precision)
        rho, sie = torch.as_tensor(rho_h, device="cuda"), torch.as_tensor(sie_h, device="cuda")
        T, P, bm, cs = (torch.zeros_like(rho) for _ in range(4))
        lam = torch.full((2 * n,), float("nan"), dtype=torch.float64, device="cuda")
        sgx.fill_eos(tab, rho, T, sie, P, None, bm, q, lam=lam, lam_stride=2, cs=cs,
                     precision=precision)
        torch.cuda.synchronize()
        for h, d in zip(host + [lam_h], (T, P, bm, cs, lam)):
            assert np.array_equal(h.view(np.uint64), d.cpu().numpy().view(np.uint64))
    finally:
        sgx.load().sgx_eos_finalize(C.byref(tab))


def test_autotune_fill_keeps_a_valid_shape_and_the_results(sgx):
    # the autotuner tries every (blocks per SM, staging) pair on the batch,
    # keeps the fastest, and the results stay the default's bits
    import ctypes as C
    from sgx import sp5lite
    L = sgx.load()
    path, _ = stiffgas_table_path()
    tab = sgx.spiner_eos(path, 1)
    saved = []
    for k in (sgx.TUNE_LOOKUP_BLOCKS_PER_SM, sgx.TUNE_LOOKUP_STAGE):
        v = C.c_int()
        assert L.sgx_tune_get(k, C.byref(v)) == 0
        saved.append(v.value)
    try:
        rho_h, sie_h = sp5lite.stiffgas_queries(1 << 20, seed=19)
        rho = torch.as_tensor(rho_h, device="cuda")
        sie = torch.as_tensor(sie_h, device="cuda")
        q = sgx.Q_TEMPERATURE | sgx.Q_PRESSURE | sgx.Q_BULK_MODULUS

        def run():
            T, P, bm = (torch.zeros_like(rho) for _ in range(3))
            sgx.fill_eos(tab, rho, T, sie, P, None, bm, q, precision=sgx.PREC_MIXED)
            torch.cuda.synchronize()
            return np.stack([x.cpu().numpy() for x in (T, P, bm)])

        base = run()
        T, P, bm = (torch.zeros_like(rho) for _ in range(3))
        b, st = sgx.autotune_fill(tab, rho, T, sie, P, None, bm, q, reps=2)
        assert 4 <= b <= 6 and 0 <= st <= 2
        got = []
        for k in (sgx.TUNE_LOOKUP_BLOCKS_PER_SM, sgx.TUNE_LOOKUP_STAGE):
            v = C.c_int()
            L.sgx_tune_get(k, C.byref(v))
            got.append(v.value)
        assert got == [b, st]
        np.testing.assert_array_equal(run(), base)
    finally:
        for k, v in zip((sgx.TUNE_LOOKUP_BLOCKS_PER_SM, sgx.TUNE_LOOKUP_STAGE), saved):
            L.sgx_tune_set(k, v)
        L.sgx_eos_finalize(C.byref(tab))


def test_autotune_pte_keeps_results_within_the_contract(sgx):
    """sgx_tune_autotune_pte times block size, count order and the lane-group
    threshold on the batch and keeps the fastest: the knobs it sets are in
    range, the block size and the count order leave the result bit for bit
    as it was, and the arrays end holding a solve that meets the bar."""
    import ctypes as C
    from sgx import workloads as W
    L = sgx.load()
    knobs = (sgx.TUNE_PTE_MIXED_BLOCK, sgx.TUNE_PTE_COUNT_ORDER, sgx.TUNE_PTE_GROUP_MIN_N)
    saved = []
    for k in knobs:
        v = C.c_int()
        assert L.sgx_tune_get(k, C.byref(v)) == 0
        saved.append(v.value)
    try:
        wl = W.pte_batched(1 << 16, seed=8)
        base, _ = run_pte(sgx, wl, sgx.PREC_MIXED)
        for blk, order in ((32, 1), (64, 0)):
            assert L.sgx_tune_set(sgx.TUNE_PTE_MIXED_BLOCK, blk) == 0
            assert L.sgx_tune_set(sgx.TUNE_PTE_COUNT_ORDER, order) == 0
            got, _ = run_pte(sgx, wl, sgx.PREC_MIXED)
            for k in base:
                assert np.array_equal(got[k], base[k], equal_nan=True), (blk, order, k)
        for k, v in zip(knobs, saved):
            L.sgx_tune_set(k, v)
        eos = [sgx.make_eos(k, p) for k, p in wl["materials"]]
        t = {k: torch.as_tensor(wl[k], device="cuda") for k in ("rho", "vfrac", "sie", "temp",
                                                                 "press")}
        status = torch.zeros(wl["sie_tot"].size * 16, dtype=torch.uint8, device="cuda")
        chosen = sgx.autotune_pte(eos, torch.as_tensor(wl["eos_idx"], device="cuda"),
                                  torch.as_tensor(wl["vfrac_tot"], device="cuda"),
                                  torch.as_tensor(wl["sie_tot"], device="cuda"), t["rho"],
                                  t["vfrac"], t["sie"], t["temp"], t["press"], status=status,
                                  reps=1)
        assert chosen[0] in (32, 64, 128) and chosen[1] in (0, 1) and 2 <= chosen[2] <= 7
        got = []
        for k in knobs:
            v = C.c_int()
            L.sgx_tune_get(k, C.byref(v))
            got.append(v.value)
        assert tuple(got) == tuple(chosen)
        # the arrays hold the chosen setting's solve: the same as a fresh call
        again, _ = run_pte(sgx, wl, sgx.PREC_MIXED)
        for k in again:
            assert np.array_equal(t[k].cpu().numpy(), again[k], equal_nan=True), k
    finally:
        for k, v in zip(knobs, saved):
            L.sgx_tune_set(k, v)
