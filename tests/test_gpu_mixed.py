"""The mixed-precision lookup path (FP32 bracket search + FP64 root and
outputs) against the reference fixtures and against the plain FP64 path.

Error bar. Both paths return a root of the same piecewise-linear function
sie(log10 T) at fixed rho; the reference stops regula falsi within 1e-14 in
log10 T, the mixed path solves the bracketing cell exactly. Where sie is
dominated by its cold (T-independent) part, rounding of sie itself limits
the root to about eps * sie / (d sie / d log10 T): for this table up to
~1e-12 relative in T at 100 K and low density. The tests therefore require
T within 1e-11 relative everywhere and within 1e-12 for 99.9% of queries.
P, bmod, cv and cs are interpolated at that T; their differences are bounded
by 1e-10 relative to the larger of the value and 1e-6 of the batch's
largest magnitude (P crosses zero inside the table)."""
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


def scaled_err(a, b):
    floor = 1e-6 * np.max(np.abs(b))
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


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
        for name, t in (("P", P), ("bmod", bm), ("cv", cv)):
            e = scaled_err(t.cpu().numpy(), fx["fill_" + name])
            assert e.max() <= 1e-10, (name, e.max())
        want_cs = np.sqrt(fx["fill_bmod"] / fx["rho"])
        assert scaled_err(cs.cpu().numpy(), want_cs).max() <= 1e-10
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
        for k in (1, 2, 3):
            assert scaled_err(a[k], b[k]).max() <= 1e-10
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
            for k in (1, 2, 3):
                assert scaled_err(a[k], b[k]).max() <= 1e-10, k
            if cached:
                # the cache holds log10 rho (the reference's rounding, exactly)
                # and log10 T (the root, within T's error / ln 10)
                assert np.array_equal(a[4][0::2], b[4][0::2])
                assert np.abs(a[4][1::2] - b[4][1::2]).max() <= 1e-11 / np.log(10.0)
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


@pytest.mark.parametrize("kind", ["two_material", "batched"])
def test_mixed_pte_accuracy(sgx, kind):
    from sgx import workloads as W
    wl = W.pte_two_material(65536, seed=5) if kind == "two_material" else \
        W.pte_batched(1 << 18, seed=6)
    ref, st_ref = run_pte(sgx, wl, sgx.PREC_FP64, params=sgx.mix_params(**TIGHT))
    got, st = run_pte(sgx, wl, sgx.PREC_MIXED)
    present = wl["eos_idx"] >= 0 if wl["eos_idx"] is not None else np.ones_like(wl["rho"], bool)
    both = st["converged"] & st_ref["converged"]
    resolved = st["resolved_fp64"].mean()
    print(f"{kind}: converged mixed {st['converged'].mean():.4f} tight {st_ref['converged'].mean():.4f}"
          f" fp64 re-solve {resolved:.4f}")
    assert st["converged"].mean() >= st_ref["converged"].mean() - 1e-3
    sel = both[None, :] & present
    for k in ("temp", "press"):
        e = scaled_err(got[k][sel], ref[k][sel])
        print(f"  {k}: max {e.max():.2e} p99.9 {np.quantile(e, 0.999):.2e}")
        assert np.quantile(e, 0.999) <= 1e-10, k
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
