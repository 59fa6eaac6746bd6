"""The serving loop (sgx_server_*): requests of different sizes submitted at
once are folded into merged solves (their cells end to end in one binned
batch), and each result must be exactly the one sgx_pte_solve gives for
that request alone (same kernels, every cell independent of the others);
admission keeps the arena within its budget; oversized requests are refused
at submission."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

OUT = ("rho", "vfrac", "sie", "temp", "press")


@pytest.fixture(scope="module")
def sgx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sgx import lib
    lib.load()
    return lib


@pytest.fixture(scope="module")
def eos_list(sgx, tmp_path_factory):
    """The batched workload's 8 analytic EOS plus the tabulated StiffGas."""
    import ctypes as C
    from sgx import sp5lite, workloads as W
    path = str(tmp_path_factory.mktemp("serve") / "stiffgas.sp5")
    sp5lite.stiffgas_table(path)
    eos = [sgx.make_eos(k, p) for k, p in W.material_pool(0)]
    tab = sgx.spiner_eos(path, 1)
    yield eos + [tab]
    sgx.load().sgx_eos_finalize(C.byref(tab))


_pinned = []


def pinned(a):
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    _pinned.append(t)
    return t.numpy()


def make_request(ncell, seed):
    from sgx import workloads as W
    req = W.serve_request(ncell, seed, pool=list(range(9)))
    for k in list(req):
        if isinstance(req[k], np.ndarray):
            req[k] = pinned(req[k])
    for k in OUT:
        req[k + "_out"] = pinned(np.zeros_like(req[k + "_in"]))
    req["status"] = pinned(np.zeros(ncell * 16, np.uint8))
    return req


def solve_alone(sgx, eos_list, req, precision):
    dev = {k: torch.as_tensor(req[k + "_in"], device="cuda").clone() for k in OUT}
    idx = torch.as_tensor(req["eos_idx"], device="cuda")
    status = torch.zeros(req["ncell"] * 16, dtype=torch.uint8, device="cuda")
    sgx.pte_solve(sgx.PTE_RHOT, eos_list, idx, torch.as_tensor(req["vfrac_tot"], device="cuda"),
                  torch.as_tensor(req["sie_tot"], device="cuda"), dev["rho"], dev["vfrac"],
                  dev["sie"], dev["temp"], dev["press"], status=status, precision=precision)
    torch.cuda.synchronize()
    out = {k: v.cpu().numpy() for k, v in dev.items()}
    out["status"] = status.cpu().numpy()
    return out


def same(req, want):
    for k in OUT:
        assert np.array_equal(req[k + "_out"].view(np.uint64), want[k].view(np.uint64)), k
    assert np.array_equal(req["status"], want["status"])


@pytest.mark.parametrize("precision", [0, 1])
def test_each_result_is_the_same_alone_and_in_the_mix(sgx, eos_list, precision):
    rng = np.random.default_rng(7 + precision)
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(1e5), 16)).astype(int)
    reqs = [make_request(int(n), seed=100 + i) for i, n in enumerate(sizes)]
    budget = 512 << 20
    srv = sgx.Server(eos_list, hbm_budget_bytes=budget, max_inflight=6, precision=precision)
    try:
        tickets = [srv.submit(r) for r in reqs]
        lat = [srv.wait(t) for t in tickets]
        st = srv.stats()
    finally:
        srv.close()
    assert all(x is not None and x > 0 for x in lat)
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["cells_completed"] == int(sizes.sum())
    assert 0 < st["arena_peak"] <= budget
    # requests waiting together were folded into shared solves
    assert 1 <= st["batches"] < len(reqs), st["batches"]
    for r in reqs:
        same(r, solve_alone(sgx, eos_list, r, precision))


def test_admission_stays_within_the_budget(sgx, eos_list):
    budget = 48 << 20  # room for about two of these requests at a time
    reqs = [make_request(90_000, seed=300 + i) for i in range(6)]
    srv = sgx.Server(eos_list, hbm_budget_bytes=budget, max_inflight=8, precision=1)
    try:
        tickets = [srv.submit(r) for r in reqs]
        for t in tickets:
            assert srv.wait(t) is not None
        st = srv.stats()
    finally:
        srv.close()
    assert st["completed"] == 6
    assert st["arena_peak"] <= budget
    for r in reqs[:2]:
        same(r, solve_alone(sgx, eos_list, r, 1))


def test_oversized_request_is_refused(sgx, eos_list):
    srv = sgx.Server(eos_list, hbm_budget_bytes=8 << 20, max_inflight=2)
    try:
        with pytest.raises(RuntimeError, match="more than the whole arena"):
            srv.submit(make_request(200_000, seed=1))
        # the server keeps working afterwards
        r = make_request(2_000, seed=2)
        assert srv.wait(srv.submit(r)) is not None
    finally:
        srv.close()
    same(r, solve_alone(sgx, eos_list, r, 1))


def test_modified_eos_serve_in_fp64_and_are_refused_in_mixed(sgx, eos_list):
    # a list with ShiftedEOS / ScaledEOS / BilinearRampEOS members serves on
    # the FP64 path with the results of sgx_pte_solve alone; the
    # mixed-precision server takes bare models only
    mod = list(eos_list)
    mod[1] = sgx.modify(mod[1], scale=1.02)
    mod[5] = sgx.modify(mod[5], shift=1e8, scale=1.02)
    mod[8] = sgx.modify(mod[8], shift=1e8)  # the table
    reqs = [make_request(n, seed=300 + i) for i, n in enumerate((3000, 20000, 700))]
    srv = sgx.Server(mod, hbm_budget_bytes=256 << 20, max_inflight=3, precision=0)
    try:
        tickets = [srv.submit(r) for r in reqs]
        for t in tickets:
            srv.wait(t)
    finally:
        srv.close()
    for r in reqs:
        same(r, solve_alone(sgx, mod, r, 0))
    with pytest.raises(RuntimeError, match="unmodified EOS only"):
        sgx.Server(mod, hbm_budget_bytes=256 << 20, max_inflight=3, precision=1)
