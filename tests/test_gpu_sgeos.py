"""sgx_get_sg_eos (host arrays, as the reference takes them) and
sgx_get_sg_eos_device (device arrays) against the reference's get_sg_eos
driver in each input mode (tests/golden/get_sg_eos*.npz, made by the oracle around the
reference's own PTESolverRhoT / FixedT / FixedP, root finder and EOS calls):
every per-cell and per-material output, within 1e-12 relative (the n >= 3
solves factor the Jacobian with a different QR than the oracle), untouched
cells left as they were."""
import numpy as np
import pytest

from common import golden, materials_from_rows

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CELLS = ("press", "pmax", "vol", "spvol", "sie", "temp", "bmod", "dpde", "cv")
FRACS = ("frac_mass", "frac_vol", "frac_ie", "frac_bmod", "frac_dpde", "frac_cv")


@pytest.fixture(scope="module")
def sgx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sgx import lib
    lib.load()
    return lib


def run(sgx, fx, precision, host=False):
    eos = [sgx.make_eos(k, p) for k, p in materials_from_rows(fx["materials"])]
    if "mods" in fx:  # ShiftedEOS / ScaledEOS / BilinearRampEOS per material
        eos = [sgx.modify(e, shift=r[1] if int(r[0]) & 1 else None,
                          scale=r[2] if int(r[0]) & 2 else None,
                          ramp=r[3:7] if int(r[0]) & 4 else None) for e, r in zip(eos, fx["mods"])]
    mode = int(fx["mode"]) if "mode" in fx else 1
    if host:
        arrs = {k: np.ascontiguousarray(fx["in_" + k], np.float64).copy() for k in CELLS + FRACS}
        sgx.get_sg_eos_host(eos, fx["eos_offsets"], np.ascontiguousarray(fx["offsets"], np.int32),
                            {k: arrs[k] for k in CELLS}, {k: arrs[k] for k in FRACS},
                            float(fx["cutoff"]), precision=precision, input_int=mode)
        return arrs
    dev = {k: torch.as_tensor(fx["in_" + k], device="cuda").clone() for k in CELLS + FRACS}
    offsets = torch.as_tensor(fx["offsets"], device="cuda")
    sgx.get_sg_eos(eos, fx["eos_offsets"], offsets, {k: dev[k] for k in CELLS},
                   {k: dev[k] for k in FRACS}, float(fx["cutoff"]), precision=precision,
                   input_int=mode)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in dev.items()}


def close(got, want, rtol, label):
    same_special = np.array_equal(np.isnan(got), np.isnan(want)) and \
        np.array_equal(np.isinf(got), np.isinf(want))
    assert same_special, f"{label}: NaN/inf pattern differs"
    ok = np.isfinite(want)
    err = np.abs(got[ok] - want[ok]) / np.maximum(np.abs(want[ok]), 1e-300)
    assert err.max(initial=0.0) <= rtol, f"{label}: max rel err {err.max():.3e}"


@pytest.mark.parametrize("arrays", ["host", "device"])
@pytest.mark.parametrize("name", ["get_sg_eos", "get_sg_eos_rho_t", "get_sg_eos_rho_p",
                                  "get_sg_eos_p_t", "get_sg_eos_modified",
                                  "get_sg_eos_p_t_modified"])
def test_get_sg_eos_matches_reference(sgx, name, arrays):
    fx = golden(name)
    got = run(sgx, fx, 0, host=arrays == "host")
    for k in CELLS + FRACS:
        close(got[k], fx["out_" + k], 1e-12, k)
    # cells outside the offset list are untouched
    untouched = np.setdiff1d(np.arange(fx["in_sie"].size), fx["offsets"] - 1)
    for k in ("press", "temp", "bmod"):
        assert np.array_equal(got[k][untouched], fx["in_" + k][untouched])


def test_get_sg_eos_mixed_precision_agrees(sgx):
    fx = golden("get_sg_eos")
    got = run(sgx, fx, 1)
    conv = fx["converged"].astype(bool)
    cells = fx["offsets"][conv] - 1
    for k in ("press", "temp"):
        w, g = fx["out_" + k][cells], got[k][cells]
        fin = np.isfinite(w)
        scale = np.maximum(np.abs(w[fin]), 1e-6 * np.abs(w[fin]).max())
        # the FP64 solve stops at the default 1e-6 relative tolerances
        assert (np.abs(g[fin] - w[fin]) / scale).max() <= 2e-5, k


def test_get_sg_eos_rejects_bad_modes(sgx):
    import ctypes as C
    lib = sgx.load()
    e = (sgx.SgxEos * 1)(sgx.make_eos(1, (0.4, 0.718e7)))
    eo = (C.c_int * 1)(1)
    for fn in (lib.sgx_get_sg_eos, lib.sgx_get_sg_eos_device):
        for mode in (-4, 2):
            rc = fn(1, 4, 4, mode, C.cast(eo, C.c_void_p), C.cast(e, C.c_void_p), 1,
                    *([None] * 16), 0.0, 0, None)
            assert rc == 1
        # the fixed-T / fixed-P solves have no mixed-precision form
        for mode in (-3, -2):
            rc = fn(1, 4, 4, mode, C.cast(eo, C.c_void_p), C.cast(e, C.c_void_p), 1,
                    *([None] * 16), 0.0, 1, None)
            assert rc == 5
        # null arrays are refused before any copy
        rc = fn(1, 4, 4, 1, C.cast(eo, C.c_void_p), C.cast(e, C.c_void_p), 1,
                *([None] * 16), 0.0, 0, None)
        assert rc == 1
