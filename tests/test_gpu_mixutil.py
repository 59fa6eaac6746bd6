"""The closure utilities against the reference (tests/golden/mix_utils.npz,
made with the reference's own ApproxTemperatureFromRhoMatU and
MixUtils::EnforceMassVolumesSum / EnforceEnergiesSum): bit-identical
results, NaN where the reference gives NaN."""
import numpy as np
import pytest

from common import golden, materials_from_rows

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sgx():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sgx import lib
    lib.load()
    return lib


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def same(got, want, label):
    assert np.array_equal(got, want, equal_nan=True), \
        f"{label}: {np.sum(~((got == want) | (np.isnan(got) & np.isnan(want))))} differ"


def test_approx_temperature_matches_reference(sgx):
    fx = golden("mix_utils")
    eos = [sgx.make_eos(k, p) for k, p in materials_from_rows(fx["materials"])]
    idx = dev(fx["eos_idx"], torch.int32)
    out = torch.zeros(fx["u_tot"].size, dtype=torch.float64, device="cuda")
    sgx.approx_temperature(eos, idx, dev(fx["u_tot"]), dev(fx["rho"]), dev(fx["vfrac"]), out)
    same(out.cpu().numpy(), fx["approx_T"], "no guess")
    sgx.approx_temperature(eos, idx, dev(fx["u_tot"]), dev(fx["rho"]), dev(fx["vfrac"]), out,
                           Tguess=dev(fx["tguess"]))
    same(out.cpu().numpy(), fx["approx_T_guess"], "with guess")


def test_enforce_sums_match_reference(sgx):
    fx = golden("mix_utils")
    idx = dev(fx["eos_idx"], torch.int32)
    rho, vfrac = dev(fx["rho"]), dev(fx["vfrac"])
    sgx.enforce_mass_volumes_sum(idx, dev(fx["vfrac_tot"]), rho, vfrac)
    torch.cuda.synchronize()
    same(rho.cpu().numpy(), fx["vol_rho"], "volumes: rho")
    same(vfrac.cpu().numpy(), fx["vol_vfrac"], "volumes: vfrac")
    sie = dev(fx["sie"])
    sgx.enforce_energies_sum(idx, dev(fx["rho_tot"]), dev(fx["sie_tot"]), dev(fx["rho"]),
                             dev(fx["vfrac"]), sie)
    torch.cuda.synchronize()
    same(sie.cpu().numpy(), fx["energy_sie"], "energies: sie")
