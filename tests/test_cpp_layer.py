"""The C++ layer (include/sgx.hpp) compiled into a caller's own program
(tests/cpp/hpp_check.cu), not through ctypes:

* the header compiles with nvcc (no GPU needed);
* on the GPU, the program's vector lookups through raw pointers and through
  a strided indexer, its tabulated FillEos with a type-indexed lambda, and
  its own kernel around PTESolverRhoT / PTESolver agree with the oracle and
  with the C ABI: bit for bit for the vector calls and the two-material
  solve, with the same convergence flags and iteration counts.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from common import PARITY_RTOL, bitwise_frac, rel_err, stiffgas_table_path

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "hpp_check.cu")
LIBDIR = os.path.join(ROOT, "singularity-eos_gb300", "lib")
_EXE = {}


def build_exe():
    """Compiles hpp_check once per session (two-material solvers only, to
    keep the build short)."""
    if "path" in _EXE:
        return _EXE["path"]
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    if not os.path.exists(os.path.join(LIBDIR, "libsgx.so")):
        pytest.skip("libsgx.so not built")
    out = os.path.join(tempfile.mkdtemp(prefix="sgx_hpp_"), "hpp_check")
    cmd = [nvcc, "-std=c++17", "-O3", "--fmad=false", "-Xcompiler", "-ffp-contract=off",
           "-gencode", "arch=compute_103a,code=sm_103a", "--expt-relaxed-constexpr",
           "-DSGX_HPP_MAX_NMAT=2", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "singularity-eos_gb300", "csrc"), SRC, "-o", out,
           "-L", LIBDIR, "-lsgx", "-Xlinker", "-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    _EXE["path"] = out
    return out


def test_header_compiles_in_a_caller_program():
    assert os.path.exists(build_exe())


@pytest.mark.gpu
def test_cpp_caller_matches_oracle_and_c_abi():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import refbind as rb
    from sgx import lib, sp5lite, workloads as W
    exe = build_exe()
    port = rb.port()
    d = tempfile.mkdtemp(prefix="sgx_hpp_run_")
    rng = np.random.default_rng(41)
    # inputs
    n = 4099
    rho = np.exp(rng.uniform(np.log(1e-3), np.log(10.0), n))
    sie = rng.uniform(1e9, 1e11, n)
    rho.tofile(os.path.join(d, "in_vec_rho.bin"))
    sie.tofile(os.path.join(d, "in_vec_sie.bin"))
    path, _ = stiffgas_table_path()
    trho, tsie = sp5lite.stiffgas_queries(8191, seed=42)
    trho.tofile(os.path.join(d, "in_tab_rho.bin"))
    tsie.tofile(os.path.join(d, "in_tab_sie.bin"))
    wl = W.pte_two_material(8192, seed=43)
    wl["rho"].tofile(os.path.join(d, "in_pte_rho.bin"))
    wl["vfrac"].tofile(os.path.join(d, "in_pte_vfrac.bin"))
    wl["sie_tot"].tofile(os.path.join(d, "in_pte_sie_tot.bin"))
    wl["vfrac_tot"].tofile(os.path.join(d, "in_pte_vfrac_tot.bin"))
    r = subprocess.run([exe, d, path], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr

    def out(name, dtype=np.float64):
        return np.fromfile(os.path.join(d, f"out_{name}.bin"), dtype=dtype)

    # 1. vector lookups: the oracle's StiffGas, bit for bit
    stiff = rb.eos_desc(rb.STIFF, (3.4, 1.816e7, 6e9, 0.0))
    T_want = port.eos_vec(stiff, 0, rho, sie)
    P_want = port.eos_vec(stiff, 3, rho, sie)
    assert bitwise_frac(out("vec_T"), T_want) == 1.0
    assert bitwise_frac(out("vec_P"), P_want) == 1.0
    T2 = out("vec_T_strided")
    assert bitwise_frac(T2[0::2], T_want) == 1.0 and np.all(T2[1::2] == 0.0)

    # 2. tabulated FillEos with VariadicIndexer<LogTemperature, LogDensity>
    #    rows against the C ABI with numbered rows [lRho, lT]
    tab = lib.spiner_eos(path, 1)
    try:
        q = lib.Q_TEMPERATURE | lib.Q_PRESSURE | lib.Q_BULK_MODULUS
        rt = torch.as_tensor(trho, device="cuda")
        st = torch.as_tensor(tsie, device="cuda")
        Tt, Pt, cvt, Bt = (torch.zeros_like(rt) for _ in range(4))
        lam = torch.zeros((trho.size, 2), dtype=torch.float64, device="cuda")
        lam[:, 1] = 1e300
        lib.fill_eos(tab, rt, Tt, st, Pt, cvt, Bt, q, lam=lam, lam_stride=2)
        torch.cuda.synchronize()
        for name, t in (("tab_T", Tt), ("tab_P", Pt), ("tab_B", Bt)):
            assert bitwise_frac(out(name), t.cpu().numpy()) == 1.0, name
        lam_h = lam.cpu().numpy()
        assert bitwise_frac(out("tab_lrho"), lam_h[:, 0]) == 1.0
        assert bitwise_frac(out("tab_lT"), lam_h[:, 1]) == 1.0
    finally:
        import ctypes as C
        lib.load().sgx_eos_finalize(C.byref(tab))

    # 3. the caller's PTESolverRhoT kernel against the oracle
    want = {k: wl[k].copy() for k in ("rho", "vfrac", "sie", "temp", "press")}
    conv, nit, _ = port.pte(0, [rb.eos_desc(k, p) for k, p in wl["materials"]], None,
                            wl["vfrac_tot"], wl["sie_tot"], want["rho"], want["vfrac"],
                            want["sie"], want["temp"], want["press"], params=port.mix_params())
    assert np.array_equal(out("pte_conv", np.int32).astype(bool), conv.astype(bool))
    assert np.array_equal(out("pte_niter", np.int32), nit)
    for k in ("rho", "vfrac", "sie", "temp", "press"):
        got = out("pte_" + k).reshape(want[k].shape)
        e = rel_err(got, want[k])
        print(f"hpp PTE {k}: max rel {e.max():.2e}, bitwise {bitwise_frac(got, want[k]):.6f}")
        assert e.max() <= PARITY_RTOL, k
