"""The float-float <-> double conversions (sgx_ff.cuh) on the device against
FP64 sums computed on the host (tests/cpp/ff_check.cu): ff2d within one ulp
of (double)hi + (double)lo for pairs of every magnitude, unnormalised pairs,
powers of two with a low part of the opposite sign, zero and subnormal low
parts; ff2d_add bit for bit against the correctly rounded FP64 sum; d2ff ->
ff2d round trips within 2^-47; and the NQT log's integer
core in 32-bit pieces (lg_nqt_int, sgx_math.cuh) bit for bit against the
reference's 64-bit formula."""
import os
import shutil
import subprocess
import tempfile

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ff_conversions():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = os.path.join(tempfile.mkdtemp(prefix="sgx_ff_"), "ff_check")
    r = subprocess.run([nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", os.path.join(ROOT, "singularity-eos_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "cpp", "ff_check.cu"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0 and "bad=0" in r.stdout, r.stdout
