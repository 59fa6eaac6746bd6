"""Builds libsgx.so (the CUDA library behind include/sgx.h) in-tree.

One nvcc invocation per translation unit, run in parallel, all for sm_103a
only; the output lands in singularity-eos_gb300/lib/. Kernels of the plain
FP64 path and the host-side table derivation are compiled without
floating-point contraction (--fmad=false, -ffp-contract=off) so that they
round exactly as the reference does; the mixed-precision kernels keep FMA.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
OBJDIR = os.path.join(HERE, "_build")
LIB = os.path.join(LIBDIR, "libsgx.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
# (object name, source, extra flags)
UNITS = [
    ("sgx_fp64", "sgx_fp64.cu", ["--fmad=false"]),
    ("sgx_mixed", "sgx_mixed.cu", ["--fmad=true"]),
    ("sgx_lookup_mixed", "sgx_lookup_mixed.cu", ["--fmad=true"]),
    ("sgx_lookup_sie", "sgx_lookup_sie.cu", ["--fmad=true"]),
    ("sgx_capi", "sgx_capi.cu", ["--fmad=false"]),
    ("sgx_table", "sgx_table.cu", ["--fmad=false"]),
    ("sgx_noalloc", "sgx_noalloc.cu", ["--fmad=false"]),
    ("sgx_helm", "sgx_helm.cu", ["--fmad=false"]),
    ("sgx_server", "sgx_server.cu", ["--fmad=false"]),
    ("sgx_sgeos", "sgx_sgeos.cu", ["--fmad=false"]),
    ("sgx_mixutil", "sgx_mixutil.cu", ["--fmad=false"]),
    ("sgx_pool", "sgx_pool.cu", ["--fmad=false"]),
    ("sgx_modifiers", "sgx_modifiers.cu", ["--fmad=false"]),
    ("sgx_sgapi", "sgx_sgapi.cu", ["--fmad=false"]),
    ("sgx_plan", "sgx_plan.cu", ["--fmad=false"]),
] + [(f"sgx_pte_fp64_n{n}", "sgx_pte_fp64_n.cu", ["--fmad=false", f"-DSGX_PTE_N={n}"])
     for n in range(1, 7)] + [
    (f"sgx_pte_fp64_bare_n{n}", "sgx_pte_fp64_n.cu",
     ["--fmad=false", f"-DSGX_PTE_N={n}", "-DSGX_BARE_MODELS"])
    for n in range(1, 7)] + [
    (f"sgx_pte_mixed_n{n}", "sgx_pte_mixed_n.cu", ["--fmad=true", f"-DSGX_PTE_N={n}"])
    for n in range(1, 7)] + [
    (f"sgx_pte_ext_n{n}", "sgx_pte_ext_n.cu", ["--fmad=false", f"-DSGX_PTE_N={n}"])
    for n in range(1, 7)] + [
    (f"sgx_pte_retry_n{n}", "sgx_pte_retry_n.cu", ["--fmad=false", f"-DSGX_PTE_N={n}"])
    for n in range(1, 7)]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(name, src, extra, verbose):
    obj = os.path.join(OBJDIR, name + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + ARCH + COMMON + extra
    if verbose:
        cmd.append("-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(len(UNITS), os.cpu_count() or 4)) as ex:
        futs = {ex.submit(_compile, n, s, e, verbose): n for n, s, e in UNITS}
        objs, logs = [], {}
        for f in cf.as_completed(futs):
            obj, log = f.result()
            objs.append(obj)
            logs[futs[f]] = log
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp] + sorted(objs) + ARCH + ["-cudart", "shared",
                                                                  "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        for k, v in logs.items():
            print(f"== {k}\n{v}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
