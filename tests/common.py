"""Helpers shared by the tests: fixture loading, EOS construction, and
comparisons in the units of the parity bar (relative error, bitwise)."""
import hashlib
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# The parity bar of the plain FP64 path: relative 1e-12 on P, T, sie_i,
# alpha_i with identical convergence flags.
PARITY_RTOL = 1e-12


def golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def materials_from_rows(rows):
    """Inverse of make_golden.mats_array: [(kind, params)]."""
    out = []
    for r in rows:
        kind = int(r[15])
        npar = {1: 2, 2: 4, 3: 4, 4: 10, 5: 0}[kind]
        out.append((kind, tuple(r[:npar])))
    return out


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    d[a == b] = 0.0
    d[both_nan] = 0.0
    return d


def bitwise_frac(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    same = (a.view(np.int64) == b.view(np.int64)) | (np.isnan(a) & np.isnan(b))
    return float(same.mean())


_TABLE = {}


def rhosie_table_path():
    """The synthetic StiffGas rho-T / rho-sie table of SpinerEOSDependsRhoSie
    (sp5lite.rhosie_table, matid 3), regenerated and cached for the session."""
    if "rhosie" not in _TABLE:
        from sgx import sp5lite
        d = tempfile.mkdtemp(prefix="sgx_table_")
        path = os.path.join(d, "rhosie.sp5")
        sp5lite.rhosie_table(path)
        _TABLE["rhosie"] = (path, hashlib.sha256(open(path, "rb").read()).hexdigest())
    return _TABLE["rhosie"]


def stiffgas_table_path():
    """The synthetic StiffGas rho-T table, regenerated deterministically and
    cached for the session; checked against the fixture's SHA-256."""
    if "path" not in _TABLE:
        from sgx import sp5lite
        d = tempfile.mkdtemp(prefix="sgx_table_")
        path = os.path.join(d, "stiffgas.sp5")
        sp5lite.stiffgas_table(path)
        _TABLE["path"] = path
        _TABLE["sha"] = hashlib.sha256(open(path, "rb").read()).hexdigest()
    return _TABLE["path"], _TABLE["sha"]
