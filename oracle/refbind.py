"""ctypes binding to the oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, tests/golden/make_golden.py,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the
product.

Two libraries share one C surface (``sg*_pte``, ``sg*_eos_vec``,
``sg*_fill_eos``, ...):

* ``oracle/_ref/libsgref.so`` -- the reference's own headers compiled against
  the shims in ``oracle/shims`` (built only where the reference sources are
  present, by ``oracle/build_ref.sh``);
* ``oracle/_build/libsgport.so`` -- ``oracle/port/sgport.cpp``, this
  project's restatement of the same algorithms, built everywhere by
  ``oracle/build_port.sh`` and pinned against the first library's output
  through the committed golden fixtures.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SO = os.path.join(HERE, "_ref", "libsgref.so")
PORT_SO = os.path.join(HERE, "_build", "libsgport.so")

# EOS type codes shared by the oracle and the product (include/sgx.h).
IDEAL, STIFF, NOBLE_ABEL, GRUNEISEN, SPINER_RHOT, HELMHOLTZ, SPINER_RHOSIE = 1, 2, 3, 4, 5, 6, 7

# thermalqs bits (singularity-eos/base/constants.hpp:22-34)
Q_DENSITY, Q_SIE, Q_PRESSURE, Q_TEMPERATURE = 1, 2, 4, 8
Q_SPECIFIC_HEAT, Q_BULK_MODULUS = 16, 32


class EosDesc(C.Structure):
    _fields_ = [
        ("type", C.c_int32),
        ("flags", C.c_int32),
        ("matid", C.c_int32),
        ("pad", C.c_int32),
        ("p", C.c_double * 16),
        ("path", C.c_char_p),
        ("mods", C.c_int32),
        ("pad2", C.c_int32),
        ("shift", C.c_double),
        ("scale", C.c_double),
        ("ramp", C.c_double * 4),
    ]


class MixParams(C.Structure):
    """Field-for-field copy of singularity::MixParams
    (mixed_cell_models.hpp:43-78)."""

    _fields_ = [
        ("verbose", C.c_int32),
        ("iterate_t_guess", C.c_int32),
        ("derivative_eps", C.c_double),
        ("pte_rel_tolerance_p", C.c_double),
        ("pte_rel_tolerance_t", C.c_double),
        ("pte_rel_tolerance_e", C.c_double),
        ("pte_rel_tolerance_v", C.c_double),
        ("pte_abs_tolerance_p", C.c_double),
        ("pte_abs_tolerance_t", C.c_double),
        ("pte_slow_convergence_thresh", C.c_double),
        ("pte_rel_tolerance_p_sufficient", C.c_double),
        ("pte_rel_tolerance_t_sufficient", C.c_double),
        ("pte_rel_tolerance_e_sufficient", C.c_double),
        ("pte_rel_tolerance_v_sufficient", C.c_double),
        ("pte_abs_tolerance_p_sufficient", C.c_double),
        ("pte_abs_tolerance_t_sufficient", C.c_double),
        ("pte_max_iter_per_mat", C.c_int64),
        ("line_search_alpha", C.c_double),
        ("line_search_max_iter", C.c_int64),
        ("line_search_fac", C.c_double),
        ("vfrac_safety_fac", C.c_double),
        ("temperature_limit", C.c_double),
        ("default_tguess", C.c_double),
        ("min_dtde", C.c_double),
        ("pte_small_step_tries", C.c_int64),
        ("pte_small_step_thresh", C.c_double),
        ("pte_max_dpdv", C.c_double),
        ("pte_reduced_system_exclude_idx", C.c_int64),
    ]


def eos_desc(type_, params=(), path=None, matid=0, flags=0, shift=None, scale=None,
             ramp=None):
    """An EOS description; shift / scale / ramp (r0, a, b, c) wrap the model
    in ShiftedEOS / ScaledEOS / BilinearRampEOS, nested ramp(scaled(shifted))."""
    d = EosDesc()
    d.type = type_
    d.flags = flags
    d.matid = matid
    for i, v in enumerate(params):
        d.p[i] = float(v)
    d.path = path.encode() if path else None
    if shift is not None:
        d.mods |= 1
        d.shift = float(shift)
    if scale is not None:
        d.mods |= 2
        d.scale = float(scale)
    if ramp is not None:
        d.mods |= 4
        for i, v in enumerate(ramp):
            d.ramp[i] = float(v)
    return d


_D = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_I = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


class Oracle:
    """One oracle library (prefix ``sgref`` or ``sgport``)."""

    def __init__(self, path, prefix):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        self.prefix = prefix
        f = self._fn
        f("mix_params_default").argtypes = [C.POINTER(MixParams)]
        f("pte").restype = C.c_int
        f("eos_vec").restype = C.c_int
        f("fill_eos").restype = C.c_int
        f("rho_sie_from_pt").restype = C.c_int
        f("eos_bounds").restype = C.c_int
        f("spiner_dump").restype = C.c_long
        f("nqt").restype = None

    def _fn(self, name):
        return getattr(self.lib, f"{self.prefix}_{name}")

    def mix_params(self, **kw):
        m = MixParams()
        self._fn("mix_params_default")(C.byref(m))
        for k, v in kw.items():
            setattr(m, k, v)
        return m

    def pte(self, solver, descs, eos_idx, vfrac_tot, sie_tot, rho, vfrac, sie, temp,
            press, params=None, lam=None, nthreads=1):
        """Runs PTESolverRhoT (solver=0), PTESolverPT (1), PTESolverRhoU (2),
        PTESolverFixedT (3) or PTESolverFixedP (4) per cell; sie_tot carries
        each cell's scalar constructor argument (T_true for FixedT, P for
        FixedP).
        Per-material arrays are [nmat_max, ncell] float64 and are updated in
        place. Returns (converged, niter, residual)."""
        nmat, ncell = rho.shape
        arr = (EosDesc * len(descs))(*descs)
        conv = np.zeros(ncell, np.int32)
        nit = np.zeros(ncell, np.int32)
        res = np.zeros(ncell, np.float64)
        rc = self._fn("pte")(
            C.c_int(solver), C.c_int(nmat), C.c_int(ncell), arr, C.c_int(len(descs)),
            _ip(eos_idx), _dp(vfrac_tot), _dp(sie_tot), _dp(rho), _dp(vfrac), _dp(sie),
            _dp(temp), _dp(press), _dp(lam),
            C.byref(params) if params is not None else None, _ip(conv), _ip(nit),
            _dp(res), C.c_int(nthreads))
        if rc != 0:
            raise RuntimeError(f"{self.prefix}_pte failed")
        return conv, nit, res

    def eos_vec(self, desc, fn, in1, in2=None, lam=None, lam_stride=0):
        n = in1.shape[0]
        out = np.zeros(n, np.float64)
        if in2 is None:
            in2 = np.zeros(n, np.float64)
        rc = self._fn("eos_vec")(C.byref(desc), C.c_int(fn), C.c_int(n), _dp(in1),
                                 _dp(in2), _dp(out), _dp(lam), C.c_int(lam_stride))
        if rc != 0:
            raise RuntimeError(f"{self.prefix}_eos_vec failed")
        return out

    def fill_eos(self, desc, rho, temp, sie, press, cv, bmod, output, lam=None,
                 lam_stride=0):
        n = rho.shape[0]
        rc = self._fn("fill_eos")(C.byref(desc), C.c_int(n), _dp(rho), _dp(temp),
                                  _dp(sie), _dp(press), _dp(cv), _dp(bmod),
                                  C.c_ulong(output), _dp(lam), C.c_int(lam_stride))
        if rc != 0:
            raise RuntimeError(f"{self.prefix}_fill_eos failed")

    def rho_sie_from_pt(self, desc, P, T, rho_guess=None):
        n = P.shape[0]
        rho = np.array(rho_guess, np.float64) if rho_guess is not None else np.zeros(n)
        sie = np.zeros(n)
        rc = self._fn("rho_sie_from_pt")(C.byref(desc), C.c_int(n), _dp(P), _dp(T),
                                         _dp(rho), _dp(sie))
        if rc != 0:
            raise RuntimeError(f"{self.prefix}_rho_sie_from_pt failed")
        return rho, sie

    def eos_bounds(self, desc, what, x):
        x = np.ascontiguousarray(x, np.float64)
        out = np.zeros_like(x)
        rc = self._fn("eos_bounds")(C.byref(desc), C.c_int(what), C.c_int(x.shape[0]),
                                    _dp(x), _dp(out))
        if rc != 0:
            raise RuntimeError(f"{self.prefix}_eos_bounds failed")
        return out

    def helm_dump(self, path):
        f = self._fn("helm_dump")
        f.restype = C.c_long
        n = f(path.encode(), None, C.c_long(0))
        if n < 0:
            raise RuntimeError("helm_dump failed")
        out = np.zeros(n)
        f(path.encode(), _dp(out), C.c_long(n))
        return out

    def helm_fill(self, path, options, rho, temp, sie, press, cv, bmod, output, lam):
        """Helmholtz FillEos over n elements (port only: sgport_helm_fill),
        OpenMP over the host threads; lam rows [Abar, Zbar, lT] (n x 3),
        updated with log10 T as the library's default mode stores it."""
        n = rho.shape[0]
        fn = self._fn("helm_fill")
        fn.restype = C.c_int
        rc = fn(C.c_char_p(path.encode()), C.c_int(options), C.c_int(n), _dp(rho), _dp(temp),
                _dp(sie), _dp(press), _dp(cv), _dp(bmod), C.c_uint(output), _dp(lam))
        if rc != 0:
            raise RuntimeError(f"{self.prefix}_helm_fill failed")

    def helm_T_from_rho_sie(self, path, rho, sie, abar, zbar):
        """T(rho, sie) of the default-option Helmholtz EOS without the lT
        cache read-back (reference library only)."""
        n = rho.shape[0]
        T = np.zeros(n)
        rc = self._fn("helm_T_from_rho_sie")(path.encode(), C.c_int(n), _dp(rho), _dp(sie),
                                             _dp(abar), _dp(zbar), _dp(T))
        if rc != 0:
            raise RuntimeError("helm_T_from_rho_sie failed")
        return T

    def get_sg_eos(self, input_int, descs, eos_offsets, offsets, cells, fracs, cutoff):
        """get_sg_eos over host arrays (reference library only) in any input
        mode (1/0 rho-sie, -1 P-T, -2 rho-P, -3 rho-T); cells / fracs are
        updated in place, as the reference does. Returns the per-cell
        converged flags."""
        nmat, cell_dim = fracs["frac_mass"].shape
        arr = (EosDesc * len(descs))(*descs)
        eo = np.ascontiguousarray(eos_offsets, np.int32)
        off = np.ascontiguousarray(offsets, np.int32)
        conv = np.zeros(off.size, np.int32)
        f = self._fn("get_sg_eos")
        f.restype = C.c_int
        rc = f(C.c_int(nmat), C.c_int(off.size), C.c_int(cell_dim), C.c_int(input_int), _ip(eo),
               arr, C.c_int(len(descs)), _ip(off),
               *(_dp(cells[k]) for k in ("press", "pmax", "vol", "spvol", "sie", "temp", "bmod",
                                         "dpde", "cv")),
               *(_dp(fracs.get(k)) for k in ("frac_mass", "frac_vol", "frac_ie", "frac_bmod",
                                             "frac_dpde", "frac_cv")),
               C.c_double(cutoff), _ip(conv))
        if rc != 0:
            raise RuntimeError("get_sg_eos failed")
        return conv

    def get_sg_eos_rho_e(self, descs, eos_offsets, offsets, cells, fracs, cutoff):
        """get_sg_eos in (rho, sie) mode."""
        return self.get_sg_eos(1, descs, eos_offsets, offsets, cells, fracs, cutoff)

    def approx_temperature(self, descs, eos_idx, u_tot, rho, vfrac, Tguess=None, lam=None):
        """ApproxTemperatureFromRhoMatU per cell (reference library only)."""
        nmat, ncell = rho.shape
        arr = (EosDesc * len(descs))(*descs)
        out = np.zeros(ncell)
        f = self._fn("approx_temperature")
        f.restype = C.c_int
        rc = f(C.c_int(nmat), C.c_int(ncell), arr, C.c_int(len(descs)), _ip(eos_idx),
               _dp(u_tot), _dp(rho), _dp(vfrac), _dp(Tguess), _dp(lam), _dp(out))
        if rc != 0:
            raise RuntimeError("approx_temperature failed")
        return out

    def enforce_sums(self, which, eos_idx, tot, rho, vfrac, tot_rho=None, sie=None):
        """MixUtils::EnforceMassVolumesSum (which=0) / EnforceEnergiesSum
        (which=1) per cell, in place (reference library only)."""
        nmat, ncell = rho.shape
        f = self._fn("enforce_sums")
        f.restype = C.c_int
        f(C.c_int(which), C.c_int(nmat), C.c_int(ncell), _ip(eos_idx), _dp(tot), _dp(tot_rho),
          _dp(rho), _dp(vfrac), _dp(sie))

    def pt_derivs(self, desc, rho, sie, P, T, lam=None, lam_stride=0):
        """PTDerivativesFromPreferred per element (reference library only):
        returns (dedP_T, drdP_T, dedT_P, drdT_P); lam (rows of lam_stride,
        updated in place) may be None."""
        n = rho.size
        out = np.zeros(4 * n)
        f = self._fn("pt_derivs")
        f.restype = C.c_int
        rc = f(C.byref(desc), C.c_int(n), _dp(np.ascontiguousarray(rho, np.float64)),
               _dp(np.ascontiguousarray(sie, np.float64)), _dp(np.ascontiguousarray(P, np.float64)),
               _dp(np.ascontiguousarray(T, np.float64)), _dp(out), _dp(lam), C.c_int(lam_stride))
        if rc != 0:
            raise RuntimeError("pt_derivs failed")
        return tuple(out.reshape(4, n))

    def p_alpha(self, desc, alpha0, Pe, Pc):
        """pAlpha2BilinearRampParams of the (shifted / scaled) EOS desc
        (reference library only): returns (r0, a, b, c)."""
        out = np.zeros(4)
        f = self._fn("p_alpha")
        f.restype = C.c_int
        rc = f(C.byref(desc), C.c_double(alpha0), C.c_double(Pe), C.c_double(Pc), _dp(out))
        if rc != 0:
            raise RuntimeError("p_alpha failed")
        return out

    def init_mods(self, desc, enabled, vals):
        """The modifier step of init_sg_* on the bare model of desc (reference
        library only): returns vals as the reference leaves them."""
        en = np.ascontiguousarray(enabled, np.int32)
        v = np.ascontiguousarray(vals, np.float64).copy()
        f = self._fn("init_mods")
        f.restype = C.c_int
        rc = f(C.byref(desc), _ip(en), _dp(v))
        if rc != 0:
            raise RuntimeError("init_mods failed")
        return v

    def spiner_dump(self, path, matid):
        scal = np.zeros(8)
        n = self._fn("spiner_dump")(path.encode(), C.c_int(matid), None, C.c_long(0),
                                    _dp(scal))
        if n < 0:
            raise RuntimeError("spiner_dump failed")
        out = np.zeros(n)
        self._fn("spiner_dump")(path.encode(), C.c_int(matid), _dp(out), C.c_long(n),
                                _dp(scal))
        return out, scal

    def spiner_sie_dump(self, path, matid):
        """SpinerEOSDependsRhoSie's tables in DBLIST order, and its scalars
        (the compiled reference only)."""
        f = self._fn("spiner_sie_dump")
        f.restype = C.c_long
        scal = np.zeros(18)
        n = f(path.encode(), C.c_int(matid), None, C.c_long(0), _dp(scal))
        if n < 0:
            raise RuntimeError("spiner_sie_dump failed")
        out = np.zeros(n)
        f(path.encode(), C.c_int(matid), _dp(out), C.c_long(n), _dp(scal))
        return out, scal

    def nqt(self, which, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.zeros_like(x)
        self._fn("nqt")(C.c_int(which), C.c_int(x.shape[0]), _dp(x), _dp(y))
        return y


def reference():
    """The compiled reference (only where oracle/_ref was built)."""
    return Oracle(REF_SO, "sgref")


def port():
    """This project's C++ restatement."""
    return Oracle(PORT_SO, "sgport")


def have_reference():
    return os.path.exists(REF_SO)
