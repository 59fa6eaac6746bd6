"""sp5-lite: this project's flat binary stand-in for singularity-eos SP5 table
files (HDF5 is not a dependency here), plus a generator of the synthetic
StiffGas-derived rho-T table used by the tabulated-lookup workload.

Image layout (little endian) -- read by singularity-eos_gb300/csrc/sgx_table.cu:
  char magic[8] = "SGXSP5L\\0"; u32 version = 1; u32 nrecords;
  record: u32 kind (1 attr f64, 2 attr i32, 3 dataset f64, 4 attr string);
          u32 len, char path[len]; u32 len, char name[len];
          kind 1: f64;  kind 2: i32;  kind 4: u32 len, bytes;
          kind 3: u32 rank, per dim (fastest first) i32 n, f64 min, f64 max,
                  then f64 data[prod n] in C order (fastest index last).
Group and field names are the reference's SP5 keys
(singularity-eos/base/sp5/singularity_eos_sp5.hpp:20-75).

The grids are uniform in the NQT "fast log10" coordinate
(singularity-eos/base/fast-math/logs.hpp:188-214, 282-292), as
SpinerEOSDependsRhoT expects: node densities and temperatures are
FastMath::pow10 of the grid coordinate, not 10**x. The NQT transforms are
reproduced bit for bit with integer arithmetic below.
"""
import struct

import numpy as np

_ONE_AS_INT = (1 << 62) - (1 << 52)
_SCALE_DOWN = 2.22044604925031e-16
_SCALE_UP = float(1 << 52)
_MANTISSA = (1 << 52) - 1
_LOW = (1 << 26) - 1
_LOG2OLOG10 = 0.301029995663981195
_LOG10OLOG2 = 3.321928094887362626
EPS = 10 * np.finfo(np.float64).eps
SMALL = 10 * np.finfo(np.float64).tiny


def lg_nqt(x):
    x = np.asarray(x, np.float64)
    xi = x.view(np.int64) - np.int64(_ONE_AS_INT)
    frac = xi & np.int64(_MANTISSA)
    hi = frac >> np.int64(26)
    lo = frac & np.int64(_LOW)
    fsq = hi * hi + ((hi * lo) >> np.int64(25))
    return (xi + (frac - fsq) // np.int64(3)).astype(np.float64) * _SCALE_DOWN


def pow2_nqt(x):
    x = np.asarray(x, np.float64)
    xi = (x * _SCALE_UP).astype(np.int64)
    frac = xi & np.int64(_MANTISSA)
    fsqrt = (67108864.0 * np.sqrt((np.int64(18014398509481984) - 3 * frac)
                                  .astype(np.float64))).astype(np.int64)
    return (xi + np.int64(9007199254740992) - fsqrt - frac + np.int64(_ONE_AS_INT)).view(np.float64)


def log10_nqt(x):
    return _LOG2OLOG10 * lg_nqt(x)


def pow10_nqt(x):
    return pow2_nqt(_LOG10OLOG2 * np.asarray(x, np.float64))


def to_log(x, offset=0.0):
    """spiner_common::to_log (eos_spiner_common.hpp:52-54)."""
    x = np.asarray(x, np.float64)
    return log10_nqt(np.abs(np.maximum(x, -offset) + offset) + EPS)


def grid(lmin, lmax, n):
    dx = (lmax - lmin) / float(n - 1)
    return lmin + np.arange(n, dtype=np.float64) * dx


class Writer:
    def __init__(self):
        self.rec = []

    def attr_f64(self, path, name, v):
        self.rec.append((1, path, name, struct.pack("<d", float(v))))

    def attr_i32(self, path, name, v):
        self.rec.append((2, path, name, struct.pack("<i", int(v))))

    def dataset(self, path, data, ranges):
        """ranges: [(n, min, max)] fastest dimension first."""
        data = np.ascontiguousarray(data, np.float64)
        assert data.size == int(np.prod([r[0] for r in ranges]))
        head = struct.pack("<I", len(ranges))
        for n, mn, mx in ranges:
            head += struct.pack("<idd", int(n), float(mn), float(mx))
        self.rec.append((3, path, "", head + data.tobytes()))

    def write(self, fname):
        with open(fname, "wb") as f:
            f.write(b"SGXSP5L\0" + struct.pack("<II", 1, len(self.rec)))
            for kind, path, name, payload in self.rec:
                p, n = path.encode(), name.encode()
                f.write(struct.pack("<I", kind) + struct.pack("<I", len(p)) + p +
                        struct.pack("<I", len(n)) + n + payload)


def read(fname):
    """An sp5-lite image as {"attrs": {path@name: value}, "datasets": {path:
    (array in C order, [(n, min, max)] fastest first)}}."""
    with open(fname, "rb") as f:
        buf = f.read()
    assert buf[:8] == b"SGXSP5L\0"
    _, nrec = struct.unpack_from("<II", buf, 8)
    off = 16
    attrs, datasets = {}, {}

    def string():
        nonlocal off
        (n,) = struct.unpack_from("<I", buf, off)
        off += 4
        v = buf[off:off + n].decode()
        off += n
        return v
    for _ in range(nrec):
        (kind,) = struct.unpack_from("<I", buf, off)
        off += 4
        path, name = string(), string()
        if kind == 1:
            attrs[path + "@" + name] = struct.unpack_from("<d", buf, off)[0]
            off += 8
        elif kind == 2:
            attrs[path + "@" + name] = struct.unpack_from("<i", buf, off)[0]
            off += 4
        elif kind == 4:
            attrs[path + "@" + name] = string()
        else:
            (rank,) = struct.unpack_from("<I", buf, off)
            off += 4
            ranges = []
            for _ in range(rank):
                ranges.append(struct.unpack_from("<idd", buf, off))
                off += 20
            count = int(np.prod([r[0] for r in ranges]))
            data = np.frombuffer(buf, np.float64, count, off).copy()
            off += 8 * count
            datasets[path] = (data.reshape([r[0] for r in reversed(ranges)]), ranges)
    return {"attrs": attrs, "datasets": datasets}


def stiffgas_table(fname, matid=1, nrho=256, nt=256, rho_range=(1e-4, 1e2),
                   t_range=(1e2, 1e6), gm1=3.4, Cv=1.816e7, Pinf=6e9, qq=0.0):
    """Writes a SpinerEOSDependsRhoT-layout table sampled from the StiffGas
    model (singularity-eos/eos/eos_stiff.hpp:63-133) on an NQT-log grid.
    Returns a dict with the grids and model parameters."""
    lr = grid(to_log(rho_range[0]), to_log(rho_range[1]), nrho)
    lt = grid(to_log(t_range[0]), to_log(t_range[1]), nt)
    rho = pow10_nqt(lr)[:, None]
    T = pow10_nqt(lt)[None, :]
    P = np.maximum(gm1 * rho * Cv * T - Pinf, -Pinf)
    sie = np.maximum((rho * Cv * T + Pinf) / (rho + SMALL) + qq, qq)
    bmod = np.maximum(gm1 * (gm1 + 1.0) * rho * Cv * T, SMALL)
    ones = np.ones_like(P)
    dPdRho = gm1 * (sie - qq)                 # (dP/drho)_e
    dPdE = gm1 * rho * ones                   # (dP/de)_rho
    dTdRho = Pinf / (rho * rho * Cv) * ones   # (dT/drho)_e
    dTdE = ones / Cv                          # (dT/de)_rho
    dEdRho = -Pinf / (rho * rho) * ones       # (de/drho)_T
    dEdT = Cv * ones                          # (de/dT)_rho
    r1 = rho[:, 0]
    cold = dict(P=np.full(nrho, -Pinf), sie=Pinf / r1 + qq,
                bmod=np.full(nrho, SMALL), dPdRho=gm1 * Pinf / r1)
    w = Writer()
    w.attr_i32("/", "log_type", 2)
    g = f"/{matid}"
    for name, v in (("rhoOffset", 0.0), ("TOffset", 0.0), ("normalDensity", 1.0),
                    ("meanAtomicMass", 1.0), ("meanAtomicNumber", 1.0)):
        w.attr_f64(g, name, v)
    w.attr_i32(g, "matid", matid)
    r2 = [(nt, lt[0], lt[-1]), (nrho, lr[0], lr[-1])]
    for key, arr in (("pressure", P), ("specific internal energy", sie),
                     ("bulk modulus", bmod), ("dPdRho", dPdRho), ("dPdE", dPdE),
                     ("dTdRho", dTdRho), ("dTdE", dTdE), ("dEdRho", dEdRho), ("dEdT", dEdT)):
        w.dataset(f"{g}/dependsLogRhoLogT/{key}", arr, r2)
    r1g = [(nrho, lr[0], lr[-1])]
    for key, arr in (("pressure", cold["P"]), ("specific internal energy", cold["sie"]),
                     ("bulk modulus", cold["bmod"]), ("dPdRho", cold["dPdRho"])):
        w.dataset(f"{g}/coldCurve/{key}", arr, r1g)
    w.write(fname)
    return dict(lrho=lr, lt=lt, gm1=gm1, Cv=Cv, Pinf=Pinf, qq=qq, matid=matid,
                rho_range=rho_range, t_range=t_range)


def rhosie_table(fname, matid=3, nrho=64, nt=96, ne=80, rho_range=(1e-3, 1e1),
                 t_range=(1e2, 1e5), gm1=3.4, Cv=1.816e7, Pinf=6e9, qq=0.0,
                 sie_offset=1e9, rho_offset=0.0):
    """Writes a SpinerEOSDependsRhoSie-layout table sampled from the StiffGas
    model: the rho-T group (as stiffgas_table), the rho-sie group on an NQT
    grid of log10(sie + sie_offset) spanning the energies the rho-T group
    reaches, and the cold curve. Below a row's cold energy the rho-sie
    group's temperature is floored at 1 K (the pressure keeps the model's
    formula). Returns a dict with the grids and model parameters."""
    lr = grid(to_log(rho_range[0], rho_offset), to_log(rho_range[1], rho_offset), nrho)
    lt = grid(to_log(t_range[0]), to_log(t_range[1]), nt)
    rho1 = pow10_nqt(lr) - rho_offset
    rho = rho1[:, None]
    T = pow10_nqt(lt)[None, :]
    e_lo = Cv * t_range[0] + Pinf / rho_range[1] + qq
    e_hi = Cv * t_range[1] + Pinf / rho_range[0] + qq
    le = grid(to_log(e_lo, sie_offset), to_log(e_hi, sie_offset), ne)
    E = (pow10_nqt(le) - sie_offset)[None, :]
    ones_t = np.ones((nrho, nt))
    ones_e = np.ones((nrho, ne))
    sie_t = (rho * Cv * T + Pinf) / rho + qq
    groups = {
        "dependsLogRhoLogT": (lt, {
            "pressure": gm1 * rho * Cv * T - Pinf,
            "specific internal energy": sie_t,
            "bulk modulus": gm1 * (gm1 + 1.0) * rho * Cv * T,
            "dPdRho": gm1 * (sie_t - qq),
            "dPdE": gm1 * rho * ones_t,
            "dTdRho": Pinf / (rho * rho * Cv) * ones_t,
            "dTdE": ones_t / Cv,
            "dEdRho": -Pinf / (rho * rho) * ones_t,
            "dEdT": Cv * ones_t}),
        "dependsLogRhoLogSie": (le, {
            "temperature": np.maximum((E - qq - Pinf / rho) / Cv, 1.0),
            "pressure": gm1 * rho * (E - qq) - (gm1 + 1.0) * Pinf,
            "bulk modulus": gm1 * (gm1 + 1.0) * rho * np.maximum(E - qq - Pinf / rho, 0.0),
            "dPdRho": gm1 * (E - qq) * ones_e,
            "dPdE": gm1 * rho * ones_e,
            "dTdRho": Pinf / (rho * rho * Cv) * ones_e,
            "dTdE": ones_e / Cv,
            "dEdRho": -Pinf / (rho * rho) * ones_e}),
    }
    w = Writer()
    w.attr_i32("/", "log_type", 2)
    g = f"/{matid}"
    for name, v in (("rhoOffset", rho_offset), ("TOffset", 0.0), ("sieOffset", sie_offset),
                    ("normalDensity", 1.0), ("meanAtomicMass", 47.9),
                    ("meanAtomicNumber", 22.0)):
        w.attr_f64(g, name, v)
    w.attr_i32(g, "matid", matid)
    for grp, (fast, fields) in groups.items():
        r2 = [(fast.size, fast[0], fast[-1]), (nrho, lr[0], lr[-1])]
        for key, arr in fields.items():
            w.dataset(f"{g}/{grp}/{key}", arr, r2)
    r1g = [(nrho, lr[0], lr[-1])]
    cold = {"pressure": np.full(nrho, -Pinf), "specific internal energy": Pinf / rho1 + qq,
            "bulk modulus": np.full(nrho, SMALL), "dPdRho": gm1 * Pinf / rho1}
    for key, arr in cold.items():
        w.dataset(f"{g}/coldCurve/{key}", arr, r1g)
    w.write(fname)
    return dict(lrho=lr, lt=lt, le=le, gm1=gm1, Cv=Cv, Pinf=Pinf, qq=qq, matid=matid,
                rho_range=rho_range, t_range=t_range, e_range=(e_lo, e_hi),
                sie_offset=sie_offset, rho_offset=rho_offset)


def rhosie_queries(n, seed=0, rho_range=(1e-3, 1e1), t_range=(1e2, 1e5), Cv=1.816e7,
                   Pinf=6e9, qq=0.0, off_table=0.05):
    """(rho, sie, T) queries for rhosie_table: rho log-uniform, T log-uniform,
    sie uniform between the model's energies at the T range's ends; a
    fraction off_table of the rows is pushed outside the table (density
    beyond either end, energy below the cold curve or above the top)."""
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(rho_range[0]), np.log(rho_range[1]), n))
    T = np.exp(rng.uniform(np.log(t_range[0]), np.log(t_range[1]), n))
    e_lo = Cv * t_range[0] + Pinf / rho + qq
    e_hi = Cv * t_range[1] + Pinf / rho + qq
    sie = e_lo + rng.random(n) * (e_hi - e_lo)
    k = rng.random(n) < off_table
    which = rng.integers(0, 4, n)
    rho = np.where(k & (which == 0), rho * 1e-2, rho)
    rho = np.where(k & (which == 1), rho * 1e2, rho)
    sie = np.where(k & (which == 2), 0.5 * (Pinf / rho + qq), sie)
    T = np.where(k & (which == 2), 0.3 * t_range[0], T)
    sie = np.where(k & (which == 3), 3.0 * e_hi, sie)
    T = np.where(k & (which == 3), 3.0 * t_range[1], T)
    return rho, sie, T


def stiffgas_queries(n, seed=0, rho_range=(1e-4, 1e2), t_range=(1e2, 1e6), gm1=3.4,
                     Cv=1.816e7, Pinf=6e9, qq=0.0):
    """Lookup queries: rho log-uniform over the table range, sie uniform
    between the model's sie at the table's minimum and maximum temperature at
    that rho."""
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(rho_range[0]), np.log(rho_range[1]), n))
    e_lo = Cv * t_range[0] + Pinf / rho + qq
    e_hi = Cv * t_range[1] + Pinf / rho + qq
    sie = e_lo + rng.random(n) * (e_hi - e_lo)
    return rho, sie
