"""Synthetic electron free-energy table in the Helmholtz EOS's ASCII format.

The Helmholtz EOS (Timmes & Swesty 2000) reads the electron-positron free
energy F(De, T) and its derivatives from ``helm_table.dat``: for each of the
101 log-spaced temperatures (log10 T = 3 .. 13) and 271 log-spaced electron
densities (log10 De = -12 .. 15), density fastest, four blocks are read in
turn (HelmElectrons::InitDataFile_, eos/eos_helmholtz.hpp:962-989):

1. f, fd, ft, fdd, ftt, fdt, fddt, fdtt, fddtt: the free energy per gram per
   Ye and its derivatives (d = d/dDe, t = d/dT);
2. dpdf, dpdfd, dpdft, dpdfdt: dP/dDe and its derivatives;
3. ef, efd, eft, efdt: the electron chemical potential (eta) and derivatives;
4. xf, xfd, xft, xfdt: the electron + positron number density and derivatives.

The real table is not available here. This module writes a table of the
same shape from a smooth analytic free energy with exact derivatives, so
the Hermite interpolation reproduces it to high order:

    F(d, T) = -a T (1.5 ln T - ln d + c0) + K d^(2/3) - b T^2 / (d^(2/3) + d0)

an ideal-gas term, a degeneracy-like term and a Sommerfeld-like thermal
correction. The heat capacity -T F_TT = 1.5 a + 2 b T / (d^(2/3) + d0) is
positive everywhere, so e(T) is monotone. P = d^2 F_d. The chemical
potential is eta = ln d - 1.5 ln T + c1 + K2 d^(2/3) / T, and the number
density is NA d + x0 T^3. The table is synthetic: it has the shape of the
real one, not its physics.
"""
import hashlib
import os
from decimal import Decimal, getcontext

import numpy as np

NTEMP, NRHO = 101, 271
LT_MIN, LT_MAX = 3.0, 13.0
LRHO_MIN, LRHO_MAX = -12.0, 15.0

A_GAS = 1.3806504e-16 * 6.02214199e23  # kB * NA
C0 = -20.0
K_DEG = 1.5e13
B_TH = 1.3e3
D0 = 1e-8
C1 = -10.0
K2 = 3e5
NA = 6.02214199e23
X0 = 1e-6


def _node_values():
    """Per-node transcendentals, computed once per density and per
    temperature in decimal arithmetic, which gives the same doubles on every
    platform (the table's SHA-256 is checked against the fixtures)."""
    getcontext().prec = 40
    ten = Decimal(10)
    dens = []
    for i in range(NRHO):
        x = Decimal(int(LRHO_MIN * 10) + i * (int((LRHO_MAX - LRHO_MIN) * 10) // (NRHO - 1)))
        d = ten ** (x / 10)
        dens.append([float(d), float(d.ln()), float(d ** (Decimal(2) / 3)),
                     float(d ** (Decimal(-1) / 3)), float(d ** (Decimal(-4) / 3)),
                     float(d ** (Decimal(-7) / 3))])
    temps = []
    for j in range(NTEMP):
        x = Decimal(int(LT_MIN * 10) + j * (int((LT_MAX - LT_MIN) * 10) // (NTEMP - 1)))
        t = ten ** (x / 10)
        temps.append([float(t), float(t.ln())])
    dv = np.array(dens).T[:, None, :]   # [6][1][NRHO]
    tv = np.array(temps).T[:, :, None]  # [2][NTEMP][1]
    return dv, tv


def _fields():
    """The 21 tabulated fields, each [NTEMP][NRHO]; only + - * / below."""
    (d, lnd, A, dm13, dm43, dm73), (T, lnT) = _node_values()
    d, lnd, A = (np.broadcast_to(x, (NTEMP, NRHO)) for x in (d, lnd, A))
    dm13, dm43, dm73 = (np.broadcast_to(x, (NTEMP, NRHO)) for x in (dm13, dm43, dm73))
    T, lnT = (np.broadcast_to(x, (NTEMP, NRHO)) for x in (T, lnT))
    a, K, b = A_GAS, K_DEG, B_TH
    A1 = (2.0 / 3.0) * dm13
    A2 = -(2.0 / 9.0) * dm43
    A3 = (8.0 / 27.0) * dm73
    g = A + D0
    g2 = g * g
    g3 = g2 * g
    h = 1.0 / g
    h1 = -A1 / g2
    h2 = -A2 / g2 + 2.0 * (A1 * A1) / g3
    h3 = -A3 / g2 + 6.0 * (A1 * A2) / g3 - 6.0 * (A1 * A1 * A1) / (g2 * g2)
    d2, T2 = d * d, T * T
    L = 1.5 * lnT - lnd + C0
    f = -a * T * L + K * A - b * T2 * h
    fd = a * T / d + K * A1 - b * T2 * h1
    fdd = -a * T / d2 + K * A2 - b * T2 * h2
    fddd = 2.0 * a * T / (d2 * d) + K * A3 - b * T2 * h3
    ft = -a * L - 1.5 * a - 2.0 * b * T * h
    ftt = -1.5 * a / T - 2.0 * b * h
    fdt = a / d - 2.0 * b * T * h1
    fddt = -a / d2 - 2.0 * b * T * h2
    fdddt = 2.0 * a / (d2 * d) - 2.0 * b * T * h3
    fdtt = -2.0 * b * h1
    fddtt = -2.0 * b * h2
    # P = d^2 F_d and its derivatives
    dpdf = 2.0 * d * fd + d2 * fdd
    dpdfd = 2.0 * fd + 4.0 * d * fdd + d2 * fddd
    dpdft = 2.0 * d * fdt + d2 * fddt
    dpdfdt = 2.0 * fdt + 4.0 * d * fddt + d2 * fdddt
    ef = lnd - 1.5 * lnT + C1 + K2 * A / T
    efd = 1.0 / d + K2 * A1 / T
    eft = -1.5 / T - K2 * A / T2
    efdt = -K2 * A1 / T2
    xf = NA * d + X0 * (T2 * T)
    xfd = np.full((NTEMP, NRHO), NA)
    xft = 3.0 * X0 * T2
    xfdt = np.zeros((NTEMP, NRHO))
    return ([f, fd, ft, fdd, ftt, fdt, fddt, fdtt, fddtt], [dpdf, dpdfd, dpdft, dpdfdt],
            [ef, efd, eft, efdt], [xf, xfd, xft, xfdt])


def table_text():
    out = []
    for blk in _fields():
        cols = np.stack([np.ascontiguousarray(x).ravel() for x in blk], axis=1)
        out.append("\n".join(" ".join(f"{v:.17e}" for v in row) for row in cols))
    return "\n".join(out) + "\n"


def helm_table(path):
    """Writes the synthetic table to `path` (unless an identical file is
    already there); returns its SHA-256."""
    text = table_text().encode()
    sha = hashlib.sha256(text).hexdigest()
    if os.path.exists(path):
        with open(path, "rb") as fh:
            if hashlib.sha256(fh.read()).hexdigest() == sha:
                return sha
    tmp = path + ".tmp"
    with open(tmp, "wb") as fh:
        fh.write(text)
    os.replace(tmp, path)
    return sha


def helm_queries(n, seed=0):
    """Cells of the Helmholtz workload: rho log-uniform on [1e-2, 1e9] g/cc,
    T log-uniform on [1e4, 1e10] K, Abar uniform on [1, 56], Zbar uniform on
    [1, min(Abar/2 + 1, 28)]."""
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(1e-2), np.log(1e9), n))
    T = np.exp(rng.uniform(np.log(1e4), np.log(1e10), n))
    abar = rng.uniform(1.0, 56.0, n)
    zbar = 1.0 + rng.random(n) * (np.minimum(abar / 2 + 1, 28.0) - 1.0)
    return rho, T, abar, zbar
