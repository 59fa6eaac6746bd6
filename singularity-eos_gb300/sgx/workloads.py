"""Seeded synthetic inputs with the shapes, sizes and value distributions of
the closure workloads (no public dataset exists for this path).

All per-material arrays are [nmat, ncell] float64, cell index fastest (the
LayoutLeft of singularity-eos get_sg_eos.hpp:30-31). Densities follow the
get_sg_eos init_functor convention (get_sg_eos_functors.hpp:107-117): every
material starts at the cell density, with volume fraction equal to its mass
fraction.
"""
import numpy as np

# EOS model codes (include/sgx.h)
IDEAL, STIFF, NOBLE_ABEL, GRUNEISEN, SPINER_RHOT, HELMHOLTZ = 1, 2, 3, 4, 5, 6

EPS = 10 * np.finfo(np.float64).eps

# Materials named by the workloads.
IDEAL_AIR = (IDEAL, (0.4, 0.718e7))                     # gamma 1.4
STIFF_WATER = (STIFF, (3.4, 1.816e7, 6e9, 0.0))         # gm1, Cv, Pinf, q
NOBLE_ABEL_GAS = (NOBLE_ABEL, (0.4, 0.718e7, 1e-3, 0.0))  # gm1, Cv, b, q
# Copper-like Gruneisen: C0, s1, s2, s3, G0, b, rho0, T0, P0, Cv
# (test_eos_gruneisen.cpp:74-83 parameters, Cv = 3.9e6).
GRUNEISEN_CU = (GRUNEISEN, (3.94e5, 1.489, 0.0, 0.0, 2.02, 0.47, 8.93, 298.0, 0.0, 3.9e6))


def gruneisen_rho_max(s1, s2, s3, rho0):
    """Gruneisen::ComputeRhoMax for the linear Us-up case
    (eos_gruneisen.hpp:231-245, 321-328) times RHOMAX_SAFETY = 0.99."""
    if abs(s2) < EPS and abs(s3) < EPS and s1 > 1.0:
        root = 1.0 / s1
        return 0.99 * (rho0 / ((1 - root) + EPS))
    raise NotImplementedError("only the linear Us-up case is tabulated here")


def pte_two_material(ncell, seed=0):
    """Plain FP64 PTE closure, 2 materials (IdealGas + StiffGas):
    rho_tot log-uniform on [1e-3, 2] g/cc, alpha_1 uniform on [0.05, 0.95],
    sie_tot uniform on [1e9, 1e11] erg/g."""
    rng = np.random.default_rng(seed)
    rho_tot = np.exp(rng.uniform(np.log(1e-3), np.log(2.0), ncell))
    a1 = rng.uniform(0.05, 0.95, ncell)
    vfrac = np.ascontiguousarray(np.stack([a1, 1.0 - a1]))
    rho = np.ascontiguousarray(np.stack([rho_tot, rho_tot]))
    sie_tot = rng.uniform(1e9, 1e11, ncell)
    return dict(
        materials=[IDEAL_AIR, STIFF_WATER], eos_idx=None, vfrac_tot=vfrac.sum(axis=0),
        sie_tot=sie_tot, rho=rho, vfrac=vfrac, sie=np.zeros_like(rho),
        temp=np.zeros_like(rho), press=np.zeros_like(rho))


def material_pool(seed=0):
    """The 8-instance EOS pool of the batched workload: 5 IdealGas with gamma
    uniform on [1.3, 1.67], StiffGas, NobleAbel and copper Gruneisen."""
    rng = np.random.default_rng(seed + 1000)
    pool = [(IDEAL, (g - 1.0, 0.718e7)) for g in rng.uniform(1.3, 1.67, 5)]
    return pool + [STIFF_WATER, NOBLE_ABEL_GAS, GRUNEISEN_CU]


def pte_batched(ncell, seed=0, nmax=5, mix=(0.55, 0.25, 0.12, 0.08)):
    """Uneven PTE batch: 2/3/4/5 materials per cell in proportions
    55/25/12/8 %, drawn without replacement from the 8-EOS pool; volume
    fractions Dirichlet(1,...,1); rho_tot log-uniform on [1e-3, 10] g/cc;
    sie_tot uniform on [1e9, 1e11] erg/g. Absent slots have eos_idx -1 and
    are packed after the present ones."""
    rng = np.random.default_rng(seed)
    pool = material_pool(seed)
    counts = rng.choice(np.arange(2, 2 + len(mix)), size=ncell, p=np.array(mix) / sum(mix))
    eos_idx = np.full((nmax, ncell), -1, np.int32)
    keys = rng.random((ncell, len(pool)))
    order = np.argsort(keys, axis=1)  # a random permutation per cell
    for m in range(nmax):
        present = counts > m
        eos_idx[m, present] = order[present, m]
    expo = rng.exponential(1.0, (nmax, ncell))
    expo[eos_idx < 0] = 0.0
    vfrac = expo / expo.sum(axis=0)
    rho_tot = np.exp(rng.uniform(np.log(1e-3), np.log(10.0), ncell))
    rho = np.where(eos_idx >= 0, rho_tot[None, :], 0.0)
    sie_tot = rng.uniform(1e9, 1e11, ncell)
    z = np.zeros((nmax, ncell))
    return dict(materials=pool, eos_idx=np.ascontiguousarray(eos_idx),
                vfrac_tot=np.ones(ncell), sie_tot=sie_tot,
                rho=np.ascontiguousarray(rho), vfrac=np.ascontiguousarray(vfrac),
                sie=z.copy(), temp=z.copy(), press=z.copy(), counts=counts)


def serve_request(ncell, seed, pool, nmax=4):
    """One closure request of the serving workload: 2..nmax materials per
    cell drawn without replacement from `pool` (a list of EOS indices into
    the server's EOS list), volume fractions Dirichlet(1,...,1), total
    density log-uniform on [1e-3, 10] g/cc, sie uniform on [1e9, 1e11]
    erg/g; zero temperature and pressure guesses. Returns a dict of
    contiguous arrays in the sgx_pte_request layout ([nmax][ncell])."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(2, nmax + 1, size=ncell)
    eos_idx = np.full((nmax, ncell), -1, np.int32)
    order = np.argsort(rng.random((ncell, len(pool))), axis=1)
    pool = np.asarray(pool, np.int32)
    for m in range(nmax):
        present = counts > m
        eos_idx[m, present] = pool[order[present, m]]
    expo = rng.exponential(1.0, (nmax, ncell))
    expo[eos_idx < 0] = 0.0
    vfrac = expo / expo.sum(axis=0)
    rho_tot = np.exp(rng.uniform(np.log(1e-3), np.log(10.0), ncell))
    rho = np.where(eos_idx >= 0, rho_tot[None, :], 0.0)
    z = np.zeros((nmax, ncell))
    return dict(nmat=nmax, ncell=ncell, eos_idx=np.ascontiguousarray(eos_idx),
                vfrac_tot=np.ones(ncell), sie_tot=rng.uniform(1e9, 1e11, ncell),
                rho_in=np.ascontiguousarray(rho), vfrac_in=np.ascontiguousarray(vfrac),
                sie_in=z.copy(), temp_in=z.copy(), press_in=z.copy())
