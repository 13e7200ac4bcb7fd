"""Seeded synthetic inputs with the shapes and value distributions of the benchmark
configurations (no datasets are involved; every draw uses numpy PCG64 with a recorded seed).

  sod            Sod shock tube along x, 128x3x3, nchem=0, reflecting x, periodic y/z.
  rayleigh_taylor  heavy-over-light RT state at n^3 with 10 passive tracers, periodic x/y,
                 reflecting z, constant -0.1 body force on z-momentum.
  primordial     10-species primordial chemistry state (number densities + specific gas
                 energy) with log-uniform mass fractions and temperatures.
  chem_hydro     planar Sod-like interface along x carrying the primordial species
                 (the multirate/IMEX chemistry-hydrodynamics workload), in the reference's
                 "Dengo-scaled" representation: chemistry state ~1, per-cell scale arrays.

Field layout matches the reference's ManyVector: rho, mx, my, mz, et as (nz, ny, nx) arrays
(x fastest, INDX of src/euler3D.hpp:62) and chemistry as (nz, ny, nx, nchem), species fastest
(BUFINDX of src/euler3D.hpp:65).
"""
from __future__ import annotations

import numpy as np

BC_PERIODIC, BC_NEUMANN, BC_DIRICHLET, BC_REFLECTING = 0, 1, 2, 3
SEED_BASE = 20261203
M_H = 1.67e-24
KBOLTZ = 1.3806488e-16
M_AMU = 1.66053904e-24


def _centres(n, lo=0.0, hi=1.0):
    return lo + (np.arange(n) + 0.5) * (hi - lo) / n


def total_energy(rho, mx, my, mz, p, gamma):
    """eos_inv (src/euler3D.hpp:1393-1398)."""
    return p / (gamma - 1.0) + (mx * mx + my * my + mz * mz) * 0.5 / rho


def sod(nx=128, ny=3, nz=3, gamma=1.4):
    x = _centres(nx)
    shp = (nz, ny, nx)
    rho = np.broadcast_to(np.where(x < 0.5, 1.0, 0.125), shp).copy()
    p = np.broadcast_to(np.where(x < 0.5, 1.0, 0.1), shp).copy()
    z0 = np.zeros(shp)
    et = total_energy(rho, z0, z0, z0, p, gamma)
    bc = (BC_REFLECTING, BC_REFLECTING, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC)
    return dict(fields=[rho, z0.copy(), z0.copy(), z0.copy(), et], nchem=0, bc=bc,
                gamma=gamma, force=None)


def rayleigh_taylor(n=128, nchem=10, gamma=1.4, seed=SEED_BASE + 1, shape=None):
    nx, ny, nz = shape if shape is not None else (n, n, n)
    rng = np.random.Generator(np.random.PCG64(seed))
    z = _centres(nz)[:, None, None]
    shp = (nz, ny, nx)
    rho = np.broadcast_to(1.5 + 0.5 * np.tanh((z - 0.5) / 0.02), shp).copy()
    # p(z) = 2.5 + 0.1 * int_z^1 rho,  int_z^1 rho = 1.5(1-z) + 0.01[ln cosh 25 - ln cosh((z-.5)/.02)]
    lc = lambda s: np.logaddexp(s, -s) - np.log(2.0)  # ln cosh, overflow-free
    integral = 1.5 * (1.0 - z) + 0.01 * (lc(25.0) - lc((z - 0.5) / 0.02))
    p = np.broadcast_to(2.5 + 0.1 * integral, shp).copy()
    vel = rng.uniform(-1e-2, 1e-2, size=(3,) + shp)
    mx, my, mz = rho * vel[0], rho * vel[1], rho * vel[2]
    et = total_energy(rho, mx, my, mz, p, gamma)
    fields = [rho, mx, my, mz, et]
    if nchem > 0:
        fields.append(rng.uniform(0.0, 1.0, size=shp + (nchem,)) * rho[..., None])
    force = np.zeros(5 + nchem)
    force[3] = -0.1
    bc = (BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_REFLECTING, BC_REFLECTING)
    return dict(fields=fields, nchem=nchem, bc=bc, gamma=gamma, force=force)


def smooth_periodic(n=96, nchem=4, gamma=1.4, seed=SEED_BASE + 4, shape=None):
    """Differentiation workload: rho = 1 + 0.2 sin(2 pi (x+y+z)), p = 1, random velocities."""
    nx, ny, nz = shape if shape is not None else (n, n, n)
    rng = np.random.Generator(np.random.PCG64(seed))
    X = _centres(nx)[None, None, :]
    Y = _centres(ny)[None, :, None]
    Z = _centres(nz)[:, None, None]
    shp = (nz, ny, nx)
    rho = np.broadcast_to(1.0 + 0.2 * np.sin(2 * np.pi * (X + Y + Z)), shp).copy()
    vel = rng.uniform(-0.1, 0.1, size=(3,) + shp)
    mx, my, mz = rho * vel[0], rho * vel[1], rho * vel[2]
    et = total_energy(rho, mx, my, mz, np.ones(shp), gamma)
    fields = [rho, mx, my, mz, et]
    if nchem > 0:
        fields.append(rng.uniform(0.0, 1.0, size=shp + (nchem,)) * rho[..., None])
    return dict(fields=fields, nchem=nchem, bc=(0,) * 6, gamma=gamma, force=None)


def primordial(ncells, seed=SEED_BASE + 2, density=1e2 * M_H, t_range=(10.0, 1e4)):
    """Physical 10-species state (H2I, H2II, HI, HII, HM, HeI, HeII, HeIII, de, ge) per cell,
    in the units of src/primordial_static.cpp:86-160: number densities, electron density in
    m_amu units, specific gas energy in erg/g.  Mass fractions log-uniform in [1e-10, 1] and
    renormalised (hydrogen 0.76 / helium 0.24), temperature log-uniform in t_range."""
    rng = np.random.Generator(np.random.PCG64(seed))
    dens = np.broadcast_to(np.asarray(density, dtype=np.float64), (ncells,)).copy()
    fr = 10.0 ** rng.uniform(-10.0, 0.0, size=(ncells, 8))
    fr[:, :5] *= 0.76 / fr[:, :5].sum(axis=1, keepdims=True)
    fr[:, 5:] *= 0.24 / fr[:, 5:].sum(axis=1, keepdims=True)
    w = np.array([2 * 1.00794, 2 * 1.00794, 1.00794, 1.00794, 1.00794,
                  4.002602, 4.002602, 4.002602]) * M_H
    n = fr * dens[:, None] / w  # number densities H2I, H2II, HI, HII, HM, HeI, HeII, HeIII
    de = (n[:, 3] + n[:, 6] + 2 * n[:, 7] - n[:, 4] + n[:, 1]) * M_H
    de = np.maximum(de, 1e-20 * M_H)
    T = 10.0 ** rng.uniform(np.log10(t_range[0]), np.log10(t_range[1]), size=ncells)
    ndens = n.sum(axis=1)
    ge = KBOLTZ * T * ndens / (dens * (5.0 / 3.0 - 1.0))
    y = np.empty((ncells, 10))
    y[:, :8] = n
    y[:, 8] = de / M_AMU
    y[:, 9] = ge
    return y, T


# Units of the primordial_blast multirate inputs (tests/primordial_blast/input_*_mr.txt)
UNITS = dict(MassUnits=3.0e70, LengthUnits=3.0857e30, TimeUnits=1.0e11)


def derived_units(MassUnits, LengthUnits, TimeUnits):
    """EulerData::UpdateUnits (src/euler3D.hpp:382-391)."""
    return dict(DensityUnits=MassUnits / LengthUnits / LengthUnits / LengthUnits,
                MomentumUnits=MassUnits / LengthUnits / LengthUnits / TimeUnits,
                EnergyUnits=MassUnits / LengthUnits / TimeUnits / TimeUnits)


def chem_hydro(n=128, seed=SEED_BASE + 3, shape=None, perturb=1e-3):
    """Chemistry-hydrodynamics state on an n^3 grid, NVAR=15.

    Density: planar Sod-like interface along x (1e2 m_H left, 0.125e2 m_H right, g/cm^3),
    temperature 2000 K left / 1600 K right (pressure ratio 0.1), random primordial mass
    fractions per cell, random velocities of up to 10% of the local sound speed.  Returned in the reference's working
    representation after prepare_Dengo_structures (src/primordial_static.cpp:227-259): the
    chemistry component is ~1 (+- perturb) and `scale` holds the physical values."""
    nx, ny, nz = shape if shape is not None else (n, n, n)
    N = nx * ny * nz
    rng = np.random.Generator(np.random.PCG64(seed))
    x = _centres(nx)
    left = np.broadcast_to(x < 0.5, (nz, ny, nx)).reshape(-1)
    dens = np.where(left, 1e2 * M_H, 0.125e2 * M_H)
    y, _ = primordial(N, seed=seed + 1000, density=dens)
    T = np.where(left, 2000.0, 1600.0)
    ndens = y[:, :8].sum(axis=1)
    y[:, 9] = KBOLTZ * T * ndens / (dens * (5.0 / 3.0 - 1.0))
    u = derived_units(**UNITS)
    shp = (nz, ny, nx)
    rho = (dens / u["DensityUnits"]).reshape(shp)
    eint = y[:, 9].reshape(shp) / u["EnergyUnits"]
    # velocity perturbations of 10% of the local sound speed c = sqrt(gamma p / rho) with
    # p = (gamma - 1) * ge / EnergyUnits (the fluid energy of src/primordial_static.cpp:152)
    gam = 5.0 / 3.0
    cs = np.sqrt(gam * (gam - 1.0) * eint / rho)
    vel = rng.uniform(-0.1, 0.1, size=(3,) + shp) * cs
    mx, my, mz = rho * vel[0], rho * vel[1], rho * vel[2]
    et = eint + 0.5 / rho * (mx * mx + my * my + mz * mz)
    scale = y.reshape(shp + (10,)).copy()
    chem = 1.0 + rng.uniform(-perturb, perturb, size=shp + (10,))
    bc = (BC_REFLECTING, BC_REFLECTING, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC, BC_PERIODIC)
    return dict(fields=[rho, mx, my, mz, et, chem], nchem=10, bc=bc, gamma=5.0 / 3.0,
                force=None, scale=scale, units={**UNITS, **u})
