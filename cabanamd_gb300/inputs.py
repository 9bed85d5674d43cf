"""Synthetic, seeded initial states for the benchmark and parity cases.

The reference's own input deck can only build exact lattices with uniform
"loop geom" velocities (src/inputFile_impl.h:536-865).  The workloads here
need Gaussian or Maxwell-Boltzmann velocities and random displacements, so
they are generated here and handed to both the GPU path and the oracle as
plain arrays (or as a LAMMPS data file, which the reference's read_data
accepts: src/read_data.h:164-275).

Lattice positions follow the reference's FCC construction
(src/inputFile_impl.h:670-689, 720-760): for iz, iy, ix, basis k in that
order, x = a * (1.0 * ix + basis[k]), ids 1..N in creation order.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# units (src/inputFile_impl.h:146-182)
UNITS = {
    "lj": dict(boltz=1.0, mvv2e=1.0, dt=0.005),
    "metal": dict(boltz=8.617343e-5, mvv2e=1.0364269e-4, dt=0.001),
    "real": dict(boltz=0.0019872067, mvv2e=48.88821291 * 48.88821291, dt=1.0),
}

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])


@dataclass
class State:
    x: np.ndarray
    v: np.ndarray
    type: np.ndarray
    id: np.ndarray
    lo: np.ndarray
    hi: np.ndarray
    mass: list
    boltz: float
    mvv2e: float
    dt: float
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.x)

    def copy(self) -> "State":
        return State(self.x.copy(), self.v.copy(), self.type.copy(), self.id.copy(),
                     self.lo.copy(), self.hi.copy(), list(self.mass), self.boltz, self.mvv2e,
                     self.dt, dict(self.meta))


def fcc_positions(nx: int, ny: int, nz: int, a: float) -> np.ndarray:
    iz, iy, ix, k = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), np.arange(4),
                                indexing="ij")
    ix = ix.ravel().astype(np.float64)
    iy = iy.ravel().astype(np.float64)
    iz = iz.ravel().astype(np.float64)
    k = k.ravel()
    x = np.empty((ix.size, 3))
    x[:, 0] = a * (1.0 * ix + FCC_BASIS[k, 0])
    x[:, 1] = a * (1.0 * iy + FCC_BASIS[k, 1])
    x[:, 2] = a * (1.0 * iz + FCC_BASIS[k, 2])
    return x


def temperature(v, mass_per_atom, boltz, mvv2e) -> float:
    """property_temperature_impl.h:55-77 for one rank."""
    n = len(v)
    smv2 = float(np.sum(np.sum(v * v, axis=1) * mass_per_atom))
    return smv2 * (mvv2e / (1.0 * (3 * n - 3) * boltz))


def gaussian_velocities(n, mass_per_atom, T, rng, boltz, mvv2e) -> np.ndarray:
    """Gaussian velocities with sigma ~ 1/sqrt(m), zero net momentum, scaled
    to temperature T (Maxwell-Boltzmann in any unit system)."""
    v = rng.standard_normal((n, 3)) / np.sqrt(mass_per_atom)[:, None]
    p = np.sum(v * mass_per_atom[:, None], axis=0) / np.sum(mass_per_atom)
    v -= p
    v *= np.sqrt(T / temperature(v, mass_per_atom, boltz, mvv2e))
    return v


def lj_fcc(ncell: int, rho: float = 0.8442, T: float = 1.44, seed: int = 12345,
           mass: float = 1.0) -> State:
    """LJ melt: FCC at reduced density rho, a = (4/rho)^(1/3)
    (inputFile_impl.h:212-214), Gaussian velocities at T."""
    a = (4.0 / rho) ** (1.0 / 3.0)
    x = fcc_positions(ncell, ncell, ncell, a)
    n = len(x)
    u = UNITS["lj"]
    rng = np.random.default_rng(seed)
    m = np.full(n, mass)
    v = gaussian_velocities(n, m, T, rng, u["boltz"], u["mvv2e"])
    L = a * ncell
    return State(x, v, np.zeros(n, np.int32), np.arange(1, n + 1, dtype=np.int32),
                 np.zeros(3), np.full(3, L), [mass], u["boltz"], u["mvv2e"], u["dt"],
                 dict(workload="lj", ncell=ncell, rho=rho, T=T, seed=seed, a=a))


def nnp_fcc(ncell: int, a: float = 3.61, mass: float = 63.546, T: float = 300.0,
            disp: float = 0.05, seed: int = 2024, dt_fs: float = 0.5) -> State:
    """NNP single element (metal units): FCC a, uniform +-disp displacement,
    Maxwell-Boltzmann velocities at T, dt in fs."""
    x = fcc_positions(ncell, ncell, ncell, a)
    n = len(x)
    rng = np.random.default_rng(seed)
    x = x + rng.uniform(-disp, disp, size=x.shape)
    u = UNITS["metal"]
    m = np.full(n, mass)
    v = gaussian_velocities(n, m, T, rng, u["boltz"], u["mvv2e"])
    L = a * ncell
    return State(x, v, np.zeros(n, np.int32), np.arange(1, n + 1, dtype=np.int32),
                 np.zeros(3), np.full(3, L), [mass], u["boltz"], u["mvv2e"], dt_fs * 1e-3,
                 dict(workload="nnp", ncell=ncell, a=a, T=T, seed=seed))


def random_box(n: int, box_min: float, box_max: float, seed: int) -> np.ndarray:
    """Uniform random positions in a cube (the geometry of the reference's
    unit tests, unit_test/tstNeighbor.hpp:247-285)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(box_min, box_max, size=(n, 3))
