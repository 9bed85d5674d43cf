"""The seeded synthetic workloads stand in for the benchmark configurations:
their shapes, densities, units and velocity statistics are the ones the
configurations state (no GPU; the serving stream's shape is checked in
test_serve.py)."""
import numpy as np

from cabanamd_gb300 import inputs


def _temperature(v, m, boltz, mvv2e):
    n = len(v)
    return mvv2e * np.sum(m[:, None] * v * v) / ((3 * n - 3) * boltz)


def test_lj_melt_configurations():
    """LJ melt: FCC at reduced density 0.8442 (a = (4/rho)^(1/3) ~ 1.6796),
    20^3 cells = 32,000 atoms (and 100^3 = 4,000,000 by the same rule),
    reduced units (boltz = mvv2e = 1, dt 0.005), Gaussian velocities with
    zero net momentum scaled to T = 1.44, seeded."""
    st = inputs.lj_fcc(20, rho=0.8442, T=1.44, seed=7)
    assert st.n == 32000
    a = (4.0 / 0.8442) ** (1.0 / 3.0)
    assert abs(a - 1.6796) < 1e-4
    assert np.allclose(st.hi - st.lo, 20 * a)
    assert np.isclose(st.n / np.prod(st.hi - st.lo), 0.8442, rtol=1e-12)
    assert (st.boltz, st.mvv2e, st.dt) == (1.0, 1.0, 0.005)
    m = np.full(st.n, st.mass[0])
    assert np.allclose((m[:, None] * st.v).sum(axis=0), 0.0, atol=1e-9)
    assert np.isclose(_temperature(st.v, m, st.boltz, st.mvv2e), 1.44, rtol=1e-12)
    assert np.all((st.x >= st.lo) & (st.x < st.hi))
    assert np.array_equal(np.sort(st.id), np.arange(1, st.n + 1))
    # seeded: the same seed gives the same state, another seed another one
    again = inputs.lj_fcc(20, rho=0.8442, T=1.44, seed=7)
    assert np.array_equal(again.v, st.v)
    assert not np.array_equal(inputs.lj_fcc(20, rho=0.8442, T=1.44, seed=8).v, st.v)
    # the 4M-atom configuration by the same rule
    assert 4 * 100 ** 3 == 4_000_000


def test_nnp_configurations():
    """NNP Cu: FCC a = 3.61 A, 10^3 cells = 4,000 atoms, each atom displaced
    uniformly by at most 0.05 A from its site, metal units (boltz
    8.617343e-5 eV/K, mvv2e 1.0364269e-4, dt 0.5 fs = 0.0005 ps),
    Maxwell-Boltzmann velocities at 300 K with zero net momentum, mass
    63.546."""
    st = inputs.nnp_fcc(10, seed=3)
    assert st.n == 4000
    assert np.allclose(st.hi - st.lo, 36.1)
    lattice = inputs.fcc_positions(10, 10, 10, 3.61)
    assert np.abs(st.x - lattice).max() <= 0.05
    assert np.abs(st.x - lattice).max() > 0.04
    assert (st.boltz, st.mvv2e) == (8.617343e-5, 1.0364269e-4)
    assert np.isclose(st.dt, 0.0005)
    assert st.mass == [63.546]
    m = np.full(st.n, 63.546)
    assert np.allclose((m[:, None] * st.v).sum(axis=0), 0.0, atol=1e-9)
    assert np.isclose(_temperature(st.v, m, st.boltz, st.mvv2e), 300.0, rtol=1e-12)
    assert inputs.nnp_fcc(40, seed=3).n == 256_000

