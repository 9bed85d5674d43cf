"""Pin the CPU oracle against the reference's own known-answer tests.

The reference holds no golden vectors for this path; its tests are
unit_test/tstNeighbor.hpp (lists equal a brute-force N^2 build; half-list
invariants; ghosts have no neighbours) and unit_test/tstIntegrator.hpp
(100 steps forward, negate v, 100 back: positions return).  Both are
restated here on the same geometry (1000 particles, 200 of them ghosts,
cutoff 2.32, cube [-5.3*2.32, 4.7*2.32]) with this project's seeded
generator, since Kokkos' XorShift stream cannot be reproduced without
Kokkos.  Analytic known answers (LJ dimer, perfect-lattice symmetry) pin
the force arithmetic.
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from cabanamd_gb300 import inputs

from conftest import pair_sets

CUT = 2.32
BOX_MIN, BOX_MAX = -5.3 * CUT, 4.7 * CUT


def _fixture(seed=342343901):
    rng = np.random.default_rng(seed)
    return rng.uniform(BOX_MIN, BOX_MAX, size=(1000, 3))


def test_tstneighbor_full_bruteforce_definition():
    """tstNeighbor.hpp:76-141: count and fill with d^2 <= rc^2, self
    excluded; an independent numpy restatement agrees exactly."""
    x = _fixture()
    nloc = 800
    off, j = O.neigh_brute(x, nloc, CUT, 0)
    d = x[:nloc, None, :] - x[None, :, :]
    d2 = d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2]
    ref = (d2 <= CUT * CUT)
    ref[np.arange(nloc), np.arange(nloc)] = False
    for i in range(nloc):
        assert sorted(j[off[i]:off[i + 1]].tolist()) == np.nonzero(ref[i])[0].tolist()


def test_tstneighbor_half_invariants():
    """tstNeighbor.hpp:193-243: sum(half) <= sum(full); per-atom half count
    <= full; j in list(i) => i not in list(j); each local pair exactly once."""
    x = _fixture()
    nloc = 800
    offf, jf = O.neigh_brute(x, nloc, CUT, 0)
    offh, jh = O.neigh_brute(x, nloc, CUT, 1)
    assert offh[-1] <= offf[-1]
    full = [set(jf[offf[i]:offf[i + 1]].tolist()) for i in range(nloc)]
    half = [set(jh[offh[i]:offh[i + 1]].tolist()) for i in range(nloc)]
    for i in range(nloc):
        assert len(half[i]) <= len(full[i])
        assert half[i] <= full[i]
        for jj in half[i]:
            if jj < nloc:
                assert i not in half[jj]
    # every local-local pair appears exactly once
    for i in range(nloc):
        for jj in full[i]:
            if jj < nloc:
                assert (jj in half[i]) != (i in half[jj])


def _periodic_system(n=1500, L=14.0, seed=7):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0.0, L, size=(n, 3))
    return x, np.zeros(3), np.full(3, L)


@pytest.mark.parametrize("half", [0, 1])
def test_cell_list_equals_bruteforce_over_halo(half):
    """The cell-stencil enumeration with in-place image shifts (the GPU's
    algorithm) gives exactly the set a brute force over the reference's
    6-phase halo ghosts gives."""
    x, lo, hi = _periodic_system()
    cut = 2.8
    g = O.make_grid(lo, hi, cut)
    typ = np.zeros(len(x), np.int32)
    ids = np.arange(1, len(x) + 1, dtype=np.int32)
    O.sort_atoms(g, x, None, None, typ, ids)
    offc, jc, ic = O.neigh_cells(x, g, hi, cut, cut, half)
    offb, jb, ib = O.periodic_brute(x, lo, hi, cut, half)
    assert pair_sets(offc, jc, ic) == pair_sets(offb, jb, ib)
    # ghosts were really needed
    assert np.any(ic != O.IMG_ZERO)


def test_halo_small_box_multiple_images():
    """A box smaller than two cutoffs gets both -L and +L images of the same
    atom and corner images, as the 6-phase halo does."""
    x, lo, hi = _periodic_system(n=60, L=5.0, seed=3)
    cut = 2.6
    g = O.make_grid(lo, hi, cut)
    assert g.nc[0] == 1
    typ = np.zeros(len(x), np.int32)
    ids = np.arange(1, len(x) + 1, dtype=np.int32)
    O.sort_atoms(g, x, None, None, typ, ids)
    for half in (0, 1):
        offc, jc, ic = O.neigh_cells(x, g, hi, cut, cut, half)
        offb, jb, ib = O.periodic_brute(x, lo, hi, cut, half)
        assert pair_sets(offc, jc, ic) == pair_sets(offb, jb, ib)


def test_tstintegrator_reversibility():
    """tstIntegrator.hpp:82-137 with EXPECT_FLOAT_EQ's 4-ulp float test."""
    rng = np.random.default_rng(342343901)
    n = 1000
    x = rng.uniform(BOX_MIN, BOX_MAX, size=(n, 3))
    v = rng.uniform(-1, 1, size=(n, 3))
    f = rng.uniform(-1, 1, size=(n, 3))
    t = np.zeros(n, np.int32)
    x0 = x.copy()
    mass = np.array([1.0])
    for _ in range(100):
        O.nve_initial(x, v, f, t, mass, 0.005, 1.0)
        O.nve_final(v, f, t, mass, 0.005, 1.0)
    v *= -1.0
    for _ in range(100):
        O.nve_initial(x, v, f, t, mass, 0.005, 1.0)
        O.nve_final(v, f, t, mass, 0.005, 1.0)
    a = x.astype(np.float32)
    b = x0.astype(np.float32)
    ulps = np.abs(a.view(np.int32).astype(np.int64) - b.view(np.int32).astype(np.int64))
    assert ulps.max() <= 4


def test_lj_dimer_analytic():
    """Known answer: two atoms at r give F = 24 eps (2 (s/r)^12 - (s/r)^6)/r
    and the shifted energy 4 eps ((s/r)^12 - (s/r)^6) - E(rc)."""
    r = 1.3
    x = np.array([[5.0, 5.0, 5.0], [5.0 + r, 5.0, 5.0]])
    lo, hi = np.zeros(3), np.full(3, 20.0)
    g = O.make_grid(lo, hi, 2.8)
    t = np.zeros(2, np.int32)
    ids = np.array([1, 2], np.int32)
    O.sort_atoms(g, x, None, None, t, ids)
    p = O.lj_params([(1, 1, 1.0, 1.0, 2.5)])
    for half in (0, 1):
        off, j, img = O.neigh_cells(x, g, hi, 2.8, 2.8, half)
        lh = O.ListHandle(off, j, img)
        f = O.lj_force(x, t, p, lh, hi - lo, half)
        fr = 24.0 * (2 * r ** -12 - r ** -6) / r
        i1 = int(np.nonzero(ids == 1)[0][0])
        assert np.isclose(f[i1, 0], -fr, rtol=1e-14)
        assert np.allclose(f.sum(axis=0), 0.0, atol=1e-12)
        e = O.lj_energy(x, t, p, lh, hi - lo, half)
        ec = 4.0 * (2.5 ** -12 - 2.5 ** -6)
        assert np.isclose(e, 4.0 * (r ** -12 - r ** -6) - ec, rtol=1e-13)


def test_perfect_fcc_forces_vanish_and_energy_known():
    """Known answer: on a perfect FCC lattice every force is zero by
    symmetry and the energy per atom equals the analytic shell sum."""
    st = inputs.lj_fcc(6, T=1.0)
    x = st.x.copy()
    g = O.make_grid(st.lo, st.hi, 2.8)
    t = st.type.copy()
    ids = st.id.copy()
    O.exchange_self(x, st.hi - st.lo)
    O.sort_atoms(g, x, None, None, t, ids)
    p = O.lj_params([(1, 1, 1.0, 1.0, 2.5)])
    off, j, img = O.neigh_cells(x, g, st.hi, 2.8, 2.8, 0)
    lh = O.ListHandle(off, j, img)
    f = O.lj_force(x, t, p, lh, st.hi - st.lo, 0)
    assert np.abs(f).max() < 1e-10
    e = O.lj_energy(x, t, p, lh, st.hi - st.lo, 0) / len(x)
    # analytic: sum over FCC shells within rc of 1/2 * 4((1/r)^12-(1/r)^6 - shift)
    a = st.meta["a"]
    pts = inputs.fcc_positions(7, 7, 7, a) - a * 3
    r = np.sqrt((pts * pts).sum(1))
    r = r[(r > 1e-9) & (r < 2.5)]
    ec = 4.0 * (2.5 ** -12 - 2.5 ** -6)
    ref = 0.5 * np.sum(4.0 * (r ** -12 - r ** -6) - ec)
    assert np.isclose(e, ref, rtol=1e-12)


def test_oracle_run_energy_conservation_small():
    """LJ melt 5^3 cells (500 atoms), full and half lists: FP64 NVE energy
    is conserved and both lists give the same trajectory forces."""
    for half in (0, 1):
        st = inputs.lj_fcc(5, T=1.44, seed=11)
        th, f = O.run_lj(st.x, st.v, st.type, st.id, st.lo, st.hi, [(1, 1, 1.0, 1.0, 2.5)],
                         force_cut=2.5, skin=0.3, half=half, rebuild_every=20, thermo_every=10,
                         nsteps=100, boltz=1.0, mvv2e=1.0, dt=0.005, mass=[1.0])
        assert th.shape == (11, 4)
        etot = th[:, 2] + th[:, 3]
        if not half:
            assert np.ptp(etot) < 5e-3
        assert np.all(np.isfinite(th))


def test_oracle_reproduces_committed_golden_trajectories():
    """tests/golden/lj_small.npz (made by tests/golden/make_golden.py) is the
    oracle's own output; a change in the oracle shows up here."""
    import sys
    from pathlib import Path
    gold = np.load(Path(__file__).resolve().parent / "golden" / "lj_small.npz")
    sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
    from make_golden import LJ_CASE, lj_small_case
    for half in (0, 1):
        st = lj_small_case()
        th, f = O.run_lj(st.x, st.v, st.type, st.id, st.lo, st.hi, [(1, 1, 1.0, 1.0, 2.5)],
                         force_cut=2.5, skin=0.3, half=half, rebuild_every=20, thermo_every=10,
                         nsteps=LJ_CASE["nsteps"], boltz=1.0, mvv2e=1.0, dt=0.005, mass=[1.0])
        o = np.argsort(st.id)
        assert np.array_equal(th, gold[f"thermo_half{half}"])
        assert np.array_equal(st.x[o], gold[f"x_half{half}"])
        assert np.array_equal(f[o], gold[f"f_half{half}"])


def test_lj_disordered_two_types_against_an_independent_restatement():
    """A disordered two-type system (FCC 4^3 cells displaced by up to 0.15
    sigma, types at random, three pair_coeff rows with their own epsilon,
    sigma and cutoff): the oracle's full- and half-list forces and shifted
    energies equal a plain numpy sum over every periodic image of
    force_lj_cabana_neigh_impl.h's expressions (lj1 = 48 eps sigma^12,
    lj2 = 24 eps sigma^6, rsq < cutsq strictly, the energy shifted to zero
    at each pair type's cutoff), within 1e-12.  The half-list energy keeps
    the reference's weights (:317-377): a pair of two local atoms counts
    once, a pair with a ghost (here: through a periodic image) one half, and
    the half list holds each image pair once, so such pairs count half."""
    st = inputs.lj_fcc(4, T=1.0, seed=31)
    rng = np.random.default_rng(31)
    x = st.x + rng.uniform(-0.15, 0.15, size=st.x.shape)
    L = st.hi - st.lo
    x = st.lo + np.mod(x - st.lo, L)
    t = rng.integers(0, 2, len(x)).astype(np.int32)
    ids = st.id.copy()
    coeffs = [(1, 1, 1.0, 1.0, 2.5), (2, 2, 0.8, 1.1, 2.5), (1, 2, 1.2, 0.95, 2.2)]
    cut = 2.5 + 0.3
    g = O.make_grid(st.lo, st.hi, cut)
    O.sort_atoms(g, x, None, None, t, ids)
    p = O.lj_params(coeffs, ntypes=2)

    # the restatement
    lj1 = np.zeros((2, 2))
    lj2 = np.zeros((2, 2))
    cutsq = np.zeros((2, 2))
    for (a, b, eps, sig, rc) in coeffs:
        for (i, j) in ((a - 1, b - 1), (b - 1, a - 1)):
            lj1[i, j] = 48.0 * eps * sig ** 12
            lj2[i, j] = 24.0 * eps * sig ** 6
            cutsq[i, j] = rc * rc
    shifts = np.array([[a, b, c] for a in (-1, 0, 1) for b in (-1, 0, 1)
                       for c in (-1, 0, 1)], dtype=float) * L
    image = np.repeat(np.any(shifts != 0.0, axis=1), len(x))
    f_ref = np.zeros_like(x)
    pe_ref = {0: 0.0, 1: 0.0}
    for i in range(len(x)):
        d = (x[i] - (x[None, :, :] + shifts[:, None, :])).reshape(-1, 3)
        tj = np.tile(t, len(shifts))
        rsq = (d * d).sum(axis=1)
        c2 = cutsq[t[i], tj]
        m = (rsq > 0.0) & (rsq < c2)
        d, rsq, tj, c2, im = d[m], rsq[m], tj[m], c2[m], image[m]
        a1, a2 = lj1[t[i], tj], lj2[t[i], tj]
        r2inv = 1.0 / rsq
        r6inv = r2inv ** 3
        fpair = r6inv * (a1 * r6inv - a2) * r2inv
        f_ref[i] = (d * fpair[:, None]).sum(axis=0)
        r6c = (1.0 / c2) ** 3
        # every ordered pair once: half of each pair's energy
        e = 0.5 * r6inv * (0.5 * a1 * r6inv - a2) / 6.0 - 0.5 * r6c * (0.5 * a1 * r6c - a2) / 6.0
        pe_ref[0] += np.sum(e)
        pe_ref[1] += np.sum(np.where(im, 0.5 * e, e))
    fmax = np.abs(f_ref).max()
    for half in (0, 1):
        off, j, img = O.neigh_cells(x, g, st.hi, cut, cut, half)
        lh = O.ListHandle(off, j, img)
        f = O.lj_force(x, t, p, lh, L, half)
        assert np.allclose(f, f_ref, rtol=0, atol=1e-12 * fmax), half
        e = O.lj_energy(x, t, p, lh, L, half)
        assert np.isclose(e, pe_ref[half], rtol=1e-12), (half, e, pe_ref[half])


def test_nve_and_thermo_against_an_independent_restatement():
    """integrator_nve.h:91-110 with integrator_nve_impl.h:49-54 (dtf =
    0.5 dt / mvv2e, dtfm = dtf / mass[type], v += dtfm f, x += dt v) in numpy
    elementwise operations, which round each product and sum separately as
    the oracle does: bit for bit over an initial + final pair of half-steps
    with two types; the kinetic sum and the temperature factor
    (property_temperature_impl.h:71-76, dof = 3N - 3) within 1e-14."""
    rng = np.random.default_rng(77)
    n = 1000
    x = rng.uniform(0.0, 20.0, size=(n, 3))
    v = rng.normal(size=(n, 3))
    f = rng.normal(size=(n, 3)) * 10.0
    t = rng.integers(0, 2, n).astype(np.int32)
    mass = np.array([1.0, 2.5])
    dt, mvv2e, boltz = 0.005, 1.0364269e-4, 8.617343e-5
    xo, vo = x.copy(), v.copy()
    O.nve_initial(xo, vo, f, t, mass, dt, mvv2e)
    dtf = 0.5 * dt / mvv2e
    dtfm = dtf / mass[t]
    vr = v + dtfm[:, None] * f
    xr = x + dt * vr
    assert np.array_equal(vo, vr) and np.array_equal(xo, xr)
    f2 = rng.normal(size=(n, 3))
    O.nve_final(vo, f2, t, mass, dt, mvv2e)
    vr = vr + dtfm[:, None] * f2
    assert np.array_equal(vo, vr)
    smv2 = O.sum_mv2(vo, t, mass)
    ref = np.sum((vr[:, 0] * vr[:, 0] + vr[:, 1] * vr[:, 1] + vr[:, 2] * vr[:, 2]) * mass[t])
    assert np.isclose(smv2, ref, rtol=1e-14)
    temp = smv2 * (mvv2e / (1.0 * (3 * n - 3) * boltz))
    assert np.isclose(temp, ref * mvv2e / ((3 * n - 3) * boltz), rtol=1e-14)


def test_sort_order_against_an_independent_restatement():
    """The cell sort's declared order: after the single-rank wrap
    (comm_mpi.h:141-168: x > L -> x - L, x < 0 -> x + L, each test on the
    pre-wrap value), atoms ordered by cell index cx + nc_x (cy + nc_y cz),
    with c = floor((x - lo) / h) clamped to [0, nc) and nc = floor(L / (cut
    (1 + 1e-10))) cells of edge h = L / nc (binning_cabana_impl.h:57-113),
    then by id inside a cell; velocities, types and ids permuted alike."""
    rng = np.random.default_rng(41)
    n = 3000
    lo, hi = np.array([0.0, 0.0, 0.0]), np.array([17.3, 12.1, 9.7])
    L = hi - lo
    x = rng.uniform(-0.4, 1.4, size=(n, 3)) * L * 0.999 + 0.0005 * L
    x = np.clip(x, -0.9 * L, 1.9 * L)
    v = rng.normal(size=(n, 3))
    t = rng.integers(0, 3, n).astype(np.int32)
    ids = rng.permutation(n).astype(np.int32) + 1
    cut = 2.8
    xr = x.copy()
    for d in range(3):
        col = x[:, d]
        xr[:, d] = np.where(col > L[d], col - L[d], np.where(col < 0.0, col + L[d], col))
    nc = np.maximum(np.floor(L / (cut * (1.0 + 1e-10))).astype(int), 1)
    h = L / nc
    c = np.clip(np.floor((xr - lo) / h), 0, nc - 1).astype(int)
    key = c[:, 0] + nc[0] * (c[:, 1] + nc[1] * c[:, 2])
    order = np.lexsort((ids, key))

    xo, vo, to, io = x.copy(), v.copy(), t.copy(), ids.copy()
    O.exchange_self(xo, L)
    assert np.array_equal(xo, xr)
    g = O.make_grid(lo, hi, cut)
    O.sort_atoms(g, xo, vo, None, to, io)
    assert np.array_equal(io, ids[order])
    assert np.array_equal(xo, xr[order]) and np.array_equal(vo, v[order])
    assert np.array_equal(to, t[order])
