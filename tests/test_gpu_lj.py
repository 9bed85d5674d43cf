"""GPU parity of the LJ hot path through the C ABI against the CPU oracle.

Bars (from the task's contract):
  - neighbour lists: bit-exact as per-atom sets (and, for this builder's
    canonical order, identical arrays);
  - FP64 forces / energies / thermo: within 1e-10 relative (full-list forces
    and the integrator are in fact bit-identical);
  - mixed precision: max force error <= 1e-4 of the RMS force.
"""
import numpy as np
import pytest

from cabanamd_gb300 import gbmd, inputs
from oracle import pyoracle as O

from conftest import by_id_sets

pytestmark = pytest.mark.gpu

LJ = [(1, 1, 1.0, 1.0, 2.5)]


def _ctx(make, st, prec=gbmd.PREC_FP64):
    c = make()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(prec)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    for (i, j, e, s, rc) in LJ:
        c.lj_coeff(i, j, e, s, rc)
    return c


def _oracle_prepare(st, cut, half):
    x = st.x.copy()
    t = st.type.copy()
    ids = st.id.copy()
    v = st.v.copy()
    O.exchange_self(x, st.hi - st.lo)
    g = O.make_grid(st.lo, st.hi, cut)
    O.sort_atoms(g, x, v, None, t, ids)
    off, j, img = O.neigh_cells(x, g, st.hi, cut, cut, half)
    return x, v, t, ids, (off, j, img)


def _displaced_fcc(ncell=6, disp=0.15, seed=5):
    st = inputs.lj_fcc(ncell, T=1.44, seed=seed)
    rng = np.random.default_rng(seed)
    st.x += rng.uniform(-disp, disp, size=st.x.shape)
    return st


@pytest.mark.parametrize("half", [0, 1])
def test_lists_bitexact(gpu_ctx_factory, half):
    st = _displaced_fcc()
    cut = 2.8
    c = _ctx(gpu_ctx_factory, st)
    c.exchange()
    c.binning(cut)
    c.neigh_build(cut, half, 50)
    a = c.download_atoms()
    off, j, img = c.neigh_download()
    x, v, t, ids, (ooff, oj, oimg) = _oracle_prepare(st, cut, half)
    # identical canonical order
    assert np.array_equal(a.id, ids)
    assert np.array_equal(a.x, x)
    assert np.array_equal(off, ooff)
    assert np.array_equal(j, oj)
    assert np.array_equal(img, oimg)
    # and equal as sets to the brute force over the reference's halo ghosts
    boff, bj, bimg = O.periodic_brute(x, st.lo, st.hi, cut, half)
    assert by_id_sets(off, j, img, a.id) == by_id_sets(boff, bj, bimg, ids)


@pytest.mark.parametrize("L,n,cut", [(5.0, 60, 2.6), (7.0, 150, 2.8), (11.3, 600, 2.8)])
def test_lists_small_boxes_multi_image(gpu_ctx_factory, L, n, cut):
    """nc = 1, 2, 4 cells per dimension: multiple images of one atom."""
    rng = np.random.default_rng(int(L * 10))
    x = rng.uniform(0, L, size=(n, 3))
    st = inputs.State(x, np.zeros_like(x), np.zeros(n, np.int32),
                      np.arange(1, n + 1, dtype=np.int32), np.zeros(3), np.full(3, L), [1.0],
                      1.0, 1.0, 0.005)
    for half in (0, 1):
        c = _ctx(gpu_ctx_factory, st)
        c.exchange()
        c.binning(cut)
        c.neigh_build(cut, half, 8)  # tiny guess exercises the regrow path
        a = c.download_atoms()
        off, j, img = c.neigh_download()
        boff, bj, bimg = O.periodic_brute(a.x, st.lo, st.hi, cut, half)
        assert by_id_sets(off, j, img, a.id) == by_id_sets(boff, bj, bimg, a.id)
        c.close()


def test_boundary_atoms_and_wrap(gpu_ctx_factory):
    """Atoms exactly on the box faces, on the ghost thresholds and slightly
    outside (wrapped by Comm::exchange) give the reference's sets."""
    L = 12.0
    cut = 2.8
    rng = np.random.default_rng(9)
    pts = rng.uniform(0, L, size=(400, 3))
    special = np.array([[0.0, 0.0, 0.0], [L, 1.0, 1.0], [L - cut, 5.0, 5.0], [cut, 6.0, 6.0],
                        [-1e-3, 3.0, 3.0], [L + 1e-3, 4.0, 4.0], [6.0, L, 0.0],
                        [L - cut, L - cut, L - cut]])
    x = np.vstack([pts, special])
    n = len(x)
    st = inputs.State(x, np.zeros_like(x), np.zeros(n, np.int32),
                      np.arange(1, n + 1, dtype=np.int32), np.zeros(3), np.full(3, L), [1.0],
                      1.0, 1.0, 0.005)
    for half in (0, 1):
        c = _ctx(gpu_ctx_factory, st)
        c.exchange()
        c.binning(cut)
        c.neigh_build(cut, half, 50)
        a = c.download_atoms()
        off, j, img = c.neigh_download()
        xo, vo, to, io, (ooff, oj, oimg) = _oracle_prepare(st, cut, half)
        assert np.array_equal(a.x, xo)
        assert np.array_equal(j, oj) and np.array_equal(img, oimg)
        boff, bj, bimg = O.periodic_brute(xo, st.lo, st.hi, cut, half)
        assert by_id_sets(off, j, img, a.id) == by_id_sets(boff, bj, bimg, io)
        c.close()


@pytest.mark.parametrize("prec", [gbmd.PREC_FP64, gbmd.PREC_MIXED])
def test_cell_boundary_coordinates_bin_like_the_oracle(gpu_ctx_factory, prec):
    """Binning takes floor((x - lo) / h) from an FP32 estimate unless the
    estimate lies within 1e-3 of a cell boundary, where the correctly
    rounded FP64 quotient decides.  Coordinates exactly on the boundaries
    lo + k h and a few ulps either side must land in the oracle's cells:
    the atom order and both lists equal the oracle's arrays."""
    L = np.array([20.0, 17.3, 23.1])
    cut = 2.8
    nc = np.floor(L / (cut * (1.0 + 1e-10)))
    h = L / nc
    rng = np.random.default_rng(17)
    n = 700
    x = rng.uniform(0.0, 1.0, size=(n, 3)) * L
    for d in range(3):
        k = rng.integers(1, int(nc[d]), n)
        b = k * h[d]
        kind = rng.integers(0, 6, n)
        near = np.select([kind == 0, kind == 1, kind == 2, kind == 3, kind == 4],
                         [b, np.nextafter(b, np.inf), np.nextafter(b, -np.inf),
                          b + 3 * np.spacing(b), b - 3 * np.spacing(b)], b + 1e-4)
        pick = rng.random(n) < 0.6
        x[pick, d] = near[pick]
    st = inputs.State(x, np.zeros_like(x), np.zeros(n, np.int32),
                      np.arange(1, n + 1, dtype=np.int32), np.zeros(3), L.copy(), [1.0],
                      1.0, 1.0, 0.005)
    for half in (0, 1):
        c = _ctx(gpu_ctx_factory, st, prec)
        c.exchange()
        c.binning(cut)
        c.neigh_build(cut, half, 50)
        a = c.download_atoms()
        off, j, img = c.neigh_download()
        c.close()
        xo, vo, to, io, (ooff, oj, oimg) = _oracle_prepare(st, cut, half)
        assert np.array_equal(a.id, io)
        assert np.array_equal(a.x, xo)
        assert by_id_sets(off, j, img, a.id) == by_id_sets(ooff, oj, oimg, io)
        if prec == gbmd.PREC_FP64:
            assert np.array_equal(off, ooff) and np.array_equal(j, oj)
            assert np.array_equal(img, oimg)


def _rel_force_err(f, fref):
    rms = np.sqrt(np.mean(fref * fref))
    return np.abs(f - fref).max() / rms


@pytest.mark.parametrize("half", [0, 1])
def test_force_energy_fp64(gpu_ctx_factory, half):
    st = _displaced_fcc(seed=21)
    cut = 2.8
    c = _ctx(gpu_ctx_factory, st)
    c.exchange()
    c.binning(cut)
    c.neigh_build(cut, half, 50)
    c.zero_force()
    c.force_compute()
    e = c.force_energy()
    a = c.download_atoms()
    x, v, t, ids, lst = _oracle_prepare(st, cut, half)
    lh = O.ListHandle(*lst)
    p = O.lj_params(LJ)
    fo = O.lj_force(x, t, p, lh, st.hi - st.lo, half)
    eo = O.lj_energy(x, t, p, lh, st.hi - st.lo, half)
    if half == 0:
        assert np.array_equal(a.f, fo)  # same list order, no contraction
    assert _rel_force_err(a.f, fo) < 1e-12
    assert abs(e - eo) <= 1e-10 * abs(eo)


def test_integrator_reversibility_gpu(gpu_ctx_factory):
    """tstIntegrator.hpp:82-137 through the C ABI, bit-identical to the
    oracle's integrator."""
    rng = np.random.default_rng(342343901)
    st = _displaced_fcc(ncell=6, disp=0.1, seed=8)
    st.v = rng.uniform(-1, 1, size=st.x.shape)
    c = _ctx(gpu_ctx_factory, st)
    # Nonzero, bounded forces held constant: one LJ evaluation of a
    # displaced lattice (the reference draws f uniformly in [-1, 1]).
    c.binning(2.8)
    c.neigh_build(2.8, 0, 50)
    c.zero_force()
    c.force_compute()
    a0 = c.download_atoms()
    assert np.abs(a0.f).max() > 0
    for _ in range(100):
        c.integrate_initial()
        c.integrate_final()
    a1 = c.download_atoms()
    # oracle: same forces, same updates, bit for bit
    xo, vo, fo = a0.x.copy(), a0.v.copy(), a0.f.copy()
    for _ in range(100):
        O.nve_initial(xo, vo, fo, a0.type, np.array([1.0]), 0.005, 1.0)
        O.nve_final(vo, fo, a0.type, np.array([1.0]), 0.005, 1.0)
    assert np.array_equal(a1.x, xo) and np.array_equal(a1.v, vo)
    # reverse and integrate back (tstIntegrator.hpp:104-128)
    c.scale_velocities(-1.0)
    for _ in range(100):
        c.integrate_initial()
        c.integrate_final()
    a2 = c.download_atoms()
    fa = a2.x.astype(np.float32).view(np.int32).astype(np.int64)
    fb = a0.x.astype(np.float32).view(np.int32).astype(np.int64)
    assert np.abs(fa - fb).max() <= 4  # EXPECT_FLOAT_EQ
    c.close()


def _run_gpu(make, st, half, nsteps, prec=gbmd.PREC_FP64, thermo_every=10):
    c = _ctx(make, st, prec)
    row0 = c.md_init(2.5, 0.3, half, 20, thermo_every)
    rows = c.md_run(nsteps)
    a = c.download_atoms()
    c.close()
    return np.vstack([row0[None, :], rows]), a


def _run_oracle(st, half, nsteps, thermo_every=10):
    s = st.copy()
    th, f = O.run_lj(s.x, s.v, s.type, s.id, s.lo, s.hi, LJ, force_cut=2.5, skin=0.3,
                     half=half, rebuild_every=20, thermo_every=thermo_every, nsteps=nsteps,
                     boltz=s.boltz, mvv2e=s.mvv2e, dt=s.dt, mass=s.mass, nthreads=4)
    return th, s, f


@pytest.mark.parametrize("half", [0, 1])
def test_md_run_small_matches_oracle(gpu_ctx_factory, half):
    st = inputs.lj_fcc(6, T=1.44, seed=77)
    gth, ga = _run_gpu(gpu_ctx_factory, st, half, 100)
    oth, os_, of = _run_oracle(st, half, 100)
    assert gth.shape == oth.shape
    assert np.allclose(gth, oth, rtol=1e-10, atol=1e-12)
    if half == 0:
        assert np.array_equal(ga.x, os_.x)  # bit-identical trajectory


def test_md_run_config0_32k_100_steps(gpu_ctx_factory):
    """LJ melt 20^3 FCC cells = 32,000 atoms, half list, 100 steps, thermo
    every 10: every thermo value within 1e-10 relative of the oracle."""
    st = inputs.lj_fcc(20, T=1.44, seed=12345)
    assert st.n == 32000
    gth, ga = _run_gpu(gpu_ctx_factory, st, 1, 100)
    oth, os_, of = _run_oracle(st, 1, 100)
    assert np.allclose(gth[:, 1:], oth[:, 1:], rtol=1e-10, atol=0)
    gx = ga.by_id().x
    ox = os_.x[np.argsort(os_.id)]
    assert np.abs(gx - ox).max() < 1e-9


@pytest.mark.parametrize("half", [0, 1])
def test_mixed_precision_force_error(gpu_ctx_factory, half):
    st = _displaced_fcc(ncell=8, seed=31)
    cut = 2.8
    res = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = _ctx(gpu_ctx_factory, st, prec)
        c.exchange()
        c.binning(cut)
        c.neigh_build(cut, half, 50)
        c.zero_force()
        c.force_compute()
        res[prec] = (c.download_atoms(), c.force_energy())
        c.close()
    f64, e64 = res[gbmd.PREC_FP64]
    fmx, emx = res[gbmd.PREC_MIXED]
    assert np.array_equal(f64.id, fmx.id)
    assert _rel_force_err(fmx.f, f64.f) <= 1e-4
    assert abs(emx - e64) <= 1e-5 * abs(e64)


def test_mixed_precision_nve_drift(gpu_ctx_factory):
    """Mixed NVE over 1000 steps conserves energy like FP64 does."""
    st = inputs.lj_fcc(8, T=1.44, seed=5)
    th, _ = _run_gpu(gpu_ctx_factory, st, 0, 1000, prec=gbmd.PREC_MIXED, thermo_every=100)
    etot = th[:, 2] + th[:, 3]
    # equilibrating LJ melt; the per-atom energy must not wander
    assert np.abs(etot[-1] - etot[2]) < 5e-3


def test_lost_atom_is_an_error_not_a_fault(gpu_ctx_factory):
    st = _displaced_fcc(ncell=4)
    st.x[3] = [np.nan, 1.0, 1.0]
    c = _ctx(gpu_ctx_factory, st)
    with pytest.raises(gbmd.GbmdError) as e:
        c.exchange()
    assert e.value.code == 4
    c.close()


def test_bad_arguments(gpu_ctx_factory):
    c = gpu_ctx_factory()
    with pytest.raises(gbmd.GbmdError):
        c.set_box([0, 0, 0], [0, 1, 1])
    with pytest.raises(gbmd.GbmdError):
        c.md_init(2.5, 0.3, 0)  # no atoms
    with pytest.raises(gbmd.GbmdError):
        c.set_types([1.0] * 9)
    with pytest.raises(gbmd.GbmdError):
        c.neigh_build(2.8, 0)  # no binning
    c.close()


def test_empty_system(gpu_ctx_factory):
    st = inputs.State(np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0, np.int32),
                      np.zeros(0, np.int32), np.zeros(3), np.full(3, 10.0), [1.0], 1.0, 1.0,
                      0.005)
    c = _ctx(gpu_ctx_factory, st)
    c.exchange()
    c.binning(2.8)
    c.neigh_build(2.8, 0)
    assert c.neigh_size() == (0, 0)
    c.force_compute()
    assert c.force_energy() == 0.0
    c.close()


@pytest.mark.parametrize("half", [0, 1])
def test_md_run_matches_committed_golden(gpu_ctx_factory, half):
    """The GPU trajectory against tests/golden/lj_small.npz (oracle output,
    no oracle run needed): full list bit-identical, half within 1e-10."""
    import sys
    from pathlib import Path
    here = Path(__file__).resolve().parent / "golden"
    sys.path.insert(0, str(here))
    from make_golden import LJ_CASE, lj_small_case
    gold = np.load(here / "lj_small.npz")
    st = lj_small_case()
    gth, ga = _run_gpu(gpu_ctx_factory, st, half, LJ_CASE["nsteps"])
    a = ga.by_id()
    if half == 0:
        assert np.array_equal(a.x, gold["x_half0"])
        assert np.array_equal(a.v, gold["v_half0"])
        assert np.allclose(gth, gold["thermo_half0"], rtol=1e-12, atol=1e-14)
    else:
        assert np.allclose(gth, gold["thermo_half1"], rtol=1e-10, atol=1e-12)
        assert np.abs(a.x - gold["x_half1"]).max() < 1e-10


@pytest.mark.parametrize("half", [0, 1])
def test_lists_without_images(gpu_ctx_factory, half):
    """gbmd_set_list_images(0): the pairs among the atoms themselves (the
    reference's tree lists over the local atoms, neighbor_tree.h:43-58)
    equal the brute force over the atoms without ghosts; periodic lists are
    restored by gbmd_set_list_images(1)."""
    st = _displaced_fcc()
    cut = 2.8
    c = _ctx(gpu_ctx_factory, st)
    c.exchange()
    c.binning(cut)
    c.set_list_images(False)
    c.neigh_build(cut, half, 50)
    a = c.download_atoms()
    off, j, img = c.neigh_download()
    assert np.all(img == O.IMG_ZERO)
    boff, bj = O.neigh_brute(a.x, len(a.x), cut, half)
    bimg = np.full(len(bj), O.IMG_ZERO, np.int8)
    assert by_id_sets(off, j, img, a.id) == by_id_sets(boff, bj, bimg, a.id)
    c.set_list_images(True)
    c.neigh_build(cut, half, 50)
    off2, j2, img2 = c.neigh_download()
    poff, pj, pimg = O.periodic_brute(a.x, st.lo, st.hi, cut, half)
    assert by_id_sets(off2, j2, img2, a.id) == by_id_sets(poff, pj, pimg, a.id)
    assert len(j2) > len(j)
    c.close()


@pytest.mark.parametrize("prec", [gbmd.PREC_FP64, gbmd.PREC_MIXED])
def test_tstneighbor_geometry_lists_without_images(gpu_ctx_factory, prec):
    """The reference's neighbour unit test (unit_test/tstNeighbor.hpp:76-379)
    on its own geometry: 1000 uniform atoms in the cube [-5.3 rc, 4.7 rc],
    rc = 2.32, lists over the raw positions with no periodic images (what
    its fixture does, and what NeighborTree builds).  The full list equals
    the brute-force N^2 set with d^2 <= rc^2 (:76-141); the half list keeps
    each pair exactly once, within the full list (:144-243).  Both
    precisions build the same lists."""
    cut = 2.32
    lo, hi = -5.3 * cut, 4.7 * cut
    x = np.random.default_rng(342343901).uniform(lo, hi, size=(1000, 3))
    st = inputs.State(x=x, v=np.zeros_like(x), type=np.zeros(1000, np.int32),
                      id=np.arange(1, 1001, dtype=np.int32), lo=np.full(3, lo),
                      hi=np.full(3, hi), mass=[1.0], boltz=1.0, mvv2e=1.0, dt=0.005)
    lists = {}
    for half in (0, 1):
        c = _ctx(gpu_ctx_factory, st, prec)
        c.binning(cut)
        c.set_list_images(False)
        c.neigh_build(cut, half, 50)
        a = c.download_atoms()
        off, j, img = c.neigh_download()
        c.close()
        assert np.all(img == O.IMG_ZERO)
        lists[half] = {k: {p for p, _ in v} for k, v in by_id_sets(off, j, img, a.id).items()}
        if half == 0:
            boff, bj = O.neigh_brute(a.x, len(a.x), cut, 0)
            bimg = np.full(len(bj), O.IMG_ZERO, np.int8)
            assert by_id_sets(off, j, img, a.id) == by_id_sets(boff, bj, bimg, a.id)
    full, halfl = lists[0], lists[1]
    assert sum(map(len, halfl.values())) * 2 == sum(map(len, full.values()))
    for i in full:
        assert halfl[i] <= full[i]
        for p in full[i]:
            assert (p in halfl[i]) != (i in halfl[p])


def test_bounded_wait_expires_and_context_survives(gpu_ctx_factory):
    """Failure detection without a fault: a device wait that nothing
    completes gives up after its bound, the host gets GBMD_ERR_TIMEOUT, and
    the same context then runs an MD segment normally."""
    import time
    st = inputs.lj_fcc(4, T=1.44, seed=2)
    c = _ctx(gpu_ctx_factory, st, gbmd.PREC_MIXED)
    t0 = time.perf_counter()
    rc = c.check_bounded_wait(0.05)
    dt = time.perf_counter() - t0
    assert rc == 5  # GBMD_ERR_TIMEOUT
    assert "timed out" in c.last_error()
    assert 0.03 < dt < 5.0
    row0 = c.md_init(2.5, 0.3, 0, 20, 10)  # clears the flags
    rows = c.md_run(20)
    assert np.all(np.isfinite(rows)) and rows.shape == (2, 4)
    assert abs(row0[2] + row0[3] - (rows[-1, 2] + rows[-1, 3])) < 1e-2
    c.close()


LJ2 = [(1, 1, 1.0, 1.0, 2.5), (1, 2, 0.8, 1.1, 2.6), (2, 2, 1.2, 0.9, 2.2)]


@pytest.mark.parametrize("half", [0, 1])
def test_two_types_fp64_matches_oracle_and_mixed_close(gpu_ctx_factory, half):
    """Multi-type LJ (pair_coeff tables, force_lj_cabana_neigh_impl.h:62-89):
    FP64 = oracle (full list bit for bit), mixed within 1e-4 of RMS F."""
    st = _displaced_fcc(ncell=7, seed=9)
    st.type = (np.arange(st.n) % 2).astype(np.int32)
    st.mass = [1.0, 2.0]
    cut = 2.9
    res = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = gpu_ctx_factory()
        c.set_units(st.boltz, st.mvv2e, st.dt)
        c.set_box(st.lo, st.hi)
        c.set_types(st.mass)
        c.set_precision(prec)
        c.upload_atoms(st.x, st.v, st.type, st.id)
        for (i, j, e, s, rc) in LJ2:
            c.lj_coeff(i, j, e, s, rc)
        c.exchange()
        c.binning(cut)
        c.neigh_build(cut, half, 50)
        c.zero_force()
        c.force_compute()
        res[prec] = (c.download_atoms(), c.force_energy())
        c.close()
    x, v, t, ids, lst = _oracle_prepare(st, cut, half)
    lh = O.ListHandle(*lst)
    p = O.lj_params(LJ2, 2)
    fo = O.lj_force(x, t, p, lh, st.hi - st.lo, half)
    eo = O.lj_energy(x, t, p, lh, st.hi - st.lo, half)
    a64, e64 = res[gbmd.PREC_FP64]
    amx, emx = res[gbmd.PREC_MIXED]
    assert np.array_equal(a64.id, ids) and np.array_equal(amx.id, ids)
    if half == 0:
        assert np.array_equal(a64.f, fo)
    assert _rel_force_err(a64.f, fo) < 1e-12
    assert abs(e64 - eo) <= 1e-10 * abs(eo)
    assert _rel_force_err(amx.f, fo) <= 1e-4
    assert abs(emx - eo) <= 1e-5 * abs(eo)


def test_list_capacity_regrows_for_a_dense_cluster(gpu_ctx_factory):
    """Atoms packed into one corner of a large box: the first build sizes the
    list from the mean density, overflows and regrows (neighbor_verlet.h:
    58-61 grows the guess), and the final list equals the brute force."""
    rng = np.random.default_rng(4)
    sub = inputs.lj_fcc(5, rho=1.1, seed=4)  # 500 atoms in a (5 a)^3 cube
    n = sub.n
    st = inputs.State(sub.x.copy() + 1.0, sub.v.copy(), sub.type.copy(), sub.id.copy(),
                      np.zeros(3), np.full(3, 30.0), [1.0], 1.0, 1.0, 0.005)
    st.x += rng.uniform(-0.05, 0.05, st.x.shape)
    cut = 2.8
    c = _ctx(gpu_ctx_factory, st)
    c.exchange()
    c.binning(cut)
    c.neigh_build(cut, 0, 8)  # a guess far below the ~90 neighbours at rho 1.1
    a = c.download_atoms()
    off, j, img = c.neigh_download()
    tot, mx = c.neigh_size()
    assert mx > 8
    poff, pj, pimg = O.periodic_brute(a.x, st.lo, st.hi, cut, 0)
    assert by_id_sets(off, j, img, a.id) == by_id_sets(poff, pj, pimg, a.id)
    c.close()


def test_upload_rejects_more_atoms_than_the_index_width(gpu_ctx_factory):
    """n above 2^27 - 2 (list entries hold a 27-bit atom index) is refused
    before any array is read."""
    import ctypes as C
    c = gpu_ctx_factory()
    c.set_types([1.0])
    small = np.zeros(3)
    ids = np.zeros(1, np.int32)
    rc = c.lib.gbmd_upload_atoms(c.h, (1 << 27), small.ctypes.data, small.ctypes.data,
                                 ids.ctypes.data, ids.ctypes.data)
    assert rc == 3  # GBMD_ERR_CAPACITY
    assert "2^27" in c.last_error()
    c.close()


def test_mixed_half_list_md_conserves_energy(gpu_ctx_factory):
    """Half list, mixed precision (partner forces by vector FP32 reductions):
    total energy over 500 steps stays as close to constant as FP64's does."""
    st = inputs.lj_fcc(8, T=1.44, seed=6)
    out = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        th, _ = _run_gpu(gpu_ctx_factory, st, 1, 500, prec=prec, thermo_every=50)
        out[prec] = th[:, 2] + th[:, 3]
    d64 = out[gbmd.PREC_FP64][-1] - out[gbmd.PREC_FP64][1]
    dmx = out[gbmd.PREC_MIXED][-1] - out[gbmd.PREC_MIXED][1]
    assert np.all(np.isfinite(out[gbmd.PREC_MIXED]))
    assert abs(dmx - d64) < 2e-3


@pytest.mark.parametrize("prec", [gbmd.PREC_FP64, gbmd.PREC_MIXED])
def test_full_list_runs_are_deterministic(gpu_ctx_factory, prec):
    """Run twice, compare bits: the full-list paths use no atomics, so two
    runs of the same state give the same trajectory and thermo exactly."""
    st = inputs.lj_fcc(10, T=1.44, seed=8)
    th1, a1 = _run_gpu(gpu_ctx_factory, st, 0, 120, prec=prec)
    th2, a2 = _run_gpu(gpu_ctx_factory, st, 0, 120, prec=prec)
    assert np.array_equal(th1, th2)
    assert np.array_equal(a1.x, a2.x) and np.array_equal(a1.v, a2.v)


@pytest.mark.parametrize("prec", [gbmd.PREC_FP64, gbmd.PREC_MIXED])
def test_md_run_graphs_match_direct_launches(gpu_ctx_factory, prec):
    """md_run replays CUDA graphs of the fused steps between thermo steps
    and list rebuilds.  Over md_run calls of uneven length (runs cut short
    by a call's end, graphs reused after rebuilds), the thermo rows and the
    final state equal those of direct launches bit for bit, and the launch
    count is the same."""
    st = _displaced_fcc(8)
    out = {}
    for graphs in (False, True):
        c = _ctx(gpu_ctx_factory, st, prec)
        c.set_graphs(graphs)
        c.md_init(2.5, 0.3, 0, 20, 10)
        rows, launches = [], 0
        for k in (37, 1, 2, 60):
            rows.append(c.md_run(k))
            launches += c.last_run()[1]
        a = c.download_atoms()
        out[graphs] = (np.vstack(rows), a, c.graph_replays(), c.step_count(), launches)
        c.close()
    (r0, a0, g0, s0, n0), (r1, a1, g1, s1, n1) = out[False], out[True]
    assert g0 == 0 and g1 >= 8 and s0 == s1 == 100
    assert n0 == n1
    assert len(r0) == 10 and np.array_equal(r0, r1)
    assert np.array_equal(a0.id, a1.id)
    assert np.array_equal(a0.x, a1.x) and np.array_equal(a0.v, a1.v)


@pytest.mark.parametrize("prec", [gbmd.PREC_FP64, gbmd.PREC_MIXED])
def test_md_run_graphs_follow_changed_dt_and_coefficients(gpu_ctx_factory, prec):
    """A cached graph replays its launches' arguments by value.  Changing the
    timestep (set_units) or the LJ coefficients (lj_coeff) between md_run
    calls must therefore select new graphs: the rows and the final state
    still equal those of direct launches bit for bit, and graphs keep being
    replayed after each change."""
    st = _displaced_fcc(8)
    out = {}
    for graphs in (False, True):
        c = _ctx(gpu_ctx_factory, st, prec)
        c.set_graphs(graphs)
        c.md_init(2.5, 0.3, 0, 20, 10)
        rows, replays = [c.md_run(37)], [c.graph_replays()]
        c.set_units(st.boltz, st.mvv2e, 0.5 * st.dt)  # new dtf/m and dtv
        rows.append(c.md_run(33))
        replays.append(c.graph_replays())
        c.lj_coeff(1, 1, 1.1, 1.02, 2.5)  # new lj1 / lj2 / energy shift
        rows.append(c.md_run(30))
        replays.append(c.graph_replays())
        a = c.download_atoms()
        out[graphs] = (np.vstack(rows), a, replays)
        c.close()
    (r0, a0, g0), (r1, a1, g1) = out[False], out[True]
    assert g0 == [0, 0, 0]
    assert g1[0] > 0 and g1[1] > g1[0] and g1[2] > g1[1]
    assert np.array_equal(r0, r1)
    assert np.array_equal(a0.x, a1.x) and np.array_equal(a0.v, a1.v)


def test_md_run_graphs_half_list_match_direct_launches(gpu_ctx_factory):
    """Half lists (force + fused final/initial integrate per step) replay
    CUDA graphs too.  FP64 half-list forces are summed by FP64 atomics, whose
    order varies from run to run, so graphs on and off agree within 1e-10
    (thermo rows relative, positions absolute), with the same launch count."""
    st = _displaced_fcc(8)
    out = {}
    for graphs in (False, True):
        c = _ctx(gpu_ctx_factory, st, gbmd.PREC_FP64)
        c.set_graphs(graphs)
        c.md_init(2.5, 0.3, 1, 20, 10)
        rows, launches = [], 0
        for k in (37, 1, 2, 60):
            rows.append(c.md_run(k))
            launches += c.last_run()[1]
        a = c.download_atoms()
        out[graphs] = (np.vstack(rows), a, c.graph_replays(), launches)
        c.close()
    (r0, a0, g0, n0), (r1, a1, g1, n1) = out[False], out[True]
    assert g0 == 0 and g1 >= 8 and n0 == n1
    assert np.allclose(r0, r1, rtol=1e-10, atol=0)
    assert np.array_equal(a0.id, a1.id)
    assert np.abs(a0.x - a1.x).max() <= 1e-10


@pytest.mark.parametrize("prec", [gbmd.PREC_FP64, gbmd.PREC_MIXED])
def test_tile_shapes_do_not_change_results(gpu_ctx_factory, prec):
    """Every compiled tile shape -- LJ atoms per block with the list rows'
    prefetch distance, list-build warps per block with the slots staged per
    lane -- and the autotuner's choice give the default shape's run bit for
    bit: thermo rows (energy and kinetic sums are per warp of 32 atoms,
    whatever the block), positions, velocities and forces."""
    st = _displaced_fcc(8)

    def run(shapes=None):
        c = _ctx(gpu_ctx_factory, st, prec)
        if shapes is None:
            c.set_tuning(True)
        else:
            c.set_shapes(*shapes)
        row0 = c.md_init(2.5, 0.3, 0, 20, 10)
        rows = np.vstack([row0[None], c.md_run(60)])
        a = c.download_atoms()
        sh = c.shapes()
        c.close()
        return rows, a, sh

    r0, a0, s0 = run((128, 16, 12, 32))
    assert s0 == {"lj_threads": 128, "lj_prefetch": 16, "nb_warps": 12, "nb_out": 32,
                  "tuned": False}
    for shapes in [(64, 0, 8, 32), (256, 8, 16, 24), (128, 32, 8, 48)]:
        r1, a1, s1 = run(shapes)
        assert (s1["lj_threads"], s1["lj_prefetch"], s1["nb_warps"], s1["nb_out"]) == shapes
        assert np.array_equal(r0, r1), shapes
        assert np.array_equal(a0.id, a1.id), shapes
        assert np.array_equal(a0.x, a1.x) and np.array_equal(a0.v, a1.v), shapes
        assert np.array_equal(a0.f, a1.f), shapes
    r2, a2, s2 = run(None)
    assert s2["tuned"]
    assert s2["lj_threads"] in (64, 128, 256) and (s2["nb_warps"], s2["nb_out"]) in [
        (12, 32), (8, 32), (16, 24), (8, 48)]
    assert np.array_equal(r0, r2)
    assert np.array_equal(a0.x, a2.x) and np.array_equal(a0.v, a2.v)


def test_set_shapes_rejects_uncompiled_shapes(gpu_ctx_factory):
    c = gpu_ctx_factory()
    for bad in [(96, 16, 12, 32), (128, -1, 12, 32), (128, 16, 12, 48)]:
        with pytest.raises(gbmd.GbmdError) as ei:
            c.set_shapes(*bad)
        assert ei.value.code == 1
    c.set_shapes(256, 0, 16, 24)
    assert c.shapes()["lj_threads"] == 256
    c.close()
