"""NNP path: n2p2 file formats, the FP64 oracle, and the GPU kernels.

Parity of the NNP arithmetic is unpinned (n2p2 v2.0.1 is not vendored and
no reference test exercises NNP results), so the oracle is checked against
what can be known: the reference fixture's files (input/nnp, read from a
copy committed in tests/golden/nnp_ni), an independent numpy evaluation of
the published symmetry-function and network definitions, finite
differences of its own energy, and symmetry (zero net force).
"""
import os
from pathlib import Path

import numpy as np
import pytest

from cabanamd_gb300 import inputs
from cabanamd_gb300 import nnp_files as NF
from oracle import pyoracle as O

from conftest import by_id_sets

GOLD = Path(__file__).resolve().parent / "golden"
NI_DIR = GOLD / "nnp_ni"


def _prepare(st, cut):
    x = st.x.copy()
    t = st.type.copy()
    ids = st.id.copy()
    O.exchange_self(x, st.hi - st.lo)
    g = O.make_grid(st.lo, st.hi, cut)
    O.sort_atoms(g, x, None, None, t, ids)
    off, j, img = O.neigh_cells(x, g, st.hi, cut, cut, 0)
    return x, t, ids, O.ListHandle(off, j, img)


def _cu_potential(st, rc=6.0, skin=1.0, seed=7):
    pot = NF.synthetic_cu_potential(seed=seed, rc=rc)
    x, t, ids, lh = _prepare(st, rc + skin)
    r = O.nnp_compute(x, lh, st.hi - st.lo, O.NNPHandle(pot), forces=False)
    NF.fit_scaling(pot, "Cu", r["G"])
    return pot


def test_reference_fixture_files_parse():
    pot = NF.read_potential(NI_DIR)
    assert pot.elements == ["Ni"]
    assert pot.nsf("Ni") == 27 and pot.nodes == [24, 24, 1] and pot.activations == "ttl"
    sf = pot.symfns["Ni"]
    assert [s.type for s in sf] == [2] * 3 + [3] * 24
    # canonical order: eta, then zeta, then lambda (scaling.data rows follow it)
    ang = [(s.eta, s.zeta, s.lam) for s in sf[3:]]
    assert ang == sorted(ang)
    assert pot.atom_energy["Ni"] == -0.97
    W, b = pot.W["Ni"], pot.b["Ni"]
    assert [w.shape for w in W] == [(24, 27), (24, 24), (1, 24)]
    assert sum(w.size for w in W) + sum(v.size for v in b) == 1297
    # scaling.data rows alternate lambda -1 / +1 within each zeta: the
    # lambda=+1 maximum exceeds the lambda=-1 one at every (eta, zeta)
    gmax = pot.gmax["Ni"][3:].reshape(3, 4, 2)
    assert np.all(gmax[..., 1] > gmax[..., 0])


def test_write_read_roundtrip(tmp_path):
    pot = NF.synthetic_cu_potential(seed=3)
    pot.gmin["Cu"] = np.linspace(0, 1, pot.nsf("Cu"))
    pot.gmax["Cu"] = pot.gmin["Cu"] + 2.0
    NF.write_potential(tmp_path, pot)
    back = NF.read_potential(tmp_path)
    assert [s.key() for s in back.symfns["Cu"]] == [s.key() for s in pot.symfns["Cu"]]
    for a, b in zip(back.W["Cu"], pot.W["Cu"]):
        assert np.array_equal(a, b)
    assert np.array_equal(back.gmin["Cu"], pot.gmin["Cu"])


@pytest.mark.parametrize("ncell", [3, 4])
def test_oracle_forces_match_finite_differences(ncell):
    st = inputs.nnp_fcc(ncell, seed=11)
    pot = _cu_potential(st)
    x, t, ids, lh = _prepare(st, 7.0)
    h = O.NNPHandle(pot)
    L = st.hi - st.lo
    r = O.nnp_compute(x, lh, L, h)
    assert np.allclose(r["f"].sum(axis=0), 0.0, atol=1e-10)
    eps = 1e-5
    rng = np.random.default_rng(ncell)
    for i in rng.choice(len(x), 4, replace=False):
        for d in range(3):
            xp = x.copy()
            xp[i, d] += eps
            xm = x.copy()
            xm[i, d] -= eps
            ep = O.nnp_compute(xp, lh, L, h, forces=False)["esum"]
            em = O.nnp_compute(xm, lh, L, h, forces=False)["esum"]
            fd = -(ep - em) / (2 * eps)
            assert abs(r["f"][i, d] - fd) <= 1e-6 * max(1.0, abs(fd))


def test_oracle_energy_assembly_reference_formula():
    pot = NF.read_potential(NI_DIR)
    h = O.NNPHandle(pot)
    n, esum = 108, 12.5
    e = O._nnp_lib().orc_nnp_energy(n, esum, O.C.byref(h.m))
    assert np.isclose(e, (esum + n * -0.97) * 27.211384021355236, rtol=1e-15)


# ---------------------------------------------------------------------------
# Several elements (no reference fixture: checked by construction)
def _binary_state(ncell=3, seed=13):
    st = inputs.nnp_fcc(ncell, seed=seed)
    rng = np.random.default_rng(seed)
    st.type = rng.integers(0, 2, st.n).astype(np.int32)
    st.mass = [58.6934, 63.546]
    return st


def _binary_potential(st, rc=6.0, skin=1.0, seed=7):
    """synthetic_binary_potential with its scaling fitted to st."""
    pot = NF.synthetic_binary_potential(seed=seed, rc=rc)
    x, t, ids, lh = _prepare(st, rc + skin)
    r = O.nnp_compute_multi(x, t, lh, st.hi - st.lo, pot, forces=False)
    for k, e in enumerate(pot.elements):
        NF.fit_scaling(pot, e, r["G"][t == k, :pot.nsf(e)])
    return pot


def test_oracle_element_channels_sum_to_one_element():
    """Summed over neighbour elements (G2) and element pairs (G3), the
    binary potential's raw functions equal those of a one-element potential
    with the same parameters on the same atoms."""
    st = _binary_state()
    pot2 = NF.synthetic_binary_potential(rc=6.0)
    e = "Cu"
    sfs1 = sorted({(s.type, s.eta, s.zeta, s.lam) for s in pot2.symfns[e]})
    pot1 = NF.synthetic_cu_potential(rc=6.0)
    pot1.symfns[e] = sorted([NF.SymFn(ty, e, (e,) if ty == 2 else (e, e), eta, lam=lam,
                                      zeta=z, rc=6.0) for (ty, eta, z, lam) in sfs1],
                            key=NF.SymFn.key)
    n1 = len(pot1.symfns[e])
    pot1.gmin[e], pot1.gmax[e] = np.zeros(n1), np.ones(n1)
    layers = [n1] + pot1.nodes
    pot1.W[e] = [np.zeros((layers[l], layers[l - 1])) for l in range(1, len(layers))]
    pot1.b[e] = [np.zeros(layers[l]) for l in range(1, len(layers))]
    x, t, ids, lh = _prepare(st, 7.0)
    L = st.hi - st.lo
    r2 = O.nnp_compute_multi(x, t, lh, L, pot2, forces=False)
    r1 = O.nnp_compute(x, lh, L, O.NNPHandle(pot1), forces=False)
    for k, el in enumerate(pot2.elements):
        rows = np.where(t == k)[0]
        assert len(rows) > 0
        want = np.zeros((len(rows), n1))
        for si, s in enumerate(pot2.symfns[el]):
            col = pot1.symfns[e].index(next(q for q in pot1.symfns[e] if
                                            (q.type, q.eta, q.zeta, q.lam) ==
                                            (s.type, s.eta, s.zeta, s.lam)))
            want[:, col] += r2["G"][rows, si]
        assert np.allclose(want, r1["G"][rows], rtol=1e-12, atol=1e-14)


def test_oracle_binary_forces_match_finite_differences():
    st = _binary_state(seed=21)
    pot = _binary_potential(st)
    x, t, ids, lh = _prepare(st, 7.0)
    L = st.hi - st.lo
    r = O.nnp_compute_multi(x, t, lh, L, pot)
    assert np.allclose(r["f"].sum(axis=0), 0.0, atol=1e-10)
    assert np.sqrt(np.mean(r["f"] ** 2)) > 1e-3
    eps = 1e-5
    rng = np.random.default_rng(5)
    for i in rng.choice(len(x), 4, replace=False):
        for d in range(3):
            xp = x.copy()
            xp[i, d] += eps
            xm = x.copy()
            xm[i, d] -= eps
            ep = O.nnp_compute_multi(xp, t, lh, L, pot, forces=False)["esum"]
            em = O.nnp_compute_multi(xm, t, lh, L, pot, forces=False)["esum"]
            fd = -(ep - em) / (2 * eps)
            assert abs(r["f"][i, d] - fd) <= 1e-6 * max(1.0, abs(fd))


def test_binary_potential_files_round_trip(tmp_path):
    st = _binary_state()
    pot = _binary_potential(st)
    NF.write_potential(tmp_path, pot)
    back = NF.read_potential(tmp_path)
    assert back.elements == ["Ni", "Cu"]
    for e in back.elements:
        assert [s.key() for s in back.symfns[e]] == [s.key() for s in pot.symfns[e]]
        assert np.array_equal(back.gmin[e], pot.gmin[e])
        for a, b in zip(back.b[e], pot.b[e]):
            assert np.array_equal(a, b)
    # an input.nn listing the heavier element first still maps Ni to index 0
    txt = (tmp_path / "input.nn").read_text().replace("elements Ni Cu", "elements Cu Ni")
    (tmp_path / "input.nn").write_text(txt)
    assert NF.read_potential(tmp_path).elements == ["Ni", "Cu"]


# ---------------------------------------------------------------------------
# GPU
def _gpu_ctx(make, st, prec, potdir, cut, cfl=1.0, cfe=1.0):
    from cabanamd_gb300 import gbmd
    c = make()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(prec)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(potdir), cfl, cfe)
    c.exchange()
    c.binning(cut)
    c.neigh_build(cut, 0, 64)
    return c


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["ni_fixture", "cu_synthetic"])
def test_gpu_nnp_fp64_matches_oracle(gpu_ctx_factory, tmp_path, which):
    from cabanamd_gb300 import gbmd
    if which == "ni_fixture":
        pot = NF.read_potential(NI_DIR)
        potdir = NI_DIR
        st = inputs.nnp_fcc(3, a=3.52, mass=58.6934, seed=5)
        rc = pot.symfns["Ni"][0].rc
    else:
        st = inputs.nnp_fcc(4, seed=5)
        pot = _cu_potential(st)
        NF.write_potential(tmp_path, pot)
        potdir = tmp_path
        rc = 6.0
    cut = rc + 0.5
    c = _gpu_ctx(gpu_ctx_factory, st, gbmd.PREC_FP64, potdir, cut)
    c.zero_force()
    c.force_compute()
    a = c.download_atoms()
    G, E = c.nnp_download()
    pe = c.force_energy()
    c.close()
    x, t, ids, lh = _prepare(st, cut)
    assert np.array_equal(a.id, ids)
    r = O.nnp_compute(x, lh, st.hi - st.lo, O.NNPHandle(pot))
    assert np.allclose(G, r["G"], rtol=1e-11, atol=1e-12)
    assert np.allclose(E, r["E"], rtol=1e-10, atol=1e-12)
    rms = np.sqrt(np.mean(r["f"] ** 2))
    assert np.abs(a.f - r["f"]).max() <= 1e-10 * max(rms, 1e-30)
    assert np.isclose(pe, O._nnp_lib().orc_nnp_energy(len(x), r["esum"], O.C.byref(
        O.NNPHandle(pot).m)), rtol=1e-10)


@pytest.mark.gpu
def test_gpu_nnp_mixed_force_error(gpu_ctx_factory, tmp_path):
    from cabanamd_gb300 import gbmd
    st = inputs.nnp_fcc(5, seed=9)
    pot = _cu_potential(st)
    NF.write_potential(tmp_path, pot)
    res = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = _gpu_ctx(gpu_ctx_factory, st, prec, tmp_path, 7.0)
        c.zero_force()
        c.force_compute()
        res[prec] = (c.download_atoms(), c.nnp_download()[1])
        c.close()
    f64, e64 = res[gbmd.PREC_FP64]
    fmx, emx = res[gbmd.PREC_MIXED]
    rms = np.sqrt(np.mean(f64.f ** 2))
    assert np.abs(fmx.f - f64.f).max() / rms <= 1e-4
    assert np.abs(emx - e64).max() <= 1e-4 * np.abs(e64).max()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_nnp_dense_state_uses_the_large_capacity(gpu_ctx_factory, tmp_path, prec):
    """Cu compressed to a = 2.6 A has 200-206 neighbours inside 6 A, past the
    common 192-neighbour capacity.  The list's largest count (inside rc +
    skin) selects the 448-neighbour kernels at the rebuild, and the forces
    match the oracle's (FP64 within 1e-10 of the RMS force, mixed within
    1e-4), as the reference's uncapped n2p2 evaluation would give them."""
    from cabanamd_gb300 import gbmd
    p = gbmd.PREC_FP64 if prec == "fp64" else gbmd.PREC_MIXED
    pot = _cu_potential(inputs.nnp_fcc(4, seed=5))
    NF.write_potential(tmp_path, pot)
    dense = inputs.nnp_fcc(4, a=2.6, seed=3)
    c = _gpu_ctx(gpu_ctx_factory, dense, p, tmp_path, 7.0)
    assert c.neigh_size()[1] > 192
    c.zero_force()
    c.force_compute()
    a = c.download_atoms()
    c.close()
    x, t, ids, lh = _prepare(dense, 7.0)
    assert np.array_equal(a.id, ids)
    r = O.nnp_compute_mt(x, t, lh, dense.hi - dense.lo, pot, os.cpu_count() or 1)
    rms = np.sqrt(np.mean(r["f"] ** 2))
    tol = 1e-10 if p == gbmd.PREC_FP64 else 1e-4
    assert np.abs(a.f - r["f"]).max() <= tol * rms


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_nnp_neighbour_capacity_is_an_error(gpu_ctx_factory, tmp_path, prec):
    """More than 448 neighbours inside the NNP cutoff (Cu compressed to
    a = 1.95 A: ~490 within 6 A) is GBMD_ERR_CAPACITY, reported with the
    largest count by force_compute (which reads the device flags), by
    force_energy and by md_init.  The kernels cap their shared-memory writes
    at the capacity, so the GPU does not fault: the same context then runs a
    normal-density state (a = 3.9 A, same box) after md_init clears the
    flag."""
    from cabanamd_gb300 import gbmd
    p = gbmd.PREC_FP64 if prec == "fp64" else gbmd.PREC_MIXED
    NF.write_potential(tmp_path, _cu_potential(inputs.nnp_fcc(4, seed=5)))
    dense = inputs.nnp_fcc(8, a=1.95, seed=3)
    c = _gpu_ctx(gpu_ctx_factory, dense, p, tmp_path, 7.0)
    c.zero_force()
    with pytest.raises(gbmd.GbmdError) as ei:
        c.force_compute()
    assert ei.value.code == 3 and "448 neighbours" in str(ei.value)
    with pytest.raises(gbmd.GbmdError) as ei:
        c.force_energy()
    assert ei.value.code == 3
    with pytest.raises(gbmd.GbmdError) as ei:
        c.md_init(6.0, 1.0, 0, 20, 10)
    assert ei.value.code == 3
    normal = inputs.nnp_fcc(4, a=3.9, seed=3)
    assert np.allclose(normal.hi, dense.hi)
    c.upload_atoms(normal.x, normal.v, normal.type, normal.id)
    c.md_init(6.0, 1.0, 0, 20, 10)
    rows = c.md_run(20)
    assert len(rows) == 2 and np.all(np.isfinite(rows))
    c.close()


@pytest.mark.gpu
def test_gpu_nnp_md_conserves_energy(gpu_ctx_factory, tmp_path):
    """NVE with the NNP: sum E_i + KE stays constant over 200 steps."""
    from cabanamd_gb300 import gbmd
    st = inputs.nnp_fcc(4, seed=13)
    pot = _cu_potential(st)
    NF.write_potential(tmp_path, pot)
    c = gpu_ctx_factory()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(tmp_path), 1.0, 1.0)
    c.md_init(6.0, 1.0, 0, 20, 0)
    etot = []
    for _ in range(20):
        c.md_run(10)
        G, E = c.nnp_download()
        T, KE = c.thermo()
        etot.append(E.sum() + KE)
    c.close()
    n = st.n
    etot = np.array(etot) / n
    # velocity-Verlet fluctuation at dt = 0.5 fs stays ~1e-5 eV/atom and
    # there is no drift beyond it
    assert np.ptp(etot) < 1e-4
    slope = np.polyfit(np.arange(len(etot)) * 10.0, etot, 1)[0]
    assert abs(slope) * 1000.0 < 1e-4


@pytest.mark.gpu
def test_gpu_nnp_mixed_is_reproducible_and_G_accurate(gpu_ctx_factory, tmp_path):
    """The compacted-triplet FP32 path: forces accumulate through fixed-point
    integer atomics, so two evaluations are bit-identical; its symmetry
    functions (downloaded unscaled) agree with the FP64 path's."""
    from cabanamd_gb300 import gbmd
    st = inputs.nnp_fcc(5, seed=19)
    pot = _cu_potential(st)
    NF.write_potential(tmp_path, pot)
    out = []
    for _ in range(2):
        c = _gpu_ctx(gpu_ctx_factory, st, gbmd.PREC_MIXED, tmp_path, 7.0)
        c.zero_force()
        c.force_compute()
        out.append((c.download_atoms().f, c.nnp_download()[0]))
        c.close()
    assert np.array_equal(out[0][0], out[1][0])
    c = _gpu_ctx(gpu_ctx_factory, st, gbmd.PREC_FP64, tmp_path, 7.0)
    c.zero_force()
    c.force_compute()
    g64 = c.nnp_download()[0]
    c.close()
    # relative to each function's fitted range (what the network sees: the
    # scaling multiplies G's error by up to ~50 x 2 here).  FP32 geometry
    # (positions rounded to ~1e-7 of a cell, single-precision terms) puts the
    # floor near 1e-5; the forces this feeds stay within 3e-5 of FP64.
    span = pot.gmax["Cu"] - pot.gmin["Cu"]
    assert (np.abs(out[0][1] - g64).max(axis=0) / span).max() <= 3e-5


@pytest.mark.gpu
@pytest.mark.parametrize("zeta", [(1.0, 3.0), (1.0, 2.0, 8.0, 32.0)])
def test_gpu_nnp_mixed_other_zeta_sets(gpu_ctx_factory, tmp_path, zeta):
    """zeta = 3 is not a power of two (generic FP32 kernels); {1, 2, 8, 32}
    uses the full power ladder.  Both stay within 1e-4 of FP64."""
    from cabanamd_gb300 import gbmd
    st = inputs.nnp_fcc(4, seed=23)
    pot = NF.synthetic_cu_potential(seed=5)
    e = "Cu"
    sfs = [s for s in pot.symfns[e] if s.type == 2]
    sfs += [NF.SymFn(3, e, (e, e), eta, lam=lam, zeta=z, rc=6.0)
            for eta in (0.001, 0.01, 0.05) for z in zeta for lam in (-1.0, 1.0)]
    pot.symfns[e] = sorted(sfs, key=NF.SymFn.key)
    n = len(sfs)
    rng = np.random.default_rng(3)
    pot.W[e][0] = rng.normal(0.0, 1.0 / np.sqrt(n), size=(pot.nodes[0], n))
    pot.gmin[e] = np.zeros(n)
    pot.gmax[e] = np.ones(n)
    x, t, ids, lh = _prepare(st, 7.0)
    r = O.nnp_compute(x, lh, st.hi - st.lo, O.NNPHandle(pot), forces=False)
    NF.fit_scaling(pot, e, r["G"])
    NF.write_potential(tmp_path, pot)
    res = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = _gpu_ctx(gpu_ctx_factory, st, prec, tmp_path, 7.0)
        c.zero_force()
        c.force_compute()
        res[prec] = c.download_atoms().f
        c.close()
    rms = np.sqrt(np.mean(res[gbmd.PREC_FP64] ** 2))
    assert np.abs(res[gbmd.PREC_MIXED] - res[gbmd.PREC_FP64]).max() / rms <= 1e-4


@pytest.mark.gpu
def test_gpu_nnp_mixed_reference_fixture(gpu_ctx_factory):
    """The reference's own Ni potential (input/nnp) in mixed precision
    against FP64 on its 108-atom example geometry (3^3 FCC cells, a = 3.52).
    The potential is trained in Bohr / Hartree: with input/in.nnp's
    conversion factors (cflength 1.8897261328, cfenergy 0.0367493254) its
    inputs are in range; with 1 / 1 every tanh unit saturates and the forces
    are exactly zero."""
    from cabanamd_gb300 import gbmd
    st = inputs.nnp_fcc(3, a=3.52, mass=58.6934, seed=5)
    cfl, cfe = 1.8897261328, 0.0367493254
    rc = NF.read_potential(NI_DIR).symfns["Ni"][0].rc / cfl
    res = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = _gpu_ctx(gpu_ctx_factory, st, prec, NI_DIR, rc + 0.5, cfl, cfe)
        c.zero_force()
        c.force_compute()
        res[prec] = (c.download_atoms().f, c.nnp_download()[1])
        c.close()
    f64, e64 = res[gbmd.PREC_FP64]
    fmx, emx = res[gbmd.PREC_MIXED]
    rms = np.sqrt(np.mean(f64 ** 2))
    assert rms > 1e-3
    assert np.abs(fmx - f64).max() / rms <= 1e-4
    assert np.abs(emx - e64).max() <= 1e-4 * np.abs(e64).max()


@pytest.mark.gpu
def test_gpu_nnp_fp64_length_energy_units(gpu_ctx_factory):
    """cflength / cfenergy (input/in.nnp: Angstrom / eV positions against a
    Bohr / Hartree network): the GPU evaluates the network on positions x
    cflength and returns forces x cflength / cfenergy -- the oracle run on the
    scaled geometry gives the same symmetry functions and forces."""
    from cabanamd_gb300 import gbmd
    cfl, cfe = 1.8897261328, 0.0367493254
    pot = NF.read_potential(NI_DIR)
    st = inputs.nnp_fcc(3, a=3.52, mass=58.6934, seed=5)
    cut = pot.symfns["Ni"][0].rc / cfl + 0.5
    c = _gpu_ctx(gpu_ctx_factory, st, gbmd.PREC_FP64, NI_DIR, cut, cfl, cfe)
    c.zero_force()
    c.force_compute()
    a = c.download_atoms()
    G, E = c.nnp_download()
    c.close()
    o = np.argsort(a.id)
    sc = st.copy()
    sc.x = st.x * cfl
    sc.lo = st.lo * cfl
    sc.hi = st.hi * cfl
    x, t, ids, lh = _prepare(sc, cut * cfl)
    r = O.nnp_compute(x, lh, sc.hi - sc.lo, O.NNPHandle(pot))
    q = np.argsort(ids)
    assert np.allclose(G[o], r["G"][q], rtol=1e-10, atol=1e-12)
    f_ref = r["f"][q] * cfl / cfe
    rms = np.sqrt(np.mean(f_ref ** 2))
    assert rms > 1e-3
    assert np.abs(a.f[o] - f_ref).max() <= 1e-9 * rms


# ---------------------------------------------------------------------------
# GPU, several elements
def _binary_gpu(gpu_ctx_factory, tmp_path, prec, ncell=4, seed=13):
    st = _binary_state(ncell, seed)
    pot = _binary_potential(st)
    NF.write_potential(tmp_path, pot)
    c = _gpu_ctx(gpu_ctx_factory, st, prec, tmp_path, 6.5)
    c.zero_force()
    c.force_compute()
    a = c.download_atoms()
    G, E = c.nnp_download()
    pe = c.force_energy()
    c.close()
    return st, pot, a, G, E, pe


@pytest.mark.gpu
def test_gpu_nnp_two_elements_fp64_matches_oracle(gpu_ctx_factory, tmp_path):
    """Per-element function sets, networks and scaling; radial functions
    filtered by neighbour element, angular ones by element pair."""
    from cabanamd_gb300 import gbmd
    st, pot, a, G, E, pe = _binary_gpu(gpu_ctx_factory, tmp_path, gbmd.PREC_FP64)
    x, t, ids, lh = _prepare(st, 6.5)
    assert np.array_equal(a.id, ids)
    r = O.nnp_compute_multi(x, t, lh, st.hi - st.lo, pot)
    assert G.shape == r["G"].shape
    assert np.allclose(G, r["G"], rtol=1e-11, atol=1e-12)
    assert np.allclose(E, r["E"], rtol=1e-10, atol=1e-12)
    rms = np.sqrt(np.mean(r["f"] ** 2))
    assert rms > 1e-3
    assert np.abs(a.f - r["f"]).max() <= 1e-10 * rms
    assert np.isclose(pe, r["energy"], rtol=1e-10)


@pytest.mark.gpu
def test_gpu_nnp_two_elements_mixed_force_error(gpu_ctx_factory, tmp_path):
    from cabanamd_gb300 import gbmd
    _, _, a64, _, _, pe64 = _binary_gpu(gpu_ctx_factory, tmp_path / "a", gbmd.PREC_FP64)
    _, _, amx, _, _, pemx = _binary_gpu(gpu_ctx_factory, tmp_path / "b", gbmd.PREC_MIXED)
    assert np.array_equal(a64.id, amx.id)
    rms = np.sqrt(np.mean(a64.f ** 2))
    assert np.abs(amx.f - a64.f).max() <= 1e-4 * rms
    assert abs(pemx - pe64) <= 1e-5 * abs(pe64)


@pytest.mark.gpu
def test_gpu_nnp_two_elements_needs_matching_types(gpu_ctx_factory, tmp_path):
    from cabanamd_gb300 import gbmd
    st = _binary_state(3)
    NF.write_potential(tmp_path, _binary_potential(st))
    st.type[:] = 0
    st.mass = [58.6934]
    c = _gpu_ctx(gpu_ctx_factory, st, gbmd.PREC_FP64, tmp_path, 6.5)
    with pytest.raises(gbmd.GbmdError) as ei:
        c.force_compute()
    assert "elements" in str(ei.value)
    c.close()


@pytest.mark.gpu
def test_gpu_nnp_two_elements_md_conserves_energy(gpu_ctx_factory, tmp_path):
    """NVE with the two-element potential: sum E_i + KE stays constant (the
    reference's energy assembly multiplies by 27.211 but its forces do not,
    so the conserved sum is the networks' own)."""
    from cabanamd_gb300 import gbmd
    st = _binary_state(4, seed=3)
    NF.write_potential(tmp_path, _binary_potential(st))
    c = gpu_ctx_factory()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(gbmd.PREC_FP64)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(tmp_path), 1.0, 1.0)
    c.md_init(6.0, 1.0, 0, 20, 0)
    etot = []
    for _ in range(10):
        c.md_run(10)
        G, E = c.nnp_download()
        T, KE = c.thermo()
        etot.append(E.sum() + KE)
    c.close()
    etot = np.array(etot) / st.n
    assert np.all(np.isfinite(etot))
    assert np.ptp(etot) < 1e-4


@pytest.mark.gpu
def test_gpu_nnp_two_elements_unequal_function_counts(gpu_ctx_factory, tmp_path):
    """Elements with different function counts (Ni 32, Cu 20): G / dE/dG rows
    are padded to the larger count, every kernel indexes them by that stride,
    and both precisions match the oracle as in the equal-count case."""
    from cabanamd_gb300 import gbmd
    st = _binary_state(4, seed=17)
    pot = NF.synthetic_binary_potential(seed=5, rc=6.0)
    e = "Cu"
    keep = [s for k, s in enumerate(pot.symfns[e]) if s.type == 2 or k % 2 == 0][:20]
    pot.symfns[e] = keep
    n1 = len(keep)
    layers = [n1] + pot.nodes
    rng = np.random.default_rng(9)
    pot.W[e] = [rng.normal(0.0, 1.0 / np.sqrt(layers[l - 1]), size=(layers[l], layers[l - 1]))
                for l in range(1, len(layers))]
    pot.gmin[e], pot.gmax[e] = np.zeros(n1), np.ones(n1)
    x, t, ids, lh = _prepare(st, 7.0)
    r = O.nnp_compute_multi(x, t, lh, st.hi - st.lo, pot, forces=False)
    for k, el in enumerate(pot.elements):
        NF.fit_scaling(pot, el, r["G"][t == k, :pot.nsf(el)])
    NF.write_potential(tmp_path, pot)
    ro = O.nnp_compute_multi(x, t, lh, st.hi - st.lo, pot)
    res = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = _gpu_ctx(gpu_ctx_factory, st, prec, tmp_path, 6.5)
        c.zero_force()
        c.force_compute()
        a = c.download_atoms()
        G, E = c.nnp_download()
        res[prec] = (a, G, E, c.force_energy())
        c.close()
    a64, G64, E64, pe64 = res[gbmd.PREC_FP64]
    amx, Gmx, Emx, pemx = res[gbmd.PREC_MIXED]
    assert np.array_equal(a64.id, ids)
    assert G64.shape == (len(x), 32)
    assert np.all(G64[t == 1, n1:] == 0.0)
    assert np.allclose(G64, ro["G"], rtol=1e-11, atol=1e-12)
    assert np.allclose(E64, ro["E"], rtol=1e-10, atol=1e-12)
    rms = np.sqrt(np.mean(ro["f"] ** 2))
    assert np.abs(a64.f - ro["f"]).max() <= 1e-10 * rms
    assert np.abs(amx.f - ro["f"]).max() <= 1e-4 * rms
    assert abs(pemx - pe64) <= 1e-5 * abs(pe64)


# ---------------------------------------------------------------------------
# The NNP workload's trajectory (4,000 atoms, 200 steps) against the oracle's,
# from the committed fixture (tests/golden/make_golden.py --nnp)
NNP_CU_DIR = GOLD / "nnp_cu"
NNP_CU_NPZ = GOLD / "nnp_cu_4000.npz"


def _nnp_cu_state():
    """The 10^3-cell Cu state of the fixture (initial x, v from the file)."""
    d = np.load(NNP_CU_NPZ)
    st = inputs.nnp_fcc(10, a=3.61, mass=63.546, T=300.0, disp=0.05, seed=20261204,
                        dt_fs=0.5)
    st.x = d["x0"].copy()
    st.v = d["v0"].copy()
    return st, d


def test_nnp_fixture_step0_matches_oracle():
    """The committed trajectory still starts where the oracle does: the
    step-0 thermo row of one oracle force evaluation equals the fixture's."""
    from oracle import pyoracle as O2
    st, d = _nnp_cu_state()
    pot = NF.read_potential(NNP_CU_DIR)
    th, _, _ = O2.run_nnp(st.x, st.v, st.type, st.id, st.lo, st.hi, pot, force_cut=6.0,
                          skin=1.0, rebuild_every=20, thermo_every=10, nsteps=0,
                          boltz=st.boltz, mvv2e=st.mvv2e, dt=st.dt, mass=st.mass,
                          nthreads=os.cpu_count() or 1)
    assert th.shape == (1, 4)
    assert np.allclose(th[0], d["thermo"][0], rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_gpu_nnp_fp64_trajectory_matches_oracle(gpu_ctx_factory):
    """FP64 NNP NVE on the workload's 4,000-atom Cu state (10^3 FCC cells,
    32 symmetry functions, 32-25-25-1 softplus network, 0.5 fs, full list of
    7.0 A rebuilt every 20 steps) against the oracle's 200-step trajectory:
    every thermo row (step, T, PE/N, KE/N) within 1e-10 relative, the forces
    after step 100 within 1e-10 of the RMS force, and the positions and
    velocities after step 200 within 1e-9 (A, A/ps) of the oracle's."""
    from cabanamd_gb300 import gbmd
    st, d = _nnp_cu_state()
    c = gpu_ctx_factory()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(gbmd.PREC_FP64)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(NNP_CU_DIR), 1.0, 1.0)
    row0 = c.md_init(6.0, 1.0, 0, 20, 10)
    r1 = c.md_run(100)
    a100 = c.download_atoms().by_id()
    r2 = c.md_run(100)
    a200 = c.download_atoms().by_id()
    c.close()
    rows = np.vstack([row0[None], r1, r2])
    th = d["thermo"]
    assert rows.shape == th.shape == (21, 4)
    assert np.array_equal(rows[:, 0], th[:, 0])
    rel = np.abs(rows[:, 1:] - th[:, 1:]) / np.abs(th[:, 1:])
    assert rel.max() <= 1e-10, rel.max(axis=0)
    f = d["f100"]
    rms = np.sqrt(np.mean(f * f))
    assert np.abs(a100.f - f).max() <= 1e-10 * rms
    assert np.abs(a200.x - d["x200"]).max() <= 1e-9
    assert np.abs(a200.v - d["v200"]).max() <= 1e-9


@pytest.mark.gpu
def test_gpu_nnp_mixed_trajectory_tracks_oracle(gpu_ctx_factory):
    """Mixed precision (FP32 symmetry functions and force chain, tensor-core
    MLP, FP64 integration) on the same 200 steps: the temperature and
    energies track the oracle's FP64 trajectory, and the conserved energy
    sum E_i + KE drifts no more than the FP64 oracle's plus 1e-5 eV/atom
    per 1000 steps."""
    from cabanamd_gb300 import gbmd
    st, d = _nnp_cu_state()
    c = gpu_ctx_factory()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(gbmd.PREC_MIXED)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(NNP_CU_DIR), 1.0, 1.0)
    row0 = c.md_init(6.0, 1.0, 0, 20, 10)
    rows = np.vstack([row0[None], c.md_run(200)])
    c.close()
    th = d["thermo"]
    hartree = 27.211384021355236
    assert np.abs(rows[:, 1] - th[:, 1]).max() <= 1e-3 * th[:, 1].max()
    assert np.abs(rows[:, 2] - th[:, 2]).max() / hartree <= 1e-4
    e_mx = rows[:, 2] / hartree + rows[:, 3]
    e_64 = th[:, 2] / hartree + th[:, 3]
    s_mx = np.polyfit(rows[:, 0], e_mx, 1)[0] * 1000.0
    s_64 = np.polyfit(th[:, 0], e_64, 1)[0] * 1000.0
    assert abs(s_mx - s_64) <= 1e-5, (s_mx, s_64)


@pytest.mark.gpu
@pytest.mark.parametrize("reps", [3, 6])
def test_gpu_nnp_two_elements_periodic_replicas(gpu_ctx_factory, tmp_path, reps):
    """The per-element atom groups at sizes whose grouping scan runs over
    several warps of blocks (reps 3: 55,296 atoms) and over several chunks of
    1,024 blocks (reps 6: 442,368 atoms).  The state is a 2,048-atom
    two-element system (8^3 cells) repeated reps^3 times: every copy of an
    atom has the same periodic environment, so its energy and force equal
    those of the atom in the small system (FP64: within 1e-10 relative of
    the RMS; mixed: within 1e-4).  An atom left out of its group, taken
    twice, or run with the other element's network breaks that."""
    from cabanamd_gb300 import gbmd
    small = _binary_state(8, seed=41)
    pot = _binary_potential(_binary_state(4, seed=41))
    NF.write_potential(tmp_path, pot)
    ns = small.n
    L = small.hi - small.lo
    shifts = np.array([(a, b, c) for c in range(reps) for b in range(reps) for a in range(reps)],
                      dtype=np.float64) * L
    big = small.copy()
    big.x = (small.x[None, :, :] + shifts[:, None, :]).reshape(-1, 3)
    big.v = np.zeros_like(big.x)
    big.type = np.tile(small.type, reps ** 3)
    big.id = np.arange(1, len(big.x) + 1, dtype=np.int32)
    big.hi = small.lo + reps * L
    for prec, tol in ((gbmd.PREC_FP64, 1e-10), (gbmd.PREC_MIXED, 1e-4)):
        out = []
        for st in (small, big):
            c = _gpu_ctx(gpu_ctx_factory, st, prec, tmp_path, 7.0)
            c.zero_force()
            c.force_compute()
            a = c.download_atoms()
            _, E = c.nnp_download()
            c.close()
            src = (a.id - 1) % ns  # the small-system atom each copy repeats
            out.append((src, a.f, E))
        (s0, f0, e0), (s1, f1, e1) = out
        fs = np.zeros_like(f0)
        es = np.zeros_like(e0)
        fs[s0], es[s0] = f0, e0
        assert np.bincount(s1, minlength=ns).tolist() == [reps ** 3] * ns
        rms = np.sqrt(np.mean(f0 ** 2))
        assert np.abs(f1 - fs[s1]).max() <= tol * rms, prec
        assert np.abs(e1 - es[s1]).max() <= tol * np.abs(e0).max(), prec


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_gpu_nnp_md_run_graphs_match_direct_launches(gpu_ctx_factory, prec):
    """md_run captures the NNP steps between thermo steps and rebuilds (force
    + fused final/initial integrate) into CUDA graphs and replays them.  Over
    md_run calls of uneven length, graphs on and off give the same thermo
    rows and final state -- bit for bit in mixed precision (fixed-point
    force sums); within 1e-10 in FP64, whose forces are summed by FP64
    atomics in an order that varies from run to run -- with the same launch
    count."""
    from cabanamd_gb300 import gbmd
    p = gbmd.PREC_FP64 if prec == "fp64" else gbmd.PREC_MIXED
    st = inputs.nnp_fcc(5, seed=13)
    out = {}
    for graphs in (False, True):
        c = gpu_ctx_factory()
        c.set_units(st.boltz, st.mvv2e, st.dt)
        c.set_box(st.lo, st.hi)
        c.set_types(st.mass)
        c.set_precision(p)
        c.upload_atoms(st.x, st.v, st.type, st.id)
        c.nnp_load(str(NNP_CU_DIR), 1.0, 1.0)
        c.set_graphs(graphs)
        c.md_init(6.0, 1.0, 0, 20, 10)
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
    assert len(r0) == 10
    assert np.array_equal(a0.id, a1.id)
    if p == gbmd.PREC_MIXED:
        assert np.array_equal(r0, r1)
        assert np.array_equal(a0.x, a1.x) and np.array_equal(a0.v, a1.v)
    else:
        assert np.allclose(r0, r1, rtol=1e-10, atol=0)
        assert np.abs(a0.x - a1.x).max() <= 1e-10
        assert np.abs(a0.v - a1.v).max() <= 1e-10 * np.abs(a0.v).max()


# ---------------------------------------------------------------------------
# An independent restatement of the NNP arithmetic: the oracle's symmetry
# functions, atomic energies and forces against a plain numpy evaluation of
# the published definitions, written without the oracle's neighbour list.
def _restated_nnp(x, L, pot, elem, types=None):
    """Behler-Parrinello radial G2 = sum_j exp(-eta (r_ij - rs)^2) fc(r_ij)
    and angular G3 = 2^(1 - zeta) sum_{j<k} (1 + lambda cos theta_ijk)^zeta
    exp(-eta ((r_ij - rs)^2 + (r_ik - rs)^2 + (r_jk - rs)^2)) fc(r_ij)
    fc(r_ik) fc(r_jk) (n2p2 symmetry-function types 2 and 3) with the cosine
    cutoff fc(r) = (cos(pi r / rc) + 1) / 2 for r < rc; every periodic image
    of every atom inside the cutoff (rc < L, so images one box away suffice);
    then the scaling to [smin, smax] and the atomic network (t: tanh,
    p: softplus ln(1 + e^x), l: linear).  Returns raw G and E_i.  With
    types (each atom's index into pot.elements), the atoms of element elem
    are evaluated, a radial function summing the neighbours of its
    neighbour element and an angular one the pairs of its unordered element
    pair; rows of the other atoms stay zero."""
    sfs = pot.symfns[elem]
    n = len(x)
    ei = pot.elements.index(elem)
    el = np.zeros(n, int) if types is None else np.asarray(types)
    shifts = np.array([[a, b, c] for a in (-1, 0, 1) for b in (-1, 0, 1)
                       for c in (-1, 0, 1)], dtype=float) * L
    G = np.zeros((n, len(sfs)))

    def fcut(r, rc):
        return np.where(r < rc, 0.5 * (np.cos(np.pi * r / rc) + 1.0), 0.0)

    for i in range(n):
        if el[i] != ei:
            continue
        d = (x[None, :, :] + shifts[:, None, :] - x[i]).reshape(-1, 3)
        ne = np.tile(el, len(shifts))
        r = np.sqrt((d * d).sum(axis=1))
        keep = (r > 0.0) & (r < max(s.rc for s in sfs))
        d, r, ne = d[keep], r[keep], ne[keep]
        jj, kk = np.triu_indices(len(r), 1)
        djk = d[jj] - d[kk]
        rjk = np.sqrt((djk * djk).sum(axis=1))
        cos = (d[jj] * d[kk]).sum(axis=1) / (r[jj] * r[kk])
        lo_el, hi_el = np.minimum(ne[jj], ne[kk]), np.maximum(ne[jj], ne[kk])
        for s, sf in enumerate(sfs):
            fc = fcut(r, sf.rc)
            nb = sorted(pot.elements.index(e) for e in sf.neighbors)
            if sf.type == 2:
                m = ne == nb[0]
                G[i, s] = np.sum(np.exp(-sf.eta * (r[m] - sf.rs) ** 2) * fc[m])
            else:
                m = (lo_el == nb[0]) & (hi_el == nb[-1])
                rad = np.exp(-sf.eta * ((r[jj] - sf.rs) ** 2 + (r[kk] - sf.rs) ** 2 +
                                        (rjk - sf.rs) ** 2))
                G[i, s] = 2.0 ** (1.0 - sf.zeta) * np.sum(
                    ((1.0 + sf.lam * cos) ** sf.zeta * rad * fc[jj] * fc[kk] *
                     fcut(rjk, sf.rc))[m])
    a = pot.smin + (pot.smax - pot.smin) * (G - pot.gmin[elem]) / (pot.gmax[elem] - pot.gmin[elem])
    for W, b, act in zip(pot.W[elem], pot.b[elem], pot.activations):
        a = a @ np.asarray(W).T + np.asarray(b)
        if act == "t":
            a = np.tanh(a)
        elif act == "p":
            a = np.log1p(np.exp(a))
    E = np.where(el == ei, a[:, 0], 0.0)
    return G, E


@pytest.mark.parametrize("which", ["cu_synthetic", "ni_fixture"])
def test_oracle_matches_an_independent_restatement(which):
    """The oracle's raw symmetry functions, atomic energies and their sum
    equal a plain numpy evaluation of the published Behler-Parrinello
    definitions over every periodic image (1e-12 relative), for the
    workloads' Cu potential (softplus network, 8 G2 + 24 G3 with zeta up to
    16) and for the reference's trained Ni fixture (tanh network, its 27
    functions, lengths in Bohr); and the oracle's forces equal the negative
    gradient of the restated total energy by central differences."""
    if which == "cu_synthetic":
        st = inputs.nnp_fcc(3, seed=21)
        pot = _cu_potential(st)
        cut = 7.0
    else:
        bohr = 1.8897261254578281
        st = inputs.nnp_fcc(3, a=3.52 * bohr, mass=58.6934, disp=0.05 * bohr, seed=22)
        pot = NF.read_potential(NI_DIR)
        cut = 7.3699319 + 0.5
    elem = pot.elements[0]
    x, t, ids, lh = _prepare(st, cut)
    L = st.hi - st.lo
    r = O.nnp_compute(x, lh, L, O.NNPHandle(pot))
    G, E = _restated_nnp(x, L, pot, elem)
    assert np.allclose(r["G"], G, rtol=1e-12, atol=1e-12 * np.abs(G).max())
    assert np.allclose(r["E"], E, rtol=1e-12, atol=1e-12 * np.abs(E).max())
    assert np.isclose(r["esum"], E.sum(), rtol=1e-12)
    # forces: the restated energy's central differences for a few atoms
    eps = 1e-5
    rng = np.random.default_rng(5)
    for i in rng.choice(len(x), 2, replace=False):
        for d in range(3):
            xp = x.copy()
            xp[i, d] += eps
            xm = x.copy()
            xm[i, d] -= eps
            fd = -(_restated_nnp(xp, L, pot, elem)[1].sum() -
                   _restated_nnp(xm, L, pot, elem)[1].sum()) / (2 * eps)
            assert abs(r["f"][i, d] - fd) <= 1e-6 * max(1.0, abs(fd)), (i, d, r["f"][i, d], fd)


def test_oracle_two_elements_match_an_independent_restatement():
    """Two elements (Ni/Cu at random on a displaced FCC lattice, the
    workloads' binary potential): for each element's atoms, the oracle's raw
    symmetry functions and atomic energies equal the numpy restatement with
    radial functions over the neighbours of their element and angular ones
    over the pairs of their unordered element pair (1e-12), and the total
    energy is the sum of both elements' restated atomic energies."""
    st = _binary_state(3, seed=23)
    pot = _binary_potential(st)
    x, t, ids, lh = _prepare(st, 7.0)
    L = st.hi - st.lo
    r = O.nnp_compute_multi(x, t, lh, L, pot)
    Etot = 0.0
    for k, e in enumerate(pot.elements):
        G, E = _restated_nnp(x, L, pot, e, types=t)
        sel = t == k
        nsf = pot.nsf(e)
        assert np.allclose(r["G"][sel, :nsf], G[sel], rtol=1e-12,
                           atol=1e-12 * np.abs(G[sel]).max())
        assert np.allclose(r["E"][sel], E[sel], rtol=1e-12, atol=1e-12 * np.abs(E[sel]).max())
        Etot += E.sum()
    assert np.isclose(r["esum"], Etot, rtol=1e-12)
