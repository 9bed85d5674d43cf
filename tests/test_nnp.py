"""NNP path: n2p2 file formats, the FP64 oracle, and the GPU kernels.

Parity of the NNP arithmetic is unpinned (n2p2 v2.0.1 is not vendored and
no reference test exercises NNP results), so the oracle is checked against
what can be known: the reference fixture's files (input/nnp, read from a
copy committed in tests/golden/nnp_ni), finite differences of its own
energy, and symmetry (zero net force).
"""
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
