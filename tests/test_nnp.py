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
def _gpu_ctx(make, st, prec, potdir, cut):
    from cabanamd_gb300 import gbmd
    c = make()
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(prec)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(potdir), 1.0, 1.0)
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
