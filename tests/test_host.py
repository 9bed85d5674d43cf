"""The C++ host driver (cabanamd_gb300/host): input decks, lattice and
velocity set-up, LAMMPS data files, and the two run loops.

CPU tests build the driver and exercise what needs no GPU (--parse-only,
--init-only); the velocity generator is checked against an independent
restatement of the LAMMPS geom generator the reference uses
(src/inputFile.h:66-148).  GPU tests run decks end to end and compare the
fused loop, the module-by-module loop and the oracle.
"""
import math
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cabanamd_gb300 import inputs
from cabanamd_gb300.build import build_host, build_lib
from conftest import read_data

ROOT = Path(__file__).resolve().parents[1]
DECKS = ROOT / "cabanamd_gb300" / "host" / "decks"


@pytest.fixture(scope="module")
def exe():
    build_lib()
    return build_host()


def run(exe, *args, check=True):
    r = subprocess.run([str(exe), *map(str, args)], capture_output=True, text=True, cwd=ROOT)
    if check and r.returncode != 0:
        raise AssertionError(f"driver failed ({r.returncode}): {r.stderr}")
    return r


class GeomRandomRef:
    """Independent restatement of the reference's LAMMPS geom generator:
    Jenkins one-at-a-time style hash of (seed, x, y, z) bytes taken as signed
    char (x86-64, the reference's CI), 27 kept bits, 5 warm-up draws of a
    Park-Miller minimal-standard stream."""

    def __init__(self, seed, coord):
        h = 0
        data = struct.pack("<i", seed) + struct.pack("<3d", *coord)
        for byte in data:
            sb = byte - 256 if byte > 127 else byte
            h = (h + (sb & 0xFFFFFFFF)) & 0xFFFFFFFF
            h = (h + (h << 10)) & 0xFFFFFFFF
            h ^= h >> 6
        h = (h + (h << 3)) & 0xFFFFFFFF
        h ^= h >> 11
        h = (h + (h << 15)) & 0xFFFFFFFF
        self.s = (h & 0x7FFFFFF) or 1
        for _ in range(5):
            self.uniform()

    def uniform(self):
        self.s = (16807 * self.s) % 2147483647
        return self.s / 2147483647.0


def test_parse_only(exe):
    import json
    d = json.loads(run(exe, "-il", DECKS / "in.lj_melt", "--parse-only").stdout)
    assert d["lattice_constant"] == pytest.approx((4 / 0.8442) ** (1 / 3), rel=1e-15)
    assert d["box_hi"] == pytest.approx([20 * d["lattice_constant"]] * 3, rel=1e-15)
    assert d["force"] == "lj/cut" and d["force_cutoff"] == 2.5 and d["skin"] == 0.3
    assert d["half"] == 1 and d["rebuild_every"] == 20 and d["nsteps"] == 100
    d = json.loads(run(exe, "-il", DECKS / "in.lj_melt", "--parse-only",
                       "--force-iteration", "NEIGH_FULL").stdout)
    assert d["half"] == 0
    d = json.loads(run(exe, "-il", DECKS / "in.nnp_ni", "--parse-only").stdout)
    assert d["force"] == "nnp" and d["force_cutoff"] == 3.9 and d["dt"] == 0.0005
    assert d["mvv2e"] == 1.0364269e-4


def test_unknown_keyword_is_an_error(exe, tmp_path):
    deck = tmp_path / "in.bad"
    deck.write_text("units lj\nfrobnicate 3\n")
    r = run(exe, "-il", deck, "--parse-only", check=False)
    assert r.returncode == 1 and "unknown keyword" in r.stderr


def test_init_lattice_and_velocities(exe, tmp_path):
    """create_lattice: FCC in the reference's loop order, ids 1..N, zero
    momentum, T = target, and each velocity from the geom generator."""
    out = tmp_path / "init.data"
    run(exe, "-il", DECKS / "in.lj_small", "--init-only", out)
    box, ids, types, x, v = read_data(out)
    a = (4 / 0.8442) ** (1 / 3)
    assert np.array_equal(ids, np.arange(1, 865))
    assert np.all(types == 1)
    assert np.array_equal(x, inputs.fcc_positions(6, 6, 6, a))
    assert box["x"] == (0.0, 6 * a)
    assert np.abs(v.sum(axis=0)).max() < 1e-12
    T = (v * v).sum() / (3 * 864 - 3)
    assert T == pytest.approx(1.44, rel=1e-13)
    # independent generator: raw uniform velocities, then the same
    # momentum removal and scaling
    raw = np.array([[g.uniform() - 0.5 for _ in range(3)]
                    for g in (GeomRandomRef(4711, xi) for xi in x)])
    raw -= raw.mean(axis=0)
    raw *= math.sqrt(1.44 / ((raw * raw).sum() / (3 * 864 - 3)))
    assert np.allclose(v, raw, rtol=1e-12, atol=1e-14)


def test_read_data_round_trip(exe, tmp_path):
    first = tmp_path / "a.data"
    run(exe, "-il", DECKS / "in.lj_small", "--init-only", first)
    deck = tmp_path / "in.read"
    deck.write_text(f"units lj\natom_style atomic\nread_data {first}\nmass 1 1.0\n"
                    "pair_style lj/cut 2.5\npair_coeff 1 1 1.0 1.0 2.5\nrun 10\n")
    second = tmp_path / "b.data"
    run(exe, "-il", deck, "--init-only", second)
    a, b = read_data(first), read_data(second)
    for p, q in zip(a[1:], b[1:]):
        assert np.array_equal(p, q)


@pytest.mark.parametrize("damage", ["truncate_atoms", "bad_number", "missing_velocity",
                                    "atom_outside", "no_file"])
def test_damaged_data_files_are_errors(exe, tmp_path, damage):
    """Host-side fault injection: truncated or corrupt data files stop the
    driver with an error message (the reference's log_err), never a crash."""
    good = tmp_path / "a.data"
    run(exe, "-il", DECKS / "in.lj_small", "--init-only", good)
    lines = good.read_text().splitlines()
    ia = lines.index(next(ln for ln in lines if ln.strip().startswith("Atoms")))
    iv = lines.index(next(ln for ln in lines if ln.strip().startswith("Velocities")))
    bad = tmp_path / "bad.data"
    if damage == "truncate_atoms":
        out = lines[:ia + 2 + 100]
    elif damage == "bad_number":
        out = list(lines)
        w = out[ia + 5].split()
        w[2] = "1.0e"  # not a number
        out[ia + 5] = " ".join(w)
    elif damage == "missing_velocity":
        out = lines[:iv + 2] + lines[iv + 3:]
    elif damage == "atom_outside":
        out = list(lines)
        w = out[ia + 5].split()
        w[2] = "1.0e9"
        out[ia + 5] = " ".join(w)
    else:
        out = None
    if out is not None:
        bad.write_text("\n".join(out) + "\n")
    deck = tmp_path / "in.read"
    deck.write_text(f"units lj\natom_style atomic\nread_data {bad}\nmass 1 1.0\n"
                    "pair_style lj/cut 2.5\npair_coeff 1 1 1.0 1.0 2.5\nrun 10\n")
    r = run(exe, "-il", deck, "--init-only", tmp_path / "out.data", check=False)
    assert r.returncode == 1, (r.returncode, r.stderr)
    assert r.stderr.startswith("cbnmd_gb300: ") and len(r.stderr.strip()) > 14


# ---------------------------------------------------------------------------
def thermo_rows(text):
    rows = []
    for ln in text.splitlines():
        w = ln.split()
        if len(w) == 6 and w[0].isdigit():
            rows.append([float(t) for t in w[:4]])
    return np.array(rows)


@pytest.mark.gpu
def test_driver_runs_deck_like_the_oracle(exe, tmp_path):
    """in.lj_small (full list, FP64): the fused loop and the module-by-module
    loop print the same thermo, and the final state equals the oracle's
    trajectory from the same initial data file."""
    from oracle import pyoracle as O
    init = tmp_path / "init.data"
    run(exe, "-il", DECKS / "in.lj_small", "--init-only", init)
    deck_text = (DECKS / "in.lj_small").read_text()
    deck = tmp_path / "in.run"
    deck.write_text(deck_text + f"write_data {tmp_path / 'final.data'}\n")
    fused = run(exe, "-il", deck, "--precision", "fp64").stdout
    deck2 = tmp_path / "in.run2"
    deck2.write_text(deck_text + f"write_data {tmp_path / 'final2.data'}\n")
    modules = run(exe, "-il", deck2, "--precision", "fp64", "--modules").stdout
    ta, tb = thermo_rows(fused), thermo_rows(modules)
    assert ta.shape == (11, 4)
    assert np.array_equal(ta[:, :3], tb[:, :3])
    assert "Atomsteps/s" in fused
    box, ids, types, x0, v0 = read_data(init)
    st = inputs.State(x0.copy(), v0.copy(), np.zeros(len(ids), np.int32), ids.astype(np.int32),
                      np.zeros(3), np.array([box["x"][1], box["y"][1], box["z"][1]]), [1.0],
                      1.0, 1.0, 0.005, {})
    th, f = O.run_lj(st.x, st.v, st.type, st.id, st.lo, st.hi, [(1, 1, 1.0, 1.0, 2.5)],
                     force_cut=2.5, skin=0.3, half=0, rebuild_every=20, thermo_every=10,
                     nsteps=100, boltz=1.0, mvv2e=1.0, dt=0.005, mass=[1.0], nthreads=4)
    o = np.argsort(st.id)
    _, fid, _, xf, vf = read_data(tmp_path / "final.data")
    assert np.array_equal(xf, st.x[o])
    assert np.array_equal(vf, st.v[o])
    _, _, _, xm, _ = read_data(tmp_path / "final2.data")
    assert np.array_equal(xm, xf)
    assert np.allclose(ta[:, 1:3], np.round(th[:, 1:3], 6), atol=2e-6)


@pytest.mark.gpu
def test_driver_runs_reference_nnp_example(exe):
    """The reference's Ni NNP example deck runs (mixed precision) and
    conserves energy over its 100 steps.  This potential was trained in
    Hartree and Bohr (pair_style cfenergy 0.0367493254 = 1 / 27.211...), so
    the reference's fixed Hartree -> eV factor in the energy assembly
    (force_nnp_cabana_neigh_impl.h:101-130) makes the printed PotE an energy
    in eV, consistent with the forces: ETot = PotE + KE is the conserved sum
    per atom."""
    out = run(exe, "-il", DECKS / "in.nnp_ni", "--precision", "mixed").stdout
    t = thermo_rows(out)
    assert t.shape == (11, 4)
    assert np.all(np.isfinite(t))
    assert 300 < t[0, 1] < 900
    ke = t[:, 3] - t[:, 2]
    assert np.all(ke > 0)
    # the kinetic energy does change (a potential with forces), while the
    # total stays put: velocity Verlet at 0.5 fs fluctuates by ~1e-5
    # eV/atom and does not drift
    assert np.ptp(ke) > 1e-3
    etot = t[:, 3]
    assert np.ptp(etot) < 2e-4, etot
    slope = np.polyfit(t[:, 0], etot, 1)[0] * 1000.0
    assert abs(slope) < 1e-3, slope


def test_vacuum_and_neigh_type_options(exe, tmp_path):
    """--vacuum R scales the domain's high corner and leaves the lattice
    (positions, ids, velocities) as the deck makes it
    (inputFile_impl.h:553-559); bad values are the reference's errors."""
    a, b = tmp_path / "a.data", tmp_path / "b.data"
    run(exe, "-il", DECKS / "in.lj_small", "--init-only", a)
    run(exe, "-il", DECKS / "in.lj_small", "--init-only", b, "--vacuum", 2.5,
        "--neigh-type", "TREE_2D")
    boxa, ida, ta, xa, va = read_data(a)
    boxb, idb, tb, xb, vb = read_data(b)
    for k in "xyz":
        assert boxb[k][0] == boxa[k][0]
        assert boxb[k][1] == pytest.approx(2.5 * boxa[k][1], rel=1e-15)
    assert np.array_equal(ida, idb)
    assert np.array_equal(xa, xb)
    assert np.array_equal(va, vb)
    r = run(exe, "-il", DECKS / "in.lj_small", "--init-only", b, "--vacuum", 1.0, check=False)
    assert r.returncode != 0 and "Vacuum multiplier" in r.stderr
    r = run(exe, "-il", DECKS / "in.lj_small", "--neigh-type", "OCTREE", check=False)
    assert r.returncode != 0 and "--neigh-type" in r.stderr


@pytest.mark.gpu
def test_tree_lists_in_vacuum_match_verlet(exe, tmp_path):
    """In a vacuum box no pair crosses the periodic boundary until the first
    rebuild wraps atoms that left through the low face (the lattice starts at
    0), so up to step 19 TREE lists (no images) and VERLET lists give the
    same trajectory bit for bit; in the periodic box they differ from the
    first step.  (After a wrap a TREE list loses the wrapped atom's partners,
    as the reference's ghost-free tree query does.)"""
    outs = {}
    deck_text = (DECKS / "in.lj_small").read_text().replace("run             100",
                                                            "run             19")
    assert "run             19" in deck_text
    for nt in ("VERLET_2D", "TREE_2D"):
        deck = tmp_path / f"in.{nt}"
        deck.write_text(deck_text + f"write_data {tmp_path / (nt + '.data')}\n")
        run(exe, "-il", deck, "--precision", "fp64", "--vacuum", 2.0, "--neigh-type", nt)
        outs[nt] = read_data(tmp_path / (nt + ".data"))
    assert np.array_equal(outs["VERLET_2D"][3], outs["TREE_2D"][3])
    assert np.array_equal(outs["VERLET_2D"][4], outs["TREE_2D"][4])
    deck = tmp_path / "in.p"
    deck.write_text(deck_text + f"write_data {tmp_path / 'tree_periodic.data'}\n")
    run(exe, "-il", deck, "--precision", "fp64", "--neigh-type", "TREE_2D")
    xp = read_data(tmp_path / "tree_periodic.data")[3]
    deck.write_text(deck_text + f"write_data {tmp_path / 'verlet_periodic.data'}\n")
    run(exe, "-il", deck, "--precision", "fp64")
    assert not np.array_equal(xp, read_data(tmp_path / "verlet_periodic.data")[3])



@pytest.mark.gpu
def test_driver_runs_two_element_nnp_deck(exe, tmp_path):
    """A deck with two atom types and a two-element potential: read_data
    gives types 1 (Ni) and 2 (Cu), `mass` sets both, and the fused and
    module-by-module loops print the same thermo in FP64."""
    from cabanamd_gb300 import nnp_files as NF
    st = inputs.nnp_fcc(4, seed=3)
    rng = np.random.default_rng(3)
    types = rng.integers(1, 3, st.n)
    pot = NF.synthetic_binary_potential(seed=7, rc=6.0)
    for e in pot.elements:  # scaling over a generous range: the run stays in it
        pot.gmin[e] = np.zeros(pot.nsf(e))
        pot.gmax[e] = np.full(pot.nsf(e), 50.0)
    potdir = tmp_path / "pot"
    NF.write_potential(potdir, pot)
    data = tmp_path / "two.data"
    L = float(st.hi[0])
    st.x = np.mod(st.x, L)  # displaced lattice sites back inside the box
    lines = ["two-element state", "", f"{st.n} atoms", "2 atom types", "",
             f"0 {L!r} xlo xhi", f"0 {L!r} ylo yhi", f"0 {L!r} zlo zhi", "",
             "Masses", "", "1 58.6934", "2 63.546", "", "Atoms # atomic", ""]
    lines += [f"{i + 1} {types[i]} {float(st.x[i, 0])!r} {float(st.x[i, 1])!r} "
              f"{float(st.x[i, 2])!r}" for i in range(st.n)]
    lines += ["", "Velocities", ""]
    lines += [f"{i + 1} 0.0 0.0 0.0" for i in range(st.n)]
    data.write_text("\n".join(lines) + "\n")
    deck = tmp_path / "in.two"
    deck.write_text(f"units metal\natom_style atomic\nread_data {data}\n"
                    "mass 1 58.6934\nmass 2 63.546\n"
                    f"pair_style nnp dir {potdir} showew no cflength 1.0 cfenergy 1.0\n"
                    "pair_coeff * * 6.0\nneighbor 1.0 bin\ntimestep 0.0005\nthermo 10\n"
                    "fix 1 all nve\nrun 30\n")
    fused = thermo_rows(run(exe, "-il", deck, "--precision", "fp64").stdout)
    mods = thermo_rows(run(exe, "-il", deck, "--precision", "fp64", "--modules").stdout)
    assert fused.shape == (4, 4) and np.all(np.isfinite(fused))
    assert np.allclose(fused[:, 1:3], mods[:, 1:3], rtol=1e-9, atol=1e-9)
    mixed = thermo_rows(run(exe, "-il", deck, "--precision", "mixed").stdout)
    assert np.allclose(mixed[:, 1:3], fused[:, 1:3], rtol=1e-3, atol=1e-4)


# ---------------------------------------------------------------------------
# Several regions, types and masses; VTK particle output (the reference's
# input/in.lb exercises the same commands)
REGIONS = {1: (0, 8, 0, 8, 0, 3), 2: (3, 6, 3, 6, 4, 7), 3: (0, 2, 0, 2, 4, 8)}
MASS = {1: 1.0, 2: 2.0, 3: 0.5}
VEL = {1: (1.0, 1234), 2: (0.5, 5678), 3: (2.0, 91011)}


def test_multi_region_deck_lattice_types_and_velocities(exe, tmp_path):
    """in.lj_regions: the FCC sites inside each region get that region's
    type (lattice units, lo <= u < hi), and the velocities follow the
    reference's per-type set-up (inputFile_impl.h:795-865): the type's seed
    in the geom generator, divided by sqrt(m), the mass-weighted momentum
    removed, then every atom scaled by sqrt(T_target(type) / T)."""
    import json
    d = json.loads(run(exe, "-il", DECKS / "in.lj_regions", "--parse-only").stdout)
    assert d["ntypes"] == 3 and d["pair_coeff_rows"] == 6
    assert d["vtk_rate"] == 10 and d["vtk_file"] == "regions%_*.vtu"
    out = tmp_path / "init.data"
    run(exe, "-il", DECKS / "in.lj_regions", "--init-only", out)
    box, ids, types, x, v = read_data(out)
    a = (4 / 0.8442) ** (1 / 3)
    assert box["z"] == (0.0, 8 * a)
    # independent site list: every FCC site of the 8^3 box inside a region
    sites = inputs.fcc_positions(8, 8, 8, a)
    u = sites
    want_t = np.zeros(len(sites), int)
    for t, (x0, x1, y0, y1, z0, z1) in REGIONS.items():
        # the bounds scaled to the lattice constant, as the reference tests
        inside = ((u[:, 0] >= a * x0) & (u[:, 0] < a * x1) & (u[:, 1] >= a * y0)
                  & (u[:, 1] < a * y1) & (u[:, 2] >= a * z0) & (u[:, 2] < a * z1))
        want_t[inside & (want_t == 0)] = t
    keep = want_t > 0
    assert len(ids) == keep.sum() == 768 + 108 + 64
    order = np.lexsort(x.T)
    worder = np.lexsort(sites[keep].T)
    assert np.array_equal(x[order], sites[keep][worder])
    assert np.array_equal(types[order], want_t[keep][worder])
    m = np.array([MASS[t] for t in types])
    raw = np.array([[g.uniform() - 0.5 for _ in range(3)]
                    for g in (GeomRandomRef(VEL[t][1], xi) for t, xi in zip(types, x))])
    raw /= np.sqrt(m)[:, None]
    raw -= (m[:, None] * raw).sum(axis=0) / m.sum()
    T = (m[:, None] * raw * raw).sum() / (3 * len(m) - 3)
    raw *= np.sqrt(np.array([VEL[t][0] for t in types]) / T)[:, None]
    assert np.allclose(v, raw, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("line,msg", [
    ("dump d all xyz 10 a*%.vtu", "only supports 'vtk'"),
    ("dump d 1 vtk 10 a*%.vtu", "'all' types"),
    ("dump d all vtk 10 a%.vtu", "'*' in file name"),
    ("dump d all vtk 10 a*.vtu", "'%' in file name"),
    ("dump d all vtk 0 a*%.vtu", "rate >= 1"),
])
def test_dump_command_errors(exe, tmp_path, line, msg):
    """dump: the reference's checks (inputFile_impl.h:327-357)."""
    deck = tmp_path / "in.bad"
    deck.write_text((DECKS / "in.lj_small").read_text() + line + "\n")
    r = run(exe, "-il", deck, "--parse-only", check=False)
    assert r.returncode == 1 and msg in r.stderr


def read_vtu(path):
    """Velocity, Id, Type and Points of a VTK particle piece."""
    import xml.etree.ElementTree as ET
    piece = ET.parse(path).getroot().find("UnstructuredGrid/Piece")
    n = int(piece.get("NumberOfPoints"))
    assert piece.get("NumberOfCells") == "0"
    arr = {}
    for da in piece.iter("DataArray"):
        txt = (da.text or "").split()
        if da.get("Name") in ("connectivity", "offsets", "types"):
            assert txt == []
            continue
        dt = float if da.get("type") == "Float64" else int
        arr[da.get("Name")] = np.array([dt(t) for t in txt])
    return (n, arr["Velocity"].reshape(n, 3), arr["Id"], arr["Type"],
            arr["Points"].reshape(n, 3))


@pytest.mark.gpu
@pytest.mark.parametrize("loop", ["fused", "modules"])
def test_multi_region_deck_writes_vtk_particles(exe, tmp_path, loop):
    """in.lj_regions end to end: VTK particle files after steps 10, 20, ...,
    100 (none at step 0, no .pvtu on one rank), named by the reference's
    pattern, each holding the state of the binary snapshot of the same step
    to the 6 significant digits of %g."""
    from cabanamd_gb300.snapshot import read_snapshot, snapshot_path
    text = (DECKS / "in.lj_regions").read_text().replace(
        "regions%_*.vtu", str(tmp_path / "regions%_*.vtu"))
    deck = tmp_path / "in.regions"
    deck.write_text(text)
    dump = tmp_path / "bin"
    dump.mkdir()
    args = ["-il", deck, "--dumpbinary", 10, dump] + (["--modules"] if loop == "modules" else [])
    out = run(exe, *args).stdout
    assert len(thermo_rows(out)) == 11
    names = sorted(p.name for p in tmp_path.glob("regions*"))
    assert names == [f"regions_0_{s:04d}.vtu" for s in range(10, 101, 10)]
    for step in range(10, 101, 10):
        n, vv, vid, vtype, vx = read_vtu(tmp_path / f"regions_0_{step:04d}.vtu")
        s = read_snapshot(snapshot_path(dump, step)).by_id()
        o = np.argsort(vid)
        assert n == 940 and np.array_equal(vid[o], s.id)
        assert np.array_equal(vtype[o], s.type)
        for got, want in ((vx[o], s.x), (vv[o], s.v)):
            assert np.all(np.abs(got - want) <= 5.0001e-6 * np.abs(want) + 1e-300)
