"""Regenerate the committed fixtures in tests/golden/.

1. nnp_ni/: the reference's own NNP fixture (CabanaMD input/nnp: a trained
   Ni potential, n2p2 format), copied verbatim so the loader and NNP tests
   can run where the reference tree is absent.
2. lj_small.npz: oracle trajectories of a small LJ melt (4^3 FCC cells = 256
   atoms, rho 0.8442, T 1.44, rc 2.5, skin 0.3, rebuild 20, 60 steps, thermo
   every 10) for the full and the half list, with the final state by id.
   The GPU tests compare against these without running the oracle, and the
   CPU tests check the oracle still reproduces them.

3. nnp_cu/ + nnp_cu_4000.npz: the NNP workload's Cu potential (8 G2 + 24 G3,
   rc 6.0 A cosine cutoff, 32-25-25-1 softplus network with N(0, 1/fan_in)
   weights from seed 2024, zero biases) with its scaling fitted to the
   oracle's symmetry functions of the 10^3-cell state (4,000 atoms, a 3.61 A,
   +-0.05 A displacements and 300 K velocities from seed 20261204), and the
   oracle's FP64 NVE trajectory of that state: 200 steps of 0.5 fs, full
   list of cutoff 7.0 A rebuilt every 20 steps, thermo every 10 steps; the
   forces after step 100 and the positions and velocities after step 200,
   by id.  Takes ~15 minutes on 8 cores (`--nnp`).

Usage (from the repository root, where the reference tree is mounted):
    python tests/golden/make_golden.py [/path/to/CabanaMD] [--nnp]
"""
from __future__ import annotations

import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

LJ_CASE = dict(ncell=4, rho=0.8442, T=1.44, seed=4242, nsteps=60)


def lj_small_case():
    from cabanamd_gb300 import inputs
    return inputs.lj_fcc(LJ_CASE["ncell"], rho=LJ_CASE["rho"], T=LJ_CASE["T"],
                         seed=LJ_CASE["seed"])


def make_lj_small(out: Path):
    from oracle import pyoracle as O
    data = {}
    for half in (0, 1):
        st = lj_small_case()
        th, f = O.run_lj(st.x, st.v, st.type, st.id, st.lo, st.hi, [(1, 1, 1.0, 1.0, 2.5)],
                         force_cut=2.5, skin=0.3, half=half, rebuild_every=20, thermo_every=10,
                         nsteps=LJ_CASE["nsteps"], boltz=1.0, mvv2e=1.0, dt=0.005, mass=[1.0])
        o = np.argsort(st.id)
        data[f"thermo_half{half}"] = th
        data[f"x_half{half}"] = st.x[o]
        data[f"v_half{half}"] = st.v[o]
        data[f"f_half{half}"] = f[o]
    np.savez_compressed(out, **data)


NNP_CASE = dict(ncell=10, a=3.61, mass=63.546, T=300.0, disp=0.05, seed=20261204, dt_fs=0.5,
                wseed=2024, rc=6.0, skin=1.0, rebuild_every=20, thermo_every=10, nsteps=200,
                snap_step=100)


def nnp_cu_case():
    from cabanamd_gb300 import inputs
    c = NNP_CASE
    return inputs.nnp_fcc(c["ncell"], a=c["a"], mass=c["mass"], T=c["T"], disp=c["disp"],
                          seed=c["seed"], dt_fs=c["dt_fs"])


def make_nnp_cu(potdir: Path, out: Path, nthreads: int):
    """The potential, fitted by the oracle, then the oracle's trajectory."""
    import os
    from cabanamd_gb300 import nnp_files as NF
    from oracle import pyoracle as O
    c = NNP_CASE
    st = nnp_cu_case()
    pot = NF.synthetic_cu_potential(seed=c["wseed"], rc=c["rc"])
    cut = c["rc"] + c["skin"]
    x, t, ids = st.x.copy(), st.type.copy(), st.id.copy()
    O.exchange_self(x, st.hi - st.lo)
    g = O.make_grid(st.lo, st.hi, cut)
    O.sort_atoms(g, x, None, None, t, ids)
    off, j, img = O.neigh_cells(x, g, st.hi, cut, cut, 0, nthreads)
    r = O.nnp_compute_mt(x, t, O.ListHandle(off, j, img), st.hi - st.lo, pot, nthreads,
                         forces=False)
    NF.fit_scaling(pot, "Cu", r["G"])
    NF.write_potential(potdir, pot)
    pot = NF.read_potential(potdir)  # what the tests load
    s = st.copy()
    th, _, snap = O.run_nnp(s.x, s.v, s.type, s.id, s.lo, s.hi, pot, force_cut=c["rc"],
                            skin=c["skin"], rebuild_every=c["rebuild_every"],
                            thermo_every=c["thermo_every"], nsteps=c["nsteps"], boltz=s.boltz,
                            mvv2e=s.mvv2e, dt=s.dt, mass=s.mass, nthreads=nthreads,
                            snap_step=c["snap_step"])
    o = np.argsort(s.id)
    os_ = np.argsort(snap["id"])
    np.savez_compressed(out, x0=st.x, v0=st.v, thermo=th, f100=snap["f"][os_],
                        x100=snap["x"][os_], x200=s.x[o], v200=s.v[o])


def copy_nnp_fixture(reference: Path, out: Path):
    src = reference / "input" / "nnp"
    out.mkdir(parents=True, exist_ok=True)
    for name in ("input.nn", "scaling.data", "weights.028.data"):
        shutil.copyfile(src / name, out / name)


if __name__ == "__main__":
    import os
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = Path(args[0]) if args else None
    if ref is not None:
        copy_nnp_fixture(ref, HERE / "nnp_ni")
    make_lj_small(HERE / "lj_small.npz")
    if "--nnp" in sys.argv:
        make_nnp_cu(HERE / "nnp_cu", HERE / "nnp_cu_4000.npz", os.cpu_count() or 1)
    print("golden fixtures written to", HERE)
