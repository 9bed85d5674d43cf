"""Regenerate the committed fixtures in tests/golden/.

1. nnp_ni/: the reference's own NNP fixture (CabanaMD input/nnp: a trained
   Ni potential, n2p2 format), copied verbatim so the loader and NNP tests
   can run where the reference tree is absent.
2. lj_small.npz: oracle trajectories of a small LJ melt (4^3 FCC cells = 256
   atoms, rho 0.8442, T 1.44, rc 2.5, skin 0.3, rebuild 20, 60 steps, thermo
   every 10) for the full and the half list, with the final state by id.
   The GPU tests compare against these without running the oracle, and the
   CPU tests check the oracle still reproduces them.

Usage (from the repository root, where the reference tree is mounted):
    python tests/golden/make_golden.py /path/to/CabanaMD
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


def copy_nnp_fixture(reference: Path, out: Path):
    src = reference / "input" / "nnp"
    out.mkdir(parents=True, exist_ok=True)
    for name in ("input.nn", "scaling.data", "weights.028.data"):
        shutil.copyfile(src / name, out / name)


if __name__ == "__main__":
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else None
    if ref is not None:
        copy_nnp_fixture(ref, HERE / "nnp_ni")
    make_lj_small(HERE / "lj_small.npz")
    print("golden fixtures written to", HERE)
