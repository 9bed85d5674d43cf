import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libgbmd.so")


def pair_sets(off, j, img, ids=None):
    """Per-atom sorted sets of (partner, image code); partners mapped to ids
    when given so lists from differently ordered atoms compare."""
    out = []
    for i in range(len(off) - 1):
        jj = j[off[i]:off[i + 1]]
        mm = img[off[i]:off[i + 1]]
        if ids is not None:
            jj = ids[jj]
        out.append(sorted(zip(jj.tolist(), mm.tolist())))
    return out


def by_id_sets(off, j, img, ids):
    """dict id -> sorted list of (partner id, image code)."""
    s = pair_sets(off, j, img, ids)
    return {int(ids[i]): s[i] for i in range(len(s))}


@pytest.fixture(scope="session")
def gpu_ctx_factory():
    from cabanamd_gb300 import gbmd
    from cabanamd_gb300.build import build_lib
    build_lib()

    def make():
        return gbmd.Context(0)
    return make


def read_data(path):
    """Atoms / Velocities of a LAMMPS data file, sorted by id."""
    lines = Path(path).read_text().splitlines()
    box, atoms, vel, sec = {}, [], [], None
    for ln in lines:
        w = ln.split("#")[0].split()
        if not w:
            continue
        if len(w) == 4 and w[2] in ("xlo", "ylo", "zlo"):
            box[w[2][0]] = (float(w[0]), float(w[1]))
        elif w[0] in ("Atoms", "Velocities", "Masses"):
            sec = w[0]
        elif sec == "Atoms" and len(w) == 5:
            atoms.append((int(w[0]), int(w[1]), float(w[2]), float(w[3]), float(w[4])))
        elif sec == "Velocities" and len(w) == 4:
            vel.append((int(w[0]), float(w[1]), float(w[2]), float(w[3])))
    a = np.array(sorted(atoms))
    v = np.array(sorted(vel))
    return box, a[:, 0].astype(int), a[:, 1].astype(int), a[:, 2:], v[:, 1:]
