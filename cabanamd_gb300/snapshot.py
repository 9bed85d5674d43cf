"""Binary configuration snapshots: the record of CabanaMD's --dumpbinary and
--correctness (CbnMD::dump_binary / check_correctness,
src/cabanamd_impl.h:434-642), as the cbnmd_gb300 driver writes them.

One file per step and rank, ``<dir>/output.<step:%010d>.<rank:%03d>``:

    int32 n | int32 id[n] | int32 type[n] | float64 q[n] |
    float64 x[n][3] | float64 v[n][3] | float64 f[n][3]

x, v and f are atom-major xyz triples (the reference's writer and reader
disagree on this layout; the driver's snapshot.cpp fixes it this way), all
little-endian as written on both supported hosts.
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

HEADER = "# timestep deltarnorm maxdelr deltavnorm maxdelv deltafnorm maxdelf"


@dataclass
class Snapshot:
    id: np.ndarray    # [n] int32
    type: np.ndarray  # [n] int32, 0-based
    q: np.ndarray     # [n] float64
    x: np.ndarray     # [n, 3] float64
    v: np.ndarray     # [n, 3] float64
    f: np.ndarray     # [n, 3] float64

    @property
    def n(self) -> int:
        return len(self.id)

    def by_id(self) -> "Snapshot":
        """The same atoms in increasing id order."""
        o = np.argsort(self.id, kind="stable")
        return Snapshot(self.id[o], self.type[o], self.q[o], self.x[o], self.v[o], self.f[o])


def snapshot_path(directory, step: int, rank: int = 0) -> Path:
    return Path(directory) / f"output.{step:010d}.{rank:03d}"


def write_snapshot(path, s: Snapshot) -> None:
    n = s.n
    with open(path, "wb") as fh:
        fh.write(np.int32(n).astype("<i4").tobytes())
        for a, dt, shape in ((s.id, "<i4", (n,)), (s.type, "<i4", (n,)), (s.q, "<f8", (n,)),
                             (s.x, "<f8", (n, 3)), (s.v, "<f8", (n, 3)), (s.f, "<f8", (n, 3))):
            a = np.asarray(a)
            if a.shape != shape:
                raise ValueError(f"snapshot array of shape {a.shape}, expected {shape}")
            fh.write(np.ascontiguousarray(a, dtype=dt).tobytes())


def read_snapshot(path) -> Snapshot:
    raw = Path(path).read_bytes()
    if len(raw) < 4:
        raise ValueError(f"Error reading reference data: {path}")
    n = int(np.frombuffer(raw, "<i4", 1)[0])
    if n < 0 or len(raw) != 4 + n * (4 + 4 + 8 + 72):
        raise ValueError(f"Error reading reference data: {path}")
    off = 4
    out = []
    for dt, count, shape in (("<i4", n, (n,)), ("<i4", n, (n,)), ("<f8", n, (n,)),
                             ("<f8", 3 * n, (n, 3)), ("<f8", 3 * n, (n, 3)),
                             ("<f8", 3 * n, (n, 3))):
        a = np.frombuffer(raw, dt, count, off).reshape(shape)
        off += a.nbytes
        out.append(a.astype(a.dtype.newbyteorder("=")))
    return Snapshot(*out)


def snapshot_diff(cur: Snapshot, ref: Snapshot) -> tuple[float, ...]:
    """(|dr|, max|dr_k|, |dv|, max|dv_k|, |df|, max|df_k|) of current minus
    reference with atoms matched by id (cabanamd_impl.h:560-640)."""
    if cur.n != ref.n:
        raise ValueError("Mismatch in current and reference atom counts")
    order = np.argsort(cur.id, kind="stable")
    pos = np.searchsorted(cur.id[order], ref.id)
    pos = np.minimum(pos, max(cur.n - 1, 0))
    if cur.n and not np.array_equal(cur.id[order][pos], ref.id):
        raise ValueError("Unable to find current id matching reference id")
    j = order[pos]
    out = []
    for a, b in ((cur.x, ref.x), (cur.v, ref.v), (cur.f, ref.f)):
        d = a[j] - b
        out += [float(np.sqrt(np.sum(d * d))), float(np.max(np.abs(d), initial=0.0))]
    return tuple(out)


def read_correctness(path) -> np.ndarray:
    """Rows [step, |dr|, max|dr|, |dv|, max|dv|, |df|, max|df|] of a
    correctness file."""
    lines = Path(path).read_text().splitlines()
    if not lines or lines[0] != HEADER:
        raise ValueError(f"not a correctness file: {path}")
    return np.array([[float(t) for t in ln.split()] for ln in lines[1:]]).reshape(-1, 7)
