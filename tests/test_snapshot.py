"""Binary snapshots and the correctness diff (--dumpbinary / --correctness,
src/cabanamd_impl.h:434-642).

CPU tests: the Python reader / writer against the driver's C++ reader
(--snapdiff), atom matching by id, and the reference's error cases.  GPU
tests: the driver's snapshots of an FP64 run equal the oracle's trajectory,
a run checked against its own snapshots gives zero deltas, and a
mixed-precision run checked against FP64 snapshots stays close.
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from cabanamd_gb300.build import build_host, build_lib
from conftest import read_data
from cabanamd_gb300.snapshot import (HEADER, Snapshot, read_correctness, read_snapshot,
                                     snapshot_diff, snapshot_path, write_snapshot)

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


def random_snapshot(rng, n):
    return Snapshot(rng.permutation(n).astype(np.int32) + 1, rng.integers(0, 3, n, dtype=np.int32),
                    np.zeros(n), rng.normal(size=(n, 3)) * 10, rng.normal(size=(n, 3)),
                    rng.normal(size=(n, 3)) * 100)


def test_path_and_layout(tmp_path):
    assert snapshot_path("d", 120, 3).as_posix() == "d/output.0000000120.003"
    s = random_snapshot(np.random.default_rng(1), 37)
    p = tmp_path / "a"
    write_snapshot(p, s)
    raw = p.read_bytes()
    assert len(raw) == 4 + 37 * (4 + 4 + 8 + 3 * 24)
    # atom-major xyz triples right after n, id, type, q
    off = 4 + 37 * 16
    assert np.array_equal(np.frombuffer(raw, "<f8", 3, off), s.x[0])
    r = read_snapshot(p)
    for k in ("id", "type", "q", "x", "v", "f"):
        assert np.array_equal(getattr(r, k), getattr(s, k))


def test_snapdiff_matches_numpy(exe, tmp_path):
    """The C++ reader and diff (--snapdiff) on files the Python writer made:
    atoms in a different order are matched by id."""
    rng = np.random.default_rng(7)
    ref = random_snapshot(rng, 500)
    o = rng.permutation(500)
    cur = Snapshot(ref.id[o], ref.type[o], ref.q[o], ref.x[o] + rng.normal(size=(500, 3)) * 1e-9,
                   ref.v[o] * (1 + 1e-12), ref.f[o] + 1e-6)
    write_snapshot(tmp_path / "cur", cur)
    write_snapshot(tmp_path / "ref", ref)
    out = run(exe, "--snapdiff", tmp_path / "cur", tmp_path / "ref").stdout.splitlines()
    assert out[0].startswith("# deltarnorm")
    got = np.array([float(t) for t in out[1].split()])
    want = np.array(snapshot_diff(cur, ref))
    assert np.allclose(got, want, rtol=1e-14, atol=0)
    assert want[5] == pytest.approx(1e-6, rel=1e-6)
    same = run(exe, "--snapdiff", tmp_path / "ref", tmp_path / "ref").stdout.splitlines()[1]
    assert [float(t) for t in same.split()] == [0.0] * 6


def test_snapdiff_errors(exe, tmp_path):
    rng = np.random.default_rng(3)
    a = random_snapshot(rng, 20)
    write_snapshot(tmp_path / "a", a)
    b = Snapshot(a.id[:19], a.type[:19], a.q[:19], a.x[:19], a.v[:19], a.f[:19])
    write_snapshot(tmp_path / "b", b)
    r = run(exe, "--snapdiff", tmp_path / "a", tmp_path / "b", check=False)
    assert r.returncode != 0 and "atom counts" in r.stderr
    c = Snapshot(a.id.copy(), a.type, a.q, a.x, a.v, a.f)
    c.id[4] = 999
    write_snapshot(tmp_path / "c", c)
    r = run(exe, "--snapdiff", tmp_path / "a", tmp_path / "c", check=False)
    assert r.returncode != 0 and "999" in r.stderr
    (tmp_path / "short").write_bytes((tmp_path / "a").read_bytes()[:-8])
    r = run(exe, "--snapdiff", tmp_path / "a", tmp_path / "short", check=False)
    assert r.returncode != 0 and "Error reading reference data" in r.stderr
    with pytest.raises(ValueError):
        read_snapshot(tmp_path / "short")
    r = run(exe, "--snapdiff", tmp_path / "a", tmp_path / "missing", check=False)
    assert r.returncode != 0 and "Cannot open" in r.stderr


# ---------------------------------------------------------------------------
def _deck(tmp_path, name, extra=""):
    d = tmp_path / name
    d.write_text((DECKS / "in.lj_small").read_text() + extra)
    return d


@pytest.mark.gpu
def test_dumpbinary_matches_oracle(exe, tmp_path):
    """in.lj_small, FP64 full list: the step-0, 50 and 100 snapshots of both
    run loops are the oracle's state bit for bit (x, v and f by id)."""
    from oracle import pyoracle as O
    init = tmp_path / "init.data"
    run(exe, "-il", DECKS / "in.lj_small", "--init-only", init)
    deck = _deck(tmp_path, "in.a")
    dump = tmp_path / "dump"
    dump.mkdir()
    run(exe, "-il", deck, "--precision", "fp64", "--dumpbinary", 50, dump)
    assert sorted(p.name for p in dump.iterdir()) == [
        "output.0000000000.000", "output.0000000050.000", "output.0000000100.000"]
    dump2 = tmp_path / "dump2"
    dump2.mkdir()
    run(exe, "-il", deck, "--precision", "fp64", "--modules", "--dumpbinary", 50, dump2)
    box, ids, types, x0, v0 = read_data(init)
    lo, hi = np.zeros(3), np.array([box["x"][1], box["y"][1], box["z"][1]])
    x, v = x0.copy(), v0.copy()
    typ, idv = np.zeros(len(ids), np.int32), ids.astype(np.int32)
    for step in (0, 50, 100):
        if step:
            th, f = O.run_lj(x, v, typ, idv, lo, hi, [(1, 1, 1.0, 1.0, 2.5)], force_cut=2.5,
                             skin=0.3, half=0, rebuild_every=20, thermo_every=10, nsteps=step,
                             boltz=1.0, mvv2e=1.0, dt=0.005, mass=[1.0], nthreads=4)
            o = np.argsort(idv)
            want = (x[o], v[o], f[o])
            x, v = x0.copy(), v0.copy()
            typ, idv = np.zeros(len(ids), np.int32), ids.astype(np.int32)
        for d in (dump, dump2):
            s = read_snapshot(snapshot_path(d, step)).by_id()
            assert np.array_equal(s.id, np.sort(ids))
            assert np.all(s.type == 0) and np.all(s.q == 0)
            if step == 0:
                assert np.array_equal(s.x, x0[np.argsort(ids)])
                assert np.array_equal(s.v, v0[np.argsort(ids)])
            else:
                assert np.array_equal(s.x, want[0])
                assert np.array_equal(s.v, want[1])
                assert np.array_equal(s.f, want[2])


@pytest.mark.gpu
def test_correctness_against_snapshots(exe, tmp_path):
    """--correctness: an FP64 run against its own snapshots gives zero deltas.
    A mixed-precision run against them starts from the same x and v with
    forces within 1e-4 of the melt's RMS force; later steps drift apart as
    trajectories of a liquid do, and stay close over 100 steps."""
    deck = _deck(tmp_path, "in.b")
    dump = tmp_path / "dump"
    dump.mkdir()
    run(exe, "-il", deck, "--precision", "fp64", "--dumpbinary", 20, dump)
    out = tmp_path / "corr.txt"
    run(exe, "-il", deck, "--precision", "fp64", "--correctness", 20, dump, out)
    assert out.read_text().splitlines()[0] == HEADER
    rows = read_correctness(out)
    assert np.array_equal(rows[:, 0], [0, 20, 40, 60, 80, 100])
    assert np.all(rows[:, 1:] == 0)
    out2 = tmp_path / "corr_mixed.txt"
    run(exe, "-il", deck, "--precision", "mixed", "--correctness", 100, dump, out2)
    rows = read_correctness(out2)
    assert np.array_equal(rows[:, 0], [0, 100])
    # the deck starts on the perfect lattice (zero forces): the force scale is
    # the melt's at step 100
    f_rms = np.sqrt(np.mean(read_snapshot(snapshot_path(dump, 100)).f ** 2) * 3)
    assert f_rms > 1.0
    assert rows[0, 1] == 0 and rows[0, 3] == 0   # same initial x, v
    assert rows[0, 6] < 1e-4 * f_rms
    assert np.all(rows[1:, 2] < 1e-3)
