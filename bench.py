#!/usr/bin/env python
"""Benchmark of the GB300 MD hot path: atom-steps/s on the 4,000,000-atom
LJ FCC melt (100^3 cells, rho 0.8442, T 1.44, rc 2.5, skin 0.3, rebuild
every 20 steps, thermo every 10, dt 0.005).

A "step" is one CbnMD timestep (src/cabanamd_impl.h:284-399): initial
integrate, [exchange + sort + list rebuild every 20th step], force, final
integrate, [thermo every 10th step].  `value` is device time of K steps
with the state resident in HBM; `e2e` goes through the C ABI from host
buffers (upload, init, K steps, thermo readbacks, download).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbmd|reference]
                  [--precision mixed|fp64] [--list full|half] [--cells C]

--impl reference times the CPU restatement of the reference's algorithm
(oracle/, OpenMP on all host cores; the reference itself needs Kokkos,
Cabana and MPI, which are not installable here) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("atom-steps/s (LJ, NNP) mixed vs FP64 at ≤1e-4 force err; serving p50/p99")
LJ = [(1, 1, 1.0, 1.0, 2.5)]
FORCE_CUT, SKIN, REBUILD, THERMO = 2.5, 0.3, 20, 10


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.lines:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [t.strip() for t in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def make_state(cells):
    from cabanamd_gb300 import inputs
    return inputs.lj_fcc(cells, rho=0.8442, T=1.44, seed=20261203)


def new_ctx(dev, st, prec):
    from cabanamd_gb300 import gbmd
    c = gbmd.Context(dev)
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(prec)
    for (i, j, e, s, rc) in LJ:
        c.lj_coeff(i, j, e, s, rc)
    return c


def run_device(dev, st, prec, half, steps, warmup, profile=True):
    """Resident-state run: returns dict with ms, rows, launches, force time."""
    c = new_ctx(dev, st, prec)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.md_init(FORCE_CUT, SKIN, half, REBUILD, THERMO)
    if warmup:
        c.md_run(warmup)
    tot, _ = c.neigh_size()
    c.set_profiling(profile)
    with ClockSampler(dev) as clk:
        rows = c.md_run(steps)
    ms, launches = c.last_run()
    fms, fcount = c.kernel_time("force")
    nms, ncount = c.kernel_time("neigh")
    ims, icount = c.kernel_time("integrate")
    sms, scount = c.kernel_time("sort")
    c.set_profiling(False)
    a = c.download_atoms()
    c.close()
    return dict(ms=ms, rows=rows, launches=launches, force_ms=fms, force_n=fcount,
                neigh_ms=nms, neigh_n=ncount, int_ms=ims, int_n=icount, sort_ms=sms,
                sort_n=scount, list_entries=tot, clocks=clk.summary(), atoms=a)


def force_error(dev, atoms, st, half):
    """Mixed vs FP64 forces on identical positions (max |df| / rms f)."""
    from cabanamd_gb300 import gbmd
    out = {}
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = new_ctx(dev, st, prec)
        c.upload_atoms(atoms.x, atoms.v, atoms.type, atoms.id)
        c.exchange()
        c.binning(FORCE_CUT + SKIN)
        c.neigh_build(FORCE_CUT + SKIN, half, 96)
        c.zero_force()
        c.force_compute()
        out[prec] = (c.download_atoms().by_id().f, c.force_energy())
        c.close()
    f64, e64 = out[gbmd.PREC_FP64]
    fmx, emx = out[gbmd.PREC_MIXED]
    rms = float(np.sqrt(np.mean(f64 * f64)))
    return {"max_rel_force_err": float(np.abs(fmx - f64).max() / rms),
            "rms_rel_force_err": float(np.sqrt(np.mean((fmx - f64) ** 2)) / rms),
            "pe_rel_err": float(abs(emx - e64) / abs(e64))}


def run_e2e(dev, st, prec, half, steps):
    """Through the public C ABI from host buffers: upload, md_init, K steps
    (thermo rows read back every 10 steps), download."""
    c = new_ctx(dev, st, prec)
    x = np.ascontiguousarray(st.x)
    v = np.ascontiguousarray(st.v)
    c.synchronize()
    t0 = time.perf_counter()
    c.upload_atoms(x, v, st.type, st.id)
    c.md_init(FORCE_CUT, SKIN, half, REBUILD, THERMO)
    rows = c.md_run(steps)
    a = c.download_atoms()
    t1 = time.perf_counter()
    c.close()
    n = st.n
    h2d = n * (24 + 24 + 4 + 4)
    d2h = n * (24 * 3 + 4 + 4) + (len(rows) + 1) * 32
    return {"value": n * steps / (t1 - t0), "unit": "atom-steps/s",
            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "seconds": t1 - t0}


def cpu_baseline(st, half, steps, threads):
    from oracle import pyoracle as O
    s = st.copy()
    tm = {}
    O.run_lj(s.x, s.v, s.type, s.id, s.lo, s.hi, LJ, force_cut=FORCE_CUT, skin=SKIN, half=half,
             rebuild_every=REBUILD, thermo_every=THERMO, nsteps=steps, boltz=s.boltz,
             mvv2e=s.mvv2e, dt=s.dt, mass=s.mass, nthreads=threads, time_from_step=0,
             timing=tm)
    return st.n * steps / tm["loop_seconds"], tm["loop_seconds"]


def profile_traffic(workload_key, atoms):
    """DRAM bytes per force launch from the committed ncu summary (scaled
    by atoms when the capture used a smaller case)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text()).get(workload_key)
    if not d:
        return None
    return d["dram_bytes_per_launch"] * atoms / d["atoms"]


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local, dist


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbmd", choices=["gbmd", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--list", default="full", choices=["full", "half"])
    ap.add_argument("--cells", type=int, default=100)
    ap.add_argument("--cpu-steps", type=int, default=20)
    ap.add_argument("--no-variants", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    half = 1 if args.list == "half" else 0
    rank, ws, local, dist = dist_setup()
    st = make_state(args.cells)
    n = st.n
    threads = os.cpu_count() or 1
    workload = f"lj_fcc_{args.cells}^3_cells_{n}_atoms"
    config = {"workload": workload, "atoms": n, "rho": 0.8442, "T": 1.44, "cutoff": FORCE_CUT,
              "skin": SKIN, "rebuild_every": REBUILD, "thermo_every": THERMO, "dt": 0.005,
              "list": args.list, "precision": args.precision,
              "l2": "inputs larger than L2 (positions, velocities, forces, Verlet list "
                    "> 1 GB resident per GPU)",
              "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"}

    if args.impl == "reference":
        if rank != 0:
            return
        total = args.warmup + args.steps
        from oracle import pyoracle as O
        s = st.copy()
        tm = {}
        O.run_lj(s.x, s.v, s.type, s.id, s.lo, s.hi, LJ, force_cut=FORCE_CUT, skin=SKIN,
                 half=half, rebuild_every=REBUILD, thermo_every=THERMO, nsteps=total,
                 boltz=s.boltz, mvv2e=s.mvv2e, dt=s.dt, mass=s.mass, nthreads=threads,
                 time_from_step=args.warmup, timing=tm)
        sec = tm["loop_seconds"]
        val = n * args.steps / sec
        line = {"metric": METRIC, "value": val, "unit": "atom-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * sec / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(config, precision="fp64"), "impl": "reference",
                "cpu_baseline": {"value": val, "unit": "atom-steps/s", "cores": threads,
                                 "kind": "port",
                                 "sample": f"full {n}-atom system, {args.steps} timed steps "
                                           f"after {args.warmup} warm-up steps (CPU "
                                           "restatement of the reference, OpenMP)"},
                "e2e": {"value": val, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    from cabanamd_gb300 import gbmd
    prec = gbmd.PREC_MIXED if args.precision == "mixed" else gbmd.PREC_FP64
    dev = local
    if dist:
        dist.barrier()
    r = run_device(dev, st, prec, half, args.steps, args.warmup)
    ms = r["ms"]
    if dist:
        import torch
        t = torch.tensor([ms], dtype=torch.float64,
                         device="cuda" if torch.cuda.is_available() else "cpu")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    value = ws * n * args.steps / (ms * 1e-3)
    if rank != 0:
        return

    # roofline of the dominant kernel (LJ force): algorithmic bytes per launch
    K = r["list_entries"] / n
    if prec == gbmd.PREC_MIXED:
        per_atom = 16 + 4 + 4 * K + 24 + (24 if half else 0)
    else:
        per_atom = 32 + 4 + 4 + 4 * K + 24 + (24 if half else 0)
    f_avg_s = r["force_ms"] * 1e-3 / max(r["force_n"], 1)
    achieved = n * per_atom / f_avg_s / 1e9
    peak, peak_kind = peaks()
    traffic = profile_traffic(f"lj_force_{args.precision}_{args.list}", n)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
            "kernel": "k_lj_mixed" if prec == gbmd.PREC_MIXED else "k_lj_fp64",
            "algorithmic_bytes_per_atom": per_atom, "list_entries_per_atom": K,
            "avg_launch_ms": f_avg_s * 1e3, "launches": r["force_n"]}
    phase_ms = {"force": r["force_ms"], "neigh": r["neigh_ms"], "sort": r["sort_ms"],
                "integrate": r["int_ms"], "total": r["ms"]}

    cpu_val, cpu_sec = cpu_baseline(st, half, args.cpu_steps, threads)
    e2e = run_e2e(dev, st, prec, half, args.steps)
    rows = r["rows"]
    drift = None
    if len(rows) >= 2:
        etot = rows[:, 2] + rows[:, 3]
        drift = float((etot[-1] - etot[0]) / (rows[-1, 0] - rows[0, 0]) * 1000.0)

    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32/f64" if prec == gbmd.PREC_MIXED else "f64", "data": "synthetic",
            "config": config, "roofline": roof,
            "cpu_baseline": {"value": cpu_val, "unit": "atom-steps/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{args.cpu_steps} steps (incl. one list rebuild) of the "
                                       f"same {n}-atom system, FP64 CPU restatement of the "
                                       f"reference, {cpu_sec:.1f} s"},
            "e2e": e2e, "gpu_launches": r["launches"], "clocks": r["clocks"],
            "phase_ms": phase_ms, "nve_drift_per_atom_per_1000_steps": drift}
    if prec == gbmd.PREC_MIXED:
        line["accuracy_vs_fp64"] = force_error(dev, r["atoms"], st, half)
    if not args.no_variants:
        var = {}
        for pname, p in (("fp64", gbmd.PREC_FP64), ("mixed", gbmd.PREC_MIXED)):
            for lname, h in (("full", 0), ("half", 1)):
                if p == prec and h == half:
                    var[f"{pname}_{lname}"] = value
                    continue
                vsteps = min(args.steps, 40)
                rv = run_device(dev, st, p, h, vsteps, 3, profile=False)
                var[f"{pname}_{lname}"] = n * vsteps / (rv["ms"] * 1e-3)
        line["variants_atom_steps_per_s"] = var
        line["mixed_over_fp64"] = var["mixed_full"] / var["fp64_full"]
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
