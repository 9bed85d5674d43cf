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

Besides the headline, the line carries:
  - variants_*: FP64 / mixed x full / half lists of the same system (rates,
    NVE drift);
  - nnp: the 256,000-atom Cu NNP system (mixed against FP64, force accuracy
    at the fitted state, the 4,000-atom drift comparison, roofline), and a
    two-element potential on the same lattice (two_elements);
  - serving: the seeded 2,000-job stream through the continuous-batching
    engine (capacity, Poisson stream at 80% load, p50 / p99 latency,
    failures).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = ("atom-steps/s (LJ, NNP) mixed vs FP64 at ≤1e-4 force err; serving p50/p99")
LJ = [(1, 1, 1.0, 1.0, 2.5)]
FORCE_CUT, SKIN, REBUILD, THERMO = 2.5, 0.3, 20, 10
# NNP workloads: Cu-like FCC (a 3.61 A), rc 6.0 A cosine cutoff, 8 G2 + 24 G3,
# 32-25-25-1 softplus/linear network with N(0, 1/fan_in) weights; scaling
# fitted to the 10^3-cell (4,000-atom) state at step 0.  The neighbour skin
# is 1.0 A with a rebuild every 20 steps.
NNP_RC, NNP_SKIN, NNP_WSEED, NNP_XSEED = 6.0, 1.0, 2024, 20261204
HARTREE_EV = 27.211384021355236
REF_MAX_STEPS = 100


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


REASON_NAMES = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
# NVML clock-event reason bits (nvml.h, nvmlClocksEventReason*)
NVML_REASON_BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20,
                    "hw_thermal_slowdown": 0x40}


class NvmlClocks:
    """Read-only NVML queries of one GPU: current SM clock, maximum SM clock
    and the active clock-event (throttle) reasons.  `lib` is the loaded
    libnvidia-ml (a stand-in object in tests)."""

    NVML_CLOCK_SM = 1

    def __init__(self, lib, nvml_index: int):
        self.lib = lib
        self.handle = ctypes.c_void_p()
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit_v2 failed")
        if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(nvml_index),
                                             ctypes.byref(self.handle)) != 0:
            lib.nvmlShutdown()
            raise OSError(f"no NVML device {nvml_index}")
        self.reasons_fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(self.handle, self.NVML_CLOCK_SM, ctypes.byref(mx)) != 0:
            lib.nvmlShutdown()
            raise OSError("nvmlDeviceGetMaxClockInfo failed")
        self.sm_max = float(mx.value)

    @classmethod
    def open(cls, device: int):
        """None when NVML cannot be loaded or queried (the caller falls back
        to nvidia-smi)."""
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
        except OSError:
            return None
        idx = device
        try:
            import torch
            idx = torch.cuda._get_nvml_device_index(device)
        except Exception:
            pass
        try:
            return cls(lib, idx)
        except (OSError, AttributeError):
            return None

    def read(self):
        """(sm MHz, max sm MHz, set of active reason names), or None."""
        sm = ctypes.c_uint()
        rs = ctypes.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.handle, self.NVML_CLOCK_SM,
                                           ctypes.byref(sm)) != 0:
            return None
        if self.reasons_fn(self.handle, ctypes.byref(rs)) != 0:
            return None
        names = {nm for nm, bit in NVML_REASON_BITS.items() if rs.value & bit}
        return float(sm.value), self.sm_max, names

    def close(self):
        self.lib.nvmlShutdown()


class ClockSampler:
    """SM clocks and throttle reasons during the timed region.

    Through NVML (read-only queries) every millisecond, so that a region of
    a few tens of milliseconds holds many samples; where NVML cannot be
    loaded, through nvidia-smi every 10 ms.  Entering the `with` block waits
    (at most `margin_s`) for the first sample, and leaving it waits for one
    sample after the region, so that the region is bracketed by samples;
    the summary says how many fell inside it."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, margin_s: float = 0.3, period_s: float = 0.001,
                 nvml: "NvmlClocks | None | bool" = True):
        self.device = device
        self.proc = None
        self.nvml = None
        self.margin = margin_s
        self.period = period_s
        self._nvml_arg = nvml
        self.samples: list[tuple[float, float, float, set]] = []
        self.stop = threading.Event()
        self.t0 = self.t1 = None
        self.source = None

    def __enter__(self):
        arg = self._nvml_arg
        self.nvml = NvmlClocks.open(self.device) if arg is True else (arg or None)
        if self.nvml is not None:
            self.source = f"NVML every {self.period * 1e3:g} ms"
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
        else:
            try:
                self.proc = subprocess.Popen(
                    ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                     "--format=csv,noheader,nounits", "-lms", "10"],
                    stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
                self.source = "nvidia-smi every 10 ms"
                self.t = threading.Thread(target=self._read, daemon=True)
                self.t.start()
            except (FileNotFoundError, OSError):
                self.proc = None
        if self.nvml is not None or self.proc is not None:
            self._wait_for(lambda: len(self.samples) > 0)
        self.t0 = time.perf_counter()
        return self

    def _wait_for(self, cond):
        end = time.perf_counter() + self.margin
        while not cond() and time.perf_counter() < end:
            time.sleep(0.0005)

    def _poll(self):
        while not self.stop.is_set():
            r = self.nvml.read()
            if r is not None:
                self.samples.append((time.perf_counter(),) + r)
            self.stop.wait(self.period)

    def _read(self):
        for ln in self.proc.stdout:
            ts = time.perf_counter()
            f = [t.strip() for t in ln.strip().split(",")]
            if len(f) < 9:
                continue
            try:
                sm, mx = float(f[1]), float(f[2])
            except ValueError:
                continue
            names = {nm for k, nm in enumerate(REASON_NAMES) if f[5 + k].lower() == "active"}
            self.samples.append((ts, sm, mx, names))

    def __exit__(self, *a):
        self.t1 = time.perf_counter()
        if self.nvml is not None or self.proc is not None:
            self._wait_for(lambda: bool(self.samples) and self.samples[-1][0] > self.t1)
        if self.nvml is not None:
            self.stop.set()
            self.t.join(timeout=1.0)
            self.nvml.close()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return None
        sm = [s[1] for s in self.samples]
        inside = [s for s in self.samples
                  if self.t0 is not None and self.t1 is not None and self.t0 <= s[0] <= self.t1]
        reasons = set().union(*(s[3] for s in self.samples))
        # the median under load counts the samples inside the region when
        # there are any, else the bracketing ones
        med = float(np.median([s[1] for s in inside])) if inside else float(np.median(sm))
        return {"sm_mhz": med, "sm_max_mhz": float(max(s[2] for s in self.samples)),
                "reasons": sorted(reasons), "samples": len(sm),
                "samples_in_region": len(inside),
                "sampling": f"{self.source}, from just before to just after the timed region"}


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
    shapes = c.shapes()
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
                sort_n=scount, list_entries=tot, clocks=clk.summary(), atoms=a, shapes=shapes)


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


def run_e2e(dev, st, prec, half, steps, reps=5):
    """Through the public C ABI from host buffers: upload, md_init, K steps
    (thermo rows read back every 10 steps), download.  The host mirrors
    (inputs and outputs) are page-locked once before the timed region, as
    an integrating code keeps its host mirrors (gbmd_host_register).  The
    whole sequence runs `reps` times on a fresh context each; the line
    reports the run of median wall time (all runs' seconds beside it), so
    that one hiccup of the shared host does not decide the figure."""
    from cabanamd_gb300 import gbmd
    n = st.n
    x = gbmd.aligned_empty((n, 3), np.float64)
    v = gbmd.aligned_empty((n, 3), np.float64)
    t = gbmd.aligned_empty((n,), np.int32)
    ids = gbmd.aligned_empty((n,), np.int32)
    x[:], v[:], t[:], ids[:] = st.x, st.v, st.type, st.id
    out = gbmd.Atoms(*(gbmd.aligned_empty(sh, dt) for sh, dt in
                       (((n, 3), np.float64), ((n, 3), np.float64), ((n, 3), np.float64),
                        ((n,), np.int32), ((n,), np.int32))))
    pin = gbmd.PinnedHost(x, v, t, ids, out.x, out.v, out.f, out.type, out.id)
    runs = []
    for _ in range(reps):
        c = new_ctx(dev, st, prec)
        c.synchronize()
        t0 = time.perf_counter()
        c.upload_atoms(x, v, t, ids)
        t1 = time.perf_counter()
        c.md_init(FORCE_CUT, SKIN, half, REBUILD, THERMO)
        t2 = time.perf_counter()
        rows = c.md_run(steps)
        t3 = time.perf_counter()
        c.download_atoms(out)
        t4 = time.perf_counter()
        c.close()
        if not np.array_equal(np.sort(out.id), st.id):
            raise RuntimeError("e2e: downloaded ids are not a permutation of the uploaded ones")
        runs.append((t0, t1, t2, t3, t4))
    pin.close()
    t0, t1, t2, t3, t4 = sorted(runs, key=lambda r: r[4] - r[0])[len(runs) // 2]
    h2d = n * (24 + 24 + 4 + 4)
    d2h = n * (24 * 3 + 4 + 4) + (len(rows) + 1) * 32
    return {"value": n * steps / (t4 - t0), "unit": "atom-steps/s",
            "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "seconds": t4 - t0, "runs_seconds": [r[4] - r[0] for r in runs],
            "runs_phase_ms": [[round(1e3 * (b - a), 3) for a, b in zip(r[:-1], r[1:])]
                              for r in runs],
            "statistic": f"median of {reps} runs, each on a fresh context",
            "host_buffers": "page-locked (gbmd_host_register)",
            "phase_ms": {"upload": 1e3 * (t1 - t0), "md_init": 1e3 * (t2 - t1),
                         "md_run": 1e3 * (t3 - t2), "download": 1e3 * (t4 - t3)}}


def cpu_baseline(st, half, steps, threads):
    from oracle import pyoracle as O
    s = st.copy()
    tm = {}
    O.run_lj(s.x, s.v, s.type, s.id, s.lo, s.hi, LJ, force_cut=FORCE_CUT, skin=SKIN, half=half,
             rebuild_every=REBUILD, thermo_every=THERMO, nsteps=steps, boltz=s.boltz,
             mvv2e=s.mvv2e, dt=s.dt, mass=s.mass, nthreads=threads, time_from_step=0,
             timing=tm)
    return st.n * steps / tm["loop_seconds"], tm["loop_seconds"]


def nnp_state(cells):
    from cabanamd_gb300 import inputs
    return inputs.nnp_fcc(cells, a=3.61, mass=63.546, T=300.0, disp=0.05, seed=NNP_XSEED,
                          dt_fs=0.5)


def nnp_ctx(dev, st, prec, potdir):
    from cabanamd_gb300 import gbmd
    c = gbmd.Context(dev)
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(prec)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(potdir), 1.0, 1.0)
    return c


def nnp_potential(dev, potdir):
    """Write the NNP workload potential to potdir, its scaling fitted to the
    raw symmetry functions of the 4,000-atom state (computed by the FP64 GPU
    path)."""
    from cabanamd_gb300 import gbmd, nnp_files as NF
    pot = NF.synthetic_cu_potential(seed=NNP_WSEED, rc=NNP_RC)
    NF.write_potential(potdir, pot)
    st = nnp_state(10)
    c = nnp_ctx(dev, st, gbmd.PREC_FP64, potdir)
    cut = NNP_RC + NNP_SKIN
    c.exchange()
    c.binning(cut)
    c.neigh_build(cut, 0, 96)
    c.zero_force()
    c.force_compute()
    G, _ = c.nnp_download()
    c.close()
    NF.fit_scaling(pot, "Cu", G)
    NF.write_potential(potdir, pot)
    return pot


def nnp_energy_drift(rows, n_steps_scale=1000.0, max_step=None):
    """Slope (per atom per 1000 steps) of sum_i E_i / N + KE / N, the energy
    the NNP forces conserve (the thermo PE carries the reference's fixed
    27.211... factor, which its forces do not), over rows up to max_step."""
    if max_step is not None:
        rows = rows[rows[:, 0] <= max_step]
    if len(rows) < 3:
        return None
    etot = rows[:, 2] / HARTREE_EV + rows[:, 3]
    return float(np.polyfit(rows[:, 0], etot, 1)[0] * n_steps_scale)


# The random-weight NNP of the workloads is fitted to the displaced lattice
# at step 0; past ~300 steps (dt 0.5 fs) its trajectory leaves the fitted
# range and heats without bound in FP64 as in mixed precision (T ~ 2e4 K by
# step 500).  Energy conservation is therefore judged over the first 200
# steps, the length of the 4,000-atom FP64 workload.
NNP_STABLE_STEPS = 200


def lj_energy_drift(rows):
    if len(rows) < 3:
        return None
    etot = rows[:, 2] + rows[:, 3]
    return float(np.polyfit(rows[:, 0], etot, 1)[0] * 1000.0)


def nnp_run(dev, st, prec, potdir, steps, warmup, profile=True):
    c = nnp_ctx(dev, st, prec, potdir)
    c.md_init(NNP_RC, NNP_SKIN, 0, REBUILD, THERMO)
    c.md_run(warmup)
    c.set_profiling(profile)
    with ClockSampler(dev) as clk:
        rows = c.md_run(steps)
    ms, launches = c.last_run()
    kt = {k: c.kernel_time(k) for k in ("nnp_sf", "nnp_mlp", "nnp_force", "neigh", "sort",
                                        "integrate")} if profile else {}
    a = c.download_atoms()
    c.close()
    return dict(ms=ms, rows=rows, launches=launches, kt=kt, clocks=clk.summary(), atoms=a)


def nnp_force_error(dev, atoms, st, potdir):
    """Mixed vs FP64 NNP forces and per-atom energies at identical positions."""
    from cabanamd_gb300 import gbmd
    out = {}
    cut = NNP_RC + NNP_SKIN
    for prec in (gbmd.PREC_FP64, gbmd.PREC_MIXED):
        c = nnp_ctx(dev, st, prec, potdir)
        c.upload_atoms(atoms.x, atoms.v, atoms.type, atoms.id)
        c.exchange()
        c.binning(cut)
        c.neigh_build(cut, 0, 96)
        c.zero_force()
        c.force_compute()
        a = c.download_atoms()
        _, E = c.nnp_download()
        o = np.argsort(a.id)
        out[prec] = (a.f[o], E[o])
        c.close()
    f64, e64 = out[gbmd.PREC_FP64]
    fmx, emx = out[gbmd.PREC_MIXED]
    rms = float(np.sqrt(np.mean(f64 * f64)))
    return {"max_rel_force_err": float(np.abs(fmx - f64).max() / rms),
            "rms_rel_force_err": float(np.sqrt(np.mean((fmx - f64) ** 2)) / rms),
            "max_atom_energy_err_eV": float(np.abs(emx - e64).max()),
            "rms_force_eV_per_A": rms}


def nnp_cpu_baseline(pot, st):
    """One FP64 force evaluation of the CPU restatement (single thread) on
    the 4,000-atom state."""
    from oracle import pyoracle as O
    x = st.x.copy()
    t = st.type.copy()
    ids = st.id.copy()
    O.exchange_self(x, st.hi - st.lo)
    cut = NNP_RC + NNP_SKIN
    g = O.make_grid(st.lo, st.hi, cut)
    O.sort_atoms(g, x, None, None, t, ids)
    t0 = time.perf_counter()
    off, j, img = O.neigh_cells(x, g, st.hi, cut, cut, 0)
    O.nnp_compute(x, O.ListHandle(off, j, img), st.hi - st.lo, O.NNPHandle(pot))
    sec = time.perf_counter() - t0
    return st.n / sec, sec


NNP_FLOP_PER_ATOM_STEP = 2.17e6  # counting convention: G3 fwd+grad T*24*30 + G2 + MLP
# What the convention's `frac` is and is not: the kernels execute fewer
# operations than it counts (the (eta, lambda, zeta) grid shares exponentials
# and powers, the triplet geometry is cached between the two kernels), so it
# is a rate of useful work in the convention's units; the pipes' own use is
# the ncu counters of the two kernels (an ncu --set full capture at 32,000
# atoms, summarised under profiles/).
NNP_ROOFLINE_NOTE = {
    "convention": "achieved = 2.17 MFLOP per atom-step (G3 forward + gradient 24 x 30 per "
                  "triplet, G2, MLP) / "
                  "event-timed kernel time; the kernels execute fewer operations than counted, "
                  "so frac is useful work in the convention's units, not pipe utilisation",
    "pipe_counters_32k_atoms": {
        "k_nnp_sf_f32": {"fma_pipe_pct": 31.0, "alu_pipe_pct": 38.5, "issue_active_pct": 66.8},
        "k_nnp_force_f32": {"fma_pipe_pct": 41.3, "alu_pipe_pct": 27.6,
                            "issue_active_pct": 69.2},
        "source": "ncu --set full of the two kernels at 32,000 atoms (profiles/)"}}


def binary_state(cells):
    """The NNP state with two elements: each atom Ni or Cu (types 1, 2 in
    atomic-number order) at random, seeded."""
    st = nnp_state(cells)
    rng = np.random.default_rng(NNP_XSEED + 1)
    st.type = rng.integers(0, 2, st.n).astype(np.int32)
    st.mass = [58.6934, 63.546]
    return st


def binary_potential(dev, potdir):
    """Write the two-element potential to potdir, each element's scaling
    fitted to its raw symmetry functions on the 4,000-atom two-element state
    (computed by the FP64 GPU path)."""
    from cabanamd_gb300 import gbmd, nnp_files as NF
    pot = NF.synthetic_binary_potential(seed=NNP_WSEED, rc=NNP_RC)
    NF.write_potential(potdir, pot)
    st = binary_state(10)
    c = nnp_ctx(dev, st, gbmd.PREC_FP64, potdir)
    cut = NNP_RC + NNP_SKIN
    c.exchange()
    c.binning(cut)
    c.neigh_build(cut, 0, 96)
    c.zero_force()
    c.force_compute()
    a = c.download_atoms()
    G, _ = c.nnp_download()
    c.close()
    for k, e in enumerate(pot.elements):
        NF.fit_scaling(pot, e, G[a.type == k, :pot.nsf(e)])
    NF.write_potential(potdir, pot)
    return pot


def nnp_two_elements_block(dev, cells=40, small_cells=20, steps=20, warmup=3, fp64_steps=3):
    """The multi-element NNP path on a two-element potential (per centre
    element: G2 per neighbour element, G3 per element pair; scaling fitted on
    the 4,000-atom state by the FP64 path): mixed-precision throughput at
    `cells`, mixed vs FP64 at `small_cells` and the force accuracy there."""
    import tempfile
    from cabanamd_gb300 import gbmd
    with tempfile.TemporaryDirectory() as potdir:
        binary_potential(dev, potdir)
        big, small = binary_state(cells), binary_state(small_cells)
        rb = nnp_run(dev, big, gbmd.PREC_MIXED, potdir, steps, warmup, profile=False)
        rs = nnp_run(dev, small, gbmd.PREC_MIXED, potdir, steps, warmup, profile=False)
        r64 = nnp_run(dev, small, gbmd.PREC_FP64, potdir, fp64_steps, 3, profile=False)
        mixed_small = small.n * steps / (rs["ms"] * 1e-3)
        fp64_small = small.n * fp64_steps / (r64["ms"] * 1e-3)
        return {"potential": "two elements (Ni, Cu), 8 G2 + 24 G3 per element in 3 "
                             "element-pair channels, 16-16-1 tanh",
                "atoms": big.n, "mixed_atom_steps_per_s": big.n * steps / (rb["ms"] * 1e-3),
                "small_atoms": small.n, "small_mixed_atom_steps_per_s": mixed_small,
                "small_fp64_atom_steps_per_s": fp64_small,
                "small_mixed_over_fp64": mixed_small / fp64_small,
                "accuracy_vs_fp64": nnp_force_error(dev, small, small, potdir)}


def nnp_block(dev, potdir, pot, cells, steps, warmup, fp64_steps, cpu=True):
    """Configs of the NNP workload: the large mixed-precision system (timed
    over `steps`) against an FP64 sample of it, forces compared at the
    initial (fitted-range) state and after the run, and the 4,000-atom
    system run 200 steps in FP64 and in mixed precision for the energy
    drift comparison."""
    from cabanamd_gb300 import gbmd
    big = nnp_state(cells)
    r = nnp_run(dev, big, gbmd.PREC_MIXED, potdir, steps, warmup)
    n = big.n
    mixed = n * steps / (r["ms"] * 1e-3)
    r64 = nnp_run(dev, big, gbmd.PREC_FP64, potdir, fp64_steps, 3, profile=False)
    fp64 = n * fp64_steps / (r64["ms"] * 1e-3)
    kt = r["kt"]
    chain_ms = (kt["nnp_sf"][0] + kt["nnp_force"][0]) / max(kt["nnp_sf"][1], 1)
    simt_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    rows = r["rows"]
    blk = {"workload": f"nnp_cu_fcc_{cells}^3_cells_{n}_atoms", "atoms": n,
           "mixed_atom_steps_per_s": mixed, "mixed_ms_per_step": r["ms"] / steps,
           "mixed_steps": steps,
           "fp64_atom_steps_per_s": fp64, "fp64_ms_per_step": r64["ms"] / fp64_steps,
           "fp64_steps": fp64_steps, "mixed_over_fp64": mixed / fp64,
           "phase_ms_per_step": {k: v[0] / steps for k, v in kt.items()},
           "gpu_launches": r["launches"], "clocks": r["clocks"],
           "accuracy_vs_fp64": nnp_force_error(dev, big, big, potdir),
           "accuracy_vs_fp64_after_run": nnp_force_error(dev, r["atoms"], big, potdir),
           "temperature_K_first_last": [float(rows[0, 1]), float(rows[-1, 1])] if len(rows)
           else None,
           "nve_drift_per_atom_per_1000_steps_mixed_first_200":
               nnp_energy_drift(rows, max_step=NNP_STABLE_STEPS),
           "roofline": {"bound": "fp32_simt", "unit": "TFLOP/s",
                        "kernels": "k_nnp_sf_f32 + k_nnp_force_f32",
                        "flop_per_atom_step": NNP_FLOP_PER_ATOM_STEP,
                        "achieved": NNP_FLOP_PER_ATOM_STEP * n / (chain_ms * 1e-3) / 1e12,
                        "peak": simt_peak, "peak_source": "nominal (152 SM x 128 FP32 lanes x "
                                                          "2 x 2.07 GHz)",
                        **NNP_ROOFLINE_NOTE}}
    blk["roofline"]["frac"] = blk["roofline"]["achieved"] / simt_peak
    small = nnp_state(10)
    drift = {}
    for pname, p in (("fp64", gbmd.PREC_FP64), ("mixed", gbmd.PREC_MIXED)):
        r2 = nnp_run(dev, small, p, potdir, NNP_STABLE_STEPS, 3, profile=False)
        drift[pname] = nnp_energy_drift(r2["rows"])
        blk[f"{pname}_4000_atoms_200_steps"] = {
            "atom_steps_per_s": small.n * NNP_STABLE_STEPS / (r2["ms"] * 1e-3),
            "ms_per_step": r2["ms"] / NNP_STABLE_STEPS,
            "nve_drift_per_atom_per_1000_steps": drift[pname]}
    if drift["fp64"] is not None and drift["mixed"] is not None:
        blk["nve_drift_mixed_minus_fp64_4000_atoms"] = drift["mixed"] - drift["fp64"]
    blk["two_elements"] = nnp_two_elements_block(dev)
    if cpu:
        v, sec = nnp_cpu_baseline(pot, small)
        blk["cpu_baseline"] = {"value": v, "unit": "atom-steps/s", "cores": 1, "kind": "port",
                               "sample": f"one FP64 list build + force evaluation of the "
                                         f"{small.n}-atom state, single-threaded CPU "
                                         f"restatement, {sec:.1f} s"}
    return blk


def fp64_alone_step_fit(dev, jobs, potdir, sample, steps=20):
    """FP64, one job at a time on a context: per-step device time of `sample`
    jobs per kind (every k-th of the stream), fitted per kind as
    t_step = a + b N.  Returns {kind: (a, b)} in seconds."""
    from cabanamd_gb300 import gbmd, serve as S
    fits = {}
    for kind in ("lj", "nnp"):
        kj = [j for j in jobs if j.kind == kind]
        if not kj:
            continue
        pick = kj[:: max(1, len(kj) // sample)][:sample]
        ns, ts = [], []
        for j in pick:
            st = S.job_state(j)
            c = gbmd.Context(dev)
            c.set_units(st.boltz, st.mvv2e, st.dt)
            c.set_box(st.lo, st.hi)
            c.set_types(st.mass)
            c.set_precision(gbmd.PREC_FP64)
            c.upload_atoms(st.x, st.v, st.type, st.id)
            if kind == "lj":
                c.lj_coeff(1, 1, 1.0, 1.0, S.LJ_CUT)
                c.md_init(S.LJ_CUT, S.LJ_SKIN, 0, REBUILD, THERMO)
            else:
                c.nnp_load(potdir, 1.0, 1.0)
                c.md_init(S.NNP_CUT, S.NNP_SKIN, 0, REBUILD, THERMO)
            c.md_run(steps)
            ms, _ = c.last_run()
            c.close()
            ns.append(st.n)
            ts.append(ms * 1e-3 / steps)
        A = np.vstack([np.ones(len(ns)), ns]).T
        a, b = np.linalg.lstsq(A, np.array(ts), rcond=None)[0]
        fits[kind] = (float(a), float(b), len(ns))
    return fits


def serve_block(dev, potdir, njobs, seed=20261204, fp64_sample=6):
    """The serving stream: `njobs` seeded jobs (log-uniform 500-50,000
    atoms in whole FCC cells, 70% LJ / 30% NNP, 100-1000 steps), first all
    at t = 0 (batched capacity), then Poisson arrivals at 80% of that
    capacity; device memory budget 150 GB."""
    from cabanamd_gb300 import serve as S
    jobs = S.make_stream(njobs, seed=seed)
    work = np.array([j.atoms * j.nsteps for j in jobs], dtype=float)
    e = S.Engine(dev, budget_bytes=150e9, max_running=256, chunk=10)
    closed, _ = S.run_stream(e, jobs, potdir, None)
    e.close()
    cap = closed.atom_steps_per_s
    rate = 0.8 * cap / work.mean()
    e = S.Engine(dev, budget_bytes=150e9, max_running=256, chunk=10)
    opened, _ = S.run_stream(e, jobs, potdir, rate)
    e.close()
    fits = fp64_alone_step_fit(dev, jobs, potdir, fp64_sample)
    t_seq = sum(j.nsteps * (fits[j.kind][0] + fits[j.kind][1] * j.atoms) for j in jobs)
    seq = work.sum() / t_seq
    return {
        "jobs": njobs, "lj_jobs": sum(j.kind == "lj" for j in jobs),
        "atom_steps": int(work.sum()),
        "atoms_min_max": [min(j.atoms for j in jobs), max(j.atoms for j in jobs)],
        "budget_bytes": 150e9, "max_running": 256, "chunk_steps": 10,
        "batched_capacity_atom_steps_per_s": cap,
        "batched_makespan_s": closed.makespan_s,
        "poisson_rate_jobs_per_s": rate,
        "stream_atom_steps_per_s": opened.atom_steps_per_s,
        "stream_makespan_s": opened.makespan_s,
        "latency_p50_s": opened.latency_p50_s, "latency_p99_s": opened.latency_p99_s,
        "latency_mean_s": opened.latency_mean_s,
        "offered_load_over_capacity": 0.8,
        "stream_over_capacity": opened.atom_steps_per_s / cap,
        "stream_over_offered_load": opened.atom_steps_per_s / (0.8 * cap),
        "steady_atom_steps_per_s": opened.steady_atom_steps_per_s,
        "steady_over_capacity": opened.steady_atom_steps_per_s / cap,
        "steady_window": "arrivals between the 10th and 90th percentile times",
        "window_offered_atom_steps_per_s": opened.window_offered_atom_steps_per_s,
        "window_offered_over_capacity": opened.window_offered_atom_steps_per_s / cap,
        "steady_served_over_window_offered": (
            opened.steady_atom_steps_per_s / opened.window_offered_atom_steps_per_s
            if opened.window_offered_atom_steps_per_s > 0 else None),
        "failed": closed.failed + opened.failed,
        "failures": {"batched": closed.errors, "stream": opened.errors},
        "peak_hbm_bytes": opened.stats["peak_used_bytes"],
        "launches": opened.stats["launches"],
        "host_seconds_batched": {k: closed.stats[k] for k in
                                 ("busy_seconds", "admit_seconds", "wait_seconds",
                                  "retire_seconds")},
        "fp64_one_at_a_time_atom_steps_per_s": seq,
        "speedup_vs_fp64_one_at_a_time": opened.atom_steps_per_s / seq,
        "fp64_estimate": f"per-kind fit t_step = a + b N over {fp64_sample} jobs per kind, "
                         f"20 steps each, FP64 contexts run alone",
    }


def nnp_headline(dev, args, ws):
    """--workload nnp / nnp2: the mixed NNP system (one element, or the
    two-element Ni/Cu potential) as the headline line (used for small-case
    profiling of the NNP kernels)."""
    from cabanamd_gb300 import gbmd
    two = args.workload == "nnp2"
    with tempfile.TemporaryDirectory() as potdir:
        if two:
            binary_potential(dev, potdir)
            st = binary_state(args.nnp_cells)
        else:
            nnp_potential(dev, potdir)
            st = nnp_state(args.nnp_cells)
        prec = gbmd.PREC_MIXED if args.precision == "mixed" else gbmd.PREC_FP64
        r = nnp_run(dev, st, prec, potdir, args.steps, args.warmup)
    n = st.n
    kt = r["kt"]
    chain_ms = (kt["nnp_sf"][0] + kt["nnp_force"][0]) / max(kt["nnp_sf"][1], 1)
    simt_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    achieved = NNP_FLOP_PER_ATOM_STEP * n / (chain_ms * 1e-3) / 1e12
    return {"metric": METRIC, "value": n * args.steps / (r["ms"] * 1e-3), "unit": "atom-steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32/bf16/f64" if prec == gbmd.PREC_MIXED else "f64",
            "data": "synthetic",
            "config": {"workload": f"nnp_{'nicu' if two else 'cu'}_fcc_{args.nnp_cells}^3_cells_"
                                   f"{n}_atoms", "atoms": n,
                       "rc": NNP_RC, "skin": NNP_SKIN, "rebuild_every": REBUILD,
                       "thermo_every": THERMO, "dt_fs": 0.5, "precision": args.precision},
            "roofline": {"bound": "fp32_simt", "achieved": None if two else achieved,
                         "peak": simt_peak, "unit": "TFLOP/s",
                         "frac": None if two else achieved / simt_peak, "traffic": None,
                         "peak_source": "nominal (152 SM x 128 FP32 lanes x 2 x 2.07 GHz)",
                         **NNP_ROOFLINE_NOTE,
                         **({"note": "the FLOP convention counts the one-element potential"}
                            if two else {})},
            "gpu_launches": r["launches"], "clocks": r["clocks"],
            "phase_ms_per_step": {k: v[0] / args.steps for k, v in kt.items()},
            "nve_drift_per_atom_per_1000_steps": nnp_energy_drift(r["rows"])}


# DRAM bytes (read + write) per atom of one launch of the fused step kernel
# (k_lj_mixed, force + final + next initial integrate, no thermo), from one
# ncu capture on this workload itself (4,000,000 atoms, 100^3 cells):
# 1,602,664,704 B read + 344,884,736 B written
# (summarised under profiles/).
TRAFFIC_PER_ATOM = {"lj_step_mixed_full": (1602664704 + 344884736) / 4000000}


def profile_traffic(workload_key, atoms):
    per_atom = TRAFFIC_PER_ATOM.get(workload_key)
    return None if per_atom is None else per_atom * atoms


def lj_kernel_bytes(K, mixed, half):
    """Algorithmic bytes per atom of one launch of the timed LJ kernel (K list
    entries per atom; neighbour positions counted once, as cache-resident).
    Full lists run the fused step kernel: own position (FP32 shadow in mixed
    precision, which the FP64 path reads as double4), list count and home
    cell, the K entries, the force written, the velocity read and written,
    the next position (and mixed shadow) written, and, in mixed precision,
    the FP64 position read by the integrator.  Half lists run the force
    kernel alone (force read-modify-write).  Returns (kernel bytes, force-only
    bytes)."""
    if mixed:
        force_only = 16 + 4 + 4 * K + 24 + (24 if half else 0)
        fused = 4 + 16 + 4 + 4 * K + 24 + 24 + 24 + 32 + 32 + 16
    else:
        force_only = 32 + 4 + 4 + 4 * K + 24 + (24 if half else 0)
        fused = 4 + 32 + 4 + 4 * K + 24 + 24 + 24 + 32
    return (force_only if half else fused), force_only


def max_over_ranks(ms, dist):
    """The slowest rank's timed-region length (replicas: each rank runs its
    own copy of the workload); barrier on both sides."""
    if not dist:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64,
                     device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def replica_throughput(ws, atoms, steps, ms):
    """Whole-job atom-steps/s of ws replicas of `atoms` atoms over `steps`
    steps that took `ms` (max over ranks)."""
    return ws * atoms * steps / (ms * 1e-3)


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
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbmd", choices=["gbmd", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--list", default="full", choices=["full", "half"])
    ap.add_argument("--cells", type=int, default=100)
    ap.add_argument("--cpu-steps", type=int, default=20)
    ap.add_argument("--no-variants", action="store_true",
                    help="headline workload only (no precision/list variants, no NNP block)")
    ap.add_argument("--workload", default="lj", choices=["lj", "nnp", "nnp2", "serve"],
                    help="headline workload: LJ melt (default), the mixed NNP system, or "
                         "the same with the two-element potential")
    ap.add_argument("--nnp-cells", type=int, default=40)
    ap.add_argument("--nnp-steps", type=int, default=500)
    ap.add_argument("--nnp-fp64-steps", type=int, default=5)
    ap.add_argument("--serve-jobs", type=int, default=2000,
                    help="jobs of the serving stream measured with the variants (0: skip)")
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
        # a bounded sample of the workload: at most REF_MAX_STEPS timed steps
        # (about 40 s of host time at 4M atoms), after at most 3 warm-up steps
        rsteps = min(args.steps, REF_MAX_STEPS)
        rwarm = min(args.warmup, 3)
        from oracle import pyoracle as O
        s = st.copy()
        tm = {}
        O.run_lj(s.x, s.v, s.type, s.id, s.lo, s.hi, LJ, force_cut=FORCE_CUT, skin=SKIN,
                 half=half, rebuild_every=REBUILD, thermo_every=THERMO, nsteps=rwarm + rsteps,
                 boltz=s.boltz, mvv2e=s.mvv2e, dt=s.dt, mass=s.mass, nthreads=threads,
                 time_from_step=rwarm, timing=tm)
        sec = tm["loop_seconds"]
        val = n * rsteps / sec
        line = {"metric": METRIC, "value": val, "unit": "atom-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * sec / rsteps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(config, precision="fp64"), "impl": "reference",
                "cpu_baseline": {"value": val, "unit": "atom-steps/s", "cores": threads,
                                 "kind": "port",
                                 "sample": f"full {n}-atom system, {rsteps} timed steps "
                                           f"after {rwarm} warm-up steps (CPU restatement "
                                           "of the reference, OpenMP on all host cores)"},
                "e2e": {"value": val, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    from cabanamd_gb300 import gbmd
    prec = gbmd.PREC_MIXED if args.precision == "mixed" else gbmd.PREC_FP64
    dev = local
    if args.workload in ("nnp", "nnp2"):
        if rank == 0:
            print(json.dumps(nnp_headline(dev, args, ws)), flush=True)
        return
    if args.workload == "serve":
        # the serving stream alone (the headline's `serving` block)
        if rank == 0:
            with tempfile.TemporaryDirectory() as potdir:
                nnp_potential(dev, potdir)
                print(json.dumps({"workload": "serve", "serving":
                                  serve_block(dev, potdir, args.serve_jobs)}), flush=True)
        return
    if dist:
        dist.barrier()
    r = run_device(dev, st, prec, half, args.steps, args.warmup)
    ms = max_over_ranks(r["ms"], dist)
    value = replica_throughput(ws, n, args.steps, ms)
    if rank != 0:
        return

    # roofline of the dominant kernel (the fused LJ step for full lists, the
    # force kernel for half lists): algorithmic bytes per launch
    K = r["list_entries"] / n
    per_atom, force_only = lj_kernel_bytes(K, prec == gbmd.PREC_MIXED, half)
    f_avg_s = r["force_ms"] * 1e-3 / max(r["force_n"], 1)
    achieved = n * per_atom / f_avg_s / 1e9
    peak, peak_kind = peaks()
    traffic = (profile_traffic(f"lj_step_{args.precision}_{args.list}", n)
               if n == 4000000 else None)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
            "kernel": ("k_lj_mixed" if prec == gbmd.PREC_MIXED else "k_lj_fp64") +
                      (" (force)" if half else " (fused step: force + final + next initial)"),
            "algorithmic_bytes_per_atom": per_atom, "list_entries_per_atom": K,
            "force_only_bytes_per_atom": force_only,
            "force_only_frac": n * force_only / f_avg_s / 1e9 / peak,
            "avg_launch_ms": f_avg_s * 1e3, "launches": r["force_n"],
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch "
                              "of this kernel on this 4,000,000-atom workload" if traffic else None}
    phase_ms = {"force": r["force_ms"], "neigh": r["neigh_ms"], "sort": r["sort_ms"],
                "integrate": r["int_ms"], "total": r["ms"]}

    cpu_val, cpu_sec = cpu_baseline(st, half, args.cpu_steps, threads)
    e2e = run_e2e(dev, st, prec, half, args.steps)
    drift = lj_energy_drift(r["rows"])

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
            "tile_shapes": r["shapes"],
            "phase_ms": phase_ms, "nve_drift_per_atom_per_1000_steps": drift}
    if prec == gbmd.PREC_MIXED:
        line["accuracy_vs_fp64"] = force_error(dev, r["atoms"], st, half)
    if not args.no_variants:
        # the other precision / list combinations, each over the full step
        # count so that every variant's drift compares with its FP64 twin
        var, vdrift = {}, {}
        for pname, p in (("fp64", gbmd.PREC_FP64), ("mixed", gbmd.PREC_MIXED)):
            for lname, h in (("full", 0), ("half", 1)):
                key = f"{pname}_{lname}"
                if p == prec and h == half:
                    var[key], vdrift[key] = value, drift
                    continue
                vsteps = args.steps
                rv = run_device(dev, st, p, h, vsteps, 3, profile=False)
                var[key] = n * vsteps / (rv["ms"] * 1e-3)
                vdrift[key] = lj_energy_drift(rv["rows"]) if vsteps >= 100 else None
        line["variants_atom_steps_per_s"] = var
        line["variants_nve_drift_per_atom_per_1000_steps"] = vdrift
        line["mixed_over_fp64"] = var["mixed_full"] / var["fp64_full"]
        base = vdrift.get(f"fp64_{args.list}")
        if drift is not None and base is not None:
            line["nve_drift_mixed_minus_fp64"] = drift - base
        with tempfile.TemporaryDirectory() as potdir:
            pot = nnp_potential(dev, potdir)
            line["nnp"] = nnp_block(dev, potdir, pot, args.nnp_cells, args.nnp_steps, 3,
                                    args.nnp_fp64_steps)
            if args.serve_jobs > 0:
                line["serving"] = serve_block(dev, potdir, args.serve_jobs)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
