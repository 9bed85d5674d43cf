"""Serving engine binding (include/gbmd_serve.h) and the job-stream driver.

:class:`Engine` wraps the C engine: jobs (an initial state plus a
:class:`JobSpec`) are submitted at any time, :meth:`Engine.step` admits what
fits and advances every running job by one chunk of timesteps, finished jobs
hand back their final state and thermo rows.

:func:`make_stream` generates the seeded serving workload (independent
periodic FCC boxes, LJ or NNP, uneven sizes and step counts) and
:func:`run_stream` plays it against an engine: closed (everything submitted at
t = 0, the batched capacity) or open with Poisson arrivals, reporting per-job
latency percentiles and aggregate atom-steps/s.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import gbmd, inputs

JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class JobSpecC(C.Structure):
    _fields_ = [("force_type", C.c_int), ("precision", C.c_int),
                ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("boltz", C.c_double), ("mvv2e", C.c_double), ("dt", C.c_double),
                ("mass", C.c_double),
                ("lj_epsilon", C.c_double), ("lj_sigma", C.c_double), ("lj_cut", C.c_double),
                ("nnp_dir", C.c_char_p), ("nnp_cflength", C.c_double),
                ("nnp_cfenergy", C.c_double),
                ("md", gbmd.MDParams), ("nsteps", C.c_int64)]


class EngineStatsC(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("admitted", C.c_int64), ("finished", C.c_int64),
                ("failed", C.c_int64), ("running", C.c_int64), ("queued", C.c_int64),
                ("budget_bytes", C.c_uint64), ("used_bytes", C.c_uint64),
                ("peak_used_bytes", C.c_uint64), ("atom_steps", C.c_int64),
                ("chunks", C.c_int64), ("launches", C.c_int64), ("busy_seconds", C.c_double),
                ("atom_steps_run", C.c_int64), ("cancelled", C.c_int64),
                ("admit_seconds", C.c_double), ("wait_seconds", C.c_double),
                ("retire_seconds", C.c_double), ("batched_rebuilds", C.c_int64)]


def declare(L: C.CDLL) -> None:
    """ctypes signatures of the serving entry points."""
    vp = C.c_void_p
    i64 = C.c_int64
    D = C.POINTER(C.c_double)
    I = C.POINTER(C.c_int)
    L.gbmd_engine_create.argtypes = [C.POINTER(vp), C.c_int, C.c_uint64, C.c_int, C.c_int]
    L.gbmd_engine_destroy.argtypes = [vp]
    L.gbmd_engine_destroy.restype = None
    L.gbmd_engine_last_error.argtypes = [vp]
    L.gbmd_engine_last_error.restype = C.c_char_p
    L.gbmd_engine_now.argtypes = [vp]
    L.gbmd_engine_now.restype = C.c_double
    L.gbmd_job_submit.argtypes = [vp, C.POINTER(JobSpecC), i64, vp, vp, vp, vp, C.c_double,
                                  C.POINTER(i64)]
    L.gbmd_engine_step.argtypes = [vp, I, I, I]
    L.gbmd_job_poll.argtypes = [vp, i64, I, I, D]
    L.gbmd_job_error.argtypes = [vp, i64]
    L.gbmd_job_error.restype = C.c_char_p
    L.gbmd_job_result.argtypes = [vp, i64, C.POINTER(i64), vp, vp, vp, vp, vp, vp, C.c_int, I]
    L.gbmd_job_release.argtypes = [vp, i64]
    L.gbmd_job_cancel.argtypes = [vp, i64]
    L.gbmd_engine_get_stats.argtypes = [vp, C.POINTER(EngineStatsC)]


@dataclass
class JobSpec:
    """One MD job (a CbnMD run): force, precision, box, units, MD cadence."""
    force: int                     # gbmd.FORCE_LJ / gbmd.FORCE_NNP
    nsteps: int
    lo: tuple
    hi: tuple
    boltz: float
    mvv2e: float
    dt: float
    mass: float
    force_cut: float
    skin: float
    precision: int = gbmd.PREC_MIXED
    half: int = 0
    rebuild_every: int = 20
    thermo_every: int = 10
    lj: tuple = (1.0, 1.0, 2.5)    # epsilon, sigma, cutoff
    nnp_dir: str | None = None

    def to_c(self) -> JobSpecC:
        s = JobSpecC()
        s.force_type = self.force
        s.precision = self.precision
        s.lo = (C.c_double * 3)(*self.lo)
        s.hi = (C.c_double * 3)(*self.hi)
        s.boltz, s.mvv2e, s.dt, s.mass = self.boltz, self.mvv2e, self.dt, self.mass
        s.lj_epsilon, s.lj_sigma, s.lj_cut = self.lj
        s.nnp_dir = self.nnp_dir.encode() if self.nnp_dir else None
        s.nnp_cflength = 1.0
        s.nnp_cfenergy = 1.0
        s.md = gbmd.MDParams(self.force_cut, self.skin, self.half, self.rebuild_every,
                             self.thermo_every, 50)
        s.nsteps = self.nsteps
        return s


@dataclass
class JobResult:
    x: np.ndarray
    v: np.ndarray
    f: np.ndarray
    id: np.ndarray
    thermo: np.ndarray
    arrival: float
    admitted: float
    finished: float


class Engine:
    """Continuous-batching MD engine on one GPU."""

    def __init__(self, device: int = 0, budget_bytes: float = 150e9, max_running: int = 256,
                 chunk: int = 10):
        self.lib = gbmd.load_library()
        self.h = C.c_void_p()
        rc = self.lib.gbmd_engine_create(C.byref(self.h), device, int(budget_bytes),
                                         max_running, chunk)
        if rc:
            raise gbmd.GbmdError(rc, "engine creation failed")

    def _chk(self, rc):
        if rc:
            raise gbmd.GbmdError(rc, self.lib.gbmd_engine_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.gbmd_engine_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def now(self) -> float:
        return self.lib.gbmd_engine_now(self.h)

    def submit(self, spec: JobSpec, st: "inputs.State", arrival: float = -1.0) -> int:
        x = np.ascontiguousarray(st.x, dtype=np.float64)
        v = np.ascontiguousarray(st.v, dtype=np.float64)
        t = np.ascontiguousarray(st.type, dtype=np.int32)
        i = np.ascontiguousarray(st.id, dtype=np.int32)
        cs = spec.to_c()
        jid = C.c_int64()
        self._chk(self.lib.gbmd_job_submit(self.h, C.byref(cs), len(x), x.ctypes.data,
                                           v.ctypes.data, t.ctypes.data, i.ctypes.data,
                                           float(arrival), C.byref(jid)))
        return jid.value

    def step(self):
        r, q, f = C.c_int(), C.c_int(), C.c_int()
        self._chk(self.lib.gbmd_engine_step(self.h, C.byref(r), C.byref(q), C.byref(f)))
        return r.value, q.value, f.value

    def poll(self, jid: int):
        s, e = C.c_int(), C.c_int()
        t = np.zeros(3)
        self._chk(self.lib.gbmd_job_poll(self.h, jid, C.byref(s), C.byref(e), gbmd._dp(t)))
        return s.value, e.value, t

    def error(self, jid: int) -> str:
        return self.lib.gbmd_job_error(self.h, jid).decode()

    def result(self, jid: int) -> JobResult:
        n = C.c_int64()
        nr = C.c_int()
        self._chk(self.lib.gbmd_job_result(self.h, jid, C.byref(n), None, None, None, None, None,
                                           None, 0, C.byref(nr)))
        x = np.zeros((n.value, 3))
        v = np.zeros((n.value, 3))
        f = np.zeros((n.value, 3))
        ids = np.zeros(n.value, np.int32)
        rows = np.zeros((max(nr.value, 1), 4))
        self._chk(self.lib.gbmd_job_result(self.h, jid, C.byref(n), x.ctypes.data,
                                           v.ctypes.data, f.ctypes.data, None, ids.ctypes.data,
                                           rows.ctypes.data, nr.value, C.byref(nr)))
        _, _, t = self.poll(jid)
        return JobResult(x, v, f, ids, rows[:nr.value], t[0], t[1], t[2])

    def release(self, jid: int):
        self._chk(self.lib.gbmd_job_release(self.h, jid))

    def cancel(self, jid: int):
        """Cancel a queued or running job (it ends FAILED, error CANCELLED)."""
        self._chk(self.lib.gbmd_job_cancel(self.h, jid))

    def stats(self) -> dict:
        s = EngineStatsC()
        self._chk(self.lib.gbmd_engine_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in EngineStatsC._fields_}

    def drain(self, sleep: float = 0.0):
        """Step until no job is queued or running."""
        while True:
            r, q, _ = self.step()
            if r == 0 and q == 0:
                return
            if sleep:
                time.sleep(sleep)


# ---------------------------------------------------------------------------
# Serving workload
LJ_CUT, LJ_SKIN = 2.5, 0.3
NNP_CUT, NNP_SKIN = 6.0, 1.0


@dataclass
class StreamJob:
    kind: str            # "lj" or "nnp"
    cells: int           # FCC cells per edge (atoms = 4 cells^3)
    nsteps: int
    rho: float = 0.0     # LJ density
    T: float = 0.0       # LJ temperature (NNP: 300 K)
    seed: int = 0
    gap: float = 0.0     # unit-rate exponential inter-arrival gap

    @property
    def atoms(self) -> int:
        return 4 * self.cells ** 3


def make_stream(njobs: int, seed: int = 20261204, nmin: int = 500, nmax: int = 50000,
                lj_frac: float = 0.7, smin: int = 100, smax: int = 1000) -> list[StreamJob]:
    """Seeded serving workload: atom counts log-uniform in [nmin, nmax]
    rounded to whole FCC cells (4 m^3 atoms), LJ with density U[0.7, 0.9] and
    T U[0.8, 1.5] or NNP at 300 K, steps U[smin, smax], unit-rate Poisson
    gaps (scaled to the arrival rate by the caller)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(njobs):
        n = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        m = max(2, int(round((n / 4.0) ** (1.0 / 3.0))))
        kind = "lj" if rng.uniform() < lj_frac else "nnp"
        steps = int(rng.integers(smin, smax + 1))
        rho = float(rng.uniform(0.7, 0.9))
        T = float(rng.uniform(0.8, 1.5))
        out.append(StreamJob(kind, m, steps, rho if kind == "lj" else 0.0,
                             T if kind == "lj" else 300.0, int(rng.integers(1 << 30)),
                             float(rng.exponential(1.0))))
    return out


def job_state(j: StreamJob) -> "inputs.State":
    if j.kind == "lj":
        return inputs.lj_fcc(j.cells, rho=j.rho, T=j.T, seed=j.seed)
    return inputs.nnp_fcc(j.cells, seed=j.seed)


def job_spec(j: StreamJob, st: "inputs.State", nnp_dir: str | None,
             precision: int = gbmd.PREC_MIXED) -> JobSpec:
    if j.kind == "lj":
        return JobSpec(gbmd.FORCE_LJ, j.nsteps, tuple(st.lo), tuple(st.hi), st.boltz, st.mvv2e,
                       st.dt, float(st.mass[0]), LJ_CUT, LJ_SKIN, precision=precision,
                       lj=(1.0, 1.0, LJ_CUT))
    return JobSpec(gbmd.FORCE_NNP, j.nsteps, tuple(st.lo), tuple(st.hi), st.boltz, st.mvv2e,
                   st.dt, float(st.mass[0]), NNP_CUT, NNP_SKIN, precision=precision,
                   nnp_dir=nnp_dir)


@dataclass
class StreamReport:
    jobs: int
    atom_steps: int
    makespan_s: float
    atom_steps_per_s: float
    latency_p50_s: float
    latency_p99_s: float
    latency_mean_s: float
    failed: int
    stats: dict = field(default_factory=dict)
    latencies: list = field(default_factory=list)
    steady_atom_steps_per_s: float = 0.0   # over the middle 80% of the arrivals
    errors: dict = field(default_factory=dict)  # failure message -> count
    # work of the jobs that arrived in the same window, per second of it
    window_offered_atom_steps_per_s: float = 0.0


def run_stream(engine: Engine, jobs: list[StreamJob], nnp_dir: str | None, rate: float | None,
               precision: int = gbmd.PREC_MIXED, keep_results: bool = False):
    """Play the stream: rate None submits every job at t = 0 (closed batch);
    otherwise job k arrives at sum of gaps / rate (jobs per second).
    Returns (StreamReport, {index: JobResult} if keep_results)."""
    states = [job_state(j) for j in jobs]
    specs = [job_spec(j, s, nnp_dir, precision) for j, s in zip(jobs, states)]
    arr = np.zeros(len(jobs))
    if rate:
        arr = np.cumsum([j.gap for j in jobs]) / rate
        arr -= arr[0]
    t0 = engine.now()
    ids = [None] * len(jobs)
    nxt = 0
    live = 0
    trace = []  # (time since t0, atom-steps run so far)
    while nxt < len(jobs) or live:
        now = engine.now() - t0
        while nxt < len(jobs) and arr[nxt] <= now:
            ids[nxt] = engine.submit(specs[nxt], states[nxt], t0 + arr[nxt])
            nxt += 1
            live += 1
        if live:
            _, _, fin = engine.step()
            live -= fin
            trace.append((engine.now() - t0, engine.stats()["atom_steps_run"]))
        elif nxt < len(jobs):
            time.sleep(max(0.0, min(0.01, arr[nxt] - (engine.now() - t0))))
    steady = offered = 0.0
    if rate and len(trace) > 2:
        ta, tb = np.percentile(arr, 10), np.percentile(arr, 90)
        tt = np.array([p[0] for p in trace])
        ww = np.array([p[1] for p in trace], dtype=float)
        ia, ib = np.searchsorted(tt, ta), np.searchsorted(tt, tb)
        if ib > ia:
            steady = (ww[ib] - ww[ia]) / (tt[ib] - tt[ia]) if ib < len(tt) else 0.0
        inwin = (arr >= ta) & (arr < tb)
        if tb > ta:
            offered = float(sum(j.atoms * j.nsteps for j, w in zip(jobs, inwin) if w)) / (tb - ta)
    lat, results, failed, errors = [], {}, 0, {}
    first, last, work = math.inf, 0.0, 0
    for k, jid in enumerate(ids):
        state, err, t = engine.poll(jid)
        if state != JOB_DONE:
            failed += 1
            msg = f"{jobs[k].kind}: {engine.error(jid)[:100]}"
            errors[msg] = errors.get(msg, 0) + 1
            continue
        lat.append(t[2] - t[0])
        first = min(first, t[0])
        last = max(last, t[2])
        work += jobs[k].atoms * jobs[k].nsteps
        if keep_results:
            results[k] = engine.result(jid)
        engine.release(jid)
    span = last - first if last > first else float("nan")
    lat = np.array(lat)
    rep = StreamReport(len(jobs), work, span, work / span if span == span else 0.0,
                       float(np.percentile(lat, 50)) if len(lat) else float("nan"),
                       float(np.percentile(lat, 99)) if len(lat) else float("nan"),
                       float(lat.mean()) if len(lat) else float("nan"), failed,
                       engine.stats(), lat.tolist(), steady, errors, offered)
    return rep, results
