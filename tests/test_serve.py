"""Serving engine: continuous batching of independent MD jobs.

CPU tests cover the seeded workload generator and the no-device error; the
GPU tests check that a job's result does not depend on what ran beside it
(bit-identical alone, in a mix, and through the single-system md_run path),
that the FP64 engine path reproduces the oracle, and admission by slots and
device-memory budget.
"""
from pathlib import Path

import numpy as np
import pytest

from cabanamd_gb300 import gbmd, inputs
from cabanamd_gb300 import serve as S
from oracle import pyoracle as O

LJ = [(1, 1, 1.0, 1.0, 2.5)]


def test_stream_is_seeded_and_shaped():
    a = S.make_stream(400, seed=5)
    b = S.make_stream(400, seed=5)
    assert [(j.kind, j.cells, j.nsteps, j.seed) for j in a] == \
           [(j.kind, j.cells, j.nsteps, j.seed) for j in b]
    atoms = np.array([j.atoms for j in a])
    assert atoms.min() >= 4 * 5 ** 3 - 1 and atoms.max() <= 4 * 23 ** 3
    assert all(j.atoms == 4 * j.cells ** 3 for j in a)
    frac = np.mean([j.kind == "lj" for j in a])
    assert 0.6 < frac < 0.8
    steps = np.array([j.nsteps for j in a])
    assert steps.min() >= 100 and steps.max() <= 1000
    lj = [j for j in a if j.kind == "lj"]
    assert all(0.7 <= j.rho <= 0.9 and 0.8 <= j.T <= 1.5 for j in lj)
    # log-uniform sizes: about as many jobs below the geometric mean as above
    gm = np.sqrt(500 * 50000)
    assert 0.35 < np.mean(atoms < gm) < 0.65


def test_engine_without_device_is_an_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from cabanamd_gb300.build import build_lib
    build_lib()
    with pytest.raises(gbmd.GbmdError) as e:
        S.Engine(0)
    assert e.value.code == 7


# ---------------------------------------------------------------------------
def _lj_job(cells, nsteps, seed, rho=0.8442, T=1.44, prec=gbmd.PREC_MIXED):
    st = inputs.lj_fcc(cells, rho=rho, T=T, seed=seed)
    spec = S.JobSpec(gbmd.FORCE_LJ, nsteps, tuple(st.lo), tuple(st.hi), st.boltz, st.mvv2e,
                     st.dt, float(st.mass[0]), 2.5, 0.3, precision=prec, lj=(1.0, 1.0, 2.5))
    return spec, st


def _ctx_run(st, nsteps, prec):
    c = gbmd.Context(0)
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(prec)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    for (i, j, e, s, rc) in LJ:
        c.lj_coeff(i, j, e, s, rc)
    row0 = c.md_init(2.5, 0.3, 0, 20, 10)
    rows = c.md_run(nsteps)
    a = c.download_atoms().by_id()
    c.close()
    return np.vstack([row0[None, :], rows]), a


def _engine_run(jobs, chunk=10, budget=8e9, max_running=64, stagger=False):
    """jobs: list of (spec, state); with stagger, job k is submitted after
    k engine steps.  Returns the results in job order."""
    e = S.Engine(0, budget_bytes=budget, max_running=max_running, chunk=chunk)
    ids = []
    k = 0
    while k < len(jobs) or True:
        if k < len(jobs):
            if stagger:
                ids.append(e.submit(*jobs[k]))
                k += 1
            else:
                ids += [e.submit(*j) for j in jobs]
                k = len(jobs)
        r, q, _ = e.step()
        if k == len(jobs) and r == 0 and q == 0:
            break
    out = []
    for jid in ids:
        state, err, _ = e.poll(jid)
        assert state == S.JOB_DONE, e.error(jid)
        out.append(e.result(jid))
    stats = e.stats()
    e.close()
    return out, stats


@pytest.mark.gpu
def test_engine_job_is_md_run_bit_for_bit():
    """One mixed LJ job through the engine (95 steps: not a multiple of the
    chunk, rebuilds at 20, 40, ...) equals md_init + md_run on a context."""
    spec, st = _lj_job(5, 95, seed=3)
    (res,), _ = _engine_run([(spec, st)])
    rows, a = _ctx_run(st, 95, gbmd.PREC_MIXED)
    assert np.array_equal(res.id, a.id)
    assert np.array_equal(res.x, a.x)
    assert np.array_equal(res.v, a.v)
    assert np.array_equal(res.f, a.f)
    assert np.array_equal(res.thermo, rows)


@pytest.mark.gpu
def test_engine_result_same_alone_and_in_the_mix():
    """Job A alone, then A among jobs of other sizes, step counts, potentials
    and arrival times: A's trajectory is bit-identical."""
    a_spec, a_st = _lj_job(6, 120, seed=11)
    (alone,), _ = _engine_run([(a_spec, a_st)])
    mix = [_lj_job(4, 50, seed=1), _lj_job(7, 200, seed=2, rho=0.75, T=0.9),
           (a_spec, a_st), _lj_job(5, 130, seed=4, rho=0.88, T=1.3),
           _lj_job(3, 70, seed=5, prec=gbmd.PREC_FP64)]
    res, stats = _engine_run(mix, stagger=True)
    b = res[2]
    assert np.array_equal(alone.x, b.x)
    assert np.array_equal(alone.v, b.v)
    assert np.array_equal(alone.f, b.f)
    assert np.array_equal(alone.thermo, b.thermo)
    # the batched launches really covered several jobs at once
    assert stats["finished"] == 5


NNP_DIR = Path(__file__).resolve().parent / "golden" / "nnp_cu"


def _nnp_job(cells, nsteps, seed, prec=gbmd.PREC_MIXED):
    st = inputs.nnp_fcc(cells, seed=seed)
    spec = S.JobSpec(gbmd.FORCE_NNP, nsteps, tuple(st.lo), tuple(st.hi), st.boltz, st.mvv2e,
                     st.dt, float(st.mass[0]), 6.0, 1.0, precision=prec, nnp_dir=str(NNP_DIR))
    return spec, st


def _ctx_run_nnp(st, nsteps, prec):
    c = gbmd.Context(0)
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(prec)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    c.nnp_load(str(NNP_DIR), 1.0, 1.0)
    row0 = c.md_init(6.0, 1.0, 0, 20, 10)
    rows = c.md_run(nsteps)
    a = c.download_atoms().by_id()
    c.close()
    return np.vstack([row0[None, :], rows]), a


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [gbmd.PREC_MIXED, gbmd.PREC_FP64])
def test_engine_nnp_job_same_alone_in_the_mix_and_through_md_run(prec):
    """An NNP job (the workload's Cu potential, 500 atoms, 75 steps) alone in
    the engine, then among LJ and other NNP jobs of other sizes, step counts,
    precisions and arrival times, and through md_init + md_run on a context.
    Mixed precision: the three trajectories are bit-identical (forces are
    summed in fixed point, so the order in which contributions land does not
    matter).  FP64: its force sums are FP64 atomic additions, whose order
    varies from run to run, so the trajectories agree within 1e-10."""
    a_spec, a_st = _nnp_job(5, 75, seed=31, prec=prec)
    (alone,), _ = _engine_run([(a_spec, a_st)])
    mix = [_lj_job(6, 90, seed=1), _nnp_job(4, 40, seed=32),
           (a_spec, a_st), _lj_job(5, 130, seed=4, rho=0.88, T=1.3),
           _nnp_job(6, 30, seed=33, prec=gbmd.PREC_FP64),
           _lj_job(4, 70, seed=5, prec=gbmd.PREC_FP64), _nnp_job(4, 120, seed=34)]
    res, stats = _engine_run(mix, stagger=True)
    b = res[2]
    rows, ref = _ctx_run_nnp(a_st, 75, prec)
    if prec == gbmd.PREC_MIXED:
        def same(a, b):
            return np.array_equal(a, b)
    else:
        def same(a, b):
            return np.allclose(a, b, rtol=1e-10, atol=1e-10 * np.abs(a).max())
    for other in (b, ref):
        assert np.array_equal(alone.id, other.id)
        assert same(alone.x, other.x)
        assert same(alone.v, other.v)
        assert same(alone.f, other.f)
    assert same(alone.thermo, b.thermo)
    assert same(alone.thermo, rows)
    assert stats["finished"] == len(mix)


@pytest.mark.gpu
def test_engine_fp64_job_matches_oracle():
    """The FP64 engine path reproduces the CPU restatement of the reference
    (full list: bit-identical trajectory, thermo within 1e-10)."""
    spec, st = _lj_job(5, 60, seed=21, prec=gbmd.PREC_FP64)
    (res,), _ = _engine_run([(spec, st)])
    s = st.copy()
    th, f = O.run_lj(s.x, s.v, s.type, s.id, s.lo, s.hi, LJ, force_cut=2.5, skin=0.3, half=0,
                     rebuild_every=20, thermo_every=10, nsteps=60, boltz=s.boltz,
                     mvv2e=s.mvv2e, dt=s.dt, mass=s.mass, nthreads=4)
    o = np.argsort(s.id)
    assert np.array_equal(res.x, s.x[o])
    assert np.allclose(res.thermo, th, rtol=1e-10, atol=1e-12)


@pytest.mark.gpu
def test_engine_admits_by_memory_budget():
    """A budget that holds one job at a time: the others queue, run one after
    another, and the peak footprint stays inside the budget."""
    # 4,000-atom jobs: admission estimate ~4.1 MB, measured footprint
    # ~2.9 MB, so 5.5 MB admits one job and not a second beside it
    jobs = [_lj_job(10, 40, seed=s) for s in range(3)]
    e = S.Engine(0, budget_bytes=5.5e6, max_running=8, chunk=10)
    ids = [e.submit(*j) for j in jobs]
    seen_running = []
    while True:
        r, q, _ = e.step()
        seen_running.append(r)
        if r == 0 and q == 0:
            break
    st = e.stats()
    assert max(seen_running) == 1
    assert st["finished"] == 3 and st["peak_used_bytes"] <= st["budget_bytes"]
    times = [e.poll(j)[2] for j in ids]
    assert times[0][2] <= times[1][1] and times[1][2] <= times[2][1]  # FIFO, one at a time
    e.close()


@pytest.mark.gpu
def test_engine_slots_and_oversized_job():
    e = S.Engine(0, budget_bytes=64e6, max_running=2, chunk=10)
    small = [e.submit(*_lj_job(4, 30, seed=s)) for s in range(4)]
    big = e.submit(*_lj_job(30, 10, seed=9))  # 108,000 atoms: over 64 MB
    peak = 0
    while True:
        r, q, _ = e.step()
        peak = max(peak, r)
        if r == 0 and q == 0:
            break
    assert peak == 2
    assert all(e.poll(j)[0] == S.JOB_DONE for j in small)
    state, err, _ = e.poll(big)
    assert state == S.JOB_FAILED and err == 3
    e.close()


@pytest.mark.gpu
def test_engine_cancel_queued_and_running_jobs():
    """Fault injection on the host: a queued job and a running job are
    cancelled; both end FAILED / CANCELLED, the running one's slot and memory
    go to the next job, and that job's result is still bit-identical to
    md_run alone."""
    e = S.Engine(0, budget_bytes=1e9, max_running=1, chunk=10)
    a = e.submit(*_lj_job(4, 200, seed=1))
    b = e.submit(*_lj_job(4, 50, seed=2))
    c_spec, c_st = _lj_job(5, 60, seed=3)
    c = e.submit(c_spec, c_st)
    r, q, _ = e.step()
    assert (r, q) == (1, 2) and e.poll(a)[0] == S.JOB_RUNNING
    e.cancel(b)  # queued
    assert e.poll(b)[:2] == (S.JOB_FAILED, 8)
    assert e.error(b) == "cancelled"
    e.step()
    used = e.stats()["used_bytes"]
    assert used > 0
    e.cancel(a)  # running, between steps
    assert e.poll(a)[:2] == (S.JOB_FAILED, 8)
    assert e.stats()["used_bytes"] < used
    with pytest.raises(gbmd.GbmdError):
        e.cancel(a)  # already finished
    while True:
        r, q, _ = e.step()
        if r == 0 and q == 0:
            break
    assert e.poll(c)[0] == S.JOB_DONE
    res = e.result(c)
    st = e.stats()
    assert st["cancelled"] == 2 and st["finished"] == 1
    e.close()
    rows, ref = _ctx_run(c_st, 60, gbmd.PREC_MIXED)
    assert np.array_equal(res.x, ref.x)
    assert np.array_equal(res.thermo, rows)


@pytest.mark.gpu
def test_engine_batches_nnp_jobs_into_job_table_launches():
    """Mixed-precision NNP jobs of the common potential shape advance in
    job-table launches (six per step for all of them, plus per-job thermo
    reductions), not ~8 launches per job and step; their results equal
    md_init + md_run on a context bit for bit."""
    jobs = [_nnp_job(4 + (k % 2), 40, seed=50 + k) for k in range(6)]
    res, stats = _engine_run(jobs)
    per_job_launches = 6 * 40 * 7
    assert stats["launches"] < per_job_launches, stats["launches"]
    for (spec, st), r in zip(jobs, res):
        rows, ref = _ctx_run_nnp(st, 40, gbmd.PREC_MIXED)
        assert np.array_equal(r.x, ref.x)
        assert np.array_equal(r.f, ref.f)
        assert np.array_equal(r.thermo, rows)


def _spec_run(spec, st):
    """md_init + md_run of one job's system on a context of its own, with
    the job's precision, list kind and rebuild cadence."""
    c = gbmd.Context(0)
    c.set_units(st.boltz, st.mvv2e, st.dt)
    c.set_box(st.lo, st.hi)
    c.set_types(st.mass)
    c.set_precision(spec.precision)
    c.upload_atoms(st.x, st.v, st.type, st.id)
    if spec.force == gbmd.FORCE_LJ:
        c.lj_coeff(1, 1, *spec.lj)
    else:
        c.nnp_load(spec.nnp_dir, 1.0, 1.0)
    row0 = c.md_init(spec.force_cut, spec.skin, spec.half, spec.rebuild_every,
                     spec.thermo_every)
    rows = c.md_run(spec.nsteps)
    a = c.download_atoms().by_id()
    c.close()
    return np.vstack([row0[None, :], rows]), a


@pytest.mark.gpu
def test_engine_rebuilds_run_in_job_table_launches():
    """The rebuilds (wrap, cell sort, Verlet list) of jobs that share an
    engine stream run in job-table launches, one per phase for all of them.
    LJ jobs of several sizes and densities in mixed precision and FP64, one
    with a half list and one rebuilt every step, and a mixed NNP job: every
    rebuild after md_init goes through the batch, and every trajectory
    equals md_init + md_run on a context of its own -- bit for bit where the
    force sums do not depend on their order, within 1e-9 for the half
    list's FP64 atomic partner sums."""
    def lj(cells, nsteps, seed, rho=0.8442, T=1.44, prec=gbmd.PREC_MIXED, half=0, every=20):
        st = inputs.lj_fcc(cells, rho=rho, T=T, seed=seed)
        spec = S.JobSpec(gbmd.FORCE_LJ, nsteps, tuple(st.lo), tuple(st.hi), st.boltz,
                         st.mvv2e, st.dt, float(st.mass[0]), 2.5, 0.3, precision=prec,
                         half=half, rebuild_every=every, lj=(1.0, 1.0, 2.5))
        return spec, st

    jobs = [lj(4, 60, 61), lj(6, 85, 62, rho=0.75, T=0.9), lj(5, 45, 63, rho=0.88),
            lj(3, 100, 64, prec=gbmd.PREC_FP64), lj(4, 50, 65, prec=gbmd.PREC_FP64, half=1),
            lj(3, 12, 66, prec=gbmd.PREC_FP64, every=1), _nnp_job(4, 45, seed=67)]
    res, stats = _engine_run(jobs)
    # rebuilds before steps rebuild_every, 2 rebuild_every, ... <= nsteps
    assert stats["batched_rebuilds"] == sum(s.nsteps // s.rebuild_every for s, _ in jobs)
    for (spec, st), r in zip(jobs, res):
        rows, ref = _spec_run(spec, st)
        assert np.array_equal(r.id, ref.id)
        if spec.half:
            for a, b in ((r.x, ref.x), (r.v, ref.v), (r.f, ref.f), (r.thermo, rows)):
                assert np.allclose(a, b, rtol=1e-9, atol=1e-9 * np.abs(b).max())
        else:
            assert np.array_equal(r.x, ref.x)
            assert np.array_equal(r.v, ref.v)
            assert np.array_equal(r.f, ref.f)
            assert np.array_equal(r.thermo, rows)
