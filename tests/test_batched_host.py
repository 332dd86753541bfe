"""The batched engine (tnalg_gb300/batched.py) on the CPU through the test double of the C ABI:
continuous batching of uneven jobs gives every job the result it gets alone and the result of the
one-job scheduler; admission keeps to the slot limit and the memory budget."""
import ctypes

import numpy as np
import pytest

import fake_lib
from tnalg_gb300 import batched, serving


@pytest.fixture(autouse=True)
def _fake():
    fake_lib.install()
    yield
    fake_lib.uninstall()


SPECS = [(8, 4, 1.0, 0.0), (10, 6, 0.5, 0.2), (12, 4, 1.5, 0.1), (6, 4, 1.0, 0.3), (9, 8, 0.2, 0.6)]


def _jobs(kind="batch"):
    out = []
    for k, (l, chi, jz, hz) in enumerate(SPECS):
        para = serving.chain_job_para(l, chi, jz=jz, hz=hz, sweeps=3, device="cpu")
        cls = batched.BatchJob if kind == "batch" else serving.DMRGJob
        out.append(cls(k, para, seed=100 + k))
    return out


def _run(jobs, precision="fp64", **kw):
    eng = batched.BatchEngine("cpu", precision=precision, **kw)
    for j in jobs:
        eng.submit(j)
    done = eng.run()
    return eng, {j.job_id: j.result for j in done}


def test_batched_results_match_alone_and_the_single_job_path():
    alone = {}
    for j in _jobs():
        _, r = _run([j])
        alone.update(r)
    eng, mix = _run(_jobs())
    assert eng.max_concurrent == len(SPECS)
    single = {}
    for j in _jobs("serial"):
        s = serving.Scheduler("cpu", max_active=1)
        s.submit(j)
        s.run()
        single[j.job_id] = j.result
    for k in range(len(SPECS)):
        assert mix[k]["e_per_site"] == pytest.approx(alone[k]["e_per_site"], abs=1e-13)
        np.testing.assert_allclose(mix[k]["eb_full"], alone[k]["eb_full"], atol=1e-12)
        assert mix[k]["solves"] == alone[k]["solves"] == 3 * 2 * (SPECS[k][0] - 1)
        # the one-job path (serving.DMRGJob, dmrg_finite_size's schedule) reaches the same state
        assert mix[k]["e_per_site"] == pytest.approx(single[k]["e_per_site"], abs=1e-10)
        np.testing.assert_allclose(mix[k]["mz"], single[k]["mz"], atol=1e-8)


def test_slots_and_budget_limit_admission_and_late_jobs_join_running_ones():
    jobs = _jobs()
    eng, res = _run(jobs, max_active=2)
    assert eng.max_concurrent == 2 and len(res) == len(SPECS)
    # a job admitted after others started shares steps with them and still gets its own result
    _, ref = _run(_jobs())
    for k in res:
        assert res[k]["e_per_site"] == pytest.approx(ref[k]["e_per_site"], abs=1e-13)
    fps = sorted(j.footprint_bytes() for j in _jobs())
    budget = fps[-1] + fps[-2]
    eng2, res2 = _run(_jobs(), budget_bytes=budget)
    assert len(res2) == len(SPECS) and eng2.max_used <= budget and eng2.max_concurrent < len(SPECS)
    summ = eng2.summary()
    assert summ["jobs"] == len(SPECS) and summ["solves"] == sum(r["solves"] for r in res2.values())
    assert summ["latency_p99_s"] >= summ["latency_p50_s"] >= 0.0


def test_grouped_path_matches_the_per_job_path():
    """The grouped path (job arenas; gauge moves, environment updates and block assembly as
    grouped launches) against the per-job path, through the test double: same states (the test
    double's batched QR is LAPACK's, as the per-job path's), chains and a ladder with straddling
    couplings."""
    def jobs():
        out = _jobs()
        lad = serving.ladder_job_para(4, 8, j_rung=1.3, jz=0.7, hz=0.2, sweeps=3, device="cpu")
        out.append(batched.BatchJob(len(out), lad, seed=77))
        return out
    _, per_job = _run(jobs(), grouped=False)
    eng, grouped = _run(jobs(), grouped=True)
    assert all(isinstance(j, batched.ArenaJob) for j in eng.done)
    for k in per_job:
        assert grouped[k]["e_per_site"] == pytest.approx(per_job[k]["e_per_site"], abs=1e-11), k
        np.testing.assert_allclose(grouped[k]["eb_full"], per_job[k]["eb_full"], atol=1e-9)
        np.testing.assert_allclose(grouped[k]["mz"], per_job[k]["mz"], atol=1e-8)
        assert grouped[k]["solves"] == per_job[k]["solves"]


def test_unconverged_solves_continue_in_the_next_step():
    """A local solve of the grouped path that stops unconverged at its per-step cycle limit stays at
    its site and continues from its Ritz vector in the next step (its gauge move and environment
    update are not repeated); the job's sweeps and result are those of an undisturbed run."""
    from tnalg_gb300 import _lib
    _, ref = _run(_jobs(), grouped=True)
    fake = fake_lib.install()
    orig = fake.tn_batched_lanczos
    calls = {"n": 0, "held": 0}

    def flaky(jobs, count, opts, ws, wsb, results, stream):
        st = orig(jobs, count, opts, ws, wsb, results, stream)
        res = ctypes.cast(results, ctypes.POINTER(_lib.LanczosResult))
        calls["n"] += 1
        if calls["n"] % 3 == 0:      # every third batched call leaves its first job unconverged
            res[0].converged = 0
            calls["held"] += 1
        return st
    fake.tn_batched_lanczos = flaky
    eng, got = _run(_jobs(), grouped=True)
    assert calls["held"] > 0 and eng.steps > max(3 * 2 * (l - 1) for l, *_ in SPECS)
    for k in ref:
        assert got[k]["solves"] == ref[k]["solves"] == 3 * 2 * (SPECS[k][0] - 1)
        assert got[k]["unconverged"] == 0
        assert got[k]["e_per_site"] == pytest.approx(ref[k]["e_per_site"], abs=1e-11)


def test_prepared_admission_joins_in_groups_and_keeps_each_result():
    """Admission with the host side prepared ahead on worker threads (the grouped path): jobs are
    prepared while admitted ones step, join in groups of at least admit_chunk (fewer when nothing
    else is being prepared), and every job's result equals the one it gets with admission done all
    at once (prefetch = 0)."""
    def jobs():
        out = _jobs()
        for k in range(3):
            para = serving.chain_job_para(7 + k, 4, jz=0.3 * k, hz=0.1, sweeps=2, device="cpu")
            out.append(batched.BatchJob(len(out), para, seed=300 + k, arrival=0.0))
        return out
    _, ref = _run(jobs(), grouped=True, prefetch=0)
    eng, res = _run(jobs(), grouped=True, prefetch=3, admit_chunk=2, workers=2)
    assert sorted(res) == sorted(ref)
    assert eng.max_concurrent <= len(SPECS) + 3
    for k in ref:
        assert res[k]["e_per_site"] == pytest.approx(ref[k]["e_per_site"], abs=1e-13), k
        np.testing.assert_allclose(res[k]["mz"], ref[k]["mz"], atol=1e-12)
        assert res[k]["solves"] == ref[k]["solves"]
    assert all(j.admitted is not None for j in eng.done)
    assert not eng._prep


def test_large_jobs_run_alone_beside_the_batch():
    """Jobs with chi >= alone_chi run the single-job path on worker threads beside the grouped
    batch: each gets the result of the one-job scheduler (same draws, same kernels), the batched
    jobs keep theirs, and every job is reported once with its latency."""
    _, ref = _run(_jobs(), grouped=True, alone_chi=0)
    eng, res = _run(_jobs(), grouped=True, alone_chi=6, alone_workers=2)
    assert sorted(res) == sorted(ref) and len(eng.done) == len(SPECS)
    big = [k for k, s in enumerate(SPECS) if s[1] >= 6]
    assert big and not isinstance(next(j for j in eng.done if j.job_id == big[0]), batched.ArenaJob)
    for k, (l, chi, jz, hz) in enumerate(SPECS):
        if k in big:
            j = _jobs("serial")[k]
            s = serving.Scheduler("cpu", max_active=1)
            s.submit(j)
            s.run()
            assert res[k]["e_per_site"] == pytest.approx(j.result["e_per_site"], abs=1e-12), k
            np.testing.assert_allclose(res[k]["mz"], j.result["mz"], atol=1e-10)
        else:
            assert res[k]["e_per_site"] == pytest.approx(ref[k]["e_per_site"], abs=1e-13), k
    assert all(j.finished is not None and j.finished >= j.arrival for j in eng.done)


def test_poisson_stream_with_prepared_admission_and_large_jobs_alone():
    """The serving configuration of the engine at once: arrivals spread in time, the host side of
    admission prepared ahead (small groups), large jobs on the single-job path beside the batch. Every
    job finishes once, after it arrived, with the result it gets when it runs alone."""
    def stream():
        out = []
        for k, (l, chi, jz, hz) in enumerate(SPECS):
            para = serving.chain_job_para(l, chi, jz=jz, hz=hz, sweeps=2, device="cpu")
            out.append(batched.BatchJob(k, para, seed=500 + k, arrival=0.004 * k))
        return out
    alone = {}
    for j in stream():
        j.arrival = 0.0
        _, r = _run([j], grouped=True, alone_chi=6, prefetch=0)
        alone.update(r)
    eng, res = _run(stream(), grouped=True, alone_chi=6, alone_workers=2, prefetch=2, admit_chunk=2, workers=2)
    assert sorted(res) == sorted(alone) and len(eng.done) == len(SPECS)
    for j in eng.done:
        assert j.finished >= j.arrival
        assert res[j.job_id]["e_per_site"] == pytest.approx(alone[j.job_id]["e_per_site"], abs=1e-13), j.job_id
    summ = eng.summary()
    assert summ["jobs"] == len(SPECS) and summ["latency_p99_s"] >= summ["latency_p50_s"] > 0
