"""The multi-job scheduler (tnalg_gb300/serving.py) on the CPU through the test double of the C ABI:
admission against a device-memory budget, round-robin interleaving, and each job's result is the
same alone and in a mix."""
import numpy as np
import pytest

import fake_lib
from tnalg_gb300 import serving


@pytest.fixture(autouse=True)
def _fake():
    fake_lib.install()
    yield


def _jobs(device="cpu"):
    out = []
    for k, (l, chi, jz, hz) in enumerate([(8, 4, 1.0, 0.0), (10, 6, 0.5, 0.2), (12, 4, 1.5, 0.1), (6, 4, 1.0, 0.3)]):
        para = serving.chain_job_para(l, chi, jz=jz, hz=hz, sweeps=3, device=device)
        out.append(serving.DMRGJob(k, para, seed=100 + k))
    return out


def test_result_is_the_same_alone_and_in_the_mix():
    alone = {}
    for j in _jobs():
        s = serving.Scheduler("cpu", max_active=1)
        s.submit(j)
        s.run()
        alone[j.job_id] = j.result
    mix = serving.Scheduler("cpu")
    for j in _jobs():
        mix.submit(j)
    done = mix.run()
    assert mix.max_concurrent == 4 and len(done) == 4
    for j in done:
        ref = alone[j.job_id]
        assert j.result["e_per_site"] == pytest.approx(ref["e_per_site"], abs=1e-12)
        np.testing.assert_allclose(j.result["mz"], ref["mz"], atol=1e-12)
        np.testing.assert_allclose(j.result["eb_full"], ref["eb_full"], atol=1e-12)
        assert j.result["solves"] == ref["solves"] > 0
        assert np.isfinite(j.result["e_per_site"]) and j.result["e_per_site"] < 0


def test_admission_respects_the_memory_budget():
    jobs = _jobs()
    fps = sorted(j.footprint_bytes() for j in jobs)
    s = serving.Scheduler("cpu", budget_bytes=fps[-1] + fps[-2])  # room for two jobs at most
    for j in jobs:
        s.submit(j)
    done = s.run()
    assert len(done) == 4 and 1 <= s.max_concurrent <= 2
    summ = s.summary()
    assert summ["jobs"] == 4 and summ["solves"] == sum(j.solves for j in done)
    assert summ["latency_p99_s"] >= summ["latency_p50_s"] >= 0.0


def test_arrivals_and_job_parameters_are_independent_of_the_rate():
    a = serving.make_jobs(6, seed=3, device="cpu")
    b = serving.make_jobs(6, seed=3, device="cpu", rate=100.0)
    for x, y in zip(a, b):
        assert x.para["l"] == y.para["l"] and x.para["chi"] == y.para["chi"] and x.seed == y.seed
        assert x.arrival == 0.0
    assert all(y.arrival > 0 for y in b) and all(b[i].arrival < b[i + 1].arrival for i in range(5))


def _held_bytes(A):
    dev = A._dev
    ts = [t for t in dev.EL + dev.ER if t is not None] + list(dev.mps)
    return 8 * sum(int(t.numel()) for t in ts)


@pytest.mark.parametrize("kind", ["chain", "ladder"])
def test_footprint_bounds_the_tensors_a_job_holds(kind):
    """The admission estimate covers the MPS and every environment stack the engine holds after
    its sweeps (both sides of every bond), for chains and for ladders with straddling terms."""
    import contextlib
    import io
    from tnalg_gb300 import DMRG_anyH
    if kind == "chain":
        para = serving.chain_job_para(14, 8, jz=0.7, hz=0.2, sweeps=2, device="cpu")
    else:
        para = serving.ladder_job_para(6, 8, j_rung=1.3, jz=0.7, hz=0.2, sweeps=2, device="cpu")
    np.random.seed(0)
    with contextlib.redirect_stdout(io.StringIO()):
        ob, A, info, _ = DMRG_anyH.dmrg_finite_size(para)
    held = _held_bytes(A)
    est = serving.estimate_device_bytes(para)
    assert est >= held
    assert est < 40 * held   # an estimate, not a blanket reservation
    assert np.isfinite(ob["e_per_site"])


def test_ladder_jobs_alone_and_mixed_with_chains():
    ladder = serving.ladder_job_para(5, 6, j_rung=1.5, jz=0.8, hz=0.3, sweeps=3, device="cpu")
    assert ladder["l"] == 10 and np.asarray(ladder["index2"]).shape == (3 * (5 + 2 * 4), 4)
    alone = serving.DMRGJob(7, ladder, seed=9)
    s = serving.Scheduler("cpu", max_active=1)
    s.submit(alone)
    s.run()
    mix = serving.Scheduler("cpu")
    jobs = _jobs() + [serving.DMRGJob(7, ladder, seed=9)]
    for j in jobs:
        mix.submit(j)
    mix.run()
    got = [j for j in mix.done if j.job_id == 7][0]
    assert got.result["e_per_site"] == pytest.approx(alone.result["e_per_site"], abs=1e-12)
    np.testing.assert_allclose(got.result["mz"], alone.result["mz"], atol=1e-12)
    # a ladder carries more environment slots than a chain of the same length and bond dimension
    chain = serving.chain_job_para(10, 6, sweeps=3, device="cpu")
    assert serving.estimate_device_bytes(ladder) > serving.estimate_device_bytes(chain)


def test_ladder_mix_in_the_request_stream():
    plain = serving.make_jobs(12, seed=4, device="cpu")
    again = serving.make_jobs(12, seed=4, device="cpu", ladder_fraction=0.0)
    assert [j.para["l"] for j in plain] == [j.para["l"] for j in again]
    mixed = serving.make_jobs(12, seed=4, device="cpu", ladder_fraction=0.5)
    lattices = [j.para["lattice"] for j in mixed]
    assert "arbitrary" in lattices and "chain" in lattices
    for j in mixed:
        if j.para["lattice"] == "arbitrary":
            assert j.para["l"] % 2 == 0 and 16 <= j.para["l"] <= 96


def test_command_line_compares_the_mix_with_sequential_fp64(capsys):
    """`python -m tnalg_gb300.serving` (the serving leg of the benchmark): the one-at-a-time pass
    runs in the baseline precision and the JSON line reports both, with latencies of both passes."""
    import json
    serving.main(["--jobs", "4", "--sweeps", "2", "--device", "cpu", "--precision", "tf32x3",
                  "--baseline-precision", "fp64", "--ladders", "0.5", "--lengths", "8,12", "--chis", "4,8",
                  "--ladder-rungs", "3,5"])
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert out["jobs"] == 4 and out["precision"] == "tf32x3" and out["baseline_precision"] == "fp64"
    assert out["solves_per_s"] > 0 and out["sequential_solves_per_s"] > 0
    assert out["sequential_latency_p99_s"] >= out["sequential_latency_p50_s"] > 0
    assert out["latency_p99_s"] >= out["latency_p50_s"] > 0
    assert out["max_abs_de_per_site_mix_vs_alone"] < 1e-8


def test_worker_threads_give_the_results_of_one_thread():
    """Scheduler(workers=4): jobs advanced by a thread pool (one task per job in flight) finish
    with the results they give alone, and admission still keeps to the budget."""
    alone = {}
    for j in _jobs():
        s = serving.Scheduler("cpu", max_active=1)
        s.submit(j)
        s.run()
        alone[j.job_id] = j.result
    mix = serving.Scheduler("cpu", workers=4)
    for j in _jobs():
        mix.submit(j)
    done = mix.run()
    assert len(done) == 4 and mix.max_concurrent == 4
    for j in done:
        assert j.result["e_per_site"] == pytest.approx(alone[j.job_id]["e_per_site"], abs=1e-12)
        np.testing.assert_allclose(j.result["mz"], alone[j.job_id]["mz"], atol=1e-12)
        assert j.result["solves"] == alone[j.job_id]["solves"]
    fps = sorted(j.footprint_bytes() for j in _jobs())
    tight = serving.Scheduler("cpu", budget_bytes=fps[-1] + fps[-2], workers=4)
    for j in _jobs():
        tight.submit(j)
    assert len(tight.run()) == 4 and 1 <= tight.max_concurrent <= 2


def test_command_line_threaded_mix_without_sequential_pass(capsys):
    import json
    serving.main(["--jobs", "3", "--sweeps", "2", "--device", "cpu", "--workers", "3", "--no-sequential",
                  "--lengths", "8,12", "--chis", "4,8", "--rate", "200"])
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert out["workers"] == 3 and out["jobs"] == 3 and "sequential_solves_per_s" not in out
    assert len(out["e_per_site"]) == 3 and all(v < 0 for v in out["e_per_site"].values())


@pytest.mark.parametrize("workers", [1, 3])
def test_requests_submitted_while_running(workers):
    """run(wait=True) is a request loop: jobs submitted from another thread while it runs (arrival
    None: stamped at submission) are admitted and finished, each with its single-job result; the
    loop returns after close() once everything submitted has finished."""
    import threading
    import time as _time
    alone = {}
    for j in _jobs():
        s = serving.Scheduler("cpu", max_active=1)
        s.submit(j)
        s.run()
        alone[j.job_id] = j.result["e_per_site"]
    sched = serving.Scheduler("cpu", workers=workers)
    live = _jobs()
    for j in live:
        j.arrival = None

    def producer():
        for j in live:
            _time.sleep(0.05)
            sched.submit(j)
        sched.close()

    t = threading.Thread(target=producer)
    t.start()
    done = sched.run(wait=True)
    t.join()
    assert sorted(j.job_id for j in done) == [0, 1, 2, 3]
    for j in done:
        assert j.result["e_per_site"] == pytest.approx(alone[j.job_id], abs=1e-12)
        assert j.arrival > 0 and j.finished >= j.admitted >= j.arrival
    arrivals = [j.arrival for j in sorted(done, key=lambda j: j.job_id)]
    assert arrivals == sorted(arrivals)


def test_power_of_two_scaling_of_the_random_start_changes_nothing():
    """The job engines scale their random tensors by powers of two (so that centring a long chain at
    large chi cannot overflow FP64); the scaling is exact, so a job's result is the one
    dmrg_finite_size gives from the unscaled draws of the same seed."""
    import contextlib
    import io
    from tnalg_gb300 import DMRG_anyH, MPSClass
    t = MPSClass.random_open_mps(6, 2, 4)
    for a, b in zip(t, serving.pow2_scaled(t)):
        e = np.log2(np.abs(a[a != 0]) / np.abs(b[a != 0]))
        assert np.all(e == np.round(e)) and np.ptp(e) == 0      # one exact power of two per tensor
    para = serving.chain_job_para(10, 6, jz=0.7, hz=0.2, sweeps=3, device="cpu")
    para["break_tol"] = -1.0
    job = serving.DMRGJob(0, dict(para), seed=42)
    s = serving.Scheduler("cpu", max_active=1)
    s.submit(job)
    s.run()
    np.random.seed(42)
    with contextlib.redirect_stdout(io.StringIO()):
        ob, _, _, _ = DMRG_anyH.dmrg_finite_size(dict(para))
    assert job.result["e_per_site"] == pytest.approx(ob["e_per_site"], abs=1e-12)
    np.testing.assert_allclose(job.result["mz"], np.ravel(ob["mz"]), atol=1e-10)
