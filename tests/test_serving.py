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
