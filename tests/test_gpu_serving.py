"""The multi-job scheduler on the GPU: every job on its own CUDA stream, interleaved with the
others, gives the result it gives alone (FP64 path: bit-for-bit arithmetic; split TF32: within
the rounding order of its GEMM atomics)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from tnalg_gb300 import serving  # noqa: E402


def _jobs(precision):
    out = []
    for k, (l, chi, jz, hz) in enumerate([(16, 16, 1.0, 0.0), (24, 32, 0.5, 0.2), (20, 16, 1.5, 0.1),
                                          (12, 8, 1.0, 0.3), (32, 32, 0.8, 0.0)]):
        para = serving.chain_job_para(l, chi, jz=jz, hz=hz, sweeps=3, precision=precision, device="cuda")
        out.append(serving.DMRGJob(k, para, seed=200 + k))
    return out


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("tf32x3", 1e-8)])
def test_jobs_alone_and_interleaved_agree(cuda_lib, precision, tol):
    if precision == "tf32x3":
        from tnalg_gb300 import _lib as L
        if not L.tf32x3_available():
            pytest.skip("tf32x3 needs an sm_103 device")
    alone = {}
    for j in _jobs(precision):
        s = serving.Scheduler("cuda", max_active=1)
        s.submit(j)
        s.run()
        alone[j.job_id] = j.result
    mix = serving.Scheduler("cuda")
    for j in _jobs(precision):
        mix.submit(j)
    done = mix.run()
    assert mix.max_concurrent == 5 and len(done) == 5
    for j in done:
        ref = alone[j.job_id]
        assert abs(j.result["e_per_site"] - ref["e_per_site"]) <= tol
        np.testing.assert_allclose(j.result["mz"], ref["mz"], atol=10 * tol)
        assert j.result["e_per_site"] < 0
    summ = mix.summary()
    assert summ["solves"] > 0 and summ["latency_p99_s"] >= summ["latency_p50_s"]
