"""Many independent DMRG jobs advanced together on one GPU (continuous batching).

A job is one finite-size DMRG run (the sweeps of dmrg_finite_size, DMRG_anyH.py:18-101): its
coupling lists, bond dimension, sweep count and seed. The engine holds every admitted job's MPS and
environments on the device across its sweeps and advances all of them one local update per step:

* each job moves its orthogonality centre to its next site and assembles its effective
  Hamiltonian (the gauge move, environment update and block assembly of its own DeviceMPS,
  MPSClass.py:143-198, 474-530, 684-733);
* the local solves of all jobs (update_tensor_eigs, MPSClass.py:778-809) then run in ONE
  tn_batched_lanczos call: one grouped matvec launch per Lanczos step for every job, grouped
  Gram-Schmidt kernels, and the convergence test on the device;
* a job that finishes its sweeps is observed (bond energies, magnetisations, energy per site)
  and leaves; jobs waiting in the queue are admitted as slots and device memory free up, so
  requests that arrive while others run share the next steps with them.

Every job draws its random MPS from its own seed and touches only its own buffers, and the batched
solver's arithmetic per job does not depend on the other jobs of the batch, so a job's result is
the same alone and in any mix (tests/test_gpu_batched.py).
"""
import ctypes
import time

import numpy as np
import torch

from . import _lib as L
from .MPSClass import MpsOpenBoundaryClass


class BatchJob:
    """One DMRG request: para (generate_parameters_dmrg conventions), seed, arrival time."""

    def __init__(self, job_id, para, seed, arrival=0.0):
        self.job_id = job_id
        self.para = para
        self.seed = int(seed)
        self.arrival = float(arrival)
        self.result = None
        self.admitted = None
        self.finished = None
        self.solves = 0
        self.matvecs = 0
        self.A = None
        self._order = None
        self._k = 0
        self._t = 0

    def footprint_bytes(self, krylov=24):
        """Device memory the job holds while admitted (its MPS, environments and solver space)."""
        if getattr(self, "_footprint", None) is None:
            from .serving import estimate_device_bytes
            self._footprint = estimate_device_bytes(self.para, krylov=krylov)
        return self._footprint

    # -- lifecycle --------------------------------------------------------------------
    def start(self, device, precision):
        p = self.para
        np.random.seed(self.seed)
        self.A = MpsOpenBoundaryClass(length=p["l"], d=p["d"], chi=p["chi"], operators=p["op"], device=device,
                                      precision=precision)
        self.A.correct_orthogonal_center(p["ob_position"])
        self.A._model(p["index1"], p["index2"], p["coeff1"], p["coeff2"], p["eigs_tol"])
        ob = p["ob_position"]
        self._order = list(range(ob + 1, p["l"])) + list(range(p["l"] - 2, -1, -1)) + list(range(1, ob))
        self._k = 0
        self._t = 0

    def site(self):
        return self._order[self._k]

    def prepare(self):
        """Centre to this step's site and its effective Hamiltonian: (desc, keep-alive, psi)."""
        dev = self.A._dev
        p = self.site()
        dev.move_center_for_solve(p)
        desc, keep = dev.site_operator(p)
        psi = dev.mps[p].contiguous()
        dev.mps[p] = psi
        return desc, keep, psi

    def solved(self, res):
        """Book the local solve; returns True when the job's last sweep is done."""
        dev = self.A._dev
        p = self.site()
        dev.unit_norm = True
        dev.tensor_changed(p)
        dev.stats["solves"] += 1
        dev.stats["matvecs"] += res.matvecs
        if not res.converged:
            dev.stats["unconverged"] += 1
        self.solves += 1
        self.matvecs += res.matvecs
        self._k += 1
        if self._k == len(self._order):
            self._k = 0
            self._t += 1
            return self._t >= self.para["sweep_time"]
        return False

    def observe(self):
        p, A = self.para, self.A
        eb = A.observe_bond_energy(p["index2"], p["coeff2"])
        mx = A.observe_magnetization(1)
        mz = A.observe_magnetization(3)
        e = float((np.sum(eb) - p["hx"] * np.sum(mx) - p["hz"] * np.sum(mz)) / p["l"])
        self.result = {"e_per_site": e, "eb_full": np.ravel(eb), "mx": np.ravel(mx), "mz": np.ravel(mz),
                       "sweeps": self._t, "solves": self.solves, "matvecs": self.matvecs,
                       "unconverged": int(A.stats["unconverged"])}
        self.A = None   # release the device tensors


class BatchEngine:
    """Continuous batching of DMRG jobs: admission by device memory, one batched local solve per
    step for all admitted jobs, p50/p99 latency from arrival to result."""

    def __init__(self, device="cuda", precision="tf32x3", budget_bytes=None, max_active=1024, max_krylov=24,
                 check_every=3, mixed_floor=2e-6, workers=8, streams=16):
        self.device = device
        self.workers = max(1, int(workers))
        self.nstreams = max(1, int(streams))
        self._streams = None
        self._pool = None
        self.precision = precision
        self.prec = L.PRECISIONS[precision]
        self.budget = budget_bytes
        self.max_active = int(max_active)
        self.krylov = int(max_krylov)
        self.check_every = int(check_every)
        self.mixed_floor = float(mixed_floor)
        self.pending = []
        self.active = []
        self.done = []
        self.steps = 0
        self.max_concurrent = 0
        self.max_used = 0
        self._used = 0
        self._ws = None
        self._t0 = None
        self.step_ms = []

    def submit(self, job):
        self.pending.append(job)
        self.pending.sort(key=lambda j: (j.arrival, j.job_id))

    def _budget(self):
        if self.budget is not None:
            return int(self.budget)
        if str(self.device).startswith("cuda"):
            free, _ = torch.cuda.mem_get_info(torch.device(self.device))
            return int(0.8 * free) + self._used
        return 1 << 62

    def _admit(self, now):
        budget = self._budget()
        while self.pending and self.pending[0].arrival <= now and len(self.active) < self.max_active:
            fp = self.pending[0].footprint_bytes(self.krylov)
            if self.active and self._used + fp > budget:
                break
            job = self.pending.pop(0)
            job.admitted = now
            job.start(self.device, self.precision)
            self.active.append(job)
            self._used += fp
        self.max_concurrent = max(self.max_concurrent, len(self.active))
        self.max_used = max(self.max_used, self._used)

    def _prepare_all(self, jobs):
        """Every job's gauge move, environment update and block assembly. On a GPU the jobs are
        spread over `streams` CUDA streams and prepared by `workers` host threads (the library's
        calls release the GIL), so their small latency-bound kernels overlap; the batched solve
        on the current stream waits for all of them."""
        cuda = str(self.device).startswith("cuda") and not L._host_test
        if not cuda or self.workers == 1:
            return [job.prepare() for job in jobs]
        if self._streams is None:
            self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.nstreams)]
            from concurrent.futures import ThreadPoolExecutor
            self._pool = ThreadPoolExecutor(max_workers=self.workers)
        main = torch.cuda.current_stream(self.device)
        ready = torch.cuda.Event()
        ready.record(main)          # the previous step's solve wrote the site tensors
        # a job keeps its stream for life: the caching allocator then sees every allocation and
        # release of the job's tensors on one stream
        groups = [[] for _ in range(self.nstreams)]
        for i, job in enumerate(jobs):
            groups[job.job_id % self.nstreams].append(i)

        def run(k):
            st = self._streams[k]
            st.wait_event(ready)
            with torch.cuda.stream(st):
                out = [(i, jobs[i].prepare()) for i in groups[k]]
            ev = torch.cuda.Event()
            ev.record(st)
            return out, ev

        results = [None] * len(jobs)
        for out, ev in self._pool.map(run, [k for k in range(self.nstreams) if groups[k]]):
            main.wait_event(ev)
            for i, r in out:
                results[i] = r
        return results

    def step(self):
        """One local update of every admitted job (one batched solve)."""
        jobs = list(self.active)
        if not jobs:
            return []
        keep, solves = [], (L.BatchSolve * len(jobs))()
        for i, (desc, kp, psi) in enumerate(self._prepare_all(jobs)):
            keep.append((kp, psi))
            solves[i].site = desc
            solves[i].psi_in = psi.data_ptr()
            solves[i].psi_out = psi.data_ptr()
        lib = L.load()
        opts = L.LanczosOpts(float(jobs[0].para["eigs_tol"]), float(jobs[0].para["tau"]), 0.0, self.mixed_floor,
                             self.krylov, 50, self.check_every, self.prec, 0, 0)
        if len({(float(j.para["eigs_tol"]), float(j.para["tau"])) for j in jobs}) > 1:
            raise ValueError("jobs of one batch share eigs_tol and tau")
        table = ctypes.cast(solves, ctypes.c_void_p)
        need = lib.tn_batched_lanczos_workspace_bytes(table, len(jobs), ctypes.byref(opts))
        if self._ws is None:
            self._ws = L.Workspace(torch.device(self.device))
        wp, wb = self._ws.args(need + 1024)
        res = (L.LanczosResult * len(jobs))()
        st = lib.tn_batched_lanczos(table, len(jobs), ctypes.byref(opts), wp, wb, ctypes.cast(res, ctypes.c_void_p),
                                    L.stream_handle())
        if st not in (L.TN_OK, L.TN_ERR_NOCONV):
            L.check(st, "batched lanczos")
        finished = []
        for i, job in enumerate(jobs):
            if job.solved(res[i]):
                finished.append(job)
        del keep
        self.steps += 1
        return finished

    def run(self, progress=None):
        """Admit (by arrival time and memory), step, retire, until every submitted job is done."""
        self._t0 = t0 = time.perf_counter()
        while self.pending or self.active:
            now = time.perf_counter() - t0
            self._admit(now)
            if not self.active:
                time.sleep(max(0.0, min(self.pending[0].arrival - now, 0.01)))
                continue
            ts = time.perf_counter()
            finished = self.step()
            for job in finished:
                job.observe()
                job.finished = time.perf_counter() - t0
                self.active.remove(job)
                self._used -= job.footprint_bytes(self.krylov)
                self.done.append(job)
            self.step_ms.append(1000.0 * (time.perf_counter() - ts))
            if progress:
                progress(self)
        if str(self.device).startswith("cuda"):
            torch.cuda.synchronize()
        return self.done

    def summary(self):
        lat = np.array([j.finished - j.arrival for j in self.done]) if self.done else np.zeros(1)
        span = max((j.finished for j in self.done), default=0.0)
        solves = sum(j.solves for j in self.done)
        return {"jobs": len(self.done), "solves": solves, "wall_s": span,
                "solves_per_s": solves / span if span > 0 else 0.0,
                "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                "max_concurrent": self.max_concurrent, "steps": self.steps,
                "step_ms_p50": float(np.percentile(self.step_ms, 50)) if self.step_ms else 0.0,
                "matvecs_per_solve": (sum(j.matvecs for j in self.done) / solves) if solves else 0.0}


def batch_jobs(njobs, seed=0, sweeps=8, precision="tf32x3", device="cuda", rate=None, lengths=(16, 64),
               chis=(32, 64, 128), ladder_fraction=0.0, ladder_lengths=(8, 48), rung=(0.5, 2.0)):
    """The request stream of serving.make_jobs (same draws: XXZ chains with Jz ~ U[0,2], hz ~ U[0,1],
    N ~ U{lengths}, chi from `chis`, optional 2 x L ladders, Poisson arrivals at `rate`) as BatchJobs.
    Every job observes once, after its last sweep."""
    from . import serving
    out = []
    for j in serving.make_jobs(njobs, seed=seed, sweeps=sweeps, precision=precision, device=device, rate=rate,
                               lengths=lengths, chis=chis, ladder_fraction=ladder_fraction,
                               ladder_lengths=ladder_lengths, rung=rung):
        j.para["dt_ob"] = int(sweeps)
        out.append(BatchJob(j.job_id, j.para, j.seed, arrival=j.arrival))
    return out


def main(argv=None):
    """Batched / serving workloads against sequential plain-FP64 solves, one JSON line."""
    import argparse
    import json
    from . import serving
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--jobs", type=int, default=512)
    ap.add_argument("--sweeps", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--rate", type=float, default=None, help="Poisson arrival rate (requests/s); default all at t=0")
    ap.add_argument("--precision", default="tf32x3")
    ap.add_argument("--lengths", default="16,64")
    ap.add_argument("--chis", default="32,64,128")
    ap.add_argument("--ladders", type=float, default=0.0)
    ap.add_argument("--ladder-rungs", default="8,48")
    ap.add_argument("--max-active", type=int, default=1024)
    ap.add_argument("--krylov", type=int, default=24)
    ap.add_argument("--baseline-jobs", type=int, default=12,
                    help="how many of the jobs also run one at a time on the plain FP64 GPU path (0: none)")
    ap.add_argument("--baseline-precision", default="fp64")
    ap.add_argument("--device", default="cuda")
    a = ap.parse_args(argv)
    lengths = tuple(int(x) for x in a.lengths.split(","))
    chis = tuple(int(x) for x in a.chis.split(","))
    rungs = tuple(int(x) for x in a.ladder_rungs.split(","))
    shape = dict(lengths=lengths, chis=chis, ladder_fraction=a.ladders, ladder_lengths=rungs)
    L.load()
    dev = a.device
    # warm-up (first launches, tensor-core attributes, QR graphs)
    warm = BatchEngine(dev, a.precision, max_krylov=a.krylov)
    for j in batch_jobs(4, seed=a.seed + 10 ** 6, sweeps=1, precision=a.precision, device=dev, **shape):
        warm.submit(j)
    warm.run()
    eng = BatchEngine(dev, a.precision, max_active=a.max_active, max_krylov=a.krylov)
    for j in batch_jobs(a.jobs, seed=a.seed, sweeps=a.sweeps, precision=a.precision, device=dev, rate=a.rate,
                        **shape):
        eng.submit(j)
    eng.run()
    out = eng.summary()
    out.update({"precision": a.precision, "sweeps": a.sweeps, "rate_per_s": a.rate, "lengths": list(lengths),
                "chis": list(chis), "ladder_fraction": a.ladders, "krylov": a.krylov,
                "unconverged_solves": int(sum(j.result["unconverged"] for j in eng.done))})
    if a.baseline_jobs > 0:
        # the first jobs of the same stream, one at a time on the single-job path
        seq = serving.make_jobs(min(a.baseline_jobs, a.jobs), seed=a.seed, sweeps=a.sweeps,
                                precision=a.baseline_precision, device=dev, **shape)
        for j in batch_jobs(1, seed=a.seed + 2 * 10 ** 6, sweeps=1, precision=a.baseline_precision, device=dev,
                            **shape):
            s = serving.Scheduler(dev, max_active=1)
            s.submit(serving.DMRGJob(0, j.para, j.seed))
            s.run()
        wall, solves, lat = 0.0, 0, []
        for j in seq:
            j.para["dt_ob"] = int(a.sweeps)
            j.arrival = 0.0
            s = serving.Scheduler(dev, max_active=1)
            s.submit(j)
            t0 = time.perf_counter()
            s.run()
            if str(dev).startswith("cuda"):
                torch.cuda.synchronize()
            wall += time.perf_counter() - t0
            solves += j.solves
            lat.append(time.perf_counter() - t0)
        done = {j.job_id: j for j in eng.done}
        de = [abs(done[j.job_id].result["e_per_site"] - j.result["e_per_site"]) for j in seq]
        out["sequential"] = {"precision": a.baseline_precision, "jobs": len(seq), "solves": solves, "wall_s": wall,
                             "solves_per_s": solves / wall, "latency_per_job_p50_s": float(np.percentile(lat, 50)),
                             "latency_per_job_p99_s": float(np.percentile(lat, 99))}
        out["speedup_vs_sequential"] = out["solves_per_s"] / (solves / wall)
        out["max_abs_de_per_site_vs_sequential"] = float(max(de))
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
