"""Many independent DMRG jobs on one GPU: admission, interleaving, latency.

A job is one finite-size DMRG run (the sweeps of `dmrg_finite_size`, DMRG_anyH.py:18-101, with
its coupling lists, chi schedule, sweep count and convergence test) that returns its energy per
site, bond energies and magnetisations. The scheduler

* admits a job once it has arrived and its estimated device memory (MPS, environments and the
  workspaces of its solver and gauge moves) fits the free part of a budget;
* gives every admitted job its own CUDA stream, MPS, environments and workspaces, and advances
  the admitted jobs one local update (solve + gauge move + environment update) at a time in
  turn: a job's host-side wait for its own Lanczos convergence check then leaves the kernels
  already queued by the other jobs running beside it, so small jobs fill the GPU together;
* records each job's latency from arrival to result (p50 and p99 over the jobs) and the
  aggregate solves/s.

A job touches only its own buffers and draws its random MPS from its own seed, so its result is
the same alone and in a mix (up to the rounding order of floating-point atomics in the split-TF32
GEMMs; the FP64 path is deterministic). The interleaved jobs are advanced by one host thread, or
with `workers=N` by a pool of host threads (the C library's calls release the GIL and its shared
host state is synchronised; each job keeps its own stream and workspaces).

    python -m tnalg_gb300.serving --jobs 16 --sweeps 4 [--rate 200] [--precision fp64|tf32x3] [--ladders 0.5]
"""
import argparse
import contextlib
import json
import threading
import time

import numpy as np

from . import Parameters as pm


def chain_job_para(length, chi, jz=1.0, hz=0.0, sweeps=4, precision="fp64", device="cuda", eigs_tol=1e-10,
                   break_tol=1e-9):
    """An XXZ open chain (Parameters.py:170-186 conventions) as a job description."""
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=int(length), chi=int(chi), jxy=1.0, jz=float(jz), hx=0.0, hz=float(hz), sweep_time=int(sweeps),
                dt_ob=1, eigs_tol=eigs_tol, break_tol=break_tol, precision=precision, device=device)
    return pm.make_consistent_parameter_dmrg(para)


def ladder_job_para(length, chi, j_rung=1.0, jz=1.0, hz=0.0, sweeps=4, precision="fp64", device="cuda",
                    eigs_tol=1e-10, break_tol=1e-9):
    """A 2 x length spin-1/2 ladder as an 'arbitrary'-lattice job (Parameters.py:205-212): sites
    (2r, 2r+1) form rung r; XXZ legs (Jxy = 1, Jz = jz) between rungs r and r+1, Heisenberg rungs
    of strength j_rung; uniform field hz. Bonds reach two sites along the chain, so every bond
    carries straddling terms."""
    para = pm.generate_parameters_dmrg("arbitrary")
    para["hx"], para["hz"] = 0.0, float(hz)
    para["op"] = list(para["op"][:6])
    para["op"].append(-para["hx"] * para["op"][1] - para["hz"] * para["op"][3])
    index2, coeff2 = [], []
    for r in range(int(length)):
        bonds = [(2 * r, 2 * r + 1, float(j_rung), float(j_rung))]
        if r + 1 < length:
            bonds += [(2 * r, 2 * r + 2, 1.0, float(jz)), (2 * r + 1, 2 * r + 3, 1.0, float(jz))]
        for i, j, jxy, jzz in bonds:
            index2 += [[i, j, 4, 5], [i, j, 5, 4], [i, j, 3, 3]]
            coeff2 += [jxy / 2, jxy / 2, jzz]
    n = 2 * int(length)
    para.update(index1=[[q, 6] for q in range(n)], coeff1=[1.0] * n, index2=index2, coeff2=coeff2, chi=int(chi),
                sweep_time=int(sweeps), dt_ob=1, eigs_tol=eigs_tol, break_tol=break_tol, tau=1e-4,
                precision=precision, device=device)
    return pm.make_consistent_parameter_dmrg(para)


def estimate_device_bytes(para, krylov=40):
    """Upper estimate of the device memory a job holds: the MPS, both environment stacks of every
    bond (slot 0 plus one chi_b x chi_b slot per open operator; after a sweep the engine holds EL[b]
    and ER[b] for all b), the block operators and straddling slots of one site, and the solver's
    Krylov basis (krylov + 1 site vectors) plus ~20 site tensors of gauge-move and GEMM staging."""
    from .engine import canonical_terms
    l, d, chi = int(para["l"]), int(para["d"]), int(para["chi"])
    dims = [min(chi, d ** min(b, l - b, 60)) for b in range(l + 1)]
    _, two = canonical_terms(para["index1"], para["coeff1"], para["index2"], para["coeff2"], para["op"],
                             para.get("eigs_tol", 1e-12))
    jmax, imin = {}, {}
    for i, j, a, b, c in two:
        jmax[(i, a)] = max(jmax.get((i, a), -1), j)
        imin[(j, b)] = min(imin.get((j, b), l), i)
    nl = np.zeros(l + 2)
    for (i, a), j in jmax.items():      # open on the left at bonds i+1..j
        nl[i + 1] += 1
        nl[j + 1] -= 1
    nr = np.zeros(l + 2)
    for (j, b), i in imin.items():      # open on the right at bonds i+1..j
        nr[i + 1] += 1
        nr[j + 1] -= 1
    nl, nr = np.cumsum(nl)[: l + 1], np.cumsum(nr)[: l + 1]
    mps = sum(dims[q] * d * dims[q + 1] for q in range(l))
    env = sum((2 + nl[b] + nr[b]) * dims[b] ** 2 for b in range(l + 1))
    cmax = max(dims)
    site = d * cmax * cmax
    strad = int(max(min(nl[b], nr[b + 1]) for b in range(l))) if l > 1 else 0
    scratch = 2 * (d * cmax) ** 2 + 2 * strad * cmax * cmax + (krylov + 1 + 20) * site
    return int(8 * (mps + env + scratch))


def pow2_scaled(tensors):
    """The random tensors of a job, each scaled by the power of two nearest 1 / sqrt(its size). A
    Gaussian site multiplies the norm of the state by ~sqrt(size), so centring a long chain at large
    chi would carry ~724^N on the centre (chi = 512) and overflow FP64 beyond ~100 sites; a
    power-of-two scaling is exact, leaves every QR factor Q bit for bit as it was and only rescales
    the state, which the first local solve normalises."""
    out = []
    for t in tensors:
        e = int(np.round(0.5 * np.log2(max(t.size, 1))))
        out.append(np.ldexp(t, -e))
    return out


class DMRGJob:
    """One DMRG run advanced one local update at a time (`advance`)."""

    def __init__(self, job_id, para, seed, arrival=0.0):
        self.job_id = job_id
        self.para = para
        self.seed = int(seed)
        self.arrival = float(arrival)
        self.result = None
        self.admitted = None
        self.finished = None
        self.solves = 0
        self.stream = None
        self._steps = None
        self.A = None

    def footprint_bytes(self):
        """Upper estimate of the device memory the job holds while admitted (estimate_device_bytes),
        computed once from its coupling lists."""
        if getattr(self, "_footprint", None) is None:
            self._footprint = estimate_device_bytes(self.para)
        return self._footprint

    def start(self, device):
        import torch
        from .MPSClass import MpsOpenBoundaryClass as Mob
        if str(device).startswith("cuda"):
            self.stream = torch.cuda.Stream(device=device)
        with self._on_stream():
            from .MPSClass import random_open_mps
            np.random.seed(self.seed)
            p = self.para
            tensors = pow2_scaled(random_open_mps(p["l"], p["d"], p["chi"]))
            self.A = Mob(length=p["l"], d=p["d"], chi=p["chi"], operators=p["op"], device=p.get("device", device),
                         precision=p.get("precision", "fp64"), tensors=tensors)
            self.A.correct_orthogonal_center(p["ob_position"])
        self._steps = self._run()

    def _on_stream(self):
        if self.stream is None:
            return contextlib.nullcontext()
        import torch
        return torch.cuda.stream(self.stream)

    def _run(self):
        """The sweeps of dmrg_finite_size (DMRG_anyH.py:47-77), yielding after every local update."""
        p, A = self.para, self.A
        l = p["l"]
        e0 = 0.0
        conv = 1.0
        out = {}
        schedule = p.get("chi_schedule")
        for t in range(p["sweep_time"]):
            if schedule:
                A.grow_bond_dimension(int(schedule[min(t, len(schedule) - 1)]), noise=p.get("chi_noise", 1e-3),
                                      method=p.get("chi_growth", "expand"),
                                      model=(p["index1"], p["index2"], p["coeff1"], p["coeff2"], p["eigs_tol"]),
                                      seed=t)
            order = list(range(p["ob_position"] + 1, l)) + list(range(l - 2, -1, -1)) + \
                list(range(1, p["ob_position"]))
            for k, n in enumerate(order):
                if k == len(order) - 1:
                    A.refine_next_solve()
                A.update_tensor_eigs(n, p["index1"], p["index2"], p["coeff1"], p["coeff2"], p["tau"], p["is_real"],
                                     tol=p["eigs_tol"])
                self.solves += 1
                yield False
            if ((t + 1) % p["dt_ob"] == 0) or t == p["sweep_time"] - 1:
                eb = A.observe_bond_energy(p["index2"], p["coeff2"])
                mx = A.observe_magnetization(1)
                mz = A.observe_magnetization(3)
                e = float((np.sum(eb) - p["hx"] * np.sum(mx) - p["hz"] * np.sum(mz)) / l)
                out = {"e_per_site": e, "eb_full": np.ravel(eb), "mx": np.ravel(mx), "mz": np.ravel(mz),
                       "sweeps": t + 1}
                conv = abs(e - e0)
                e0 = e
                if conv < p["break_tol"]:
                    break
        out["convergence"] = conv
        out["solves"] = self.solves
        self.result = out
        yield True

    def advance(self):
        """One local update (or the final observation); True once the result is ready."""
        with self._on_stream():
            done = next(self._steps)
        if done:
            self.A = None  # release the device tensors
            self._steps = None
        return done


class Scheduler:
    """Admission by device-memory budget and round-robin interleaving of admitted jobs."""

    def __init__(self, device="cuda", budget_bytes=None, max_active=64, workers=1):
        self.device = device
        self.budget = budget_bytes
        self.max_active = int(max_active)
        self.workers = max(1, int(workers))
        self.pending = []
        self.done = []
        self.max_concurrent = 0
        self._lock = threading.Lock()
        self._closed = False
        self._t0 = None

    def submit(self, job):
        """Queue a job; safe to call from any thread. While run(wait=True) executes, a job submitted
        with arrival=None is stamped with its submission time and admitted as slots and memory
        allow (latency is measured from that time)."""
        with self._lock:
            if job.arrival is None and self._t0 is not None:
                job.arrival = time.perf_counter() - self._t0
            self.pending.append(job)

    def close(self):
        """No more submissions: run(wait=True) returns once every submitted job has finished."""
        with self._lock:
            self._closed = True

    def _take_new(self, pending):
        """Submissions made since the last call, merged into the arrival-ordered pending list."""
        with self._lock:
            new, self.pending = self.pending, []
        if new:
            for j in new:
                if j.arrival is None:
                    j.arrival = time.perf_counter() - self._t0
            pending = sorted(pending + new, key=lambda j: (j.arrival, j.job_id))
        return pending

    def _open(self, wait):
        with self._lock:
            return wait and not self._closed

    def _budget(self):
        if self.budget is not None:
            return int(self.budget)
        if str(self.device).startswith("cuda"):
            import torch
            free, _ = torch.cuda.mem_get_info(torch.device(self.device))
            return int(0.8 * free)
        return 1 << 62

    def run(self, wait=False):
        """Runs every submitted job; returns the finished jobs in completion order. wait=True keeps
        accepting submissions (from other threads) until close() has been called."""
        if self.workers > 1:
            return self._run_threaded(wait)
        budget = self._budget()
        self._t0 = t0 = time.perf_counter()
        pending = self._take_new([])
        active, used = [], 0
        while pending or active or self._open(wait):
            pending = self._take_new(pending)
            now = time.perf_counter() - t0
            # admit in arrival order while the budget allows (a job larger than the whole budget
            # runs alone)
            while pending and pending[0].arrival <= now and len(active) < self.max_active:
                fp = pending[0].footprint_bytes()
                if active and used + fp > budget:
                    break
                job = pending.pop(0)
                job.admitted = time.perf_counter() - t0
                job.start(self.device)
                active.append(job)
                used += fp
            self.max_concurrent = max(self.max_concurrent, len(active))
            if not active:
                time.sleep(max(0.0, min(pending[0].arrival - now, 0.01)) if pending else 0.001)
                continue
            for job in list(active):
                if job.advance():
                    job.finished = time.perf_counter() - t0
                    active.remove(job)
                    used -= job.footprint_bytes()
                    self.done.append(job)
        return self.done

    def _run_threaded(self, wait=False):
        """run() with `workers` host threads: admission as in run() (on this thread, which also
        builds each admitted job's MPS, so the global RNG draws stay in admission order); every
        admitted job has one local update (a task) in flight at a time on the pool. The library's
        calls release the GIL, so while one thread waits inside a job's Lanczos convergence check,
        the others run their jobs' host code and queue their kernels on their own streams."""
        from concurrent.futures import FIRST_COMPLETED, ThreadPoolExecutor
        from concurrent.futures import wait as wait_any
        budget = self._budget()
        self._t0 = t0 = time.perf_counter()
        pending = self._take_new([])
        active, used, inflight = [], 0, {}
        with ThreadPoolExecutor(max_workers=self.workers) as pool:
            while pending or active or self._open(wait):
                pending = self._take_new(pending)
                now = time.perf_counter() - t0
                while pending and pending[0].arrival <= now and len(active) < self.max_active:
                    fp = pending[0].footprint_bytes()
                    if active and used + fp > budget:
                        break
                    job = pending.pop(0)
                    job.admitted = time.perf_counter() - t0
                    job.start(self.device)
                    active.append(job)
                    used += fp
                    inflight[pool.submit(job.advance)] = job
                self.max_concurrent = max(self.max_concurrent, len(active))
                if not active:
                    time.sleep(max(0.0, min(pending[0].arrival - now, 0.01)) if pending else 0.001)
                    continue
                # wake up for the next arrival (or, while open, for new submissions) while jobs run
                if pending:
                    wake = max(0.0, min(pending[0].arrival - (time.perf_counter() - t0), 0.01))
                else:
                    wake = 0.005 if self._open(wait) else None
                finished, _ = wait_any(list(inflight), timeout=wake, return_when=FIRST_COMPLETED)
                for f in finished:
                    job = inflight.pop(f)
                    if f.result():   # a job's exception is raised here
                        job.finished = time.perf_counter() - t0
                        active.remove(job)
                        used -= job.footprint_bytes()
                        self.done.append(job)
                    else:
                        inflight[pool.submit(job.advance)] = job
        return self.done

    def summary(self):
        lat = np.array([j.finished - j.arrival for j in self.done]) if self.done else np.zeros(1)
        span = max((j.finished for j in self.done), default=0.0)
        solves = sum(j.solves for j in self.done)
        return {"jobs": len(self.done), "solves": solves, "wall_s": span,
                "solves_per_s": solves / span if span > 0 else 0.0,
                "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
                "max_concurrent": self.max_concurrent}


def make_jobs(njobs, seed=0, sweeps=4, precision="fp64", device="cuda", rate=None, lengths=(16, 48),
              chis=(16, 32, 64), ladder_fraction=0.0, ladder_lengths=(8, 48), rung=(0.5, 2.0)):
    """Uneven XXZ chains: N ~ U{lengths}, Jz ~ U[0,2], hz ~ U[0,1], chi from `chis`, per-job seed =
    seed + job id; Poisson arrivals at `rate` per second (all at time 0 when rate is None).
    With ladder_fraction > 0 that share of the jobs are 2 x L ladders instead (L ~ U{ladder_lengths},
    rung coupling ~ U[rung]), as in the mixed chain/ladder request stream of the serving workload;
    ladder_fraction = 0 draws exactly the chains it always did."""
    rng = np.random.default_rng(seed)
    arrivals = np.random.default_rng(seed + 1)  # its own stream: the jobs do not depend on the rate
    kinds = np.random.default_rng(seed + 2)     # chain or ladder, drawn only when ladders are asked for
    jobs, t = [], 0.0
    for k in range(njobs):
        if rate:
            t += arrivals.exponential(1.0 / rate)
        if ladder_fraction > 0 and kinds.uniform() < ladder_fraction:
            para = ladder_job_para(int(kinds.integers(ladder_lengths[0], ladder_lengths[1] + 1)),
                                   int(kinds.choice(chis)), j_rung=float(kinds.uniform(*rung)),
                                   jz=float(kinds.uniform(0, 2)), hz=float(kinds.uniform(0, 1)), sweeps=sweeps,
                                   precision=precision, device=device)
        else:
            para = chain_job_para(int(rng.integers(lengths[0], lengths[1] + 1)), int(rng.choice(chis)),
                                  jz=float(rng.uniform(0, 2)), hz=float(rng.uniform(0, 1)), sweeps=sweeps,
                                  precision=precision, device=device)
        jobs.append(DMRGJob(k, para, seed + k, arrival=t))
    return jobs


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--jobs", type=int, default=16)
    ap.add_argument("--sweeps", type=int, default=4)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--rate", type=float, default=None)
    ap.add_argument("--precision", default="fp64")
    ap.add_argument("--max-active", type=int, default=64)
    ap.add_argument("--ladders", type=float, default=0.0, help="share of 2 x L ladder jobs (0..1)")
    ap.add_argument("--baseline-precision", default=None,
                    help="precision of the one-at-a-time pass (default: --precision); fp64 compares the mix "
                         "with sequential plain FP64 solves")
    ap.add_argument("--device", default="cuda")
    ap.add_argument("--workers", type=int, default=1,
                    help="host threads advancing the interleaved jobs (1: one thread, round robin)")
    ap.add_argument("--no-sequential", action="store_true", help="skip the one-at-a-time pass")
    ap.add_argument("--lengths", default="16,48", help="chain length range N (ladders get half as many rungs)")
    ap.add_argument("--chis", default="16,32,64", help="bond dimensions to draw from")
    ap.add_argument("--ladder-rungs", default=None, help="rung range L of the 2 x L ladders (default: half of --lengths)")
    a = ap.parse_args(argv)
    lengths = tuple(int(x) for x in a.lengths.split(","))
    chis = tuple(int(x) for x in a.chis.split(","))
    rungs = (tuple(int(x) for x in a.ladder_rungs.split(",")) if a.ladder_rungs else
             (max(2, lengths[0] // 2), max(2, lengths[1] // 2)))
    shape = dict(lengths=lengths, chis=chis, ladder_fraction=a.ladders, ladder_lengths=rungs)
    import torch
    from . import _lib as L
    L.load()
    dev = a.device
    base_prec = a.baseline_precision or a.precision

    def sync():
        if str(dev).startswith("cuda"):
            torch.cuda.synchronize()
    # warm-up: builds, tensor maps, first-launch costs
    warm = Scheduler(dev)
    for prec in sorted({a.precision, base_prec}):
        for j in make_jobs(2, seed=a.seed + 10 ** 6, sweeps=1, precision=prec, device=dev, lengths=lengths, chis=chis):
            warm.submit(j)
    warm.run()
    sync()
    # the same jobs one at a time (in the baseline precision), then interleaved
    seq_wall, seq = 0.0, {}
    seq_lat = []
    for j in ([] if a.no_sequential else
              make_jobs(a.jobs, seed=a.seed, sweeps=a.sweeps, precision=base_prec, device=dev, **shape)):
        j.arrival = 0.0
        s = Scheduler(dev, max_active=1)
        s.submit(j)
        t0 = time.perf_counter()
        s.run()
        sync()
        seq_wall += time.perf_counter() - t0
        seq_lat.append(seq_wall)   # latency of job k when the jobs arrive together and run in turn
        seq[j.job_id] = j
    mix = Scheduler(dev, max_active=a.max_active, workers=a.workers)
    for j in make_jobs(a.jobs, seed=a.seed, sweeps=a.sweeps, precision=a.precision, device=dev, rate=a.rate,
                       **shape):
        mix.submit(j)
    mix.run()
    sync()
    out = mix.summary()
    out.update({"precision": a.precision, "baseline_precision": base_prec, "sweeps": a.sweeps, "rate_per_s": a.rate,
                "ladder_fraction": a.ladders, "lengths": list(lengths), "chis": list(chis), "workers": a.workers})
    if seq:
        solves = sum(j.solves for j in seq.values())
        out.update({"sequential_wall_s": seq_wall, "sequential_solves_per_s": solves / seq_wall,
                    "sequential_latency_p50_s": float(np.percentile(seq_lat, 50)),
                    "sequential_latency_p99_s": float(np.percentile(seq_lat, 99)),
                    "speedup_vs_sequential": out["solves_per_s"] / (solves / seq_wall) if seq_wall else None,
                    "max_abs_de_per_site_mix_vs_alone": max(abs(j.result["e_per_site"] -
                                                                seq[j.job_id].result["e_per_site"]) for j in mix.done)})
    out["e_per_site"] = {str(j.job_id): j.result["e_per_site"] for j in mix.done}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
