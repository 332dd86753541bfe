#!/usr/bin/env python
"""Benchmark of the finite-size DMRG sweep on one GB300.

Workload (one "step" = one full sweep, 2(L-1) local solves with their gauge moves and
environment updates): spin-1/2 Heisenberg open chain, N=100, J=1, d=2, seeded
random-normal initial MPS, chi ramped 64 -> 256 -> 512 during the warm-up sweeps, timed
sweeps at chi=512. Synthetic input of the stated shapes; no dataset is involved.

    python bench.py [--steps K] [--warmup W] [--precision tf32x3|fp64] [--impl ours|reference] [--no-legs]

Prints ONE JSON line. `value` = sweeps/s (inputs resident in HBM), `e2e` = sweeps/s of a full
dmrg_finite_size() job from host inputs (ramp included, final MPS copied back to the host),
`cpu_baseline` = the reference's local update (oracle/: numpy + scipy ARPACK) measured on the host
cores on the converged state of the timed sweeps. At one GPU the workload legs follow (child
processes, one shared time budget; a failure is reported in the line): chain_n12_chi16 = N=12, chi=16,
10 sweeps in full on the CPU port and the GPU path; chain_n100_chi512 = N=100, chi 64 -> 256 -> 512
over 8 sweeps, mixed against the plain FP64 GPU path; j1j2_6x6_chi512 = J1-J2 6x6 in snake order, 10
sweeps at chi=512, mixed against FP64; batched_512_xxz = 512 uneven XXZ chains advanced together
(tnalg_gb300.batched) against the same jobs one at a time on the FP64 path; serving_stream = a
Poisson stream of chain and ladder requests at several rates. `summary` (the last key) gathers
the figures the metric is quoted on.
`--impl reference` times the reference's algorithm (oracle/) on the host cores, on a seeded random
state whose interior site is converged first: W untimed and K timed steps, one step = one local
update of the sweep (eigsh + centre move), so `ms_per_step` is the measured time of one step and
`value` = 1 / (2(N-1) x ms_per_step) sweeps/s.
"""
import argparse
import contextlib
import io
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DMRG sweeps/s (N=100 Heisenberg chain, chi=512)"
UNIT = "sweeps/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default=os.environ.get("TNALG_BENCH_PRECISION", "auto"))
    p.add_argument("--length", type=int, default=100)
    p.add_argument("--chi", type=int, default=512)
    p.add_argument("--ramp", default="64,256")
    p.add_argument("--eigs-tol", type=float, default=1e-12)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-solves", type=int, default=2)
    p.add_argument("--no-legs", action="store_true",
                   help="skip the workload legs (N=12 chain in full, N=100 chain and J1-J2 6x6 mixed vs FP64, "
                        "batched jobs, serving)")
    return p.parse_args()


def chain_para(length, chi, eigs_tol, precision="fp64", device="cuda"):
    from tnalg_gb300 import Parameters as pm
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=length, chi=chi, jxy=1, jz=1, hx=0, hz=0, tau=1e-4, eigs_tol=eigs_tol, break_tol=-1.0)
    para = pm.make_consistent_parameter_dmrg(para)
    para.update(precision=precision, device=device)
    return para


# ---------------------------------------------------------------------------------------
# clocks sampler (nvidia-smi during the timed region)


class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, nm in enumerate(names):
                    if r[5 + k].lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------------------
# our arm


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def max_over_ranks(ms, world, device):
    """Slowest rank's timed-region duration (replicas: every rank runs its own job)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, steps, max_ms):
    """Whole-job sweeps/s of `world` independent replicas that each ran `steps` sweeps, timed by the
    slowest one."""
    return world * steps / (max_ms / 1000.0)


def run_ours(args, rank, world, local_rank):
    import torch
    from tnalg_gb300 import _lib as L, build
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    if not os.path.exists(L.LIB_PATH):
        build.build()
    L.load()
    torch.cuda.set_device(local_rank)
    dev = "cuda:%d" % local_rank
    precision = args.precision
    if precision == "auto":
        precision = "tf32x3" if L.tf32x3_available() else "fp64"
    ramp = [int(x) for x in args.ramp.split(",") if x]
    para = chain_para(args.length, ramp[0] if ramp else args.chi, args.eigs_tol, precision, dev)
    np.random.seed(1000 * rank)
    A = MpsOpenBoundaryClass(para["l"], para["d"], para["chi"], operators=para["op"], device=dev,
                             precision=precision)
    A.correct_orthogonal_center(0)
    L_ = para["l"]
    order = list(range(1, L_)) + list(range(L_ - 2, -1, -1))

    def sweep():
        for k, n in enumerate(order):
            if k == len(order) - 1:
                A.refine_next_solve()
            A.update_tensor_eigs(n, para["index1"], para["index2"], para["coeff1"], para["coeff2"], para["tau"],
                                 True, tol=para["eigs_tol"])

    schedule = ramp + [args.chi]
    warm = max(args.warmup, len(schedule))
    model = (para["index1"], para["index2"], para["coeff1"], para["coeff2"], para["eigs_tol"])
    for t in range(warm):
        A.grow_bond_dimension(schedule[min(t, len(schedule) - 1)], seed=t, method="expand", model=model)
        sweep()
    if A.virtual_dim.max() < min(args.chi, 2 ** (L_ // 2)):
        A.grow_bond_dimension(args.chi, seed=warm, method="expand", model=model)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    lib = L.load()
    lib.tn_profile_enable(1)
    lib.tn_profile_reset()
    solves0, mv0 = A.stats["solves"], A.stats["matvecs"]
    launches0 = L.launch_count()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local_rank) as clk:
        torch.cuda.synchronize()
        # cudaProfilerStart/Stop bracket the timed sweeps (no-ops without a profiler): a
        # `ncu --profile-from-start off` launch list then holds exactly these launches.
        torch.cuda.profiler.start()
        start.record()
        t0 = time.time()
        for _ in range(args.steps):
            sweep()
        stop.record()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        wall = time.time() - t0
    ms = start.elapsed_time(stop)
    launches = L.launch_count() - launches0
    mv_ms, mv_cnt, mv_flops = L.profile_read(0)
    qr_ms, qr_cnt, qr_flops = L.profile_read(1)
    lz_ms, lz_cnt, _ = L.profile_read(4)
    lib.tn_profile_enable(0)
    ms = max_over_ranks(ms, world, dev)
    solves = A.stats["solves"] - solves0
    matvecs = A.stats["matvecs"] - mv0
    # final energy of the timed state (FP64 observables)
    eb = A.observe_bond_energy(para["index2"], para["coeff2"])
    e_site = float(np.sum(eb)) / L_
    res = {"ms": ms, "wall": wall, "solves": solves, "matvecs": matvecs, "mv_ms": mv_ms, "mv_cnt": mv_cnt,
           "mv_flops": mv_flops, "qr_ms": qr_ms, "qr_cnt": qr_cnt, "qr_flops": qr_flops, "lz_ms": lz_ms,
           "lz_cnt": lz_cnt, "precision": precision, "e_per_site": e_site, "eb_full": np.ravel(eb),
           "clocks": clk.summary(),
           "launches": launches, "chi_max": int(A.virtual_dim.max())}
    return res, A, para


def run_e2e(args, dev, precision):
    """One full dmrg_finite_size() job from host inputs: ramp + timed schedule, MPS copied back."""
    import torch
    from tnalg_gb300 import DMRG_anyH
    ramp = [int(x) for x in args.ramp.split(",") if x]
    schedule = ramp + [args.chi] * max(1, args.steps)
    para = chain_para(args.length, schedule[0], args.eigs_tol, precision, dev)
    para.update(sweep_time=len(schedule), chi_schedule=schedule, dt_ob=len(schedule))
    np.random.seed(0)
    torch.cuda.synchronize()
    t0 = time.time()
    with contextlib.redirect_stdout(io.StringIO()):
        ob, A, info, _ = DMRG_anyH.dmrg_finite_size(para)
        host = A.mps  # device -> host copy of the final MPS
    torch.cuda.synchronize()
    wall = time.time() - t0
    d2h = sum(t.nbytes for t in host)
    h2d = sum(t.nbytes for t in _initial_host_mps(args.length, 2, schedule[0]))
    return {"value": len(schedule) / wall, "unit": UNIT, "h2d_bytes_per_step": int(h2d / len(schedule)),
            "d2h_bytes_per_step": int(d2h / len(schedule)), "sweeps": len(schedule), "wall_s": wall,
            "e_per_site": float(ob["e_per_site"])}


def _initial_host_mps(l, d, chi):
    return [np.zeros((1, d, chi))] + [np.zeros((chi, d, chi))] * (l - 2) + [np.zeros((chi, d, 1))]


# ---------------------------------------------------------------------------------------
# CPU restatement (oracle) timing: measured local updates of the bench workload


def cpu_info():
    """Host cores, CPU model and the BLAS numpy calls (the reference's dgemm/LAPACK)."""
    model = ""
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu part", "hardware")):
                    model = ln.split(":", 1)[1].strip()
                    break
    except Exception:
        pass
    blas = "unknown"
    try:
        cfg = np.__config__.CONFIG["Build Dependencies"]["blas"]
        blas = "%s %s" % (cfg.get("name", ""), cfg.get("version", ""))
    except Exception:
        pass
    try:
        import torch
        threads = torch.get_num_threads()
    except Exception:
        threads = os.cpu_count()
    return {"nproc": os.cpu_count(), "threads": threads, "cpu": model, "blas": blas.strip()}


def cpu_sample(length, chi, eigs_tol, steps, warmup=0, mps=None, seed=0):
    """The reference's local update timed on the host cores (oracle/: numpy + scipy ARPACK, the
    reference's algorithm and bookkeeping) on the two interior sites mid, mid + 1 of the N-site
    chain at `chi`. One step is one local update of a sweep, as update_tensor_eigs and the gauge
    move that follows it run in DMRG_anyH.py:43-64:
      eigsh at the current centre site (started from its own tensor; ARPACK builds at least its
      ncv = 20 vectors), then the move of the orthogonality centre to the other site with the
      rebuild of that site's operator buckets (the QR move and the transfers of every carried term
      the move invalidated).
    The centre goes back and forth across the bond (mid, mid + 1), so every step is a genuine
    interior local update; `warmup` steps run untimed, then `steps` are timed one by one. A sweep
    is 2(N-1) local updates, so sweeps/s = 1 / (2(N-1) x mean step time): measured, nothing
    assumed. `mps`: the host tensors of a converged state (the benchmark's own, after its timed
    sweeps); without it a seeded random MPS, whose site an untimed first solve converges."""
    from oracle import dmrg_oracle as O
    para = chain_para(length, chi, eigs_tol, "fp64", "cpu")
    if mps is None:
        np.random.seed(seed)
        A = O.OracleMPS(length, 2, chi, para["op"])
    else:
        A = O.OracleMPS(length, 2, chi, para["op"], mps=mps)
    one, two = O.canonical_terms(para["index1"], para["coeff1"], para["index2"], para["coeff2"], A.ops, eigs_tol)
    mid = length // 2 - 1
    t0 = time.time()
    A.correct_orthogonal_center(mid)
    A.site_buckets(mid, one, two)
    A.update_tensor_eigs(mid, one, two, 1e-4, eigs_tol)
    t_setup = time.time() - t0
    site = [mid]

    def local_update():
        p = site[0]
        mv0 = A.n_matvec
        t = time.time()
        A.update_tensor_eigs(p, one, two, 1e-4, eigs_tol)
        t_solve = time.time() - t
        q = mid + 1 if p == mid else mid
        t = time.time()
        A.correct_orthogonal_center(q)
        A.site_buckets(q, one, two)
        site[0] = q
        return t_solve, time.time() - t, A.n_matvec - mv0

    for _ in range(max(0, warmup)):
        local_update()
    rows = [local_update() for _ in range(max(1, steps))]
    solve_s = float(np.mean([r[0] for r in rows]))
    move_s = float(np.mean([r[1] for r in rows]))
    per_step = solve_s + move_s
    sweeps_per_s = 1.0 / (per_step * 2 * (length - 1))
    info = cpu_info()
    return {"value": sweeps_per_s, "unit": UNIT, "cores": info["threads"], "kind": "port",
            "cpu": info, "steps": len(rows), "warmup": max(0, warmup), "ms_per_step": 1000.0 * per_step,
            "solve_s": solve_s, "move_s": move_s, "matvecs_per_solve": float(np.mean([r[2] for r in rows])),
            "sample": "oracle (numpy/scipy ARPACK restatement of the reference) on %d host threads, N=%d chain at "
                      "chi=%d, %s state: %d timed local updates (after %d untimed) back and forth across interior "
                      "bond (%d, %d): eigsh solve %.2f s (%.0f matvecs) + centre move with its operator rebuild "
                      "%.2f s per update, measured; sweeps/s = 1 / (2(N-1) x %.2f s); %.0f s untimed setup" % (
                          info["threads"], length, chi, "converged (the GPU run's)" if mps is not None else
                          "seeded random", len(rows), max(0, warmup), mid, mid + 1, solve_s,
                          float(np.mean([r[2] for r in rows])), move_s, per_step, t_setup)}


def small_chain_leg(device):
    """The N=12 Heisenberg chain in full: chi=16, seed 0, 10 sweeps (break_tol=-1),
    eigs_tol 1e-12, on the oracle (the reference's numpy/scipy path, host cores) and on the GPU
    path (dmrg_finite_size, FP64 and split TF32); sweeps/s, solves/s and the energy against exact
    diagonalisation."""
    import torch
    from oracle import dmrg_oracle as O
    from oracle import ed as ED
    from tnalg_gb300 import DMRG_anyH
    para = chain_para(12, 16, 1e-12, "fp64", device)
    para.update(sweep_time=10, dt_ob=1, break_tol=-1.0)
    e0 = float(ED.ground_state(12, 2, para["op"], para["index1"], para["coeff1"], para["index2"],
                               para["coeff2"])[0]) / 12
    out = {"workload": "N=12 Heisenberg chain, chi=16, 10 sweeps, seed 0", "ed_e_per_site": e0}
    t = time.time()
    ob, _, _ = O.dmrg_finite_size(12, 2, 16, para["op"], para["index1"], para["coeff1"], para["index2"],
                                  para["coeff2"], para["positions_h2"], tau=1e-4, eigs_tol=1e-12, sweep_time=10,
                                  hx=0.0, hz=0.0, seed=0)
    w = time.time() - t
    out["cpu_port"] = {"sweeps_per_s": 10 / w, "solves_per_s": 10 * 22 / w, "wall_s": w,
                       "abs_de_per_site_vs_ed": abs(ob["e_per_site"] - e0), "cores": cpu_info()["threads"]}
    for prec in ("fp64", "tf32x3"):
        q = dict(para)
        q["precision"] = prec
        np.random.seed(0)
        torch.cuda.synchronize()
        t = time.time()
        with contextlib.redirect_stdout(io.StringIO()):
            obg, _, info, _ = DMRG_anyH.dmrg_finite_size(q)
        torch.cuda.synchronize()
        w = time.time() - t
        out["gpu_" + prec] = {"sweeps_per_s": 10 / w, "solves_per_s": info["solves"] / w, "wall_s": w,
                              "abs_de_per_site_vs_ed": abs(obg["e_per_site"] - e0),
                              "abs_de_per_site_vs_cpu_port": abs(obg["e_per_site"] - ob["e_per_site"])}
    return out


LEGS_BUDGET_S = 960   # the child legs together (normally ~10-12 minutes)
CHAIN_ARGS = ["chain", "--length", "100", "--chi", "512", "--ramp", "64,256", "--steps", "6"]
LATTICE_ARGS = ["j1j2", "--width", "6", "--height", "6", "--chi", "512", "--ramp", "", "--steps", "10"]
BATCH_ARGS = ["--jobs", "512", "--lengths", "16,64", "--chis", "32,64,128", "--sweeps", "8", "--baseline-jobs", "8"]
SERVING_RATES = (10.0, 100.0, 2000.0)
SERVING_ARGS = ["--jobs", "24", "--lengths", "16,128", "--ladders", "0.5", "--ladder-rungs", "8,48",
                "--chis", "32,64,128,256,512", "--sweeps", "6"]


def run_lattice_leg(args_list, precision, timeout):
    """A one-job workload (tnalg_gb300.run_lattice) in a child process, on `precision` and then on
    the plain FP64 GPU path from the same seed and schedule."""
    cmd = [sys.executable, "-m", "tnalg_gb300.run_lattice"] + args_list + ["--precision", precision]
    if precision != "fp64":
        cmd.append("--compare-fp64")
    return _child_json(cmd, timeout)


def run_batch_leg(extra, precision, timeout):
    """The batched engine (tnalg_gb300.batched) in a child process."""
    cmd = [sys.executable, "-m", "tnalg_gb300.batched"] + extra + ["--precision", precision]
    return _child_json(cmd, timeout)


def _child_json(cmd, timeout):
    """Run `cmd` (python -m ...) from the repository root; its last JSON line, or an error entry."""
    shown = "python " + " ".join(c if c else '""' for c in cmd[1:])
    if timeout < 20:
        return {"skipped": "the legs' %d s time budget was spent" % LEGS_BUDGET_S, "command": shown}
    try:
        p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout)
        lines = [x for x in p.stdout.splitlines() if x.startswith("{")]
        if p.returncode != 0 or not lines:
            tail = (p.stderr or p.stdout or "").strip().splitlines()[-1:]
            return {"error": "exit %d: %s" % (p.returncode, tail[0][:300] if tail else ""), "command": shown}
        out = json.loads(lines[-1])
        out["command"] = shown
        return out
    except Exception as e:  # timeout or unparsable output: report, keep the benchmark line
        return {"error": repr(e)[:300], "command": shown}


def _pick(d, keys):
    return {k: d[k] for k in keys if isinstance(d, dict) and k in d}


def summarise(line):
    """The figures the metric is quoted on, gathered in one compact object (last key of the line)."""
    out = {}
    c1 = line.get("chain_n12_chi16")
    if isinstance(c1, dict) and "cpu_port" in c1:
        out["chain_n12_chi16"] = {"cpu_port_sweeps_per_s": c1["cpu_port"]["sweeps_per_s"],
                                    "gpu_fp64_sweeps_per_s": c1.get("gpu_fp64", {}).get("sweeps_per_s"),
                                    "gpu_tf32x3_sweeps_per_s": c1.get("gpu_tf32x3", {}).get("sweeps_per_s"),
                                    "abs_de_per_site_vs_ed": {k: c1[k]["abs_de_per_site_vs_ed"] for k in
                                                              ("cpu_port", "gpu_fp64", "gpu_tf32x3") if k in c1}}
    for key, name in (("chain_n100_chi512", "chain_n100_chi512_8sweeps"), ("j1j2_6x6_chi512", "j1j2_6x6_chi512_10sweeps")):
        c = line.get(key)
        if isinstance(c, dict) and "fp64_path" in c:
            out[name] = {"speedup_vs_fp64": c["speedup_vs_fp64"], "abs_de_per_site_vs_fp64": c["abs_de_per_site_vs_fp64"],
                         "max_abs_d_term_energy_vs_fp64": c.get("max_abs_d_term_energy_vs_fp64"),
                         "sweeps_per_s": c["sweeps_per_s"], "fp64_sweeps_per_s": c["fp64_path"]["sweeps_per_s"],
                         "matvecs_per_solve": c["matvecs_per_solve"],
                         "fp64_matvecs_per_solve": c["fp64_path"]["matvecs_per_solve"]}
        elif isinstance(c, dict):
            out[name] = _pick(c, ["error", "skipped"])
    c4 = line.get("batched_512_xxz")
    if isinstance(c4, dict):
        out["batched_512_xxz_chains"] = _pick(c4, ["solves_per_s", "speedup_vs_sequential", "latency_p50_s",
                                                "latency_p99_s", "max_abs_de_per_site_vs_sequential", "jobs",
                                                "unconverged_solves", "error", "skipped"])
        if "sequential" in c4:
            out["batched_512_xxz_chains"]["sequential_fp64_solves_per_s"] = c4["sequential"]["solves_per_s"]
    c5 = line.get("serving_stream")
    if isinstance(c5, list):
        out["serving_poisson_stream"] = [_pick(r, ["rate_per_s", "solves_per_s", "latency_p50_s", "latency_p99_s",
                                            "speedup_vs_sequential", "max_abs_de_per_site_vs_sequential",
                                            "max_concurrent", "error", "skipped"]) for r in c5]
    return out


def run_reference(args, rank):
    if rank != 0:
        return None
    s = cpu_sample(args.length, args.chi, args.eigs_tol, max(1, args.steps), warmup=args.warmup)
    # one step = one measured local update of the sweep (a bounded sample of it): ms_per_step is the
    # time of that step, value the sweeps/s it gives (a sweep is 2(N-1) local updates)
    line = {"metric": METRIC, "value": s["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": s["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "step": "one local update of the sweep (eigsh at a converged interior site + the centre move with its "
                    "operator rebuild); sweeps/s = 1 / (2(N-1) x ms_per_step)",
            "config": {"workload": "N=%d spin-1/2 Heisenberg open chain, J=1, chi=%d, one-site DMRG sweep"
                                   % (args.length, args.chi), "global_batch": 1, "seq_len": args.length,
                       "parallelism": "replicas"},
            "cpu_baseline": s, "e2e": {"value": s["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                       "d2h_bytes_per_step": 0}}
    return line


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        line = run_reference(args, rank)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    res, A, para = run_ours(args, rank, world, local_rank)
    pk, pk_kind = peaks()
    ms_step = res["ms"] / args.steps
    value = replica_throughput(world, args.steps, res["ms"])
    mixed = res["precision"] != "fp64"
    if mixed:
        peak = pk["bf16_tflops_sustained"] / 2.0 / 3.0
        peak_note = "3xTF32 useful-flop peak = measured sustained bf16 / 2 (tf32 rate) / 3 products"
    else:
        peak = 1.25
        peak_note = "nominal GB300 FP64 1.25 TFLOP/s (no FP64 entry in MEASURED_PEAKS.json)"

    def kernel_roofline(name, t_ms, cnt, flops, figure):
        avg = t_ms / max(cnt, 1)
        ach = (flops / max(cnt, 1)) / (avg / 1000.0) / 1e12 if cnt and avg > 0 else 0.0
        return {"bound": "tensor" if mixed else "fp64", "kernel": name, "achieved": ach, "peak": peak,
                "unit": "TFLOP/s", "frac": ach / peak if peak else None, "traffic": None, "avg_launch_ms": avg,
                "launches": cnt, "flops_per_launch": flops / max(cnt, 1), "work_figure": figure,
                "device_ms_per_sweep": t_ms / args.steps, "peak_source": pk_kind, "peak_note": peak_note}

    mv_line = kernel_roofline("effective-Hamiltonian matvec (tcgen05 split-TF32 block GEMMs)" if mixed else
                              "effective-Hamiltonian matvec (FP64 block GEMMs)", res["mv_ms"], res["mv_cnt"],
                              res["mv_flops"], "F_mv = 2 d chil chir (chil (n_L + n_S) + chir (n_R + n_S))")
    qr_line = kernel_roofline("gauge-move QR (tn_qr_mixed: FP32 cluster QR + FP64 re-orthogonalisation)" if mixed
                              else "gauge-move QR (tn_qr: FP64 Householder)", res["qr_ms"], res["qr_cnt"],
                              res["qr_flops"], "F_qr = 2 m n^2 - 2 n^3 / 3, m = d chi, n = chi")
    if mixed:
        # DRAM traffic from the committed ncu captures of the same shapes (cold cache, one launch each)
        qr_line.update(traffic=4.41e6, traffic_kernel="qr32_cluster_kernel (the factorisation of tn_qr_mixed; 43% of "
                       "the sweep's device time in the launch list)",
                       traffic_source="profiles/qr32_cluster_1024x512_ncu.md: dram__bytes_read 4.41 MB + write 0 per "
                       "launch at 1024 x 512; the Q kernel reads 1.6 MB, the Gram 4.2 MB "
                       "(profiles/qr32_form_q_and_gram_1024x512_ncu.md)")
        mv_line.update(traffic_component={"kernel": "tf32x3_gemm_kernel (one block GEMM of the chi=512 matvec)",
                                          "dram_bytes": 16.8e6,
                                          "source": "profiles/tf32x3_gemm_matvec_chi512_ncu.md"})
    # the roofline object describes the kernel class with the most device time in the timed sweeps
    dominant, other = (qr_line, mv_line) if res["qr_ms"] > res["mv_ms"] else (mv_line, qr_line)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if not mixed else "tf32x3+f64", "data": "synthetic",
            "config": {"workload": "N=%d spin-1/2 Heisenberg open chain, J=1, d=2, one-site DMRG sweep at chi=%d "
                                   "(warm-up ramp %s)" % (args.length, args.chi, args.ramp),
                       "global_batch": world, "seq_len": args.length, "parallelism": "replicas",
                       "precision": res["precision"], "eigs_tol": args.eigs_tol,
                       "l2": "inputs larger than L2 (MPS ~%d MB + environments)" % int(
                           sum(t.numel() for t in A.mps_device) * 8 / 2 ** 20)},
            "solves_per_s": world * res["solves"] / (res["ms"] / 1000.0),
            "matvecs_per_solve": res["matvecs"] / max(res["solves"], 1),
            "e_per_site": res["e_per_site"],
            "roofline": dominant,
            "roofline_other": other,
            "device_ms_per_sweep": {"qr": res["qr_ms"] / args.steps, "lanczos_incl_matvec": res["lz_ms"] / args.steps,
                                    "matvec": res["mv_ms"] / args.steps,
                                    "rest": ms_step - (res["qr_ms"] + res["lz_ms"]) / args.steps},
            "clocks": res["clocks"], "gpu_launches": res["launches"]}
    if rank == 0 and not args.no_e2e:
        line["e2e"] = run_e2e(args, "cuda:%d" % local_rank, res["precision"])
    if rank == 0 and not args.no_cpu:
        # the reference's local update timed on the host cores, on the converged state of the timed sweeps
        host = [t.detach().cpu().numpy() for t in A.mps_device]
        line["cpu_baseline"] = cpu_sample(args.length, args.chi, args.eigs_tol, max(1, args.cpu_solves), mps=host)
        del host
    if rank == 0 and world == 1 and not args.no_legs:
        del A
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        try:
            line["chain_n12_chi16"] = small_chain_leg("cuda:%d" % local_rank)
        except Exception as e:
            line["chain_n12_chi16"] = {"error": repr(e)[:300]}
        # the child legs share one time budget, so a stuck leg cannot hold back the line
        end = time.time() + LEGS_BUDGET_S
        prec = res["precision"]
        line["chain_n100_chi512"] = run_lattice_leg(CHAIN_ARGS, prec, min(200.0, end - time.time()))
        line["j1j2_6x6_chi512"] = run_lattice_leg(LATTICE_ARGS, prec, min(330.0, end - time.time()))
        line["batched_512_xxz"] = run_batch_leg(BATCH_ARGS, prec, min(240.0, end - time.time()))
        serving = []
        for k, rate in enumerate(SERVING_RATES):
            # the sequential FP64 pass runs once, on the first jobs of the stream, capped at 40 s
            extra = SERVING_ARGS + ["--rate", str(rate), "--baseline-jobs", "4" if k == 0 else "0",
                                    "--baseline-seconds", "40"]
            r = run_batch_leg(extra, prec, min(200.0 if k == 0 else 150.0, end - time.time()))
            for drop in ("e_per_site",):
                r.pop(drop, None)
            serving.append(r)
        if serving and serving[0].get("sequential"):
            seq = serving[0]["sequential"]["solves_per_s"]
            for r in serving[1:]:
                if "solves_per_s" in r:
                    r["speedup_vs_sequential"] = r["solves_per_s"] / seq
        line["serving_stream"] = serving
    if rank == 0:
        line["summary"] = summarise(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
