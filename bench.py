#!/usr/bin/env python
"""Benchmark of the finite-size DMRG sweep on one GB300.

Workload (one "step" = one full sweep, 2(L-1) local solves with their gauge moves and
environment updates): spin-1/2 Heisenberg open chain, N=100, J=1, d=2, seeded
random-normal initial MPS, chi ramped 64 -> 256 -> 512 during the warm-up sweeps, timed
sweeps at chi=512. Synthetic input of the stated shapes; no dataset is involved.

    python bench.py [--steps K] [--warmup W] [--precision tf32x3|fp64] [--impl ours|reference]

Prints ONE JSON line. `value` = sweeps/s (inputs resident in HBM), `e2e` = sweeps/s of a full
dmrg_finite_size() job from host inputs (ramp included, final MPS copied back to the host).
On the split-TF32 path at one GPU, `fp64_path` repeats the same job (seed, ramp, timed sweeps) on
the plain FP64 GPU path: its sweeps/s, the speed-up of this line over it and the difference of
the energies per site (`--no-fp64-leg` skips it).
On one GPU, `serving` reports the many-jobs path (tnalg_gb300.serving: 16 uneven XXZ chains interleaved,
against the same jobs one at a time on the plain FP64 GPU path: solves/s, p50/p99 latency; `--no-serving`
skips it). `j1j2_6x6` reports the J1-J2 model on the 6 x 6 snake-ordered square lattice at chi=512
(tnalg_gb300.run_lattice, against the plain FP64 path; `--no-lattice` skips it). Both legs run in child
processes and report a failure in the line instead of stopping the benchmark.
`--impl reference` times the CPU restatement of the reference (oracle/, numpy + scipy ARPACK)
on a bounded sample of the same workload and extrapolates sweeps/s.
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
    p.add_argument("--no-fp64-leg", action="store_true",
                   help="skip the plain FP64 GPU run of the same job that the split-TF32 line is compared with")
    p.add_argument("--cpu-solves", type=int, default=1)
    p.add_argument("--no-serving", action="store_true",
                   help="skip the serving leg (many small jobs interleaved vs one at a time on the FP64 path)")
    p.add_argument("--no-lattice", action="store_true",
                   help="skip the J1-J2 6x6 lattice leg (chi=512, against the FP64 path)")
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
    for t in range(warm):
        A.grow_bond_dimension(schedule[min(t, len(schedule) - 1)], seed=t)
        sweep()
    if A.virtual_dim.max() < min(args.chi, 2 ** (L_ // 2)):
        A.grow_bond_dimension(args.chi, seed=warm)
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
# CPU restatement (oracle) timing: bounded sample of interior local solves at the bench chi


def cpu_sample(length, chi, eigs_tol, nsolves, seed=0):
    """Bounded CPU sample: local solves at full-chi interior sites of a shorter chain (the cost of an
    interior solve depends on chi, not on N), extrapolated to 2(N-1) solves per sweep of the N-site
    chain. Environment construction happens before the clock starts."""
    from oracle import dmrg_oracle as O
    try:
        import torch
        threads = torch.get_num_threads()
    except Exception:
        threads = os.cpu_count()
    short = max(8, 2 * int(np.ceil(np.log2(chi))) + 6)  # middle bonds reach chi
    para = chain_para(short, chi, eigs_tol, "fp64", "cpu")
    np.random.seed(seed)
    A = O.OracleMPS(short, 2, chi, para["op"])
    one, two = O.canonical_terms(para["index1"], para["coeff1"], para["index2"], para["coeff2"], A.ops, eigs_tol)
    mid = short // 2 - 1
    t0 = time.time()
    A.correct_orthogonal_center(mid)
    A.site_buckets(mid, one, two)      # builds the cached environments of the first site
    t_prep = time.time() - t0
    # cost of one effective-Hamiltonian application at this site
    env = A.site_buckets(mid, one, two)
    psi = A.mps[mid]
    t = time.time()
    for _ in range(3):
        A.apply_heff(env, psi)
    t_mv = (time.time() - t) / 3
    times, mvs = [], []
    for n in range(mid, mid + nsolves):
        mv0 = A.n_matvec
        t = time.time()
        A.update_tensor_eigs(n, one, two, 1e-4, eigs_tol)
        times.append(time.time() - t)
        mvs.append(A.n_matvec - mv0)
    per_solve = float(np.mean(times))
    mv_per_solve = float(np.mean(mvs))
    t_rest = max(per_solve - mv_per_solve * t_mv, 0.0)
    # the reference's eigsh builds ncv=20 Lanczos vectors before its first convergence test, so a
    # solve started from an already converged site still costs >= 20 matvecs
    t_converged = 20 * t_mv + t_rest
    sweeps_per_s = 1.0 / (t_converged * 2 * (length - 1))
    return {"value": sweeps_per_s, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "numpy/scipy ARPACK restatement of the reference, %d local solve(s) at interior chi=%d sites of a "
                      "%d-site chain from a random MPS (%.1f s setup untimed): %.2f s/solve with %.0f matvecs of "
                      "%.3f s; per-solve cost at a converged site estimated as 20 matvecs + %.2f s other work = %.2f s, "
                      "extrapolated to 2(N-1)=%d solves per N=%d sweep (the random-state sample alone would give "
                      "%.2e sweeps/s)" % (nsolves, chi, short, t_prep, per_solve, mv_per_solve, t_mv, t_rest,
                                         t_converged, 2 * (length - 1), length,
                                         1.0 / (per_solve * 2 * (length - 1)))}


LEGS_BUDGET_S = 480   # serving + lattice legs together (normally ~3 minutes)
SERVING_ARGS = ["--jobs", "16", "--sweeps", "3"]
SERVING_WORKERS = 8


def run_serving_leg(precision, timeout=240, deadline=None):
    """The serving path (tnalg_gb300.serving) in a child process: 16 uneven XXZ chains (N in [16, 48],
    chi in {16, 32, 64}, 3 sweeps, seeded) interleaved on one GPU in `precision`, against the same
    jobs run one at a time on the plain FP64 GPU path; solves/s and p50/p99 latency of both, then
    (`threaded`) the same mix advanced by SERVING_WORKERS host threads. A failure or timeout of a
    child is reported in the line instead of stopping the benchmark."""
    cmd = [sys.executable, "-m", "tnalg_gb300.serving"] + SERVING_ARGS + ["--precision", precision,
                                                                          "--baseline-precision", "fp64"]
    if deadline is not None:
        timeout = max(1.0, min(timeout, deadline - time.time()))
    out = _child_json(cmd, timeout)
    if "error" in out:
        return out
    # the same interleaved mix advanced by SERVING_WORKERS host threads (their library calls release
    # the GIL, so one job's convergence-check wait no longer holds up the others' kernels), measured
    # in its own child against the sequential FP64 pass above
    cmd = [sys.executable, "-m", "tnalg_gb300.serving"] + SERVING_ARGS + [
        "--precision", precision, "--workers", str(SERVING_WORKERS), "--no-sequential"]
    left = 150.0 if deadline is None else min(150.0, deadline - time.time())
    thr = _child_json(cmd, left) if left > 30 else {"skipped": "the legs' time budget was spent"}
    if "error" not in thr and "skipped" not in thr and out.get("sequential_solves_per_s"):
        thr["speedup_vs_sequential"] = thr["solves_per_s"] / out["sequential_solves_per_s"]
        e1, e2 = out.get("e_per_site", {}), thr.get("e_per_site", {})
        common = set(e1) & set(e2)
        thr["max_abs_de_per_site_vs_one_thread"] = max((abs(e1[k] - e2[k]) for k in common), default=None)
    out["threaded"] = thr
    return out


LATTICE_ARGS = ["j1j2", "--width", "6", "--height", "6", "--chi", "512", "--ramp", "64,256", "--steps", "1"]


def run_lattice_leg(precision, timeout=300):
    """The J1-J2 lattice workload in a child process (tnalg_gb300.run_lattice): the J1-J2 model
    (J2 = 0.5) on the 6 x 6 open square lattice in snake order, chi ramped 64 -> 256 -> 512, one
    CUDA-event-timed sweep at chi=512 in `precision`, then the same seed and schedule on the plain FP64
    path (sweeps/s, energy difference per site). Failures are reported in the line."""
    cmd = [sys.executable, "-m", "tnalg_gb300.run_lattice"] + LATTICE_ARGS + ["--precision", precision]
    if precision != "fp64":
        cmd.append("--compare-fp64")
    return _child_json(cmd, timeout)


def _child_json(cmd, timeout):
    """Run `cmd` (python -m ...) from the repository root; its last JSON line, or an error entry."""
    shown = "python " + " ".join(cmd[1:])
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


def run_reference(args, rank):
    if rank != 0:
        return None
    s = cpu_sample(args.length, args.chi, args.eigs_tol, max(1, args.cpu_solves))
    line = {"metric": METRIC, "value": s["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / s["value"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
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
    if rank == 0 and world == 1 and mixed and not args.no_fp64_leg:
        # the same job (seed, ramp, timed sweeps) on the plain FP64 GPU path: the speed-up of the
        # split-TF32 path and its energy difference per site
        import copy
        a64 = copy.copy(args)
        a64.precision = "fp64"
        r64, A64, _ = run_ours(a64, rank, 1, local_rank)
        del A64
        v64 = args.steps / (r64["ms"] / 1000.0)
        line["fp64_path"] = {"value": v64, "unit": UNIT, "ms_per_step": r64["ms"] / args.steps,
                             "e_per_site": r64["e_per_site"], "speedup_of_this_line": value / v64,
                             "abs_de_per_site": abs(res["e_per_site"] - r64["e_per_site"]),
                             # index2 rows per bond: (su, sd), (sd, su), (sz, sz) with Jz = 1
                             "max_abs_d_szsz": float(np.max(np.abs(res["eb_full"][2::3] - r64["eb_full"][2::3]))),
                             "max_abs_d_bond_energy": float(np.max(np.abs(
                                 res["eb_full"].reshape(-1, 3).sum(1) - r64["eb_full"].reshape(-1, 3).sum(1)))),
                             "device_ms_per_sweep": {"qr": r64["qr_ms"] / args.steps,
                                                     "lanczos_incl_matvec": r64["lz_ms"] / args.steps,
                                                     "matvec": r64["mv_ms"] / args.steps}}
    if rank == 0 and not args.no_e2e:
        line["e2e"] = run_e2e(args, "cuda:%d" % local_rank, res["precision"])
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(args.length, args.chi, args.eigs_tol, max(1, args.cpu_solves))
    if rank == 0 and world == 1 and not (args.no_serving and args.no_lattice):
        del A
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        # the child legs share one time budget, so a stuck leg cannot hold back the line
        legs_end = time.time() + LEGS_BUDGET_S
        if not args.no_serving:
            line["serving"] = run_serving_leg(res["precision"], deadline=legs_end)
        if not args.no_lattice:
            left = legs_end - time.time()
            line["j1j2_6x6"] = (run_lattice_leg(res["precision"], timeout=min(300.0, left)) if left > 60 else
                                {"skipped": "the legs' %d s time budget was spent" % LEGS_BUDGET_S})
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
