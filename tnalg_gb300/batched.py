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
        # the job's own generator: the draws (and their order, TensorBasicModule.py:181-186) of
        # np.random.seed(seed) followed by random_open_mps, without touching the global generator, so
        # that jobs can be started from several host threads
        rs = np.random.RandomState(self.seed)
        l, d, chi = p["l"], p["d"], p["chi"]
        tensors = [None] * l
        tensors[0] = rs.randn(1, d, chi)
        tensors[l - 1] = rs.randn(chi, d, 1)
        for n in range(1, l - 1):
            tensors[n] = rs.randn(chi, d, chi)
        self.A = MpsOpenBoundaryClass(length=l, d=d, chi=chi, operators=p["op"], device=device, precision=precision,
                                      tensors=tensors)
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


# ---------------------------------------------------------------------------------------------
# grouped path: every job's state in one device arena, every local update as table rows


def _rec(dtype, **kw):
    """One record as a tuple in the dtype's field order (tables are built with one np.array call)."""
    return tuple(kw.get(name, 0) for name in dtype.names)


def _table(dtype, recs):
    return np.array(recs, dtype=dtype) if recs else np.zeros(0, dtype=dtype)


def _gemm(M, N, K, A, sA, B, sB, C, sC, *, batch=1, sAb=0, sBb=0, sCb=0, alpha=1.0, beta=0.0, accumulate=0,
          active=0):
    return _rec(L.GEMM_PROBLEM_DTYPE, M=M, N=N, K=K, nred=1, A=A, sAm=sA[0], sAk=sA[1], B=B, sBk=sB[0], sBn=sB[1],
                C=C, sCm=sC[0], sCn=sC[1], alpha=alpha, beta=beta, accumulate=accumulate, batch=batch, sAb=sAb,
                sBb=sBb, sCb=sCb, active=active)


def _op(kind, chi, d, src, out, total, *, terms=0, nterms=0, ops=0, s_slot=0, s_row=0, chir=0, out_stride=0,
        active=0):
    return _rec(L.BATCH_OP_DTYPE, kind=kind, chi=chi, d=d, chir=chir, nterms=nterms, src=src, s_slot=s_slot,
                s_row=s_row, ops=ops, terms=terms, out=out, out_stride=out_stride, total=total, active=active)


QR_MAX_ELEMS = 32768   # m n of one matrix of tn_batched_qr_mixed


class ArenaJob(BatchJob):
    """A job of the grouped path. Its MPS, both environment stacks of every bond and its scratch live
    in one device arena allocated at admission, so every pointer of every local update is fixed and
    the launch records of each (site, direction) are built once: a step of the batch concatenates
    the records of every job's current site and runs a dozen grouped launches for all jobs. The
    arithmetic is that of DeviceMPS (gauge move, incremental environment update with the carry
    plans of engine.Model, block assembly), in the grouped kernels."""

    def start(self, device, precision):
        super().start(device, precision)
        if self.para["ob_position"] != 0:
            raise ValueError("the grouped path starts its sweeps at site 0 (ob_position = 0)")
        A = self.A
        dev = A._dev
        m = dev.model
        if m.compressed:
            raise ValueError("the grouped path runs uncompressed coupling models")
        Ln, d = A.length, A.phys_dim
        # a random MPS is centred by QR moves from the right end, which leave the bonds near the left
        # end wider than d^b; moving the centre right past them and back gives every bond its final
        # dimension min(chi, d^b, d^(L-b)) now (a reduced QR truncates nothing: the state is
        # unchanged), so the arena's shapes stay fixed for the whole run
        b = 0
        while b < Ln - 1 and int(dev.virtual_dim[b + 1]) > d ** (b + 1):
            b += 1
        if b > 0:
            A.correct_orthogonal_center(b)
            A.correct_orthogonal_center(0)
        # a random MPS centred by QR moves carries the product of all R factors' norms on its centre
        # (~1e77 for 64 sites at chi = 128), beyond FP32's range for the split-TF32 absorb of the
        # first gauge move; the state's norm is irrelevant to the solves (eigsh normalises its start
        # vector), so the centre is normalised once here
        c0 = dev.mps[0]
        c0.div_(c0.abs().max().clamp_min(1e-300))   # first to O(1), so its squared norm cannot overflow
        nrm2 = torch.empty(1, dtype=torch.float64, device=dev.device)
        lib = L.load()
        wp, wb = dev.ws.args(4096 + 64 * c0.numel())
        L.check(lib.tn_dot(c0.numel(), L.ptr(c0), L.ptr(c0), L.ptr(nrm2), wp, wb, L.stream_handle()), "dot")
        L.check(lib.tn_scale(c0.numel(), L.ptr(c0), 1.0, L.ptr(nrm2), L.stream_handle()), "scale")
        dev.unit_norm = True
        dev.ensure_envs(0)
        dims = [int(x) for x in dev.virtual_dim]
        self.dims, self.d, self.model = dims, d, m
        nl = [m.n_left(b) for b in range(Ln + 1)]
        nr = [m.n_right(b) for b in range(Ln + 1)]
        cmax = max(dims)
        ngmax = max([m.memo(("sg", p), lambda p=p: m.straddle_groups(p))[2] for p in range(Ln)] + [0])
        carry_max = max(max(nl), max(nr)) + 1
        off = 0
        lay = {}

        def take(name, n):
            nonlocal off
            lay[name] = (off, n)
            off += (n + 31) // 32 * 32   # 256-byte aligned views
        for n in range(Ln):
            take(("site", n), dims[n] * d * dims[n + 1])
        for b in range(Ln + 1):
            take(("EL", b), (1 + nl[b]) * dims[b] ** 2)
            take(("ER", b), (1 + nr[b]) * dims[b] ** 2)
        take("WL", (d * cmax) ** 2)
        take("WR", (d * cmax) ** 2)
        take("Wenv", (d * cmax) ** 2)
        take("seed", d * cmax * cmax)
        take("R", cmax * cmax)
        take("T", carry_max * d * cmax * cmax)
        take("SL", max(ngmax, 1) * cmax * cmax)
        take("SR", max(ngmax, 1) * cmax * cmax)
        self.arena = torch.zeros(off, dtype=torch.float64, device=dev.device)
        self.active = torch.ones(1, dtype=torch.int32, device=dev.device)
        self.lay = lay
        base = self.arena.data_ptr()
        self.addr = {k: base + 8 * o for k, (o, _) in lay.items()}
        for n in range(Ln):
            self.view(("site", n)).copy_(dev.mps[n].reshape(-1))
        self.view(("EL", 0)).copy_(dev.EL[0].reshape(-1))
        for b in range(1, Ln + 1):
            self.view(("ER", b)).copy_(dev.ER[b].reshape(-1))
        # the one-job state is no longer needed (observables use the arena's site tensors)
        dev.mps = [self.view(("site", n)).view(dims[n], d, dims[n + 1]) for n in range(Ln)]
        dev.EL = [None] * (Ln + 1)
        dev.ER = [None] * (Ln + 1)
        dev.el_upto, dev.er_from = -1, Ln + 1
        self._rows = {}

    def view(self, key):
        o, n = self.lay[key]
        return self.arena[o:o + n]

    def rows(self):
        """Launch records of this step's local update (built once per (site, direction))."""
        k = self._k
        hit = self._rows.get(k)
        if hit is None:
            hit = self._rows[k] = self._build(k)
        return hit

    def _build(self, k):
        p = self._order[k]
        right = k < self.para["l"] - 1   # the first half of the sweep moves right
        m, d, dims, a = self.model, self.d, self.dims, self.addr
        act = self.active.data_ptr()
        ops = m.ops.data_ptr()
        q = p - 1 if right else p + 1
        cl, cr = dims[q], dims[q + 1]
        n_q = cl * d * cr
        site_q = a[("site", q)]
        out = {"ops1": [], "qr": [], "gemm1": [], "ops2": [], "gemm2": [], "ops3": []}
        if right:
            mm, nn = cl * d, cr
            qr = _rec(L.QR_ITEM_DTYPE, m=mm, n=nn, a=site_q, sAm=cr, sAn=1, r=a["R"], sRm=nn, sRn=1, active=act)
            # seed = R (cr x cr) . site[p] (cr x d dims[p+1])
            nxt = d * dims[p + 1]
            out["gemm1"].append(_gemm(cr, nxt, cr, a["R"], (cr, 1), a[("site", p)], (nxt, 1), a["seed"], (nxt, 1),
                                      active=act))
            plan = m.memo(("lcp", q), lambda: m.left_carry_plan(q))
            terms, nt = m.table_lazy(("wl", q), lambda: m.left_block_terms(q))
            out["ops1"].append(_op(L.BOP_BLOCK_LEFT, cl, d, a[("EL", q)], a["Wenv"], (cl * d) ** 2, terms=terms.data_ptr(),
                                   nterms=nt, ops=ops, s_slot=cl * cl, s_row=cl, active=act))
            # T0 = Wenv (cl d x cl d) . Q (cl d x cr)
            out["gemm1"].append(_gemm(cl * d, cr, cl * d, a["Wenv"], (cl * d, 1), site_q, (cr, 1), a["T"], (cr, 1),
                                      active=act))
            for j, (kind, x) in enumerate(plan):
                tj = a["T"] + 8 * (1 + j) * n_q
                if kind == "carry":   # T[1+j] = EL[q][slot] (cl x cl) . Q (cl x d cr)
                    out["gemm1"].append(_gemm(cl, d * cr, cl, a[("EL", q)] + 8 * x * cl * cl, (cl, 1), site_q,
                                              (d * cr, 1), tj, (d * cr, 1), active=act))
                else:
                    oi = m.opidx(("op", x), [x])
                    out["ops2"].append(_op(L.BOP_SITE_OPS, cl, d, site_q, tj, n_q, terms=oi.data_ptr(), nterms=1,
                                           ops=ops, chir=cr, out_stride=n_q, active=act))
            ns = 1 + len(plan)
            # EL[p][s] = Q^T (cr x cl d) . T[s] (cl d x cr)
            out["gemm2"].append(_gemm(cr, cr, cl * d, site_q, (1, cr), a["T"], (cr, 1), a[("EL", p)], (cr, 1),
                                      batch=ns, sAb=0, sBb=n_q, sCb=cr * cr, active=act))
        else:
            mm, nn = d * cr, cl
            qr = _rec(L.QR_ITEM_DTYPE, m=mm, n=nn, a=site_q, sAm=1, sAn=d * cr, r=a["R"], sRm=nn, sRn=1, active=act)
            # seed = site[p] (dims[p] d x cl) . R^T
            prv = dims[p] * d
            out["gemm1"].append(_gemm(prv, cl, cl, a[("site", p)], (cl, 1), a["R"], (1, cl), a["seed"], (cl, 1),
                                      active=act))
            plan = m.memo(("rcp", q), lambda: m.right_carry_plan(q))
            terms, nt = m.table_lazy(("wrf", q), lambda: m.right_block_terms(q, with_site=True))
            out["ops1"].append(_op(L.BOP_BLOCK_RIGHT, cr, d, a[("ER", q + 1)], a["Wenv"], (d * cr) ** 2,
                                   terms=terms.data_ptr(), nterms=nt, ops=ops, s_slot=cr * cr, s_row=cr, active=act))
            # T0 = B (cl x d cr) . Wenv^T
            out["gemm1"].append(_gemm(cl, d * cr, d * cr, site_q, (d * cr, 1), a["Wenv"], (1, d * cr), a["T"],
                                      (d * cr, 1), active=act))
            for j, (kind, x) in enumerate(plan):
                tj = a["T"] + 8 * (1 + j) * n_q
                if kind == "carry":   # T[1+j] = B (cl d x cr) . ER[q+1][slot]^T
                    out["gemm1"].append(_gemm(cl * d, cr, cr, site_q, (cr, 1), a[("ER", q + 1)] + 8 * x * cr * cr,
                                              (1, cr), tj, (cr, 1), active=act))
                else:
                    oi = m.opidx(("op", x), [x])
                    out["ops2"].append(_op(L.BOP_SITE_OPS, cl, d, site_q, tj, n_q, terms=oi.data_ptr(), nterms=1,
                                           ops=ops, chir=cr, out_stride=n_q, active=act))
            ns = 1 + len(plan)
            # ER[q][s] = B (cl x d cr) . T[s]^T
            out["gemm2"].append(_gemm(cl, cl, d * cr, site_q, (d * cr, 1), a["T"], (1, d * cr), a[("ER", q)], (cl, 1),
                                      batch=ns, sAb=0, sBb=n_q, sCb=cl * cl, active=act))
        # effective Hamiltonian of site p
        pl, pr = dims[p], dims[p + 1]
        t, nt = m.table_lazy(("wl", p), lambda: m.left_block_terms(p))
        out["ops3"].append(_op(L.BOP_BLOCK_LEFT, pl, d, a[("EL", p)], a["WL"], (pl * d) ** 2, terms=t.data_ptr(),
                               nterms=nt, ops=ops, s_slot=pl * pl, s_row=pl, active=act))
        t, nt = m.table_lazy(("wr", p), lambda: m.right_block_terms(p, with_site=False))
        out["ops3"].append(_op(L.BOP_BLOCK_RIGHT, pr, d, a[("ER", p + 1)], a["WR"], (d * pr) ** 2,
                               terms=t.data_ptr(), nterms=nt, ops=ops, s_slot=pr * pr, s_row=pr, active=act))
        slt, srt, ng = m.memo(("sg", p), lambda: m.straddle_groups(p))
        if ng:
            ta, na = m.table(("sl", p), slt)
            tb, nb = m.table(("sr", p), srt)
            out["ops3"].append(_op(L.BOP_COMBINE, pl, d, a[("EL", p)], a["SL"], ng * pl * pl, terms=ta.data_ptr(),
                                   nterms=na, s_slot=pl * pl, s_row=pl, out_stride=pl * pl, active=act))
            out["ops3"].append(_op(L.BOP_COMBINE, pr, d, a[("ER", p + 1)], a["SR"], ng * pr * pr, terms=tb.data_ptr(),
                                   nterms=nb, s_slot=pr * pr, s_row=pr, out_stride=pr * pr, active=act))
        solve = _rec(L.BATCH_SOLVE_DTYPE, chil=pl, d=d, chir=pr, wl=a["WL"], wr=a["WR"], nstr=ng,
                     sl=a["SL"] if ng else 0, sr=a["SR"] if ng else 0, psi_in=a["seed"], psi_out=a[("site", p)])
        res = {key: _table(v_dtype(key), v) for key, v in out.items() if key != "qr"}
        res["qr"] = _table(L.QR_ITEM_DTYPE, [qr])
        res["solve"] = _table(L.BATCH_SOLVE_DTYPE, [solve])
        res["qr_shape"] = (mm, nn, right, q)
        res["qr_big"] = mm * nn > QR_MAX_ELEMS
        return res

    def big_qr(self, ws):
        """A gauge move whose site tensor exceeds the batched QR's shared memory (m n > 32768, e.g.
        chi > 128 at d = 2): tn_qr_mixed into a scratch Q, copied back in place."""
        mm, nn, right, q = self.rows()["qr_shape"]
        lib = L.load()
        cl, cr = self.dims[q], self.dims[q + 1]
        site = self.view(("site", q))
        Qt = torch.empty(mm * nn, dtype=torch.float64, device=site.device)
        R = self.view("R")
        wp, wb = ws.args(lib.tn_qr_mixed_workspace_bytes(mm, nn))
        if right:
            L.check(lib.tn_qr_mixed(mm, nn, L.ptr(site), nn, 1, L.ptr(Qt), nn, 1, L.ptr(R), nn, 1, wp, wb,
                                    L.stream_handle()), "qr_mixed")
            site.copy_(Qt)
        else:
            L.check(lib.tn_qr_mixed(mm, nn, L.ptr(site), 1, mm, L.ptr(Qt), 1, mm, L.ptr(R), nn, 1, wp, wb,
                                    L.stream_handle()), "qr_mixed")
            site.copy_(Qt)

    def solved(self, res):
        done = super().solved(res)
        return done

    def observe(self):
        dev = self.A._dev
        dev.center = self._order[self._k - 1] if self._k > 0 else 0
        if self._k == 0:
            dev.center = self._order[-1]
        dev.unit_norm = True
        super().observe()
        self.arena = None


def v_dtype(key):
    return L.GEMM_PROBLEM_DTYPE if key.startswith("gemm") else L.BATCH_OP_DTYPE


class BatchEngine:
    """Continuous batching of DMRG jobs: admission by device memory, one batched local solve per
    step for all admitted jobs, p50/p99 latency from arrival to result."""

    def __init__(self, device="cuda", precision="tf32x3", budget_bytes=None, max_active=1024, max_krylov=24,
                 check_every=3, mixed_floor=2e-6, workers=8, streams=16, grouped=None, profile=False):
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
        self._ws2 = None
        self._observing = []
        self._t0 = None
        self.step_ms = []
        self.times = {"admit": 0.0, "step": 0.0, "observe": 0.0, "tables": 0.0}
        # device time of the grouped step's phases (CUDA events on the stream; profile=True)
        self.profile = bool(profile)
        self.phase_ms = {}
        # grouped path (job arenas, grouped launches for the whole local update) on the split-TF32
        # path; the FP64 path prepares every job with its own DeviceMPS calls
        self.grouped = self.prec == L.PREC_TF32X3 if grouped is None else bool(grouped)

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
        t_in = time.perf_counter()
        self._admit_jobs(now)
        self.times["admit"] += time.perf_counter() - t_in

    def _admit_jobs(self, now):
        budget = self._budget()
        admit = []
        while self.pending and self.pending[0].arrival <= now and len(self.active) + len(admit) < self.max_active:
            fp = self.pending[0].footprint_bytes(self.krylov)
            if (self.active or admit) and self._used + fp > budget:
                break
            job = self.pending.pop(0)
            job.admitted = now
            if self.grouped and not isinstance(job, ArenaJob):
                job.__class__ = ArenaJob
            admit.append(job)
            self._used += fp
        self._on_workers(admit, lambda job: job.start(self.device, self.precision))
        self.active += admit
        self.max_concurrent = max(self.max_concurrent, len(self.active))
        self.max_used = max(self.max_used, self._used)

    def _on_workers(self, jobs, fn):
        """fn(job) for every job: on a GPU from `workers` host threads, each job on the stream it keeps
        for life (the library's calls release the GIL, so the jobs' small latency-bound kernels overlap);
        every stream is synchronised before the call returns."""
        cuda = str(self.device).startswith("cuda") and not L._host_test
        if not cuda or self.workers == 1 or len(jobs) < 2:
            for job in jobs:
                fn(job)
            return
        self._ensure_streams()
        main = torch.cuda.current_stream(self.device)
        ready = torch.cuda.Event()
        ready.record(main)

        def run(job):
            st = self._streams[job.job_id % self.nstreams]
            st.wait_event(ready)
            with torch.cuda.stream(st):
                fn(job)
            st.synchronize()
        for _ in self._pool.map(run, jobs):
            pass

    def _observe_async(self, jobs):
        """Observe finished jobs (bond energies, magnetisations: FP64 transfer products) on the
        observer threads, each job on its own stream, while the engine steps the remaining jobs; a
        job's device memory is released and its latency stamped when its observation is done."""
        if not jobs:
            return
        cuda = str(self.device).startswith("cuda") and not L._host_test
        if not cuda or self.workers == 1:
            for job in jobs:
                job.observe()
                self._retire(job)
            return
        self._ensure_streams()
        main = torch.cuda.current_stream(self.device)
        ready = torch.cuda.Event()
        ready.record(main)

        def run(job):
            st = self._streams[job.job_id % self.nstreams]
            st.wait_event(ready)
            with torch.cuda.stream(st):
                job.observe()
            st.synchronize()
            return job
        for job in jobs:
            self._observing.append(self._obs_pool.submit(run, job))

    def _collect_observed(self, block=False):
        if not self._observing:
            return
        if block:
            from concurrent.futures import FIRST_COMPLETED, wait
            wait(self._observing, return_when=FIRST_COMPLETED)
        still = []
        for f in self._observing:
            if f.done():
                self._retire(f.result())   # an exception of the observation is raised here
            else:
                still.append(f)
        self._observing = still

    def _retire(self, job):
        job.finished = time.perf_counter() - self._t0
        self._used -= job.footprint_bytes(self.krylov)
        self.done.append(job)

    def _ensure_streams(self):
        if self._streams is None:
            self._streams = [torch.cuda.Stream(device=self.device) for _ in range(self.nstreams)]
            from concurrent.futures import ThreadPoolExecutor
            self._pool = ThreadPoolExecutor(max_workers=self.workers)
            self._obs_pool = ThreadPoolExecutor(max_workers=max(1, self.workers // 2))

    def _prepare_all(self, jobs):
        """Every job's gauge move, environment update and block assembly. On a GPU the jobs are
        spread over `streams` CUDA streams and prepared by `workers` host threads (the library's
        calls release the GIL), so their small latency-bound kernels overlap; the batched solve
        on the current stream waits for all of them."""
        cuda = str(self.device).startswith("cuda") and not L._host_test
        if not cuda or self.workers == 1:
            return [job.prepare() for job in jobs]
        self._ensure_streams()
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

    def _grouped_step(self, jobs):
        """One local update of every job of the grouped path: ~a dozen grouped launches for all
        jobs (block assembly, gauge moves, R-absorb and environment update, effective Hamiltonian)
        and one batched solve."""
        lib = L.load()
        st = L.stream_handle()
        t_tab = time.perf_counter()
        rows = [j.rows() for j in jobs]
        self.times["tables"] += time.perf_counter() - t_tab
        marks = []

        def mark(name):
            if self.profile and not L._host_test:
                ev = torch.cuda.Event(enable_timing=True)
                ev.record()
                marks.append((name, ev))
        mark("start")
        if self._ws is None:
            self._ws = L.Workspace(torch.device(self.device))
        if self._ws2 is None:
            self._ws2 = L.Workspace(torch.device(self.device))

        def ops(key):
            tab = np.concatenate([r[key] for r in rows])
            if tab.shape[0]:
                wp, wb = self._ws2.args(lib.tn_grouped_ops_workspace_bytes(tab.shape[0]))
                L.check(lib.tn_grouped_ops(ctypes.c_void_p(tab.ctypes.data), tab.shape[0], wp, wb, st), "grouped ops")
            return tab

        def gemm(key):
            tab = np.concatenate([r[key] for r in rows])
            if tab.shape[0]:
                L.grouped_gemm(tab, precision=self.prec, ws=self._ws2)
            return tab

        keep = [ops("ops1")]
        mark("assemble_env_block")
        small = [r["qr"] for r in rows if not r["qr_big"]]
        if small:
            tab = np.concatenate(small)
            tp = ctypes.c_void_p(tab.ctypes.data)
            wp, wb = self._ws2.args(lib.tn_batched_qr_mixed_workspace_bytes(tp, tab.shape[0]))
            L.check(lib.tn_batched_qr_mixed(tp, tab.shape[0], wp, wb, st), "batched qr")
            keep.append(tab)
        for j, r in zip(jobs, rows):
            if r["qr_big"]:
                j.big_qr(self._ws2)
        mark("qr")
        keep += [gemm("gemm1"), ops("ops2")]
        mark("absorb_and_transfer")
        keep.append(gemm("gemm2"))
        mark("env_close")
        keep.append(ops("ops3"))
        mark("heff_assembly")
        solves = np.concatenate([r["solve"] for r in rows])
        out = self._solve(jobs, solves, keep)
        mark("lanczos")
        if marks:
            marks[-1][1].synchronize()
            for (_, a), (name, b) in zip(marks[:-1], marks[1:]):
                self.phase_ms[name] = self.phase_ms.get(name, 0.0) + a.elapsed_time(b)
        return out

    def _solve(self, jobs, solves, keep):
        lib = L.load()
        opts = L.LanczosOpts(float(jobs[0].para["eigs_tol"]), float(jobs[0].para["tau"]), 0.0, self.mixed_floor,
                             self.krylov, 50, self.check_every, self.prec, 0, 0)
        if len({(float(j.para["eigs_tol"]), float(j.para["tau"])) for j in jobs}) > 1:
            raise ValueError("jobs of one batch share eigs_tol and tau")
        table = ctypes.c_void_p(solves.ctypes.data)
        need = lib.tn_batched_lanczos_workspace_bytes(table, len(jobs), ctypes.byref(opts))
        wp, wb = self._ws.args(need + 1024)
        res = (L.LanczosResult * len(jobs))()
        st = lib.tn_batched_lanczos(table, len(jobs), ctypes.byref(opts), wp, wb, ctypes.cast(res, ctypes.c_void_p),
                                    L.stream_handle())
        if st not in (L.TN_OK, L.TN_ERR_NOCONV):
            L.check(st, "batched lanczos")
        finished = [job for i, job in enumerate(jobs) if job.solved(res[i])]
        del keep
        self.steps += 1
        return finished

    def step(self):
        """One local update of every admitted job (one batched solve)."""
        jobs = list(self.active)
        if not jobs:
            return []
        if self.grouped:
            return self._grouped_step(jobs)
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
        while self.pending or self.active or self._observing:
            if not self.active and not self.pending:
                self._collect_observed(block=True)
                continue
            now = time.perf_counter() - t0
            self._admit(now)
            if not self.active:
                time.sleep(max(0.0, min(self.pending[0].arrival - now, 0.01)))
                continue
            ts = time.perf_counter()
            finished = self.step()
            t1 = time.perf_counter()
            self.step_ms.append(1000.0 * (t1 - ts))
            self.times["step"] += t1 - ts
            for job in finished:
                self.active.remove(job)
            self._observe_async(finished)
            self._collect_observed(block=not self.active and not self.pending)
            self.times["observe"] += time.perf_counter() - t1
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
                "matvecs_per_solve": (sum(j.matvecs for j in self.done) / solves) if solves else 0.0,
                "host_s": {k: round(v, 3) for k, v in self.times.items()},
                "device_ms_per_step": {k: round(v / max(self.steps, 1), 3) for k, v in self.phase_ms.items()}}


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
    ap.add_argument("--profile", action="store_true", help="device time per phase of the grouped step (CUDA events)")
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
    eng = BatchEngine(dev, a.precision, max_active=a.max_active, max_krylov=a.krylov, profile=a.profile)
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
