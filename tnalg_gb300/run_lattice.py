"""One finite-size DMRG workload timed on one GPU (used by the benchmark's lattice leg).

    python -m tnalg_gb300.run_lattice j1j2 [--width 6 --height 6 --j2 0.5] [--chi 512] [--ramp 64,256]
                                           [--steps 1] [--precision tf32x3] [--compare-fp64]
    python -m tnalg_gb300.run_lattice chain [--length 100] ...

j1j2: the J1-J2 Heisenberg model (J2 = 0.5) on an open width x height square lattice in snake order
(Parameters.generate_parameters_j1j2_snake: 60 J1 and 50 J2 bonds at 6 x 6, bonds up to 11 sites
apart, so every matvec carries the straddling pairs of up to 14 bonds). chain: the N-site Heisenberg
chain. Seeded random-normal initial MPS; one sweep at every bond dimension of the ramp, then `steps`
sweeps at `chi` timed with CUDA events on the launching stream. Prints one JSON line: sweeps/s,
solves/s and matvecs per solve of the timed sweeps, the energy per site of the final state (FP64
observables), and with --compare-fp64 the same seed and schedule on the plain FP64 path with the
energy difference per site.
"""
import argparse
import json
import time

import numpy as np
import torch

from . import Parameters as pm
from .MPSClass import MpsOpenBoundaryClass


def lattice_para(a):
    if a.lattice == "j1j2":
        para = pm.generate_parameters_j1j2_snake(a.width, a.height, j1=1.0, j2=a.j2)
        name = "J1-J2 Heisenberg, %dx%d open square lattice in snake order, J1=1, J2=%g" % (a.width, a.height, a.j2)
    else:
        para = pm.generate_parameters_dmrg("chain")
        para.update(l=a.length, jxy=1, jz=1, hx=0, hz=0)
        para = pm.make_consistent_parameter_dmrg(para)
        name = "N=%d spin-1/2 Heisenberg open chain, J=1" % a.length
    para.update(tau=1e-4, eigs_tol=a.eigs_tol)
    return para, name


class _Timer:
    """CUDA events on the current stream for a CUDA device, the host clock otherwise."""

    def __init__(self, device):
        self.cuda = str(device).startswith("cuda")

    def __enter__(self):
        if self.cuda:
            torch.cuda.synchronize()
            self.a, self.b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            self.a.record()
        else:
            self.t = time.perf_counter()
        return self

    def __exit__(self, *exc):
        if self.cuda:
            self.b.record()
            torch.cuda.synchronize()
            self.ms = self.a.elapsed_time(self.b)
        else:
            self.ms = 1000.0 * (time.perf_counter() - self.t)


def run(para, precision, schedule, steps, device="cuda", seed=0, refine="off", growth="expand"):
    """Ramp over `schedule[:-1]` (one sweep per bond dimension), then `steps` timed sweeps at
    schedule[-1]. refine (split-TF32 path): 'final' refines the local solves of the last sweep to
    the FP64 tolerance (DMRG_anyH.refine_sweep), 'all' those of every sweep, 'off' none. growth: how
    bonds grow between schedule entries ('expand': subspace expansion with a truncated SVD of the
    Hamiltonian's open channels; 'noise': seeded noise)."""
    np.random.seed(seed)
    l = para["l"]
    A = MpsOpenBoundaryClass(l, para["d"], schedule[0], operators=para["op"], device=device, precision=precision)
    A.correct_orthogonal_center(0)
    order = list(range(1, l)) + list(range(l - 2, -1, -1))
    total = len(schedule) - 1 + steps
    energies = []

    def sweep(t):
        A.refine_vectors = refine == "all" or (refine == "final" and t == total - 1)
        for k, n in enumerate(order):
            if k == len(order) - 1:
                A.refine_next_solve()
            e = A.update_tensor_eigs(n, para["index1"], para["index2"], para["coeff1"], para["coeff2"],
                                     para["tau"], True, tol=para["eigs_tol"])
        energies.append(float(e) / l)

    model = (para["index1"], para["index2"], para["coeff1"], para["coeff2"], para["eigs_tol"])
    for t, chi in enumerate(schedule[:-1]):
        A.grow_bond_dimension(int(chi), seed=t, method=growth, model=model)
        sweep(t)
    A.grow_bond_dimension(int(schedule[-1]), seed=len(schedule) - 1, method=growth, model=model)
    s0, m0 = A.stats["solves"], A.stats["matvecs"]
    with _Timer(device) as tm:
        for k in range(steps):
            sweep(len(schedule) - 1 + k)
    solves, matvecs = A.stats["solves"] - s0, A.stats["matvecs"] - m0
    eb = A.observe_bond_energy(para["index2"], para["coeff2"])
    mx, mz = A.observe_magnetization(1), A.observe_magnetization(3)
    e = float((np.sum(eb) - para["hx"] * np.sum(mx) - para["hz"] * np.sum(mz)) / l)
    return {"precision": precision, "refine": refine if precision != "fp64" else None,
            "ms_per_sweep": tm.ms / steps, "sweeps_per_s": 1000.0 * steps / tm.ms,
            "solves_per_s": 1000.0 * solves / tm.ms, "matvecs_per_solve": matvecs / max(solves, 1),
            "e_per_site": e, "chi_max": int(A.virtual_dim.max()), "sweep_energies_per_site": energies,
            "unconverged_solves": int(A.stats["unconverged"]), "eb_full": np.ravel(eb)}


def straddle_max(para):
    """Largest number of straddling two-body terms (i < p < j) at one site."""
    idx = np.asarray(para["index2"]).reshape(-1, 4)
    lo, hi = np.minimum(idx[:, 0], idx[:, 1]), np.maximum(idx[:, 0], idx[:, 1])
    return int(max(np.count_nonzero((lo < p) & (p < hi)) for p in range(para["l"])))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("lattice", choices=["j1j2", "chain"])
    ap.add_argument("--width", type=int, default=6)
    ap.add_argument("--height", type=int, default=6)
    ap.add_argument("--j2", type=float, default=0.5)
    ap.add_argument("--length", type=int, default=100)
    ap.add_argument("--chi", type=int, default=512)
    ap.add_argument("--ramp", default="64,256")
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--precision", default="tf32x3")
    ap.add_argument("--compare-fp64", action="store_true")
    ap.add_argument("--eigs-tol", type=float, default=1e-12)
    ap.add_argument("--device", default="cuda")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--refine", default="off", choices=["final", "all", "off"],
                    help="split-TF32 path: local solves refined to the FP64 tolerance in the last sweep (final), "
                         "in every sweep (all) or never (off)")
    ap.add_argument("--growth", default="expand", choices=["expand", "noise"])
    a = ap.parse_args(argv)
    from . import _lib as L
    L.load()
    para, name = lattice_para(a)
    schedule = [int(x) for x in a.ramp.split(",") if x] + [a.chi]
    out = {"workload": name, "sites": int(para["l"]), "two_body_rows": int(np.asarray(para["index2"]).shape[0]),
           "straddling_terms_max": straddle_max(para), "chi_schedule": schedule, "timed_sweeps": a.steps}
    res = run(para, a.precision, schedule, a.steps, a.device, a.seed, refine=a.refine, growth=a.growth)
    eb = res.pop("eb_full")
    out.update(res)
    if a.compare_fp64 and a.precision != "fp64":
        ref = run(para, "fp64", schedule, a.steps, a.device, a.seed, growth=a.growth)
        eb64 = ref.pop("eb_full")
        out["fp64_path"] = ref
        out["speedup_vs_fp64"] = out["sweeps_per_s"] / ref["sweeps_per_s"]
        out["abs_de_per_site_vs_fp64"] = abs(out["e_per_site"] - ref["e_per_site"])
        # two-body terms: c <op_a(i) op_b(j)> per index2 row; the largest difference over all rows
        out["max_abs_d_term_energy_vs_fp64"] = float(np.max(np.abs(eb - eb64)))
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
