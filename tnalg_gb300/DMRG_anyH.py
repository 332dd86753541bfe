"""Finite-size DMRG driver (drop-in for T-Nalg's DMRG_anyH.dmrg_finite_size).

Same sweep schedule, observation cadence, convergence test, outputs and prints
as DMRG_anyH.py:18-101; the MPS and every contraction live on the GPU.
"""
import time

import numpy as np

from . import Parameters as pm


def dmrg_finite_size(para=None):
    """DMRG_anyH.py:18-101. Returns (ob, A, info, para).

    ob: 'eb_full' (nh,1), 'mx' (l,1), 'mz' (l,1), 'e_per_site', 'eb', 'corr_x', 'corr_z'.
    info: 'convergence', 't_cost', plus 'sweeps', 'solves', 'matvecs', 'sweep_times'.
    """
    from .MPSClass import MpsOpenBoundaryClass as Mob
    t_start = time.time()
    info = dict()
    print("Preparing the parameters and MPS")
    if para is None:
        para = pm.generate_parameters_dmrg()
    A = Mob(length=para["l"], d=para["d"], chi=para["chi"], way="qr", ini_way="r", operators=para["op"],
            is_parallel=para.get("isParallel", False), is_save_op=para.get("is_save_op", True),
            eig_way=para.get("eigWay", 1), is_env_parallel_lmr=para.get("isParallelEnvLMR", False),
            device=para.get("device", "cuda"), precision=para.get("precision", "fp64"))
    for key, name in (("lanczos_krylov", "max_krylov"), ("lanczos_tol_cap", "tol_cap"),
                      ("lanczos_restarts", "max_restarts"), ("lanczos_check_every", "check_every"),
                      ("lanczos_mixed_floor", "mixed_floor"), ("lanczos_refine", "refine"),
                      ("lanczos_refine_cycles", "refine_cycles")):
        if key in para:
            A.lanczos[name] = para[key]
    A.coupling_compress = para.get("mpo_compress", False)
    A.coupling_tol = float(para.get("mpo_tol", 1e-14))
    A.correct_orthogonal_center(para["ob_position"])
    print("Starting to sweep ...")
    e0_per_site = 0
    info["convergence"] = 1
    info["sweep_times"] = []
    ob = dict()
    index1, index2 = para["index1"], para["index2"]
    coeff1, coeff2 = para["coeff1"], para["coeff2"]
    l = para["l"]
    schedule = para.get("chi_schedule")
    for t in range(para["sweep_time"]):
        ts = time.time()
        if schedule:
            A.grow_bond_dimension(int(schedule[min(t, len(schedule) - 1)]), noise=para.get("chi_noise", 1e-3),
                                  seed=t, method=para.get("chi_growth", "expand"),
                                  model=(index1, index2, coeff1, coeff2, para["eigs_tol"]))
        A.refine_vectors = refine_sweep(para, t, info["convergence"])
        if_ob = ((t + 1) % para["dt_ob"] == 0) or t == (para["sweep_time"] - 1)
        if if_ob:
            print("In the %d-th round of sweep ..." % (t + 1))
        order = list(range(para["ob_position"] + 1, l)) + list(range(l - 2, -1, -1)) + \
            list(range(1, para["ob_position"]))
        for k, n in enumerate(order):
            if para["if_print_detail"]:
                print("update the %d-th tensor ..." % n)
            if k == len(order) - 1:
                A.refine_next_solve()
            A.update_tensor_eigs(n, index1, index2, coeff1, coeff2, para["tau"], para["is_real"],
                                 tol=para["eigs_tol"])
        info["sweeps"] = t + 1
        if if_ob:
            ob["eb_full"] = A.observe_bond_energy(index2, coeff2)
            ob["mx"] = A.observe_magnetization(1)
            ob["mz"] = A.observe_magnetization(3)
            ob["e_per_site"] = float((np.sum(ob["eb_full"]) - para["hx"] * np.sum(ob["mx"]) -
                                      para["hz"] * np.sum(ob["mz"])) / A.length)
            info["convergence"] = abs(ob["e_per_site"] - e0_per_site)
            info["sweep_times"].append(time.time() - ts)
            if info["convergence"] < para["break_tol"]:
                print("Converged at the %d-th sweep with error = %g of energy per site." % (t + 1, info["convergence"]))
                break
            print("Convergence error of energy per site = %g" % info["convergence"])
            e0_per_site = ob["e_per_site"]
        else:
            info["sweep_times"].append(time.time() - ts)
        if t == para["sweep_time"] - 1 and info["convergence"] > para["break_tol"]:
            print("Not converged with error = %g of eb per bond" % info["convergence"])
            print("Consider to increase para['sweep_time']")
    ob["eb"] = get_bond_energies(ob["eb_full"], para["positions_h2"], para["index2"])
    A.calculate_entanglement_spectrum()
    A.calculate_entanglement_entropy()
    ob["corr_x"] = A.observe_correlators_from_middle(1, 1)
    ob["corr_z"] = A.observe_correlators_from_middle(3, 3)
    info["t_cost"] = time.time() - t_start
    info["solves"] = A.stats["solves"]
    info["matvecs"] = A.stats["matvecs"]
    print("Simulation finished in %g seconds" % info["t_cost"])
    A.clean_to_save()
    return ob, A, info, para


def refine_sweep(para, t, convergence):
    """Whether the local solves of sweep t refine their vectors to the FP64 tolerance (split-TF32
    path only; the FP64 path always solves to it). para['mixed_refine']: 'off' (default) lets the
    local solves stop at the split-TF32 floor; 'final' refines the last para['mixed_refine_sweeps']
    (1) sweeps of the schedule, and every sweep once the observed change of the energy per site is
    below 100 x break_tol; 'all' every sweep. On GB300 the refinement does not make the returned
    state more accurate: the effective Hamiltonian is assembled from environments contracted in
    split TF32, whose error (~1e-5 of the energy per site on an N=100 chain) a tighter local solve
    cannot remove, while the state's energy error stays second order (~1e-10 per site)."""
    mode = para.get("mixed_refine", "off")
    if mode == "all":
        return True
    if mode in ("off", None, False):
        return False
    if mode != "final":
        raise ValueError("mixed_refine must be 'final', 'all' or 'off'")
    if t >= para["sweep_time"] - int(para.get("mixed_refine_sweeps", 1)):
        return True
    bt = float(para.get("break_tol", -1.0))
    return bt > 0 and convergence < 100.0 * bt


def positions_set2array(pos_set):
    """DMRG_anyH.py:217-230."""
    pos = np.array([list(p) for p in pos_set], dtype=int).reshape(-1, 2)
    pos -= np.min(pos)
    for i in range(int(np.max(pos)) - 1, 0, -1):
        if np.count_nonzero(pos == i) == 0:
            pos -= (pos > i)
    return pos


def sort_positions(pos, which="ascend"):
    """Rows sorted by first site, then by second within equal first sites (DMRG_anyH.py:233-247)."""
    pos = np.asarray(pos).astype(int).reshape(-1, 2)
    order = np.lexsort((pos[:, 1], pos[:, 0]))
    if which == "descend":
        order = np.lexsort((pos[:, 1], -pos[:, 0]))
    return pos[order]


def get_bond_energies(eb_full, positions, index2):
    """Sum the per-term energies of each bond (DMRG_anyH.py:250-258)."""
    positions = np.asarray(positions)
    index2 = np.asarray(index2).reshape(-1, 4)
    eb_full = np.ravel(eb_full)
    eb = np.zeros((positions.shape[0], 1))
    for i in range(index2.shape[0]):
        hit = np.nonzero((index2[i, 0] == positions[:, 0]) & (index2[i, 1] == positions[:, 1]))
        eb[hit] += eb_full[i]
    return eb
