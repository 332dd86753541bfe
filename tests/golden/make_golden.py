"""Generate the golden fixtures in this directory from the unmodified reference.

Run by hand where the T-Nalg sources are mounted, with ``TNALG_REFERENCE`` set to their
directory (required)::

    TNALG_REFERENCE=<path to T-Nalg> python tests/golden/make_golden.py

It imports the reference through ``ref_shim`` (compatibility patches only) and
writes small ``.npz``/``.json`` files that the test suite reads; the tests never
import the reference themselves.

Cases (all with the reference's own ``dmrg_finite_size`` from DMRG_anyH.py:18,
``np.random.seed(seed)`` immediately before the call so that
``random_open_mps`` (TensorBasicModule.py:148) draws the initial MPS):

* ``chain_n12_chi16``      spin-1/2 Heisenberg chain, J=(1,1), h=0, 10 sweeps
* ``chain_n12_chi16_h``    same with hx=0.2, hz=0.3
* ``ladder_2x4_chi8``      'arbitrary' lattice: 2x4 ladder (straddling terms), hz field
* ``jigsaw_s1_n9_chi12``   spin-1 jigsaw chain (d=3)
* ``longrange_n8_chi8``    'longRange' lattice (all-to-all couplings)
* ``j1j2_snake_4x3_chi16`` J1-J2 square lattice (J2 = 0.5) in snake order, 'arbitrary' lattice, hz field
  (``python tests/golden/make_golden.py j1j2_snake_4x3_chi16`` runs this case alone)
* ``chain_s1_n8_chi9``     spin-1 Heisenberg chain (d = 3) in a field hz = 0.3
* ``chain_n10_chi16_pbc``  Heisenberg chain with periodic boundary (bond (0, 9) straddles every site), fields
* ``chain_n10_chi8_break`` XXZ chain (Jz = 1.3) with fields, observed every 2nd sweep, stopped by break_tol=1e-9
* ``chain_n10_chi8_ob3``   XXZ chain (Jz = 0.7) with fields, sweeps starting from site 3 (``ob_position``)
* ``full_n8_chi8``         the reference's 'full' lattice (all-to-all Ising couplings, transverse field hx=0.5)
* ``square_4x2_chi8``      the reference's 'square' lattice (row-major numbering), 4x2, no field (its
  make_consistent_parameter_dmrg appends the field operator instead of rebuilding the list, Parameters.py:190,
  so a field set after generate_parameters_dmrg never reaches index1)

plus the two shipped result pickles (data_dmrg/*.pr), a dense effective
Hamiltonian at one site (MPSClass.py:532 ``effective_hamiltonian_dmrg``), the
docstring examples of the contraction primitives, and the reference's exact
diagonalisation of the N=12 chain.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shim  # noqa: E402

MPSClass = ref_shim.install()
import BasicFunctionsSJR as bf  # noqa: E402
import DMRG_anyH  # noqa: E402
import HamiltonianModule as hm  # noqa: E402
import Parameters as pm  # noqa: E402
import TensorBasicModule as tbm  # noqa: E402

COMMON = dict(tau=1e-4, eigs_tol=1e-12, break_tol=-1.0, dt_ob=1)


def _history_hook():
    """Record e_per_site after every observed sweep (DMRG_anyH.py:65-70)."""
    hist = []
    C = MPSClass.MpsOpenBoundaryClass
    orig = C.observe_magnetization

    def om(self, sn):
        out = orig(self, sn)
        if sn == 3:
            hist.append(True)
        return out

    C.observe_magnetization = om
    return hist, lambda: setattr(C, "observe_magnetization", orig)


def run_case(name, para, seed, meta):
    # the default is_save_op=True run; its corr_z reads effective operators cached
    # before calculate_entanglement_spectrum re-gauged the MPS, so the run is repeated
    # with is_save_op=False (no cache) to record the correlators of the final state.
    para_nosave = dict(para)
    para_nosave["is_save_op"] = False
    np.random.seed(seed)
    ob2, _, _, _ = DMRG_anyH.dmrg_finite_size(para_nosave)
    MPSClass._shim_counter["solves"] = 0
    np.random.seed(seed)
    t0 = time.time()
    ob, A, info, para = DMRG_anyH.dmrg_finite_size(para)
    wall = time.time() - t0
    out = {
        "eb_full": np.ravel(ob["eb_full"]),
        "mx": np.ravel(ob["mx"]),
        "mz": np.ravel(ob["mz"]),
        "e_per_site": float(np.ravel(ob["e_per_site"])[0]),
        "eb": np.ravel(ob["eb"]),
        "corr_x": np.ravel(ob["corr_x"]),
        "corr_z": np.ravel(ob["corr_z"]),
        "corr_x_nocache": np.ravel(ob2["corr_x"]),
        "corr_z_nocache": np.ravel(ob2["corr_z"]),
        "e_per_site_nocache": float(np.ravel(ob2["e_per_site"])[0]),
        "ent": np.ravel(A.ent),
        "virtual_dim": np.asarray(A.virtual_dim),
        "index1": np.asarray(para["index1"]),
        "index2": np.asarray(para["index2"]),
        "coeff1": np.ravel(np.asarray(para["coeff1"], dtype=float)),
        "coeff2": np.ravel(np.asarray(para["coeff2"], dtype=float)),
        "positions_h2": np.asarray(para["positions_h2"]).astype(int),
        "op": np.stack([np.real(o) for o in para["op"]]),
        "center": A.center,
    }
    lm = A.lm
    out["lm_len"] = np.array([len(np.ravel(x)) for x in lm])
    out["lm_flat"] = np.concatenate([np.ravel(x) for x in lm]) if lm else np.zeros(0)
    for k, t in enumerate(A.mps):
        out["mps_%d" % k] = t
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    meta[name] = {
        "seed": seed,
        "e_per_site": out["e_per_site"],
        "convergence": float(np.ravel(info["convergence"])[0]),
        "wall_s": wall,
        "l": int(para["l"]),
        "d": int(para["d"]),
        "chi": int(para["chi"]),
        "sweep_time": int(para["sweep_time"]),
        "dt_ob": int(para.get("dt_ob", 1)),
        "break_tol": float(para.get("break_tol", -1.0)),
        "tau": para["tau"],
        "eigs_tol": para["eigs_tol"],
        "hx": float(para.get("hx", 0.0)),
        "hz": float(para.get("hz", 0.0)),
        "lattice": para["lattice"],
        "ob_position": int(para.get("ob_position", 0)),
        "eig_solves": MPSClass._shim_counter["solves"],
    }
    MPSClass._shim_counter["solves"] = 0
    print(name, out["e_per_site"], "%.2fs" % wall)
    return ob, A, para


def chain_para(l, chi, jxy, jz, hx, hz, sweeps):
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=l, chi=chi, jxy=jxy, jz=jz, hx=hx, hz=hz, sweep_time=sweeps, **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def chain_s1_para(l, chi, hz, sweeps):
    """Spin-1 Heisenberg chain (d = 3); the field hz splits the open chain's edge-spin degeneracy."""
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=l, chi=chi, spin="one", jxy=1, jz=1, hx=0.0, hz=hz, sweep_time=sweeps, **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def chain_para_bc(l, chi, jxy, jz, hx, hz, sweeps, bound_cond):
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=l, chi=chi, jxy=jxy, jz=jz, hx=hx, hz=hz, sweep_time=sweeps, bound_cond=bound_cond, **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def ladder_para(length, chi, j_leg, j_rung, hz, sweeps):
    """2 x length ladder numbered rung by rung: sites (2r, 2r+1) form rung r."""
    para = pm.generate_parameters_dmrg("arbitrary")
    para["hx"] = 0.0
    para["hz"] = hz
    para["op"].append(-para["hx"] * para["op"][1] - para["hz"] * para["op"][3])
    bonds, cs = [], []
    for r in range(length):
        bonds.append((2 * r, 2 * r + 1))
        cs.append(j_rung)
        if r + 1 < length:
            bonds.append((2 * r, 2 * r + 2))
            cs.append(j_leg)
            bonds.append((2 * r + 1, 2 * r + 3))
            cs.append(j_leg)
    index2, coeff2 = [], []
    for (i, j), c in zip(bonds, cs):
        index2 += [[i, j, 4, 5], [i, j, 5, 4], [i, j, 3, 3]]
        coeff2 += [c / 2, c / 2, c]
    para["index2"] = index2
    para["coeff2"] = coeff2
    para["index1"] = [[n, 6] for n in range(2 * length)]
    para["coeff1"] = [1.0] * (2 * length)
    para.update(chi=chi, sweep_time=sweeps, **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def jigsaw_para(l, chi, sweeps):
    para = pm.generate_parameters_dmrg("jigsaw")
    para.update(l=l, chi=chi, hz=0.1, sweep_time=sweeps, **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def longrange_para(l, chi, sweeps):
    para = pm.generate_parameters_dmrg("longRange")
    para.update(l=l, chi=chi, jxy=1.0, jz=1.0, hx=0.3, hz=0.2, sweep_time=sweeps, **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def j1j2_para(width, height, chi, hz, sweeps):
    """J1-J2 (J2 = 0.5) square lattice in snake order through the reference's 'arbitrary' lattice;
    the bond list is written out here (even rows left to right, odd rows right to left)."""
    def site(x, y):
        return y * width + (x if y % 2 == 0 else width - 1 - x)

    bonds = []
    for y in range(height):
        for x in range(width):
            if x + 1 < width:
                bonds.append((site(x, y), site(x + 1, y), 1.0))
            if y + 1 < height:
                bonds.append((site(x, y), site(x, y + 1), 1.0))
    for y in range(height - 1):
        for x in range(width - 1):
            bonds.append((site(x, y), site(x + 1, y + 1), 0.5))
            bonds.append((site(x + 1, y), site(x, y + 1), 0.5))
    bonds = sorted((min(i, j), max(i, j), c) for i, j, c in bonds)
    bonds = [b for b in bonds if b[2] == 1.0] + [b for b in bonds if b[2] == 0.5]
    para = pm.generate_parameters_dmrg("arbitrary")
    para["hx"] = 0.0
    para["hz"] = hz
    para["op"].append(-para["hx"] * para["op"][1] - para["hz"] * para["op"][3])
    index2, coeff2 = [], []
    for i, j, c in bonds:
        index2 += [[i, j, 4, 5], [i, j, 5, 4], [i, j, 3, 3]]
        coeff2 += [c / 2, c / 2, c]
    para["index2"] = index2
    para["coeff2"] = coeff2
    para["index1"] = [[n, 6] for n in range(width * height)]
    para["coeff1"] = [1.0] * (width * height)
    para.update(chi=chi, sweep_time=sweeps, **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def square_para(width, height, chi, hx, hz, sweeps):
    para = pm.generate_parameters_dmrg("square")
    para.update(square_width=width, square_height=height, chi=chi, jxy=1, jz=1, hx=hx, hz=hz, sweep_time=sweeps,
                **COMMON)
    return pm.make_consistent_parameter_dmrg(para)


def full_para(l, chi, sweeps):
    para = pm.generate_parameters_dmrg("full")
    para.update(l=l, chi=chi, sweep_time=sweeps, **COMMON)   # defaults jxy=0, jz=1, hx=0.5, hz=0
    return pm.make_consistent_parameter_dmrg(para)


EXTRA = {
    "j1j2_snake_4x3_chi16": lambda meta: run_case("j1j2_snake_4x3_chi16", j1j2_para(4, 3, 16, 0.1, 40), 5, meta),
    "full_n8_chi8": lambda meta: run_case("full_n8_chi8", full_para(8, 8, 8), 7, meta),
    "chain_n10_chi8_break": lambda meta: run_case("chain_n10_chi8_break",
                                                  dict(chain_para(10, 8, 1, 1.3, 0.1, 0.25, 40), dt_ob=2,
                                                       break_tol=1e-9), 9, meta),
    "chain_s1_n8_chi9": lambda meta: run_case("chain_s1_n8_chi9", chain_s1_para(8, 9, 0.3, 80), 12, meta),
    "chain_n10_chi16_pbc": lambda meta: run_case("chain_n10_chi16_pbc",
                                                 dict(chain_para_bc(10, 16, 1, 1, 0.15, 0.2, 16, "periodic")), 10,
                                                 meta),
    "chain_n10_chi8_ob3": lambda meta: run_case("chain_n10_chi8_ob3",
                                                dict(chain_para(10, 8, 1, 0.7, 0.2, 0.3, 12), ob_position=3), 8, meta),
    "square_4x2_chi8": lambda meta: run_case("square_4x2_chi8", square_para(4, 2, 8, 0.0, 0.0, 60), 6, meta),
}


def dense_heff(A, para, p, name):
    """Dense effective Hamiltonian (MPSClass.py:532-580) of the MPS A at site p."""
    A._is_save_op = False
    A.correct_orthogonal_center(p)
    h, s = A.effective_hamiltonian_dmrg(p, np.asarray(para["index1"]), np.asarray(para["index2"]),
                                        np.ravel(para["coeff1"]), np.ravel(para["coeff2"]))
    out = {"h": h, "shape": np.array(s), "p": p}
    for k, t in enumerate(A.mps):
        out["mps_%d" % k] = t
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def pickled_fixtures(meta):
    for chi in (16, 24):
        fn = os.path.join(ref_shim.REF_ROOT, "data_dmrg", "chainN12_j(1,1)_h(0,0)_chi%dopen.pr" % chi)
        ob, A, info, para = bf.load_pr(fn, ("ob", "A", "info", "para"))
        out = {
            "eb_full": np.ravel(ob["eb_full"]).astype(float),
            "mx": np.ravel(ob["mx"]).astype(float),
            "mz": np.ravel(ob["mz"]).astype(float),
            "e_per_site": float(np.ravel(ob["e_per_site"])[0]),
            "index1": np.asarray(para["index1"]),
            "index2": np.asarray(para["index2"]),
            "coeff1": np.ravel(np.asarray(para["coeff1"], dtype=float)),
            "coeff2": np.ravel(np.asarray(para["coeff2"], dtype=float)),
            "op": np.stack([np.real(o) for o in para["op"]]),
            "virtual_dim": np.asarray(A.virtual_dim),
            "center": A.center,
            "orthogonality": np.ravel(A.orthogonality),
        }
        for k in ("corr_x", "corr_z", "eb"):
            if k in ob:
                out[k] = np.ravel(ob[k]).astype(float)
        out["ent"] = np.ravel(A.ent)
        for k, t in enumerate(A.mps):
            out["mps_%d" % k] = t
        np.savez_compressed(os.path.join(HERE, "pickle_chi%d.npz" % chi), **out)
        meta["pickle_chi%d" % chi] = {
            "e_per_site": out["e_per_site"],
            "t_cost": float(info.get("t_cost", -1)),
            "convergence": float(np.ravel(info.get("convergence", -1))[0]),
            "l": int(para["l"]),
            "chi": int(para["chi"]),
            "hx": float(para.get("hx", 0.0)),
            "hz": float(para.get("hz", 0.0)),
            "keys": sorted(ob.keys()),
        }


def docstring_kats(meta):
    T = np.array([[[1, 2, 1], [2, 1, 2]], [[2, 0, 2], [1, 3, 1]], [[3, 1, 0], [2, 2, 1]]], dtype=float)
    v = np.array([[1, 1, 1], [1, 2, 1], [2, 2, 1]], dtype=float)
    T2 = np.array([[[1, 2], [2, 3]], [[3, 4], [4, 5]]], dtype=float)
    M = np.array([[1, 3], [2, 4]], dtype=float)
    ones = np.ones((2, 2, 2))
    mats = [np.array([[1, 2], [2, 3]], float), np.array([[2, 3], [3, 4]], float), np.array([[3, 4], [4, 5]], float)]
    kat = {
        "T": T.tolist(),
        "v": v.tolist(),
        "bound_l2r": tbm.bound_vec_operator_left2right(T).tolist(),
        "bound_l2r_v": tbm.bound_vec_operator_left2right(T, v=v).tolist(),
        "bound_r2l": tbm.bound_vec_operator_right2left(T).tolist(),
        "bound_r2l_v": tbm.bound_vec_operator_right2left(T, v=v).tolist(),
        "T2": T2.tolist(),
        "M": M.tolist(),
        "absorb_bond2": tbm.absorb_matrix2tensor(T2, M, 2).tolist(),
        "absorb_bond0": tbm.absorb_matrix2tensor(T2, M, 0).tolist(),
        "absorb_bond1": tbm.absorb_matrix2tensor(T2, M, 1).tolist(),
        "mats": [m.tolist() for m in mats],
        "absorb_full": tbm.absorb_matrices2tensor_full_fast(ones, [m.copy() for m in mats]).tolist(),
        "entropy_lm": [2, 1, 0.5, 0.3, 0],
        "entropy": float(tbm.entanglement_entropy(np.array([2, 1, 0.5, 0.3, 0.0]))),
    }
    op_t = np.array([[0.5, 0.0], [0.0, -0.5]])
    kat["bound_l2r_op_v"] = tbm.bound_vec_operator_left2right(T[:, :2, :] * 0 + T[:, :2, :], op_t, v).tolist()
    kat["bound_r2l_op_v"] = tbm.bound_vec_operator_right2left(T[:, :2, :], op_t, v).tolist()
    kat["op_t"] = op_t.tolist()
    with open(os.path.join(HERE, "kat_primitives.json"), "w") as f:
        json.dump(kat, f, indent=1)


def reference_ed(meta):
    """The reference's exact diagonalisation (algorithms/ExactDiagonalizationAlgo.py:12)."""
    import types
    for m in ("matplotlib.cm", "mpl_toolkits", "mpl_toolkits.mplot3d"):
        sys.modules.setdefault(m, types.ModuleType(m))
    sys.modules["matplotlib"].cm = sys.modules["matplotlib.cm"]
    sys.modules["mpl_toolkits.mplot3d"].Axes3D = object
    try:
        from algorithms.ExactDiagonalizationAlgo import exact_ground_state
        from library.Parameters import parameters_ed_ground_state
    except Exception as exc:  # pragma: no cover - depends on the mount
        meta["ed_chain_n12"] = {"error": repr(exc)}
        return
    para = parameters_ed_ground_state("chain")
    para["l"] = 12
    para = dict(para)
    try:
        from library.Parameters import make_consistent_parameter_ed
        para = make_consistent_parameter_ed(para)
    except Exception:
        pass
    np.random.seed(0)
    a, ob = exact_ground_state(para)
    meta["ed_chain_n12"] = {
        "e_eig": float(np.ravel(ob["e_eig"])[0]),
        "e_site": float(np.ravel(ob["e_site"])[0]),
        "jx": para.get("jx"), "jy": para.get("jy"), "jz": para.get("jz"),
        "hx": para.get("hx"), "hz": para.get("hz"), "l": para.get("l"),
    }


def main(argv=()):
    if argv:   # only the named extra cases, merged into the existing metadata
        with open(os.path.join(HERE, "golden_meta.json")) as f:
            meta = json.load(f)
        for name in argv:
            EXTRA[name](meta)
        with open(os.path.join(HERE, "golden_meta.json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        return
    meta = {}
    run_case("chain_n12_chi16", chain_para(12, 16, 1, 1, 0, 0, 10), 0, meta)
    ob, A, para = run_case("chain_n12_chi16_h", chain_para(12, 16, 1, 1, 0.2, 0.3, 10), 0, meta)
    dense_heff(A, para, 5, "heff_chain_n12_chi16_h_p5")
    ob, A, para = run_case("ladder_2x4_chi8", ladder_para(4, 8, 1.0, 0.7, 0.15, 16), 1, meta)
    dense_heff(A, para, 3, "heff_ladder_2x4_chi8_p3")
    run_case("jigsaw_s1_n9_chi12", jigsaw_para(9, 12, 16), 2, meta)
    run_case("longrange_n8_chi8", longrange_para(8, 8, 8), 3, meta)
    for fn in EXTRA.values():
        fn(meta)
    pickled_fixtures(meta)
    docstring_kats(meta)
    reference_ed(meta)
    with open(os.path.join(HERE, "golden_meta.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(json.dumps(meta, indent=1, sort_keys=True, default=str))


if __name__ == "__main__":
    main(sys.argv[1:])
