"""The ``para`` dictionary of the finite-size DMRG (drop-in for T-Nalg's Parameters.py).

Keys, defaults and the coupling tables follow Parameters.py:6-281 (plus the
'husimi' lattice of library/Parameters.py:151-163,309-324). Lattice names are
compared by value, so strings built at run time work too (the reference uses
``is`` and silently falls through for non-interned strings).

Keys that only this implementation reads (ignored by the reference):
    'precision'       'fp64' (plain, the drop-in) or 'tf32x3' (tensor-core matvec and
                      environment contractions, FP64 Lanczos / QR / observables)
    'device'          CUDA device of the run (default 'cuda')
    'lanczos_krylov'  Lanczos vectors per restart (default 40)
    'lanczos_tol_cap' if > 0, cap on the relative residual of each local solve
"""
import numpy as np

from . import HamiltonianModule as hm

LATTICES = ("chain", "square", "arbitrary", "jigsaw", "full", "longRange", "husimi")


def common_parameters_dmrg():
    """Parameters.py:6-25."""
    para = dict()
    para["chi"] = 30
    para["sweep_time"] = 100
    para["if_print_detail"] = False
    para["tau"] = 1e-4
    para["eigs_tol"] = 1e-5
    para["break_tol"] = 1e-8
    para["is_real"] = True
    para["dt_ob"] = 4
    para["ob_position"] = 0
    para["eigWay"] = 1
    para["isParallel"] = False
    para["isParallelEnvLMR"] = False
    para["is_save_op"] = True
    para["data_path"] = ".\\data_dmrg\\"
    para["precision"] = "fp64"
    para["device"] = "cuda"
    return para


def _spin_op_list(spin):
    op = hm.spin_operators(spin)
    return [op["id"], op["sx"], op["sy"], op["sz"], op["su"], op["sd"]]


def parameter_dmrg_arbitrary():
    """Parameters.py:28-60."""
    para = dict()
    para["spin"] = "half"
    para["op"] = _spin_op_list(para["spin"])
    para["index1"] = [[0, 6], [1, 6], [2, 6]]
    para["coeff1"] = [0.1, 0.1, 0.1]
    para["index2"] = [[0, 1, 3, 3], [1, 2, 3, 3]]
    para["coeff2"] = [1, 1]
    para["lattice"] = "arbitrary"
    para["data_exp"] = "Put_here_your_file_name_to_save_data"
    return para


def parameter_dmrg_chain():
    """Parameters.py:64-76."""
    return {"spin": "half", "bound_cond": "open", "l": 18, "jxy": 1, "jz": 1, "hx": 0, "hz": 0, "lattice": "chain"}


def parameter_dmrg_jigsaw():
    """Parameters.py:80-93."""
    return {"spin": "one", "bound_cond": "open", "l": 21, "jxy": 1, "jz": 1, "jxy1": 1, "jz1": 1, "hx": 0, "hz": 0,
            "lattice": "jigsaw"}


def parameter_dmrg_square():
    """Parameters.py:97-111."""
    para = {"bound_cond": "open", "square_width": 4, "square_height": 4, "spin": "half"}
    para["op"] = _spin_op_list(para["spin"])
    para.update(jxy=1, jz=1, hx=0, hz=0, lattice="square")
    return para


def parameter_dmrg_full():
    """Parameters.py:115-125."""
    return {"spin": "half", "l": 6, "jxy": 0, "jz": 1, "hx": 0.5, "hz": 0, "lattice": "full"}


def parameter_dmrg_long_range():
    """Parameters.py:128-139."""
    return {"spin": "half", "alpha": 1, "l": 6, "jxy": 0, "jz": 1, "hx": 0.5, "hz": 0, "lattice": "longRange"}


def parameter_dmrg_husimi():
    """library/Parameters.py:151-163 (spin-1/2 convention of this file's other lattices)."""
    return {"spin": "half", "depth": 2, "jxy": 0, "jz": 1, "hx": 0.5, "hz": 0, "lattice": "husimi"}


def generate_parameters_dmrg(lattice="chain"):
    """Parameters.py:143-166."""
    makers = {"chain": parameter_dmrg_chain, "square": parameter_dmrg_square, "arbitrary": parameter_dmrg_arbitrary,
              "jigsaw": parameter_dmrg_jigsaw, "full": parameter_dmrg_full, "longRange": parameter_dmrg_long_range,
              "husimi": parameter_dmrg_husimi}
    if lattice not in makers:
        raise ValueError("Wrong input of lattice %r; choose one of %s" % (lattice, ", ".join(LATTICES)))
    para = makers[lattice]()
    para = dict(para, **common_parameters_dmrg())
    return make_consistent_parameter_dmrg(para)


def _uniform_heisenberg(para, positions, jxy_jz=None):
    """index1 / index2 / coeff tables of a uniform XXZ model on `positions` (Parameters.py:171-187)."""
    para["op"] = _spin_op_list(para["spin"])
    para["op"].append(-para["hx"] * para["op"][1] - para["hz"] * para["op"][3])
    l = para["l"]
    para["index1"] = np.vstack((np.arange(l), 6 * np.ones(l))).T.astype(int)
    para["positions_h2"] = positions
    para["index2"] = hm.interactions_position2full_index_heisenberg_two_body(positions)
    para["coeff1"] = np.ones((l, 1))
    nb = positions.shape[0]
    para["coeff2"] = np.zeros((nb * 3, 1))
    for n in range(nb):
        jxy, jz = (para["jxy"], para["jz"]) if jxy_jz is None else jxy_jz(n)
        para["coeff2"][n * 3] = jxy / 2
        para["coeff2"][n * 3 + 1] = jxy / 2
        para["coeff2"][n * 3 + 2] = jz


def make_consistent_parameter_dmrg(para):
    """Derived tables of Parameters.py:170-281 (re-runnable after the user edits `para`)."""
    lat = para["lattice"]
    if lat == "chain":
        _uniform_heisenberg(para, hm.positions_nearest_neighbor_1d(para["l"], para["bound_cond"]))
        para["data_exp"] = "chainN%d_j(%g,%g)_h(%g,%g)_chi%d" % (para["l"], para["jxy"], para["jz"], para["hx"],
                                                                 para["hz"], para["chi"]) + para["bound_cond"]
    elif lat == "square":
        para["l"] = para["square_width"] * para["square_height"]
        pos = hm.positions_nearest_neighbor_square(para["square_width"], para["square_height"], para["bound_cond"])
        _uniform_heisenberg(para, pos)
        para["data_exp"] = "square(%d,%d)N%d_j(%g,%g)_h(%g,%g)_chi%d" % (
            para["square_width"], para["square_height"], para["l"], para["jxy"], para["jz"], para["hx"], para["hz"],
            para["chi"]) + para["bound_cond"]
    elif lat == "arbitrary":
        para["coeff1"] = np.array(para["coeff1"], dtype=float).reshape(-1, 1)
        para["coeff2"] = np.array(para["coeff2"], dtype=float).reshape(-1, 1)
        para["index1"] = np.array(para["index1"]).reshape(-1, 2).astype(int)
        para["index2"] = np.array(para["index2"]).reshape(-1, 4).astype(int)
        para["l"] = int(max(para["index1"][:, 0].max(initial=0), para["index2"][:, 0].max(initial=0),
                            para["index2"][:, 1].max(initial=0)) + 1)
        para["positions_h2"] = from_index2_to_positions_h2(para["index2"])
        check_continuity_pos_h2(para["positions_h2"])
    elif lat == "jigsaw":
        if para["bound_cond"] == "open":
            if para["l"] % 2 == 0:
                print("Note: for OBC jigsaw, l has to be odd. Auto-change l = %g to %g" % (para["l"], para["l"] + 1))
                para["l"] += 1
        elif para["l"] % 2 == 1:
            print("Note: for PBC jigsaw, l has to be even. Auto-change l = %g to %g" % (para["l"], para["l"] + 1))
            para["l"] += 1
        pos = hm.positions_jigsaw_1d(para["l"], para["bound_cond"])
        n_chain = para["l"] - (para["bound_cond"] == "open")
        _uniform_heisenberg(para, pos, lambda n: (para["jxy"], para["jz"]) if n < n_chain
                            else (para["jxy1"], para["jz1"]))
        para["data_exp"] = "JigsawN%d_j(%g,%g,%g,%g)_h(%g,%g)_chi%d" % (
            para["l"], para["jxy"], para["jz"], para["jxy1"], para["jz1"], para["hx"], para["hz"],
            para["chi"]) + para["bound_cond"]
    elif lat == "full":
        _uniform_heisenberg(para, hm.positions_fully_connected(para["l"]))
        para["data_exp"] = "fullConnectedN%d_j(%g,%g)_h(%g,%g)_chi%d" % (para["l"], para["jxy"], para["jz"],
                                                                         para["hx"], para["hz"], para["chi"])
    elif lat == "longRange":
        pos = hm.positions_fully_connected(para["l"])
        dist = lambda n: abs(pos[n, 0] - pos[n, 1]) ** para["alpha"]  # noqa: E731
        _uniform_heisenberg(para, pos, lambda n: (para["jxy"] / dist(n), para["jz"] / dist(n)))
        para["data_exp"] = "longRangeN%d_j(%g,%g)_h(%g,%g)_chi%d_alpha%g" % (
            para["l"], para["jxy"], para["jz"], para["hx"], para["hz"], para["chi"], para["alpha"])
    elif lat == "husimi":
        pos = hm.positions_husimi(para["depth"])
        para["l"] = int(pos.max()) + 1
        _uniform_heisenberg(para, pos)
        para["data_exp"] = "HusimiDepth%d_j(%g,%g)_h(%g,%g)_chi%d" % (para["depth"], para["jxy"], para["jz"],
                                                                      para["hx"], para["hz"], para["chi"])
    else:
        raise ValueError("Wrong input of lattice %r; choose one of %s" % (lat, ", ".join(LATTICES)))
    para["d"] = physical_dim_from_spin(para["spin"])
    para["nh"] = np.asarray(para["index2"]).shape[0]
    return para


def generate_parameters_j1j2_snake(width=6, height=6, j1=1.0, j2=0.5, hx=0.0, hz=0.0, jz_ratio=1.0):
    """J1-J2 Heisenberg model on an open width x height square lattice, snake-ordered into a chain,
    as an 'arbitrary'-lattice para (the reference's route for such models, Parameters.py:205-212).

    Rows: for every bond, [i, j, su, sd], [i, j, sd, su], [i, j, sz, sz] with coefficients
    (J/2, J/2, jz_ratio J), J = j1 on nearest and j2 on diagonal bonds (J1 bonds first); one-body
    rows [n, 6] with op 6 = -hx sx - hz sz. Not in the reference.
    """
    para = generate_parameters_dmrg("arbitrary")
    para["hx"], para["hz"] = float(hx), float(hz)
    para["op"] = _spin_op_list(para["spin"])
    para["op"].append(-para["hx"] * para["op"][1] - para["hz"] * para["op"][3])
    pos1, pos2 = hm.positions_j1j2_square_snake(width, height)
    index2, coeff2 = [], []
    for pos, j in ((pos1, j1), (pos2, j2)):
        for i, k in pos:
            index2 += [[i, k, 4, 5], [i, k, 5, 4], [i, k, 3, 3]]
            coeff2 += [j / 2, j / 2, jz_ratio * j]
    n = width * height
    para.update(index1=[[q, 6] for q in range(n)], coeff1=[1.0] * n, index2=index2, coeff2=coeff2,
                square_width=width, square_height=height, j1=j1, j2=j2)
    return make_consistent_parameter_dmrg(para)


def from_index2_to_positions_h2(index2):
    """Unique sorted bond positions of index2 (Parameters.py:410-418)."""
    from .DMRG_anyH import sort_positions
    pos = sort_positions(np.asarray(index2)[:, :2])
    keep = [pos[0]]
    for row in pos[1:]:
        if not (row[0] == keep[-1][0] and row[1] == keep[-1][1]):
            keep.append(row)
    return np.array(keep)


def check_continuity_pos_h2(pos_h2):
    """Sites must be numbered 0..max without gaps (Parameters.py:421-433); raises instead of exit()."""
    p0, p1 = int(np.min(pos_h2)), int(np.max(pos_h2))
    if p0 != 0:
        raise ValueError("The numbering of sites should start with 0, not %d" % p0)
    missing = [n for n in range(p0 + 1, p1) if n not in pos_h2]
    if missing:
        raise ValueError("positions_h2 misses sites %s" % missing)


def physical_dim_from_spin(spin):
    """Parameters.py:440-446."""
    return {"half": 2, "one": 3}.get(spin, False)
