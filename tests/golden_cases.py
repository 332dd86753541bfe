"""Loaders for the golden fixtures written by tests/golden/make_golden.py."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RUN_CASES = ["chain_n12_chi16", "chain_n12_chi16_h", "ladder_2x4_chi8", "jigsaw_s1_n9_chi12", "longrange_n8_chi8"]
# further reference runs; their GPU parity test is in test_gpu_wider.py
LATER_CASES = ["j1j2_snake_4x3_chi16", "square_4x2_chi8", "full_n8_chi8", "chain_n10_chi8_ob3",
               "chain_n10_chi8_break", "chain_n10_chi16_pbc", "chain_s1_n8_chi9"]


def meta():
    with open(os.path.join(GOLDEN, "golden_meta.json")) as f:
        return json.load(f)


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def para_of(name, device="cuda", precision="fp64"):
    """The reference run's `para` (coupling tables exactly as the reference built them)."""
    g, m = load(name), meta()[name]
    return {
        "l": m["l"], "d": m["d"], "chi": m["chi"], "op": list(g["op"]), "index1": g["index1"],
        "index2": g["index2"], "coeff1": g["coeff1"], "coeff2": g["coeff2"], "positions_h2": g["positions_h2"],
        "tau": m["tau"], "eigs_tol": m["eigs_tol"], "sweep_time": m["sweep_time"], "dt_ob": m.get("dt_ob", 1), "break_tol": m.get("break_tol", -1.0),
        "hx": m["hx"], "hz": m["hz"], "ob_position": m.get("ob_position", 0), "if_print_detail": False, "is_real": True,
        "device": device, "precision": precision,
    }


def spectra(name):
    g = load(name)
    return np.split(g["lm_flat"], np.cumsum(g["lm_len"])[:-1])


def mps_of(name):
    g = load(name)
    n = len([k for k in g.files if k.startswith("mps_")])
    return [g["mps_%d" % k] for k in range(n)]


def max_spectrum_diff(a_list, b_list):
    out = 0.0
    for a, b in zip(a_list, b_list):
        a = np.sort(np.ravel(a))[::-1]
        b = np.sort(np.ravel(b))[::-1]
        k = min(len(a), len(b))
        if k:
            out = max(out, float(np.max(np.abs(a[:k] - b[:k]))))
        # extra values of the longer list must be ~0 (rank deficiency)
        out = max(out, float(np.max(np.abs(a[k:]), initial=0.0)), float(np.max(np.abs(b[k:]), initial=0.0)))
    return out
