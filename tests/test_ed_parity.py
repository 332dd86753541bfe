"""DMRG against exact diagonalisation on every lattice generator (CPU, numpy test double of the C ABI).

At the full bond dimension chi = d^(N/2) the MPS spans the whole Hilbert space, so the converged
one-site DMRG energy must equal the exact ground-state energy (oracle/ed.py, sparse eigsh on the
same coupling lists). N <= 12 here; the GPU version (tests/test_gpu_wider.py) runs 12 to 16 sites.
"""
import contextlib
import io

import numpy as np
import pytest


def _quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def lattice_para(kind, size):
    """Coupling lists of the named lattice with `size` sites (rungs for the ladder; width x height
    from SQUARE[size] for the square lattices); fields on, so ground states are unique."""
    from tnalg_gb300 import Parameters as pm, serving
    if kind == "chain":
        para = pm.generate_parameters_dmrg("chain")
        para.update(l=size, jxy=1.0, jz=0.8, hx=0.3, hz=0.2)
    elif kind == "ladder":
        return serving.ladder_job_para(size // 2, 64, j_rung=1.4, jz=0.9, hz=0.25, device="cpu")
    elif kind == "jigsaw":   # spin 1 (d = 3) by default
        para = pm.generate_parameters_dmrg("jigsaw")
        para.update(l=size, hz=0.15)
    elif kind == "full":
        para = pm.generate_parameters_dmrg("full")
        para.update(l=size, jxy=0.7, jz=1.0, hx=0.4, hz=0.1)
    elif kind == "longRange":
        para = pm.generate_parameters_dmrg("longRange")
        para.update(l=size, alpha=1.5, jxy=1.0, jz=1.0, hx=0.3)
    elif kind == "square":
        w, h = SQUARE[size]
        para = pm.generate_parameters_dmrg("square")
        para.update(square_width=w, square_height=h, hx=0.2, hz=0.1)
    elif kind == "j1j2":
        w, h = SQUARE[size]
        return pm.generate_parameters_j1j2_snake(w, h, j2=0.5, hx=0.1, hz=0.2)
    else:
        raise ValueError(kind)
    return pm.make_consistent_parameter_dmrg(para)


SQUARE = {9: (3, 3), 12: (4, 3), 16: (4, 4)}
# sites per lattice on the CPU (the test double is numpy); the GPU version runs larger ones
CPU_CASES = [("chain", 12), ("ladder", 12), ("jigsaw", 7), ("full", 10), ("longRange", 10), ("square", 9),
             ("j1j2", 9)]


def run_against_ed(kind, size, device, sweeps=2):
    from oracle import ed
    from tnalg_gb300 import DMRG_anyH
    para = dict(lattice_para(kind, size))
    l, d = para["l"], para["d"]
    para.update(chi=d ** (l // 2), sweep_time=sweeps, dt_ob=1, break_tol=1e-13, eigs_tol=1e-12, tau=1e-4,
                device=device)
    np.random.seed(11)
    ob, A, info, _ = _quiet(DMRG_anyH.dmrg_finite_size, para)
    e0 = ed.ground_state(l, d, para["op"], para["index1"], para["coeff1"], para["index2"], para["coeff2"])[0]
    return ob["e_per_site"] * l, e0


@pytest.mark.parametrize("kind,size", CPU_CASES)
def test_full_bond_dimension_reaches_the_exact_ground_state(fake_backend, kind, size):
    """Two sweeps suffice: at full bond dimension the environments of random isometries already span
    the whole space, so every local problem is the full one."""
    e, e0 = run_against_ed(kind, size, "cpu")
    assert abs(e - e0) <= 1e-9 * abs(e0), (kind, e, e0)
