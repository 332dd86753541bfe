"""Exact diagonalisation for small lattices — TEST INFRASTRUCTURE ONLY.

Restates the reference's matrix-free ED (library/EDspinClass.py:69-77,
``project_all_hamilt``; driven by algorithms/ExactDiagonalizationAlgo.py:12-34)
on the same coupling lists the DMRG consumes: H = sum_two-body c * op_a(i) op_b(j)
+ sum_one-body c * op(q). The ground state comes from scipy's eigsh ('SA') on a
sparse matrix instead of the reference's 'LM' of I - tau*H; both give the
lowest eigenvalue. Sizes: d**l <= ~2**18.
"""
import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import eigsh


def _site_op(op, q, l, d):
    left = sp.identity(d ** q, format="csr")
    right = sp.identity(d ** (l - q - 1), format="csr")
    return sp.kron(sp.kron(left, sp.csr_matrix(op)), right, format="csr")


def hamiltonian(l, d, ops, index1, coeff1, index2, coeff2):
    ops = [np.real_if_close(np.asarray(o)) for o in ops]
    dim = d ** l
    h = sp.csr_matrix((dim, dim))
    index1 = np.asarray(index1).reshape(-1, 2) if np.size(index1) else np.zeros((0, 2), int)
    index2 = np.asarray(index2).reshape(-1, 4) if np.size(index2) else np.zeros((0, 4), int)
    c1 = np.ravel(np.asarray(coeff1, dtype=float)) if np.size(coeff1) else np.zeros(0)
    c2 = np.ravel(np.asarray(coeff2, dtype=float)) if np.size(coeff2) else np.zeros(0)
    for n in range(index1.shape[0]):
        if c1[n] != 0:
            h = h + c1[n] * _site_op(ops[int(index1[n, 1])], int(index1[n, 0]), l, d)
    for n in range(index2.shape[0]):
        if c2[n] != 0:
            i, j, a, b = (int(x) for x in index2[n])
            h = h + c2[n] * (_site_op(ops[a], i, l, d) @ _site_op(ops[b], j, l, d))
    return h


def ground_state(l, d, ops, index1, coeff1, index2, coeff2):
    """Returns (E0, psi0) with psi0 a unit vector in the site-major basis |s_0 s_1 ... s_{l-1}>."""
    h = hamiltonian(l, d, ops, index1, coeff1, index2, coeff2)
    rng = np.random.default_rng(0)
    w, v = eigsh(h, k=1, which="SA", v0=rng.standard_normal(h.shape[0]), tol=1e-14)
    return float(w[0]), v[:, 0]
