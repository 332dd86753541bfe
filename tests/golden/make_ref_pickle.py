"""Write a result file with the reference's own ``save_pr`` (BasicFunctionsSJR.py:25-50).

Run by hand where the T-Nalg sources are mounted, with ``TNALG_REFERENCE`` set to their
directory (required)::

    TNALG_REFERENCE=<path to T-Nalg> python tests/golden/make_ref_pickle.py

It runs the unmodified reference ``dmrg_finite_size`` (DMRG_anyH.py:18) on an N=8
spin-1/2 XXZ chain (Jz = 0.6) with fields (chi=8, 6 sweeps, seed 4) through ``ref_shim`` and saves
``(ob, A, info, para)`` exactly as the reference's scripts do, into
``ref_result_chain_n8_h.pr``. The pickle holds the reference's ``MpsOpenBoundaryClass``
instance (module ``MPSClass``), which is what a user's existing result files contain. It also
writes ``ref_rdm_chain_n8_h.npz``: two-site reduced density matrices of that state from the
reference's ``reduced_density_matrix_two_body`` with the centre at sites 0, 4 and 7, and the
package layout's one-site density matrices and on-site entropies (library/MPSClass.py) of the
same state.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import ref_shim  # noqa: E402

ref_shim.install_package_layout()
import BasicFunctionsSJR as bf  # noqa: E402
import DMRG_anyH  # noqa: E402
import Parameters as Pm  # noqa: E402
from library import MPSClass as LibMPS  # noqa: E402


def main():
    para = Pm.generate_parameters_dmrg("chain")
    para.update(l=8, chi=8, jxy=1, jz=0.6, hx=0.7, hz=0.5, sweep_time=6, dt_ob=1, break_tol=-1.0,
                eigs_tol=1e-12, tau=1e-4, if_print_detail=False)
    para = Pm.make_consistent_parameter_dmrg(para)
    np.random.seed(4)
    ob, A, info, para = DMRG_anyH.dmrg_finite_size(para)
    # two-site reduced density matrices by the reference's own method (MPSClass.py:841-855), for
    # pairs left of, around and right of the centre
    rdm = {}
    for p1, p2 in ((0, 1), (1, 5), (2, 3), (3, 7), (6, 7)):
        for c in (0, 4, 7):
            A.correct_orthogonal_center(c)
            rdm["rdm_%d_%d_c%d" % (p1, p2, c)] = A.reduced_density_matrix_two_body(p1, p2)
    # one-site density matrices and on-site entropies by the package layout's methods
    # (library/MPSClass.py), applied to this state
    lib = LibMPS.MpsOpenBoundaryClass
    for c in (0, 4, 7):
        A.correct_orthogonal_center(c)
        ent, rho = lib.calculate_onsite_entanglement_entropy(A)
        rdm["onsite_ent_c%d" % c] = np.asarray(ent)
        rdm["onsite_rho_c%d" % c] = np.stack(rho)
        for p in (0, 3, 7):
            if p != c:   # the reference's transfer from the centre to p is empty for p == centre and fails
                rdm["rdm1_%d_c%d" % (p, c)] = lib.reduced_density_matrix_one_body(A, p)
    A.correct_orthogonal_center(0)
    np.savez_compressed(os.path.join(HERE, "ref_rdm_chain_n8_h.npz"), **rdm)
    A.clean_to_save()
    para.pop("data_path", None)   # a Windows-style path built from the working directory
    bf.save_pr(HERE, "ref_result_chain_n8_h.pr", [ob, A, info, para], ["ob", "A", "info", "para"])
    print("e_per_site", ob["e_per_site"])


if __name__ == "__main__":
    main()
