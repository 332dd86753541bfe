"""End-to-end parity of the GPU DMRG with the reference (golden fixtures) and the oracle."""
import contextlib
import io

import numpy as np
import pytest
import torch

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def _run_golden(name, precision="fp64"):
    from tnalg_gb300 import DMRG_anyH
    m = gc.meta()[name]
    np.random.seed(m["seed"])
    return _quiet(DMRG_anyH.dmrg_finite_size, gc.para_of(name, precision=precision))


@pytest.mark.parametrize("name", gc.RUN_CASES)
def test_fp64_path_matches_reference_run(cuda_lib, name):
    """Same seeded MPS, same sweep schedule: energy to 1e-10 relative, observables to 1e-8."""
    g, m = gc.load(name), gc.meta()[name]
    ob, A, info, para = _run_golden(name)
    e_ref = float(g["e_per_site"])
    assert abs(ob["e_per_site"] - e_ref) <= 1e-10 * abs(e_ref)
    obs_tol = 1e-8 if name != "jigsaw_s1_n9_chi12" else 5e-8
    np.testing.assert_allclose(np.ravel(ob["eb_full"]), g["eb_full"], atol=obs_tol)
    np.testing.assert_allclose(np.ravel(ob["mx"]), g["mx"], atol=obs_tol)
    np.testing.assert_allclose(np.ravel(ob["mz"]), g["mz"], atol=obs_tol)
    np.testing.assert_allclose(ob["corr_x"], g["corr_x_nocache"], atol=obs_tol)
    np.testing.assert_allclose(ob["corr_z"], g["corr_z_nocache"], atol=obs_tol)
    np.testing.assert_allclose(np.ravel(ob["eb"]), g["eb"], atol=obs_tol)
    np.testing.assert_allclose(np.ravel(A.ent), g["ent"], atol=obs_tol)
    assert gc.max_spectrum_diff(A.lm, gc.spectra(name)) < obs_tol
    assert (A.virtual_dim == g["virtual_dim"]).all()
    assert info["solves"] == m.get("eig_solves", 2 * (m["l"] - 1) * m["sweep_time"])


def test_chain_n12_energy_against_exact_diagonalisation(cuda_lib):
    ob, A, info, para = _run_golden("chain_n12_chi16")
    e_ed = gc.meta()["ed_chain_n12"]["e_eig"]
    e = ob["e_per_site"] * 12
    assert 0 <= e - e_ed < 1e-6  # variational, within the chi=16 truncation error


def test_device_observables_on_pickled_fixture(cuda_lib):
    """The MPS shipped in data_dmrg/chainN12_..._chi16open.pr: observables equal the pickled ones."""
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    g = gc.load("pickle_chi16")
    mps = gc.mps_of("pickle_chi16")
    A = MpsOpenBoundaryClass(12, 2, 16, operators=list(g["op"]), tensors=mps)
    A.correct_orthogonal_center(0)
    eb = A.observe_bond_energy(g["index2"], g["coeff2"])
    np.testing.assert_allclose(np.ravel(eb), g["eb_full"], atol=1e-9)
    np.testing.assert_allclose(np.ravel(A.observe_magnetization(3)), g["mz"], atol=1e-9)
    assert abs(np.sum(eb) / 12 - float(g["e_per_site"])) < 1e-12
    # moving the centre must not change gauge-invariant observables
    A.correct_orthogonal_center(7)
    np.testing.assert_allclose(np.ravel(A.observe_bond_energy(g["index2"], g["coeff2"])), g["eb_full"], atol=1e-9)


def test_dense_effective_hamiltonian_matches_reference(cuda_lib):
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    for hname, src, p in (("heff_chain_n12_chi16_h_p5", "chain_n12_chi16_h", 5),
                          ("heff_ladder_2x4_chi8_p3", "ladder_2x4_chi8", 3)):
        h, g, m = gc.load(hname), gc.load(src), gc.meta()[src]
        n = len([f for f in h.files if f.startswith("mps_")])
        A = MpsOpenBoundaryClass(n, m["d"], m["chi"], operators=list(g["op"]),
                                 tensors=[h["mps_%d" % k] for k in range(n)])
        A._dev.center = p
        A._dev.orthogonality[:p] = -1
        A._dev.orthogonality[p + 1:] = 1
        dense, s = A.effective_hamiltonian_dmrg(p, g["index1"], g["index2"], g["coeff1"], g["coeff2"])
        np.testing.assert_allclose(dense, h["h"], atol=1e-11)


def test_larger_chain_against_oracle(cuda_lib):
    """XXZ chain with fields, N=24, chi=32, 3 sweeps: GPU FP64 path vs the numpy oracle."""
    from oracle import dmrg_oracle as O
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=24, chi=32, jxy=1.0, jz=0.7, hx=0.15, hz=0.25, sweep_time=3, dt_ob=1, break_tol=-1.0,
                tau=1e-4, eigs_tol=1e-12)
    para = pm.make_consistent_parameter_dmrg(para)
    np.random.seed(7)
    ob, A, info, _ = _quiet(DMRG_anyH.dmrg_finite_size, para)
    ob_o, A_o, info_o = O.dmrg_finite_size(24, 2, 32, para["op"], para["index1"], para["coeff1"], para["index2"],
                                           para["coeff2"], para["positions_h2"], tau=1e-4, eigs_tol=1e-12,
                                           sweep_time=3, hx=0.15, hz=0.25, seed=7)
    assert abs(ob["e_per_site"] - ob_o["e_per_site"]) <= 1e-10 * abs(ob_o["e_per_site"])
    np.testing.assert_allclose(np.ravel(ob["mz"]), ob_o["mz"], atol=1e-8)
    np.testing.assert_allclose(np.ravel(ob["eb_full"]), ob_o["eb_full"], atol=1e-8)


def test_canonical_form_invariants(cuda_lib):
    """After a sweep: left tensors are left-orthonormal, right tensors right-orthonormal, centre unit-norm."""
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=16, chi=24, sweep_time=1, dt_ob=1, break_tol=-1.0, eigs_tol=1e-10)
    para = pm.make_consistent_parameter_dmrg(para)
    np.random.seed(1)
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    A = MpsOpenBoundaryClass(16, 2, 24, operators=para["op"])
    A.correct_orthogonal_center(0)
    for n in list(range(1, 16)) + list(range(14, 7, -1)):
        A.update_tensor_eigs(n, para["index1"], para["index2"], para["coeff1"], para["coeff2"], 1e-4, True, 1e-10)
    c = A.center
    assert c == 8
    for k, t in enumerate(A.mps_device):
        cl, d, cr = t.shape
        if k < c:
            m = t.reshape(cl * d, cr)
            err = torch.max(torch.abs(m.T @ m - torch.eye(cr, dtype=torch.float64, device=t.device)))
        elif k > c:
            m = t.reshape(cl, d * cr)
            err = torch.max(torch.abs(m @ m.T - torch.eye(cl, dtype=torch.float64, device=t.device)))
        else:
            err = abs(torch.linalg.vector_norm(t) - 1.0)
        assert float(err) < 1e-12, (k, float(err))

