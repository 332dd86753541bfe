"""Result files on CPU: save_pr / load_pr (BasicFunctionsSJR.py:25-89) and reference-written files.

``tests/golden/ref_result_chain_n8_h.pr`` was written by the reference's own save_pr after its
dmrg_finite_size (tests/golden/make_ref_pickle.py); it holds the reference's MpsOpenBoundaryClass.
The MPS work runs through the numpy test double of the C ABI.
"""
import os

import numpy as np
import pytest

import golden_cases as gc

REF_FILE = os.path.join(gc.GOLDEN, "ref_result_chain_n8_h.pr")


def test_reference_result_file_loads_as_device_mps(fake_backend):
    from tnalg_gb300 import BasicFunctionsSJR as bf
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    ob, A, info, para = bf.load_pr(REF_FILE, ("ob", "A", "info", "para"), device="cpu")
    assert isinstance(A, MpsOpenBoundaryClass)
    assert A.length == para["l"] == 8 and A.center == 0
    assert list(A.virtual_dim) == [1, 2, 4, 8, 8, 8, 4, 2, 1]
    assert np.ravel(A.orthogonality).tolist() == [0] + [1] * 7
    assert len(A.lm) == 7 and A.ent.shape == (7, 1)
    # observables of the restored MPS equal the ones the reference pickled beside it
    eb = A.observe_bond_energy(para["index2"], para["coeff2"])
    np.testing.assert_allclose(np.ravel(eb), np.ravel(ob["eb_full"]), atol=1e-12)
    np.testing.assert_allclose(np.ravel(A.observe_magnetization(1)), np.ravel(ob["mx"]), atol=1e-12)
    np.testing.assert_allclose(np.ravel(A.observe_magnetization(3)), np.ravel(ob["mz"]), atol=1e-12)
    # the entanglement spectrum recomputed on the device equals the pickled one
    ent = np.ravel(A.ent).copy()
    A.calculate_entanglement_spectrum()
    A.calculate_entanglement_entropy()
    np.testing.assert_allclose(np.ravel(A.ent), ent, atol=1e-10)


def test_restored_mps_continues_sweeping(fake_backend):
    """A restored, converged MPS stays at the pickled energy under another sweep of local solves."""
    from tnalg_gb300 import BasicFunctionsSJR as bf
    ob, A, info, para = bf.load_pr(REF_FILE, ("ob", "A", "info", "para"), device="cpu")
    l = para["l"]
    for p in list(range(1, l)) + list(range(l - 2, -1, -1)):
        A.update_tensor_eigs(p, para["index1"], para["index2"], para["coeff1"], para["coeff2"], para["tau"],
                             para["is_real"], tol=para["eigs_tol"])
    eb = A.observe_bond_energy(para["index2"], para["coeff2"])
    mx, mz = A.observe_magnetization(1), A.observe_magnetization(3)
    e = (np.sum(eb) - para["hx"] * np.sum(mx) - para["hz"] * np.sum(mz)) / l
    assert abs(e - ob["e_per_site"]) <= 1e-10 * abs(ob["e_per_site"])


def test_save_load_roundtrip_and_name_forms(fake_backend, tmp_path):
    from tnalg_gb300 import BasicFunctionsSJR as bf
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    np.random.seed(5)
    A = MpsOpenBoundaryClass(6, 2, 4, device="cpu")
    A.correct_orthogonal_center(2)
    folder = str(tmp_path / "results" / "run1")
    bf.save_pr(folder, "r.pr", [A, {"e": -0.4}, "note"], ["A", "ob", "s"])
    path = os.path.join(folder, "r.pr")
    whole = bf.load_pr(path, device="cpu")
    assert sorted(whole) == ["A", "ob", "s"]
    B = whole["A"]
    assert B.center == 2 and (B.virtual_dim == A.virtual_dim).all()
    for a, b in zip(A.mps, B.mps):
        np.testing.assert_array_equal(a, b)
    assert bf.load_pr(path, "s", device="cpu") == "note"
    ob, s = bf.load_pr(path, ["ob", "s"], device="cpu")
    assert ob == {"e": -0.4} and s == "note"
    assert bf.load_pr(os.path.join(folder, "missing.pr")) is False
    assert bf.mkdir(folder) is True


def test_reference_script_imports_through_compat(fake_backend):
    """`from BasicFunctionsSJR import load_pr` with the module-name shims first on sys.path."""
    import importlib
    import sys
    compat = os.path.join(gc.GOLDEN, "..", "..", "tnalg_gb300", "compat")
    sys.path.insert(0, compat)
    try:
        bfs = importlib.import_module("BasicFunctionsSJR")
        A = bfs.load_pr(REF_FILE, "A", device="cpu")
        assert type(A).__module__ == "tnalg_gb300.MPSClass"
    finally:
        sys.path.remove(compat)
        sys.modules.pop("BasicFunctionsSJR", None)


def test_mismatched_pickled_dims_are_rejected(fake_backend):
    from tnalg_gb300 import BasicFunctionsSJR as bf
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    A = bf.load_pr(REF_FILE, "A", device="cpu")
    st = {"mps": A.mps, "virtual_dim": np.array([1, 2, 4, 8, 8, 8, 4, 2, 2]), "center": 0, "phys_dim": 2}
    obj = MpsOpenBoundaryClass.__new__(MpsOpenBoundaryClass)
    from tnalg_gb300 import MPSClass as M
    token = M.LOAD_DEVICE.set("cpu")
    try:
        with pytest.raises(ValueError):
            obj.__setstate__(dict(st))
    finally:
        M.LOAD_DEVICE.reset(token)


def test_two_site_density_matrices_match_the_reference(fake_backend):
    """reduced_density_matrix_two_body (MPSClass.py:841-855) on the restored state equals the
    reference's own values (tests/golden/ref_rdm_chain_n8_h.npz) for pairs left of, around and
    right of the centre; reversed arguments give the matrix in the order passed."""
    from tnalg_gb300 import BasicFunctionsSJR as bf
    g = np.load(os.path.join(gc.GOLDEN, "ref_rdm_chain_n8_h.npz"))
    A = bf.load_pr(REF_FILE, "A", device="cpu")
    for key in [k for k in g.files if k.startswith("rdm_")]:
        _, p1, p2, c = key.split("_")
        A.correct_orthogonal_center(int(c[1:]))
        np.testing.assert_allclose(A.reduced_density_matrix_two_body(int(p1), int(p2)), g[key], atol=1e-12)
    rev = A.reduced_density_matrix_two_body(5, 1)
    want = g["rdm_1_5_c0"].reshape(2, 2, 2, 2).transpose(1, 0, 3, 2).reshape(4, 4)
    np.testing.assert_allclose(rev, want, atol=1e-12)
    with pytest.raises(ValueError):
        A.reduced_density_matrix_two_body(3, 3)


def test_one_site_density_matrices_and_onsite_entropy(fake_backend):
    """reduced_density_matrix_one_body / calculate_onsite_entanglement_entropy (library/MPSClass.py)
    equal the package layout's own values on the same state, at centres 0, 4 and 7; the site at the
    centre (where the reference's method fails) gives the matrix of the on-site entropy pass."""
    from tnalg_gb300 import BasicFunctionsSJR as bf
    g = np.load(os.path.join(gc.GOLDEN, "ref_rdm_chain_n8_h.npz"))
    A = bf.load_pr(REF_FILE, "A", device="cpu")
    for c in (0, 4, 7):
        A.correct_orthogonal_center(c)
        ent, rho = A.calculate_onsite_entanglement_entropy()
        np.testing.assert_allclose(ent, g["onsite_ent_c%d" % c], atol=1e-12)
        np.testing.assert_allclose(np.stack(rho), g["onsite_rho_c%d" % c], atol=1e-12)
        for p in (0, 3, 7):
            r = A.reduced_density_matrix_one_body(p)
            want = g["rdm1_%d_c%d" % (p, c)] if p != c else g["onsite_rho_c%d" % c][p]
            np.testing.assert_allclose(r, want, atol=1e-12)
    assert 0.4 < float(np.min(ent)) < float(np.max(ent)) < np.log(2)


def _pickled_para(name, chi, device):
    from tnalg_gb300 import Parameters as pm
    g = gc.load(name)
    para = pm.generate_parameters_dmrg("arbitrary")
    para.update(index1=g["index1"], coeff1=g["coeff1"], index2=g["index2"], coeff2=g["coeff2"], op=list(g["op"]))
    para = pm.make_consistent_parameter_dmrg(para)
    para.update(chi=chi, sweep_time=30, dt_ob=1, break_tol=1e-13, eigs_tol=1e-12, tau=1e-4, hx=0.0, hz=0.0,
                device=device)
    return g, para


@pytest.mark.parametrize("name,chi", [("pickle_chi16", 16), ("pickle_chi24", 24)])
def test_shipped_result_files_replayed(fake_backend, name, chi):
    """The coupling tables pickled in the reference's data_dmrg/ result files (EasyStart convention,
    coeff 1 on S+S- / S-S+) run through dmrg_finite_size reach the energies and bond energies those
    files record (a different random start; both runs converged at the same bond dimension)."""
    import contextlib
    import io
    from tnalg_gb300 import DMRG_anyH
    g, para = _pickled_para(name, chi, "cpu")
    np.random.seed(0)
    with contextlib.redirect_stdout(io.StringIO()):
        ob, A, info, _ = DMRG_anyH.dmrg_finite_size(para)
    assert abs(ob["e_per_site"] - float(g["e_per_site"])) <= 1e-10 * abs(float(g["e_per_site"]))
    np.testing.assert_allclose(np.ravel(ob["eb_full"]), np.ravel(g["eb_full"]), atol=1e-8)
    assert list(A.virtual_dim) == list(g["virtual_dim"])


def test_correlators_from_middle_honour_ob_len(fake_backend):
    """observe_correlators_from_middle(op1, op2, ob_len) (MPSClass.py:936-952) stops after ob_len + 1
    pairs, growing alternately to the left and right of round(L/2)."""
    from tnalg_gb300 import BasicFunctionsSJR as bf
    A = bf.load_pr(REF_FILE, "A", device="cpu")
    full = A.observe_correlators_from_middle(3, 3)
    assert full.shape == (6,)      # pairs (4,5), (3,5), (3,6), (2,6), (2,7), (1,7): then the right end is passed
    short = A.observe_correlators_from_middle(3, 3, ob_len=2)
    np.testing.assert_allclose(short, full[:3], atol=1e-14)
    assert A.observe_correlators_from_middle(1, 3, ob_len=0).shape == (1,)


def test_single_observations_norm_and_centre_moves(fake_backend):
    """observation_s1 / observation_s1_s2 (MPSClass.py:857-909) against the pickled magnetisations and
    the reference's two-site density matrix; norm_mps, central_orthogonalization and
    check_orthogonal_center (MPSClass.py:170-185, 954-1022) on the restored state; set_precision
    round trip."""
    from tnalg_gb300 import BasicFunctionsSJR as bf
    ob, A, info, para = bf.load_pr(REF_FILE, ("ob", "A", "info", "para"), device="cpu")
    g = np.load(os.path.join(gc.GOLDEN, "ref_rdm_chain_n8_h.npz"))
    ops = [np.real(np.asarray(o)) for o in para["op"]]
    for p in range(8):
        assert abs(A.observation_s1((3, p)) - float(np.ravel(ob["mz"])[p])) < 1e-12
    rho = g["rdm_1_5_c0"].reshape(2, 2, 2, 2)         # [x1, x2, y1, y2]
    for a, b in ((3, 3), (1, 3), (4, 5)):
        want = np.einsum("xy,uv,xuyv->", ops[a], ops[b], rho)
        assert abs(A.observation_s1_s2(([a, b], [1, 5])) - want) < 1e-12
        # the reference sorts the positions with their operators (MPSClass.py:878-880)
        assert abs(A.observation_s1_s2(([b, a], [5, 1])) - want) < 1e-12
    assert abs(A.norm_mps() - 1.0) < 1e-12
    A.central_orthogonalization(5)
    assert A.center == 5 and A.check_orthogonal_center(if_print=False) == 5
    assert np.ravel(A.orthogonality).tolist() == [-1] * 5 + [0] + [1] * 2
    assert abs(A.norm_mps() - 1.0) < 1e-12
    assert abs(A.observation_s1((3, 2)) - float(np.ravel(ob["mz"])[2])) < 1e-12
    A.set_precision("tf32x3")
    assert A.precision == "tf32x3"
    A.set_precision("fp64")
    assert A.precision == "fp64"
