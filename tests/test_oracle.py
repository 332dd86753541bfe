"""The CPU oracle against the reference's own outputs (golden fixtures)."""
import json
import os

import numpy as np
import pytest

import golden_cases as gc
from oracle import dmrg_oracle as O
from oracle import ed


def _run(name):
    g, m = gc.load(name), gc.meta()[name]
    return O.dmrg_finite_size(m["l"], m["d"], m["chi"], list(g["op"]), g["index1"], g["coeff1"], g["index2"],
                              g["coeff2"], g["positions_h2"], tau=m["tau"], eigs_tol=m["eigs_tol"],
                              sweep_time=m["sweep_time"], hx=m["hx"], hz=m["hz"], seed=m["seed"],
                              ob_position=m.get("ob_position", 0), dt_ob=m.get("dt_ob", 1),
                              break_tol=m.get("break_tol", -1.0))


@pytest.mark.parametrize("name", ["chain_n12_chi16", "chain_n12_chi16_h", "ladder_2x4_chi8", "longrange_n8_chi8",
                                  "j1j2_snake_4x3_chi16", "square_4x2_chi8", "full_n8_chi8", "chain_n10_chi8_ob3",
                                  "chain_n10_chi8_break", "chain_n10_chi16_pbc", "chain_s1_n8_chi9"])
def test_oracle_matches_reference_runs(name):
    g = gc.load(name)
    ob, A, info = _run(name)
    assert abs(ob["e_per_site"] - float(g["e_per_site"])) <= 1e-10 * abs(float(g["e_per_site"]))
    for k in ("eb_full", "mx", "mz"):
        np.testing.assert_allclose(np.ravel(ob[k]), g[k], atol=1e-8, rtol=0)
    np.testing.assert_allclose(ob["corr_x"], g["corr_x_nocache"], atol=1e-8)
    np.testing.assert_allclose(ob["corr_z"], g["corr_z_nocache"], atol=1e-8)
    np.testing.assert_allclose(A.ent, g["ent"], atol=1e-8)
    assert gc.max_spectrum_diff(A.lm, gc.spectra(name)) < 1e-8
    assert (A.virtual_dim == g["virtual_dim"]).all()


def test_reference_default_corr_z_uses_stale_cache():
    """The reference's default run (is_save_op=True) returns a corr_z that differs from the
    cache-free run; the oracle (and the GPU path) reproduce the cache-free values."""
    g = gc.load("chain_n12_chi16")
    assert np.max(np.abs(g["corr_z"] - g["corr_z_nocache"])) > 1e-2
    # at h=0 the state is SU(2) symmetric: corr_z == corr_x for the correct correlator
    np.testing.assert_allclose(g["corr_z_nocache"], g["corr_x_nocache"], atol=1e-9)


def test_oracle_observables_on_pickled_fixture():
    """Observables of the MPS shipped in data_dmrg/*chi16open.pr equal the values pickled with it."""
    g = gc.load("pickle_chi16")
    mps = gc.mps_of("pickle_chi16")
    A = O.OracleMPS(len(mps), 2, 16, list(g["op"]), mps=mps)
    A.center = int(g["center"]) if int(g["center"]) >= 0 else 0
    if int(g["center"]) < 0:
        A.correct_orthogonal_center(0)
    eb = A.observe_bond_energy(g["index2"], g["coeff2"])
    np.testing.assert_allclose(eb, g["eb_full"], atol=1e-9)
    np.testing.assert_allclose(A.observe_magnetization(3), g["mz"], atol=1e-9)
    assert abs(np.sum(eb) / 12 - float(g["e_per_site"])) < 1e-12


def test_exact_diagonalisation_matches_reference_ed():
    m = gc.meta()["ed_chain_n12"]
    g = gc.load("chain_n12_chi16")
    e0, _ = ed.ground_state(12, 2, list(g["op"]), g["index1"], g["coeff1"], g["index2"], g["coeff2"])
    assert abs(e0 - m["e_eig"]) < 1e-9
    # DMRG at chi=16 is within the truncation error of ED
    assert 0 < float(g["e_per_site"]) * 12 - e0 < 1e-6


def test_fixture_energy_matches_ed_in_fixture_convention():
    """The shipped chi=24 pickle uses coeff 1 on S+S-/S-S+ (EasyStart convention)."""
    g = gc.load("pickle_chi24")
    e0, _ = ed.ground_state(12, 2, list(g["op"]), g["index1"], np.zeros(12), g["index2"], g["coeff2"])
    assert abs(float(g["e_per_site"]) * 12 - e0) < 1e-6


def test_docstring_kats():
    with open(os.path.join(gc.GOLDEN, "kat_primitives.json")) as f:
        k = json.load(f)
    T, v = np.array(k["T"]), np.array(k["v"])
    np.testing.assert_allclose(O.transfer_left(T), k["bound_l2r"])
    np.testing.assert_allclose(O.transfer_left(T, v=v), k["bound_l2r_v"])
    np.testing.assert_allclose(O.transfer_right(T), k["bound_r2l"])
    np.testing.assert_allclose(O.transfer_right(T, v=v), k["bound_r2l_v"])
    op = np.array(k["op_t"])
    np.testing.assert_allclose(O.transfer_left(T[:, :2, :], op, v), k["bound_l2r_op_v"])
    np.testing.assert_allclose(O.transfer_right(T[:, :2, :], op, v), k["bound_r2l_op_v"])
    T2, M = np.array(k["T2"]), np.array(k["M"])
    np.testing.assert_allclose(O.absorb_matrix2tensor(T2, M, 2), k["absorb_bond2"])
    np.testing.assert_allclose(O.absorb_matrix2tensor(T2, M, 0), k["absorb_bond0"])
    np.testing.assert_allclose(O.absorb_matrix2tensor(T2, M, 1), k["absorb_bond1"])
    assert abs(O.entanglement_entropy(np.array(k["entropy_lm"], float)) - k["entropy"]) < 1e-12


def test_dense_heff_matches_reference():
    """The oracle's bucket matvec reproduces the reference's dense effective Hamiltonian."""
    for name, src, p in (("heff_chain_n12_chi16_h_p5", "chain_n12_chi16_h", 5), ("heff_ladder_2x4_chi8_p3", "ladder_2x4_chi8", 3)):
        h = gc.load(name)
        g, m = gc.load(src), gc.meta()[src]
        n = len([f for f in h.files if f.startswith("mps_")])
        A = O.OracleMPS(n, m["d"], m["chi"], list(g["op"]), mps=[h["mps_%d" % k] for k in range(n)])
        A.center = p
        A.orthogonality[:p] = -1
        A.orthogonality[p + 1:] = 1
        one, two = O.canonical_terms(g["index1"], g["coeff1"], g["index2"], g["coeff2"], A.ops, 1e-12)
        np.testing.assert_allclose(A.dense_heff(p, one, two), h["h"], atol=1e-11)
