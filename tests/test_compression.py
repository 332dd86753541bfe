"""Rank-compressed two-body couplings (engine.CompressedModel) on CPU.

The compressed model must describe exactly the Hamiltonian of the coupling lists: every
coupling crossing a bond is reproduced by the bond bases, the straddling core reproduces the
couplings across a site, and a DMRG through the numpy test double of the C ABI gives the
reference's results (golden runs) and exact diagonalisation's energy (fully connected chain).
"""
import contextlib
import io

import numpy as np
import pytest

import golden_cases as gc


def _quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def _terms(lattice, **kw):
    from tnalg_gb300 import Parameters as pm, engine as E
    para = pm.generate_parameters_dmrg(lattice)
    para.update(**kw)
    para = pm.make_consistent_parameter_dmrg(para)
    one, two = E.canonical_terms(para["index1"], para["coeff1"], para["index2"], para["coeff2"], para["op"], 1e-12)
    return para, one, two


@pytest.mark.parametrize("lattice,kw", [("full", dict(l=14, jxy=1.0, jz=0.7)), ("longRange", dict(l=16, alpha=1.5)),
                                        ("jigsaw", dict(l=11)), ("chain", dict(l=10))])
def test_bases_reproduce_every_coupling(lattice, kw):
    from tnalg_gb300 import engine as E
    para, one, two = _terms(lattice, **kw)
    m = E.CompressedModel(para["l"], para["d"], para["op"], one, two, "cpu")
    M, ls, rs = m.M, m.lsite, m.rsite
    for b in range(para["l"] + 1):
        U, V = m.U[b], m.V[b]
        np.testing.assert_allclose(U.T @ U, np.eye(U.shape[1]), atol=1e-12)
        np.testing.assert_allclose(V.T @ V, np.eye(V.shape[1]), atol=1e-12)
        cross = M * np.outer(ls < b, rs >= b)          # couplings across bond b
        np.testing.assert_allclose(U @ (U.T @ cross), cross, atol=1e-13)
        np.testing.assert_allclose((cross @ V) @ V.T, cross, atol=1e-13)
    for p in range(para["l"]):
        cl, cr = m.straddle_core(p)
        strad = M * np.outer(ls < p, rs > p)            # pairs i < p < j
        np.testing.assert_allclose(m.U[p] @ cl.T @ cr @ m.V[p + 1].T, strad, atol=1e-13)


def test_block_terms_reproduce_site_couplings():
    """W_L / W_R coefficients expand back to the couplings ending / starting at the site."""
    from tnalg_gb300 import engine as E
    para, one, two = _terms("longRange", l=12, alpha=1.0, jxy=1.0)
    m = E.CompressedModel(para["l"], para["d"], para["op"], one, two, "cpu")
    for p in range(para["l"]):
        want = {}
        for i, j, a, b, c in two:
            if j == p:
                want[(i, a, b)] = want.get((i, a, b), 0.0) + c
        got = {}
        for slot, op, c in m.left_block_terms(p)[1:]:
            if slot <= 0:
                continue
            for k, (i, a) in enumerate(m.lports):
                if abs(m.U[p][k, slot - 1]) > 0:
                    got[(i, a, op)] = got.get((i, a, op), 0.0) + c * m.U[p][k, slot - 1]
        for key in set(want) | set(got):
            assert abs(want.get(key, 0.0) - got.get(key, 0.0)) < 1e-13, (p, key)
        want = {}
        for i, j, a, b, c in two:
            if i == p:
                want[(j, b, a)] = want.get((j, b, a), 0.0) + c
        got = {}
        for slot, op, c in m.right_block_terms(p, with_site=False)[1:]:
            for k, (j, b) in enumerate(m.rports):
                if abs(m.V[p + 1][k, slot - 1]) > 0:
                    got[(j, b, op)] = got.get((j, b, op), 0.0) + c * m.V[p + 1][k, slot - 1]
        for key in set(want) | set(got):
            assert abs(want.get(key, 0.0) - got.get(key, 0.0)) < 1e-13, (p, key)


def test_uniform_all_to_all_carries_constant_slots():
    from tnalg_gb300 import engine as E
    para, one, two = _terms("full", l=40, jxy=1.0, jz=1.0)
    m = E.make_model(para["l"], para["d"], para["op"], one, two, "cpu")
    assert m.compressed
    # rank 1 coupling per operator pair: 3 combined slots + 3 fresh ports at most, any N
    assert max(m.n_left(b) for b in range(para["l"] + 1)) <= 6
    assert max(m.straddle_core(p)[0].shape[0] for p in range(para["l"])) <= 3
    slots, groups = E.carried_cost(two, para["l"])
    assert slots > 20 * sum(m.n_left(b) + m.n_right(b) for b in range(para["l"] + 1)) / 6


def test_auto_keeps_nearest_neighbour_models_plain():
    from tnalg_gb300 import engine as E
    for lattice, kw in (("chain", dict(l=20)), ("jigsaw", dict(l=11))):
        para, one, two = _terms(lattice, **kw)
        assert not E.make_model(para["l"], para["d"], para["op"], one, two, "cpu").compressed
    with pytest.raises(ValueError):
        E.make_model(para["l"], para["d"], para["op"], one, two, "cpu", compress="sometimes")


@pytest.mark.parametrize("name", ["longrange_n8_chi8", "ladder_2x4_chi8", "jigsaw_s1_n9_chi12", "full_n8_chi8"])
def test_compressed_sweeps_match_reference(name, fake_backend):
    from tnalg_gb300 import DMRG_anyH
    g, m = gc.load(name), gc.meta()[name]
    np.random.seed(m["seed"])
    para = gc.para_of(name, device="cpu")
    para["mpo_compress"] = True
    ob, A, info, para = _quiet(DMRG_anyH.dmrg_finite_size, para)
    atol = 5e-8 if name.startswith("jigsaw") else 1e-8
    assert abs(ob["e_per_site"] - float(g["e_per_site"])) <= 1e-10 * abs(float(g["e_per_site"]))
    np.testing.assert_allclose(np.ravel(ob["eb_full"]), g["eb_full"], atol=atol)
    np.testing.assert_allclose(np.ravel(ob["mz"]), g["mz"], atol=atol)
    np.testing.assert_allclose(np.ravel(A.ent), g["ent"], atol=atol)


def test_compressed_full_chain_matches_exact_diagonalisation(fake_backend):
    from oracle import ed
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    para = pm.generate_parameters_dmrg("full")
    para.update(l=10, chi=32, jxy=1.0, jz=0.6, hx=0.3, hz=0.2, sweep_time=6, dt_ob=6, break_tol=-1.0,
                eigs_tol=1e-12, device="cpu")
    para = pm.make_consistent_parameter_dmrg(para)
    e0 = ed.ground_state(para["l"], para["d"], para["op"], para["index1"], para["coeff1"], para["index2"],
                         para["coeff2"])[0]
    res = {}
    for mode in (False, True):
        np.random.seed(1)
        p = dict(para)
        p["mpo_compress"] = mode
        ob, A, info, _ = _quiet(DMRG_anyH.dmrg_finite_size, p)
        res[mode] = ob
    assert abs(res[True]["e_per_site"] * para["l"] - e0) <= 1e-9 * abs(e0)
    assert abs(res[True]["e_per_site"] - res[False]["e_per_site"]) <= 1e-12
    np.testing.assert_allclose(np.ravel(res[True]["mz"]), np.ravel(res[False]["mz"]), atol=1e-8)


def test_lossy_tolerance_trades_slots_for_accuracy(fake_backend):
    """mpo_tol above machine precision drops small singular values of the power-law couplings:
    fewer carried operators, energy still within the dropped weight."""
    from tnalg_gb300 import DMRG_anyH, Parameters as pm, engine as E
    para = pm.generate_parameters_dmrg("longRange")
    para.update(l=12, chi=16, alpha=1.0, jxy=1.0, jz=1.0, hx=0.2, sweep_time=4, dt_ob=4, break_tol=-1.0,
                eigs_tol=1e-12, device="cpu")
    para = pm.make_consistent_parameter_dmrg(para)
    one, two = E.canonical_terms(para["index1"], para["coeff1"], para["index2"], para["coeff2"], para["op"], 1e-12)
    exact = E.CompressedModel(para["l"], para["d"], para["op"], one, two, "cpu")
    lossy = E.CompressedModel(para["l"], para["d"], para["op"], one, two, "cpu", tol=1e-4)
    n = lambda m: sum(m.n_left(b) + m.n_right(b) for b in range(para["l"] + 1))
    assert n(lossy) < n(exact)
    out = {}
    for tol in (1e-14, 1e-4):
        np.random.seed(2)
        p = dict(para)
        p.update(mpo_compress=True, mpo_tol=tol)
        out[tol] = _quiet(DMRG_anyH.dmrg_finite_size, p)[0]["e_per_site"]
    assert 0 < abs(out[1e-4] - out[1e-14]) < 1e-3
