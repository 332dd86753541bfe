"""GPU tests of the wider paths: the J1-J2 snake lattice against its reference run, rank-compressed
couplings (mpo_compress) against the plain model and exact diagonalisation, and result files
written by the reference's save_pr. Collected after the core GPU tests."""
import contextlib
import io
import os

import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu


def _quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


@pytest.mark.parametrize("name", gc.LATER_CASES)
@pytest.mark.parametrize("compress", [False, True])
def test_fp64_path_matches_later_reference_runs(cuda_lib, name, compress):
    """Same seeded MPS and sweep schedule as the reference run: energy to 1e-10 relative, observables
    to 1e-8, with the plain and the rank-compressed coupling model."""
    from tnalg_gb300 import DMRG_anyH
    g, m = gc.load(name), gc.meta()[name]
    np.random.seed(m["seed"])
    para = gc.para_of(name)
    para["mpo_compress"] = compress
    ob, A, info, para = _quiet(DMRG_anyH.dmrg_finite_size, para)
    e_ref = float(g["e_per_site"])
    assert abs(ob["e_per_site"] - e_ref) <= 1e-10 * abs(e_ref)
    for key, ref in (("eb_full", g["eb_full"]), ("mx", g["mx"]), ("mz", g["mz"]), ("eb", g["eb"])):
        np.testing.assert_allclose(np.ravel(ob[key]), ref, atol=1e-8)
    np.testing.assert_allclose(ob["corr_x"], g["corr_x_nocache"], atol=1e-8)
    np.testing.assert_allclose(ob["corr_z"], g["corr_z_nocache"], atol=1e-8)
    np.testing.assert_allclose(np.ravel(A.ent), g["ent"], atol=1e-8)
    assert (A.virtual_dim == g["virtual_dim"]).all()

def test_compressed_couplings_on_device(cuda_lib):
    """Fully connected chain (N=10, chi=32): rank-compressed couplings give the plain model's and
    exact diagonalisation's energy, in FP64 and on the split-TF32 path."""
    from oracle import ed
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    para = pm.generate_parameters_dmrg("full")
    para.update(l=10, chi=32, jxy=1.0, jz=0.6, hx=0.3, hz=0.2, sweep_time=6, dt_ob=6, break_tol=-1.0,
                eigs_tol=1e-12)
    para = pm.make_consistent_parameter_dmrg(para)
    e0 = ed.ground_state(para["l"], para["d"], para["op"], para["index1"], para["coeff1"], para["index2"],
                         para["coeff2"])[0]
    res = {}
    for mode, prec in ((False, "fp64"), (True, "fp64"), (True, "tf32x3")):
        np.random.seed(1)
        p = dict(para)
        p.update(mpo_compress=mode, precision=prec, device="cuda")
        res[(mode, prec)] = _quiet(DMRG_anyH.dmrg_finite_size, p)[0]
    e = res[(True, "fp64")]["e_per_site"]
    assert abs(e * para["l"] - e0) <= 1e-9 * abs(e0)
    assert abs(e - res[(False, "fp64")]["e_per_site"]) <= 1e-12
    np.testing.assert_allclose(np.ravel(res[(True, "fp64")]["mz"]), np.ravel(res[(False, "fp64")]["mz"]),
                               atol=1e-8)
    assert abs(res[(True, "tf32x3")]["e_per_site"] - e) <= 1e-8


def test_reference_result_file_on_device(cuda_lib):
    """A result file written by the reference's save_pr loads onto the GPU; the observables of the
    restored MPS equal the ones pickled beside it."""
    pytest.importorskip("numpy._core")   # the file's arrays were pickled by numpy 2
    from tnalg_gb300 import BasicFunctionsSJR as bf
    ob, A, info, para = bf.load_pr(os.path.join(gc.GOLDEN, "ref_result_chain_n8_h.pr"), ("ob", "A", "info", "para"))
    assert A.mps_device[0].is_cuda and A.center == 0
    eb = A.observe_bond_energy(para["index2"], para["coeff2"])
    np.testing.assert_allclose(np.ravel(eb), np.ravel(ob["eb_full"]), atol=1e-12)
    np.testing.assert_allclose(np.ravel(A.observe_magnetization(3)), np.ravel(ob["mz"]), atol=1e-12)


def test_two_site_density_matrices_on_device(cuda_lib):
    """reduced_density_matrix_two_body on the GPU equals the reference's own values on the same state."""
    pytest.importorskip("numpy._core")   # the result file's arrays were pickled by numpy 2
    from tnalg_gb300 import BasicFunctionsSJR as bf
    g = np.load(os.path.join(gc.GOLDEN, "ref_rdm_chain_n8_h.npz"))
    A = bf.load_pr(os.path.join(gc.GOLDEN, "ref_result_chain_n8_h.pr"), "A")
    for key in [k for k in g.files if k.startswith("rdm_")]:
        _, p1, p2, c = key.split("_")
        A.correct_orthogonal_center(int(c[1:]))
        np.testing.assert_allclose(A.reduced_density_matrix_two_body(int(p1), int(p2)), g[key], atol=1e-12)


def test_one_site_density_matrices_on_device(cuda_lib):
    """One-site density matrices and on-site entropies on the GPU equal the package layout's values."""
    pytest.importorskip("numpy._core")
    from tnalg_gb300 import BasicFunctionsSJR as bf
    g = np.load(os.path.join(gc.GOLDEN, "ref_rdm_chain_n8_h.npz"))
    A = bf.load_pr(os.path.join(gc.GOLDEN, "ref_result_chain_n8_h.pr"), "A")
    for c in (0, 4, 7):
        A.correct_orthogonal_center(c)
        ent, rho = A.calculate_onsite_entanglement_entropy()
        np.testing.assert_allclose(ent, g["onsite_ent_c%d" % c], atol=1e-12)
        np.testing.assert_allclose(np.stack(rho), g["onsite_rho_c%d" % c], atol=1e-12)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("tf32x3", 1e-8)])
def test_worker_threads_on_device(cuda_lib, precision, tol):
    """Scheduler(workers=4): jobs advanced from four host threads, each on its own stream, give the
    results they give alone (exercises the library's shared host state under concurrent calls)."""
    from tnalg_gb300 import _lib as L, serving
    if precision == "tf32x3" and not L.tf32x3_available():
        pytest.skip("tf32x3 needs an sm_103 device")

    def jobs():
        out = []
        for k, (l, chi, jz, hz) in enumerate([(16, 16, 1.0, 0.0), (24, 32, 0.5, 0.2), (20, 16, 1.5, 0.1),
                                              (12, 8, 1.0, 0.3), (32, 32, 0.8, 0.0), (18, 64, 1.2, 0.4)]):
            para = serving.chain_job_para(l, chi, jz=jz, hz=hz, sweeps=3, precision=precision, device="cuda")
            out.append(serving.DMRGJob(k, para, seed=300 + k))
        return out

    alone = {}
    for j in jobs():
        s = serving.Scheduler("cuda", max_active=1)
        s.submit(j)
        s.run()
        alone[j.job_id] = j.result
    mix = serving.Scheduler("cuda", workers=4)
    for j in jobs():
        mix.submit(j)
    done = mix.run()
    assert len(done) == 6 and mix.max_concurrent == 6
    for j in done:
        ref = alone[j.job_id]
        assert abs(j.result["e_per_site"] - ref["e_per_site"]) <= tol
        np.testing.assert_allclose(j.result["mz"], ref["mz"], atol=10 * tol)


@pytest.mark.parametrize("name,chi", [("pickle_chi16", 16), ("pickle_chi24", 24)])
def test_shipped_result_files_replayed_on_device(cuda_lib, name, chi):
    """The reference's shipped data_dmrg/ result files: their pickled coupling tables run on the GPU
    reach the energies and bond energies the files record."""
    from test_persistence import _pickled_para
    from tnalg_gb300 import DMRG_anyH
    g, para = _pickled_para(name, chi, "cuda")
    np.random.seed(0)
    ob, A, info, _ = _quiet(DMRG_anyH.dmrg_finite_size, para)
    assert abs(ob["e_per_site"] - float(g["e_per_site"])) <= 1e-10 * abs(float(g["e_per_site"]))
    np.testing.assert_allclose(np.ravel(ob["eb_full"]), np.ravel(g["eb_full"]), atol=1e-8)


GPU_ED_CASES = [("chain", 16), ("ladder", 16), ("jigsaw", 9), ("full", 12), ("longRange", 12), ("square", 12),
                ("j1j2", 12), ("j1j2", 16)]


@pytest.mark.parametrize("kind,size", GPU_ED_CASES)
def test_full_bond_dimension_reaches_the_exact_ground_state_on_device(cuda_lib, kind, size):
    """Every lattice generator at N <= 16 (full bond dimension, FP64 path): the DMRG energy equals
    exact diagonalisation's to 1e-9 relative."""
    from test_ed_parity import run_against_ed
    e, e0 = run_against_ed(kind, size, "cuda")
    assert abs(e - e0) <= 1e-9 * abs(e0), (kind, size, e, e0)
