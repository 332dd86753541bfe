"""Host-side logic on CPU: the drop-in parameter API, the coupling-list compiler and the
sweep orchestration (run through a numpy test double of the C ABI), and the built library's
exported symbols."""
import contextlib
import ctypes
import io
import os
import re

import numpy as np
import pytest

import golden_cases as gc


def _quiet(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


# -- parameters -------------------------------------------------------------------------


@pytest.mark.parametrize("name", ["chain_n12_chi16", "chain_n12_chi16_h", "longrange_n8_chi8", "jigsaw_s1_n9_chi12",
                                  "full_n8_chi8"])
def test_parameters_reproduce_reference_tables(name):
    from tnalg_gb300 import Parameters as pm
    m, g = gc.meta()[name], gc.load(name)
    lat = m["lattice"]
    para = pm.generate_parameters_dmrg(lat)
    para.update(l=m["l"], chi=m["chi"], hx=m["hx"], hz=m["hz"])
    if lat == "chain":
        para.update(jxy=1, jz=1)
    if lat == "longRange":
        para.update(jxy=1.0, jz=1.0)
    para = pm.make_consistent_parameter_dmrg(para)
    np.testing.assert_array_equal(np.asarray(para["index1"]), g["index1"])
    np.testing.assert_array_equal(np.asarray(para["index2"]), g["index2"])
    np.testing.assert_allclose(np.ravel(para["coeff1"]), g["coeff1"])
    np.testing.assert_allclose(np.ravel(para["coeff2"]), g["coeff2"])
    np.testing.assert_allclose(np.stack([np.real(o) for o in para["op"]]), g["op"])
    assert para["d"] == m["d"] and para["l"] == m["l"]


def test_parameters_accept_runtime_strings():
    from tnalg_gb300 import Parameters as pm
    lat = "".join(["ch", "ain"])  # not interned
    para = pm.generate_parameters_dmrg(lat)
    assert para["index2"].shape == (3 * (para["l"] - 1), 4)
    with pytest.raises(ValueError):
        pm.generate_parameters_dmrg("kagome")


def test_square_and_husimi_generators():
    from tnalg_gb300 import HamiltonianModule as hm, Parameters as pm
    p = pm.generate_parameters_dmrg("square")
    assert p["l"] == 16 and p["positions_h2"].shape == (24, 2)
    h = pm.generate_parameters_dmrg("husimi")
    pos = hm.positions_husimi(2)
    assert h["l"] == int(pos.max()) + 1 and pos.shape[0] % 3 == 0
    full = hm.positions_fully_connected(5)
    assert full.shape == (10, 2)


def test_periodic_chain_generator_reproduces_reference_tables():
    from tnalg_gb300 import Parameters as pm
    g, m = gc.load("chain_n10_chi16_pbc"), gc.meta()["chain_n10_chi16_pbc"]
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=10, chi=16, jxy=1, jz=1, hx=m["hx"], hz=m["hz"], bound_cond="periodic")
    para = pm.make_consistent_parameter_dmrg(para)
    np.testing.assert_array_equal(np.asarray(para["index2"]), g["index2"])
    np.testing.assert_allclose(np.ravel(para["coeff2"]), g["coeff2"])
    np.testing.assert_array_equal(np.asarray(para["positions_h2"]), g["positions_h2"])
    np.testing.assert_allclose(np.stack([np.real(o) for o in para["op"]]), g["op"])


def test_square_generator_reproduces_reference_tables():
    from tnalg_gb300 import Parameters as pm
    g, m = gc.load("square_4x2_chi8"), gc.meta()["square_4x2_chi8"]
    para = pm.generate_parameters_dmrg("square")
    para.update(square_width=4, square_height=2, chi=m["chi"], jxy=1, jz=1, hx=m["hx"], hz=m["hz"])
    para = pm.make_consistent_parameter_dmrg(para)
    assert para["l"] == m["l"] == 8
    np.testing.assert_array_equal(np.asarray(para["index1"]), g["index1"])
    np.testing.assert_array_equal(np.asarray(para["index2"]), g["index2"])
    np.testing.assert_allclose(np.ravel(para["coeff2"]), g["coeff2"])
    np.testing.assert_array_equal(np.asarray(para["positions_h2"]), g["positions_h2"])
    # the reference appends a second field operator on the repeated call (both zero here); the
    # list is rebuilt here, so op 6 is the field of the current hx, hz
    ops = np.stack([np.real(o) for o in para["op"]])
    assert len(ops) == 7 and len(g["op"]) == 8
    np.testing.assert_allclose(ops, g["op"][:7])
    para.update(hx=0.1, hz=0.2)
    para = pm.make_consistent_parameter_dmrg(para)
    np.testing.assert_allclose(np.real(para["op"][6]), -0.1 * np.real(para["op"][1]) - 0.2 * np.real(para["op"][3]))


@pytest.mark.parametrize("depth", [2, 3])
def test_husimi_generator_reproduces_reference_tables(depth):
    """library/Parameters.py's 'husimi' lattice (tables written by tests/golden/make_husimi_tables.py)."""
    from tnalg_gb300 import Parameters as pm
    g = np.load(os.path.join(gc.GOLDEN, "husimi_tables.npz"))
    para = pm.generate_parameters_dmrg("husimi")
    para["depth"] = depth
    para = pm.make_consistent_parameter_dmrg(para)
    assert para["l"] == int(g["d%d_l" % depth])
    for k in ("index1", "index2", "positions_h2"):
        np.testing.assert_array_equal(np.asarray(para[k]), g["d%d_%s" % (depth, k)])
    for k in ("coeff1", "coeff2"):
        np.testing.assert_allclose(np.ravel(para[k]), np.ravel(g["d%d_%s" % (depth, k)]))
    np.testing.assert_allclose(np.stack([np.real(o) for o in para["op"]]), g["d%d_op" % depth])


def test_j1j2_snake_generator():
    """J1-J2 snake lattice: 6 x 6 gives 60 J1 + 50 J2 bonds (330 rows), spans up to 11 sites; the 4 x 3
    tables equal the ones the reference run of the golden case consumed."""
    from tnalg_gb300 import HamiltonianModule as hm, Parameters as pm
    p1, p2 = hm.positions_j1j2_square_snake(6, 6)
    assert p1.shape == (60, 2) and p2.shape == (50, 2)
    assert int(max((p1[:, 1] - p1[:, 0]).max(), (p2[:, 1] - p2[:, 0]).max())) == 11
    # consecutive chain sites are lattice neighbours
    assert all([n, n + 1] in p1.tolist() for n in range(35))
    para = pm.generate_parameters_j1j2_snake(6, 6)
    assert para["l"] == 36 and para["index2"].shape == (330, 4)
    g = gc.load("j1j2_snake_4x3_chi16")
    para = pm.generate_parameters_j1j2_snake(4, 3, hz=0.1)
    np.testing.assert_array_equal(np.asarray(para["index2"]), g["index2"])
    np.testing.assert_allclose(np.ravel(para["coeff2"]), g["coeff2"])
    np.testing.assert_array_equal(np.asarray(para["index1"]), g["index1"])
    np.testing.assert_allclose(np.stack([np.real(o) for o in para["op"]]), g["op"])


# -- coupling-list compiler ---------------------------------------------------------------


def test_term_filter_and_orientation():
    from tnalg_gb300 import engine as E
    ops = [np.eye(2), np.zeros((2, 2)), np.zeros((2, 2)), np.diag([0.5, -0.5])]
    one, two = E.canonical_terms([[0, 3], [1, 1], [2, 3]], [1.0, 1.0, 1e-13], [[3, 1, 3, 0], [0, 2, 3, 3]],
                                 [0.5, 1e-20], ops, 1e-12)
    assert one == [(0, 3, 1.0)]                 # zero operator and tiny coefficient dropped
    assert two == [(1, 3, 0, 3, 0.5)]           # oriented i < j with operators swapped
    with pytest.raises(ValueError):
        E.canonical_terms([], [], [[1, 1, 3, 3]], [1.0], ops, 1e-12)


def test_open_operator_sets_chain_and_long_range():
    from tnalg_gb300 import engine as E
    ops = [np.eye(2)] * 6
    two = [(i, i + 1, a, b, 1.0) for i in range(4) for a, b in ((4, 5), (5, 4), (3, 3))]
    m = E.Model(5, 2, ops, [], two, "cpu")
    assert len(m.open_left[0]) == 0 and len(m.open_left[5]) == 0
    assert all(len(m.open_left[b]) == 3 for b in range(1, 5))
    assert m.straddle_groups(2) == ([], [], 0)
    two = [(0, 4, 3, 3, 0.5), (0, 3, 3, 3, 0.25), (1, 3, 4, 5, 1.0)]
    m = E.Model(5, 2, ops, [], two, "cpu")
    sl, sr, ng = m.straddle_groups(2)
    assert ng == 2  # two distinct left operators, three right ones -> grouped by the left side
    assert sorted(c for _, _, c in sr) == [0.25, 0.5, 1.0]


# -- orchestration through the test double ---------------------------------------------------


# (the J1-J2 reference run, 40 sweeps, is checked on the GPU; its lattice's host path is covered on the
# CPU by the 3 x 3 case of test_ed_parity.py)
@pytest.mark.parametrize("name", ["chain_n12_chi16_h", "ladder_2x4_chi8", "longrange_n8_chi8", "square_4x2_chi8",
                                  "full_n8_chi8", "chain_n10_chi8_ob3", "chain_n10_chi8_break",
                                  "chain_n10_chi16_pbc", "chain_s1_n8_chi9"])
def test_sweep_orchestration_matches_reference(name, fake_backend):
    from tnalg_gb300 import DMRG_anyH
    g, m = gc.load(name), gc.meta()[name]
    np.random.seed(m["seed"])
    ob, A, info, para = _quiet(DMRG_anyH.dmrg_finite_size, gc.para_of(name, device="cpu"))
    assert abs(ob["e_per_site"] - float(g["e_per_site"])) <= 1e-10 * abs(float(g["e_per_site"]))
    np.testing.assert_allclose(np.ravel(ob["eb_full"]), g["eb_full"], atol=1e-8)
    np.testing.assert_allclose(np.ravel(ob["mz"]), g["mz"], atol=1e-8)
    np.testing.assert_allclose(ob["corr_z"], g["corr_z_nocache"], atol=1e-8)
    np.testing.assert_allclose(np.ravel(A.ent), g["ent"], atol=1e-8)
    assert (A.virtual_dim == g["virtual_dim"]).all()
    assert info["solves"] == m.get("eig_solves", 2 * (m["l"] - 1) * m["sweep_time"])


def test_reference_script_through_compat_modules(fake_backend):
    """testDMRG.py's call pattern with the module-name shims first on sys.path."""
    import importlib
    import sys
    compat = __import__("os").path.join(gc.GOLDEN, "..", "..", "tnalg_gb300", "compat")
    sys.path.insert(0, compat)
    try:
        Pm = importlib.import_module("Parameters")
        dmrg = importlib.import_module("DMRG_anyH").dmrg_finite_size
        assert Pm.__file__.startswith(__import__("os").path.abspath(compat)) or "compat" in Pm.__file__
        para = Pm.generate_parameters_dmrg("chain")
        para.update(l=8, chi=4, sweep_time=2, device="cpu")
        para = Pm.make_consistent_parameter_dmrg(para)
        np.random.seed(0)
        ob, A, info, para = _quiet(dmrg, para)
        assert np.isfinite(ob["e_per_site"]) and A.mps[0].shape == (1, 2, 2)
    finally:
        sys.path.remove(compat)
        for m in ("Parameters", "DMRG_anyH", "MPSClass", "HamiltonianModule"):
            sys.modules.pop(m, None)


def test_pickle_roundtrip(fake_backend):
    import pickle
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    np.random.seed(3)
    A = MpsOpenBoundaryClass(6, 2, 4, device="cpu")
    A.correct_orthogonal_center(0)
    B = pickle.loads(pickle.dumps(A))
    assert B.center == 0 and (B.virtual_dim == A.virtual_dim).all()
    for a, b in zip(A.mps, B.mps):
        np.testing.assert_array_equal(a, b)


# -- the built library -------------------------------------------------------------------------


def test_library_exports_header_symbols():
    from tnalg_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    header = open(os.path.join(os.path.dirname(gc.GOLDEN), "..", "include", "tnalg_gb300.h")).read()
    declared = set(re.findall(r"^\s*(?:const char\*|int|size_t|unsigned long long)\s+(tn_\w+)\(", header, re.M))
    assert declared, "no declarations parsed"
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    assert declared <= set(_lib.exported_symbols()) | {"tn_version"}
    assert lib.tn_version() >= 100


def test_full_coefficients_match_exact_ground_state(fake_backend):
    """full_coefficients_mps (MPSClass.py:968-985, whose dropped reshape at :983 makes the reference
    fail beyond two sites) gives the DMRG state's amplitudes: unit norm, overlap 1 with the exact
    ground state of the same N=10 chain."""
    from oracle import ed
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=10, chi=32, jxy=1.0, jz=1.0, hx=0.2, hz=0.1, sweep_time=4, dt_ob=4, break_tol=-1.0,
                eigs_tol=1e-12, device="cpu")
    para = pm.make_consistent_parameter_dmrg(para)
    np.random.seed(3)
    ob, A, info, _ = _quiet(DMRG_anyH.dmrg_finite_size, para)
    psi = A.full_coefficients_mps()
    assert psi.shape == (2 ** 10, 1)
    assert abs(np.linalg.norm(psi) - 1.0) < 1e-12
    h = ed.hamiltonian(para["l"], para["d"], para["op"], para["index1"], para["coeff1"], para["index2"],
                       para["coeff2"])
    v = np.ravel(psi)
    e0 = ed.ground_state(para["l"], para["d"], para["op"], para["index1"], para["coeff1"], para["index2"],
                         para["coeff2"])[0]
    assert abs(v @ (h @ v) - e0) < 1e-9 * abs(e0)
    assert A.full_coefficients_mps(tol_memory=1) is None


def _bench():
    import importlib
    import sys
    sys.path.insert(0, os.path.join(gc.GOLDEN, "..", ".."))
    try:
        return importlib.import_module("bench")
    finally:
        sys.path.pop(0)


def test_bench_batch_leg_reports_failures_in_the_line():
    """bench.py's workload legs run in child processes; when a child fails (here: no GPU) the leg
    returns an error entry with the command instead of raising, so the benchmark line still prints."""
    bench = _bench()
    out = bench.run_batch_leg(bench.BATCH_ARGS, "fp64", timeout=120)
    assert "error" in out and out["command"].startswith("python -m tnalg_gb300.batched --jobs 512")
    assert bench.run_batch_leg(bench.BATCH_ARGS, "fp64", timeout=1)["skipped"]


def test_lattice_runner_reports_timed_sweeps(fake_backend, capsys):
    """python -m tnalg_gb300.run_lattice (the benchmark's lattice leg) on a small J1-J2 lattice through
    the test double: one JSON line with the timed sweeps and the FP64 comparison."""
    import json
    from tnalg_gb300 import run_lattice
    run_lattice.main(["j1j2", "--width", "3", "--height", "2", "--chi", "8", "--ramp", "4", "--device", "cpu",
                      "--compare-fp64"])
    out = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert out["sites"] == 6 and out["chi_schedule"] == [4, 8] and out["chi_max"] == 8
    assert out["sweeps_per_s"] > 0 and out["solves_per_s"] > 0 and out["straddling_terms_max"] > 0
    assert out["fp64_path"]["precision"] == "fp64" and out["abs_de_per_site_vs_fp64"] < 1e-8
    assert out["e_per_site"] < 0


def test_bench_summary_gathers_the_metric_figures():
    """The last key of the benchmark line: mixed-vs-FP64 speed-up and energy difference of the
    one-job legs, the batched leg against sequential FP64 solves, and the serving rates."""
    bench = _bench()
    leg = {"speedup_vs_fp64": 12.0, "abs_de_per_site_vs_fp64": 3e-10, "max_abs_d_term_energy_vs_fp64": 2e-5,
           "sweeps_per_s": 3.0, "matvecs_per_solve": 3.5,
           "fp64_path": {"sweeps_per_s": 0.25, "matvecs_per_solve": 7.0}}
    line = {"chain_n100_chi512": leg, "j1j2_6x6_chi512": {"error": "exit 1: x"},
            "batched_512_xxz": {"solves_per_s": 9000.0, "speedup_vs_sequential": 30.0, "latency_p99_s": 20.0,
                                "sequential": {"solves_per_s": 300.0}},
            "serving_stream": [{"rate_per_s": 10.0, "solves_per_s": 500.0, "latency_p99_s": 3.0, "noise": 1}]}
    out = bench.summarise(line)
    assert out["chain_n100_chi512_8sweeps"]["speedup_vs_fp64"] == 12.0
    assert out["chain_n100_chi512_8sweeps"]["fp64_matvecs_per_solve"] == 7.0
    assert out["j1j2_6x6_chi512_10sweeps"] == {"error": "exit 1: x"}
    assert out["batched_512_xxz_chains"]["sequential_fp64_solves_per_s"] == 300.0
    assert out["serving_poisson_stream"] == [{"rate_per_s": 10.0, "solves_per_s": 500.0, "latency_p99_s": 3.0}]


def test_chi_schedule_grows_bonds_and_reaches_the_direct_energy(fake_backend):
    """para['chi_schedule'] (bond growth with seeded noise between sweeps, not in the reference):
    bonds follow the schedule capped by d^min(b, L-b), and the ramped run ends at the energy of a run
    started at the final bond dimension (N=12 chain with fields, chi 4 -> 8 -> 16)."""
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=12, chi=4, jxy=1.0, jz=0.8, hx=0.2, hz=0.1, sweep_time=8, dt_ob=1, break_tol=-1.0,
                eigs_tol=1e-12, device="cpu")
    para = pm.make_consistent_parameter_dmrg(para)
    np.random.seed(2)
    ob, A, info, _ = _quiet(DMRG_anyH.dmrg_finite_size, dict(para, chi_schedule=[4, 8, 16]))
    assert list(A.virtual_dim) == [1, 2, 4, 8, 16, 16, 16, 16, 16, 8, 4, 2, 1]
    np.random.seed(2)
    ob16, _, _, _ = _quiet(DMRG_anyH.dmrg_finite_size, dict(para, chi=16))
    assert abs(ob["e_per_site"] - ob16["e_per_site"]) < 1e-9


# -- device selection ---------------------------------------------------------------------


def test_methods_run_with_the_mps_device_current(monkeypatch):
    """Every C-ABI call works on the current device and its current stream: an MPS on cuda:1 used
    while cuda:0 is current must make cuda:1 current for the call (and only then)."""
    import torch

    from tnalg_gb300 import MPSClass
    from tnalg_gb300 import _lib as L

    entered = []

    class Recorder:
        def __init__(self, dev):
            self.dev = dev

        def __enter__(self):
            entered.append(torch.device(self.dev))

        def __exit__(self, *exc):
            return False

    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    monkeypatch.setattr(torch.cuda, "device", Recorder)
    monkeypatch.setattr(L, "_host_test", False)

    class Stub:
        def __init__(self, dev):
            self._dev = type("D", (), {"device": torch.device(dev)})()

        @MPSClass.on_device
        def work(self):
            return "ran"

    assert Stub("cuda:1").work() == "ran"
    assert entered == [torch.device("cuda:1")]
    assert Stub("cuda:0").work() == "ran"   # already current: no switch
    assert Stub("cpu").work() == "ran"
    assert entered == [torch.device("cuda:1")]


def test_bond_growth_by_expansion_keeps_the_state_and_uses_the_hamiltonian(fake_backend):
    """DeviceMPS.expand_bonds (subspace expansion + truncated SVD): the grown MPS represents the same
    state (energy and local magnetisations unchanged), every bond reaches min(chi, d^b, d^(L-b)), the
    sites right of the centre are right-canonical again, and the enlarged bond spaces pay: one sweep
    after growth ends well below one sweep at the old bond dimension."""
    import torch
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=10, chi=4, jxy=1.0, jz=0.8, hx=0.2, hz=0.1, sweep_time=2, dt_ob=1, break_tol=-1.0,
                eigs_tol=1e-12, device="cpu")
    para = pm.make_consistent_parameter_dmrg(para)
    np.random.seed(4)
    ob, A, _, _ = _quiet(DMRG_anyH.dmrg_finite_size, para)
    model = (para["index1"], para["index2"], para["coeff1"], para["coeff2"], para["eigs_tol"])
    A.correct_orthogonal_center(0)
    e0 = A.observe_bond_energy(para["index2"], para["coeff2"]).sum()
    mz0 = np.ravel(A.observe_magnetization(3))
    import copy
    B = copy.deepcopy(A)
    A.grow_bond_dimension(16, seed=1, method="expand", model=model)
    assert list(A.virtual_dim) == [1, 2, 4, 8, 16, 16, 16, 8, 4, 2, 1]
    assert A.center == 0
    e1 = A.observe_bond_energy(para["index2"], para["coeff2"]).sum()
    assert abs(e1 - e0) < 1e-12 and np.max(np.abs(np.ravel(A.observe_magnetization(3)) - mz0)) < 1e-12
    for n in range(1, 10):   # right of the centre: right-canonical
        t = A.mps_device[n].reshape(A.mps_device[n].shape[0], -1)
        assert torch.allclose(t @ t.T, torch.eye(t.shape[0], dtype=torch.float64), atol=1e-12)
    def sweep(M):
        for n in list(range(1, 10)) + list(range(8, -1, -1)):
            M.update_tensor_eigs(n, para["index1"], para["index2"], para["coeff1"], para["coeff2"], para["tau"], True,
                                 tol=para["eigs_tol"])
        return (M.observe_bond_energy(para["index2"], para["coeff2"]).sum() -
                para["hx"] * M.observe_magnetization(1).sum() - para["hz"] * M.observe_magnetization(3).sum())
    assert sweep(A) < sweep(B) - 1e-5


def test_reference_arm_times_measured_local_updates():
    """bench.py --impl reference: W untimed and K timed local updates of the oracle (the reference's
    algorithm) on the host; ms_per_step is one measured step and value the sweeps/s it gives."""
    import argparse
    import bench
    s = bench.cpu_sample(10, 8, 1e-10, 3, warmup=1)
    assert s["kind"] == "port" and s["steps"] == 3 and s["warmup"] == 1 and s["matvecs_per_solve"] > 0
    assert s["value"] == pytest.approx(1.0 / (2 * 9 * s["ms_per_step"] / 1000.0), rel=1e-12)
    assert s["ms_per_step"] == pytest.approx(1000.0 * (s["solve_s"] + s["move_s"]), rel=1e-12)
    args = argparse.Namespace(length=10, chi=8, eigs_tol=1e-10, steps=2, warmup=1, gpus=1)
    line = bench.run_reference(args, 0)
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] == line["cpu_baseline"]["value"] == line["e2e"]["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["higher_is_better"]
    assert bench.run_reference(args, 1) is None      # other ranks do no work
