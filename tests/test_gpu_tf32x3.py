"""Split-TF32 tensor-core path (tcgen05) against FP64 and plain FP32 references (GPU only)."""
import contextlib
import ctypes
import io

import numpy as np
import pytest
import torch

import golden_cases as gc

pytestmark = pytest.mark.gpu

from tnalg_gb300 import _lib as L  # noqa: E402


@pytest.fixture(scope="module")
def tf32(cuda_lib):
    if not L.tf32x3_available():
        pytest.skip("tf32x3 needs an sm_103 device")
    return cuda_lib


def _rand(*shape, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(*shape, generator=g, dtype=torch.float64).cuda()


def _fp32_error(A, B, ref):
    """Error of a plain FP32 (no TF32) product of the same operands: the accuracy bar."""
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        c32 = torch.matmul(A.float(), B.float()).double()
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old
    return torch.max(torch.abs(c32 - ref)).item()


@pytest.mark.parametrize("M,N,K", [(128, 64, 32), (1024, 512, 1024), (100, 37, 70), (512, 1024, 1024),
                                   (8, 8, 4), (256, 300, 520), (1536, 512, 1536)])
def test_tf32x3_gemm_matches_fp64(tf32, M, N, K):
    A = _rand(M, K, seed=M)
    B = _rand(K, N, seed=N + 1)
    Cin = _rand(M, N, seed=3)
    C = torch.empty_like(Cin)
    ws = L.Workspace(torch.device("cuda"))
    L.gemm(A, B, C, M, N, K, (K, 1), (N, 1), (N, 1), Cin=Cin, alpha=1.25, beta=-0.5, precision=L.PREC_TF32X3,
           ws=ws)
    L.check(L.load().tn_check_device_status(L.stream_handle()))
    ref = 1.25 * (A @ B) - 0.5 * Cin
    err = torch.max(torch.abs(C - ref)).item()
    bar = 1.25 * _fp32_error(A, B, A @ B)
    # split-TF32 with FP32 tensor-core accumulation: within 4x of a plain FP32 GEMM's error
    assert err <= 4.0 * bar + 1e-12, (err, bar)
    assert err / torch.max(torch.abs(ref)).item() < 5e-6


def test_tf32x3_batched_reduced_and_transposed(tf32):
    Z, R, M, N, K = 3, 2, 96, 80, 40
    A = _rand(Z, R, K, M, seed=1)  # A(m,k) stored transposed
    B = _rand(Z, R, N, K, seed=2)  # B(k,n) stored transposed
    C = torch.zeros(Z, M, N, dtype=torch.float64, device="cuda")
    ws = L.Workspace(torch.device("cuda"))
    L.gemm(A, B, C, M, N, K, (1, M), (1, K), (N, 1), batch=Z, bstrides=(R * K * M, R * N * K, M * N), nred=R,
           rstrides=(K * M, N * K), precision=L.PREC_TF32X3, ws=ws)
    ref = torch.einsum("zrkm,zrnk->zmn", A, B)
    assert torch.max(torch.abs(C - ref)).item() / torch.max(torch.abs(ref)).item() < 3e-6


@pytest.mark.parametrize("M,N,K,transposed_b", [(2, 8, 2, True), (2, 8, 2, False), (100, 37, 70, True),
                                                (33, 65, 5, False), (4, 4, 1, True)])
def test_tf32x3_gemm_ignores_stale_workspace(tf32, M, N, K, transposed_b):
    """K not a multiple of 4 pads the staged rows; reused scratch full of NaN bytes (as the caching
    allocator can hand back) must not reach the product (the first seed move of a sweep, R(2x2)
    times a 2x2x4 site, is the K=2 case)."""
    A = _rand(M, K, seed=M + K)
    B = _rand(K, N, seed=N + 5)
    Bs = B.T.contiguous() if transposed_b else B
    sB = (1, K) if transposed_b else (N, 1)
    C = torch.empty(M, N, dtype=torch.float64, device="cuda")
    ws = L.Workspace(torch.device("cuda"))
    ws.get(L.load().tn_gemm_workspace_bytes(L.PREC_TF32X3, M, N, K, 1, 1)).fill_(255)  # 0xFFFFFFFF: NaN
    L.gemm(A, Bs, C, M, N, K, (K, 1), sB, (N, 1), precision=L.PREC_TF32X3, ws=ws)
    L.check(L.load().tn_check_device_status(L.stream_handle()))
    ref = A @ B
    assert torch.isfinite(C).all()
    assert torch.max(torch.abs(C - ref)).item() <= 5e-6 * torch.max(torch.abs(ref)).item()


@pytest.mark.parametrize("m,n", [(1024, 512), (300, 200), (96, 200)])
def test_qr_mixed_any_fp64_magnitude(tf32, m, n):
    """tn_qr_mixed scales its input by an exact power of two before the FP32 factorisation (the
    cluster kernel for n <= m <= 1024, n <= 512, the blocked path otherwise): inputs scaled by
    2^500 and 2^-500 give bit-for-bit the same FP32 problem, hence the same Q and an exactly
    scaled R."""
    lib = L.load()
    k = min(m, n)
    A = _rand(m, n, seed=m * n)
    outs = []
    for f in (1.0, 2.0 ** 500, 2.0 ** -500):
        Q = torch.empty((m, k), dtype=torch.float64, device="cuda")
        R = torch.empty((k, n), dtype=torch.float64, device="cuda")
        ws = L.Workspace(torch.device("cuda"))
        wp, wb = ws.args(lib.tn_qr_mixed_workspace_bytes(m, n))
        L.check(lib.tn_qr_mixed(m, n, L.ptr(A * f), n, 1, L.ptr(Q), k, 1, L.ptr(R), n, 1, wp, wb, L.stream_handle()))
        L.check(lib.tn_check_device_status(L.stream_handle()))
        assert torch.isfinite(Q).all() and torch.isfinite(R).all()
        outs.append((Q, R / f))
    for Q, R in outs[1:]:
        torch.testing.assert_close(Q, outs[0][0], rtol=0, atol=1e-12)
        torch.testing.assert_close(R, outs[0][1], rtol=1e-12, atol=1e-12 * torch.max(torch.abs(outs[0][1])).item())


def test_tf32x3_gemm_reports_operands_beyond_fp32_range(tf32):
    """Split TF32 has FP32's exponent range: a finite FP64 operand of 1e103 cannot be staged, and the
    device status says so (TN_ERR_NUMERIC) instead of leaving silent NaNs."""
    lib = L.load()
    A = _rand(8, 16, seed=1) * 1e103
    B = _rand(16, 8, seed=2)
    C = torch.empty(8, 8, dtype=torch.float64, device="cuda")
    L.gemm(A, B, C, 8, 8, 16, (16, 1), (8, 1), (8, 1), precision=L.PREC_TF32X3, ws=L.Workspace(torch.device("cuda")))
    assert lib.tn_check_device_status(L.stream_handle()) == L.TN_ERR_NUMERIC
    assert b"FP32 range" in lib.tn_last_error()
    assert lib.tn_check_device_status(L.stream_handle()) == L.TN_OK  # the flag is cleared once reported


def test_seed_move_of_unnormalized_state_stays_fp64(tf32):
    """A random 100-site MPS centred by QR carries its norm (~1e100) on the centre: the first seed
    move absorbs in FP64; after a solve the centre has unit norm and seed moves use split TF32."""
    from tnalg_gb300 import Parameters as pm
    from tnalg_gb300.MPSClass import MpsOpenBoundaryClass
    para = pm.generate_parameters_dmrg("chain")
    para.update(l=100, chi=64)
    para = pm.make_consistent_parameter_dmrg(para)
    np.random.seed(0)
    A = MpsOpenBoundaryClass(100, 2, 64, operators=para["op"], precision="tf32x3")
    A.correct_orthogonal_center(0)
    dev = A._dev
    assert not dev.unit_norm
    dev.move_center_for_solve(1)
    assert torch.isfinite(dev.mps[1]).all()
    A.update_tensor_eigs(1, para["index1"], para["index2"], para["coeff1"], para["coeff2"], para["tau"], True,
                         tol=1e-12)
    assert dev.unit_norm and dev._seed_precision(True) == L.PREC_TF32X3
    dev.move_center_for_solve(2)
    assert torch.isfinite(dev.mps[2]).all()
    assert abs(torch.linalg.vector_norm(dev.mps[2]).item() - 1.0) < 1e-5
    L.check(L.load().tn_check_device_status(L.stream_handle()))


def _site(cl, d, cr, dense=True):
    wl = _rand(cl * d, cl * d, seed=cl)
    wl = wl + wl.T
    wr = _rand(d * cr, d * cr, seed=cr + 7)
    wr = wr + wr.T
    desc = L.SiteDesc(cl, d, cr, wl.data_ptr(), wr.data_ptr(), 0, None, None)
    full = None
    if dense:
        full = torch.kron(wl, torch.eye(cr, dtype=torch.float64, device="cuda")) + \
            torch.kron(torch.eye(cl, dtype=torch.float64, device="cuda"), wr)
    return desc, full, (wl, wr)


@pytest.mark.parametrize("cl,d,cr", [(64, 2, 64), (128, 2, 96), (5, 3, 7), (512, 2, 512)])
def test_tf32x3_matvec(tf32, cl, d, cr):
    """Mixed matvec against the FP64 matvec of the same site (block form, no dense matrix)."""
    lib = L.load()
    desc, _, keep = _site(cl, d, cr, dense=False)
    psi = _rand(cl * d * cr, seed=5)
    y = torch.empty_like(psi)
    ref = torch.empty_like(psi)
    ws = L.Workspace(torch.device("cuda"))
    for prec, out in ((L.PREC_TF32X3, y), (L.PREC_FP64, ref)):
        wp, wb = ws.args(lib.tn_matvec_workspace_bytes(ctypes.byref(desc), prec))
        L.check(lib.tn_matvec(ctypes.byref(desc), L.ptr(psi), L.ptr(out), 1.0, 0.5, prec, wp, wb,
                              L.stream_handle()))
    L.check(lib.tn_check_device_status(L.stream_handle()))
    assert torch.max(torch.abs(y - ref)).item() / torch.max(torch.abs(ref)).item() < 3e-6


def test_tf32x3_lanczos_fp64_refined_energy(tf32):
    lib = L.load()
    desc, dense, keep = _site(24, 2, 20)
    n = 24 * 2 * 20
    psi = _rand(n, seed=9)
    opts = L.LanczosOpts(1e-14, 0.0, 1e-12, 2e-6, 40, 200, 3, L.PREC_TF32X3, 1, 0)
    ws = L.Workspace(torch.device("cuda"))
    wp, wb = ws.args(lib.tn_lanczos_workspace_bytes(ctypes.byref(desc), ctypes.byref(opts)))
    res = L.LanczosResult()
    L.check(lib.tn_lanczos(ctypes.byref(desc), L.ptr(psi), ctypes.byref(opts), wp, wb, ctypes.byref(res),
                           L.stream_handle()))
    w0 = torch.linalg.eigvalsh(dense)[0].item()
    assert abs(res.energy_fp64 - w0) <= 1e-9 * abs(w0)
    assert abs(res.energy - w0) <= 1e-5 * abs(w0)


@pytest.mark.parametrize("m,n,cond,transposed", [(1024, 512, 1.0, False), (1024, 512, 1e10, False),
                                                 (1024, 512, 1e6, True), (512, 512, 1e8, False),
                                                 (1000, 300, 1e4, True), (256, 128, 1e6, False),
                                                 (64, 64, 1e3, False), (4, 2, 1.0, False), (96, 200, 1e3, False),
                                                 (256, 128, 0.0, False), (512, 256, -1.0, False),
                                                 (512, 256, -1.0, True), (128, 64, -1.0, True),
                                                 (128, 128, -2.0, False), (512, 256, -2.0, True)])
def test_qr_mixed_orthonormal_and_spanning(tf32, m, n, cond, transposed):
    """FP32 Householder + FP64 re-orthogonalisation: Q orthonormal to ~1e-12 at any conditioning,
    col(Q) = col(A) to FP32 accuracy, R accurate to FP32. n <= m <= 1024, n <= 512 run on the
    16-CTA cluster kernel; `transposed` reads A and writes Q through the column-major strides of a
    right gauge move; cond = 0 makes the last 16 singular values exactly zero, cond = -1 all but the
    first quarter (the centre tensor right after a bond grew by expansion: rank = the old bond), and
    cond = -2 scales those to 1e-21: sub-columns whose squares are subnormal in FP32, which the
    factorisation must take as zero instead of building a non-orthogonal reflector from them."""
    lib = L.load()
    k = min(m, n)
    g = torch.Generator(device="cpu").manual_seed(m + n)
    U, _ = torch.linalg.qr(torch.randn(m, k, generator=g, dtype=torch.float64))
    V, _ = torch.linalg.qr(torch.randn(n, k, generator=g, dtype=torch.float64))
    if cond > 0:
        s = torch.logspace(0, -np.log10(cond), k, dtype=torch.float64)
    else:
        s = torch.ones(k, dtype=torch.float64)
        if cond == 0:
            s[-16:] = 0.0
        else:
            s[k // 4:] = 0.0 if cond == -1 else 1e-21
    A = ((U * s) @ V.T).cuda()
    R = torch.empty((k, n), dtype=torch.float64, device="cuda")
    ws = L.Workspace(torch.device("cuda"))
    wp, wb = ws.args(lib.tn_qr_mixed_workspace_bytes(m, n))
    if transposed:
        At = A.T.contiguous()  # A(i, j) = At[j, i]
        Qt = torch.empty((k, m), dtype=torch.float64, device="cuda")
        L.check(lib.tn_qr_mixed(m, n, L.ptr(At), 1, m, L.ptr(Qt), 1, m, L.ptr(R), n, 1, wp, wb, L.stream_handle()))
        Q = Qt.T
    else:
        Q = torch.empty((m, k), dtype=torch.float64, device="cuda")
        L.check(lib.tn_qr_mixed(m, n, L.ptr(A), n, 1, L.ptr(Q), k, 1, L.ptr(R), n, 1, wp, wb, L.stream_handle()))
    L.check(lib.tn_check_device_status(L.stream_handle()))
    assert torch.isfinite(Q).all() and torch.isfinite(R).all()
    assert torch.equal(torch.tril(R, -1), torch.zeros_like(R))
    eye = torch.eye(k, dtype=torch.float64, device="cuda")
    assert torch.max(torch.abs(Q.T @ Q - eye)).item() < 1e-11
    resid = A - Q @ (Q.T @ A)
    assert torch.linalg.matrix_norm(resid).item() / torch.linalg.matrix_norm(A).item() < 1e-5
    assert torch.linalg.matrix_norm(Q @ R - A).item() / torch.linalg.matrix_norm(A).item() < 1e-5


def test_tf32x3_dmrg_close_to_reference(tf32):
    """Mixed path on the N=12 chain: energy per site within 1e-8 of the reference's FP64 run."""
    from tnalg_gb300 import DMRG_anyH
    g, m = gc.load("chain_n12_chi16_h"), gc.meta()["chain_n12_chi16_h"]
    np.random.seed(m["seed"])
    with contextlib.redirect_stdout(io.StringIO()):
        ob, A, info, _ = DMRG_anyH.dmrg_finite_size(gc.para_of("chain_n12_chi16_h", precision="tf32x3"))
    assert abs(ob["e_per_site"] - float(g["e_per_site"])) <= 1e-8
    np.testing.assert_allclose(np.ravel(ob["mz"]), g["mz"], atol=1e-5)


def test_tf32x3_chi128_sweeps_match_fp64(tf32):
    """An N=24 XXZ chain in a transverse field, chi ramped to 128: the split-TF32 path (cluster QR for the
    seeding moves, bond growth and spectrum pass; split-TF32 matvec, environments and correlator
    strings) against the FP64 path on the same seed: energy per site to 1e-8; one-site and
    two-site observables and entanglement entropies to 1e-5, the mixed path's bar on the N=12
    golden case (the two runs take different Lanczos trajectories, and a state converged to
    ~1e-9 in energy differs at ~1e-6 in its observables)."""
    from tnalg_gb300 import DMRG_anyH, Parameters as pm
    runs = {}
    for prec in ("fp64", "tf32x3"):
        para = pm.generate_parameters_dmrg("chain")
        para.update(l=24, chi=32, jz=0.8, hx=0.1, sweep_time=4, chi_schedule=[32, 128, 128, 128], dt_ob=4,
                    break_tol=-1.0, eigs_tol=1e-12, precision=prec)
        para = pm.make_consistent_parameter_dmrg(para)
        np.random.seed(7)
        with contextlib.redirect_stdout(io.StringIO()):
            ob, A, info, _ = DMRG_anyH.dmrg_finite_size(para)
        runs[prec] = (ob, A)
    (o64, A64), (o32, A32) = runs["fp64"], runs["tf32x3"]
    assert A32.stats["qr_mixed"] > 0 and A64.stats["qr_mixed"] == 0
    assert int(A32.virtual_dim.max()) == 128
    assert abs(o32["e_per_site"] - o64["e_per_site"]) <= 1e-8
    np.testing.assert_allclose(np.ravel(o32["mx"]), np.ravel(o64["mx"]), atol=1e-5)
    np.testing.assert_allclose(np.ravel(o32["mz"]), np.ravel(o64["mz"]), atol=1e-5)
    np.testing.assert_allclose(np.ravel(o32["corr_x"]), np.ravel(o64["corr_x"]), atol=1e-5)
    np.testing.assert_allclose(np.ravel(o32["corr_z"]), np.ravel(o64["corr_z"]), atol=1e-5)
    np.testing.assert_allclose(np.ravel(A32.ent), np.ravel(A64.ent), atol=1e-5)


@pytest.mark.parametrize("cl,d,cr,ng", [(64, 2, 48, 3), (5, 3, 7, 2), (256, 2, 256, 4)])
def test_tf32x3_matvec_straddling_pairs(tf32, cl, d, cr, ng):
    """Split-TF32 matvec with straddling pairs (sum_g SL_g (x) 1 (x) SR_g, as in ladders and
    long-range couplings) against the FP64 matvec of the same site."""
    lib = L.load()
    desc0, _, keep = _site(cl, d, cr, dense=False)
    sl = _rand(ng, cl, cl, seed=11)
    sr = _rand(ng, cr, cr, seed=12)
    desc = L.SiteDesc(cl, d, cr, keep[0].data_ptr(), keep[1].data_ptr(), ng, sl.data_ptr(), sr.data_ptr())
    psi = _rand(cl * d * cr, seed=5)
    y = torch.empty_like(psi)
    ref = torch.empty_like(psi)
    ws = L.Workspace(torch.device("cuda"))
    for prec, out in ((L.PREC_TF32X3, y), (L.PREC_FP64, ref)):
        wp, wb = ws.args(lib.tn_matvec_workspace_bytes(ctypes.byref(desc), prec))
        L.check(lib.tn_matvec(ctypes.byref(desc), L.ptr(psi), L.ptr(out), 0.75, 0.5, prec, wp, wb,
                              L.stream_handle()))
    L.check(lib.tn_check_device_status(L.stream_handle()))
    assert torch.max(torch.abs(y - ref)).item() / torch.max(torch.abs(ref)).item() < 3e-6


def test_tf32x3_ladder_with_straddling_couplings(tf32):
    """The 2x4 ladder of the reference runs (its rungs straddle the centre) on the split-TF32 path:
    energy per site within 1e-7 of the reference's FP64 run."""
    from tnalg_gb300 import DMRG_anyH
    g, m = gc.load("ladder_2x4_chi8"), gc.meta()["ladder_2x4_chi8"]
    np.random.seed(m["seed"])
    with contextlib.redirect_stdout(io.StringIO()):
        ob, A, info, _ = DMRG_anyH.dmrg_finite_size(gc.para_of("ladder_2x4_chi8", precision="tf32x3"))
    assert abs(ob["e_per_site"] - float(g["e_per_site"])) <= 1e-7


def test_tf32x3_j1j2_lattice_matches_fp64_after_ten_sweeps(tf32):
    """The frustrated J1-J2 model (J2 = 0.5) on a 4 x 4 open square lattice in snake order (straddling
    couplings up to 7 sites apart), 10 sweeps at chi = 64 from the same seeded random MPS on both
    paths: the split-TF32 state's energy per site (FP64 observables) within 1e-8 of the plain FP64
    path's, the energy per site of the metric's tolerance."""
    from tnalg_gb300 import Parameters as pm
    from tnalg_gb300 import run_lattice
    para = pm.generate_parameters_j1j2_snake(4, 4, j1=1.0, j2=0.5)
    para.update(tau=1e-4, eigs_tol=1e-12)
    mixed = run_lattice.run(para, "tf32x3", [64], 10, "cuda", seed=0)
    fp64 = run_lattice.run(para, "fp64", [64], 10, "cuda", seed=0)
    assert mixed["chi_max"] == fp64["chi_max"] == 64
    assert abs(mixed["e_per_site"] - fp64["e_per_site"]) <= 1e-8, (mixed["e_per_site"], fp64["e_per_site"])
    assert np.max(np.abs(mixed["eb_full"] - fp64["eb_full"])) < 1e-5


@pytest.mark.parametrize("m,n,zero", [(1024, 512, "tail"), (512, 256, "every_third"), (256, 128, "tail")])
def test_qr_mixed_exactly_zero_columns(tf32, m, n, zero):
    """Gauge moves right after a bond grew by expansion factor matrices whose columns for the new
    directions are exactly zero (the zero rows of the site right of the bond, transposed): Q must still
    have orthonormal columns and Q R = A."""
    lib = L.load()
    A = _rand(m, n, seed=m + 3 * n)
    if zero == "tail":
        A[:, n // 2:] = 0.0
    else:
        A[:, ::3] = 0.0
    Q = torch.empty((m, n), dtype=torch.float64, device="cuda")
    R = torch.empty((n, n), dtype=torch.float64, device="cuda")
    for fn in ("tn_qr_mixed", "tn_qr"):
        ws = L.Workspace(torch.device("cuda"))
        wp, wb = ws.args(getattr(lib, fn + "_workspace_bytes")(m, n))
        L.check(getattr(lib, fn)(m, n, L.ptr(A), n, 1, L.ptr(Q), n, 1, L.ptr(R), n, 1, wp, wb, L.stream_handle()))
        L.check(lib.tn_check_device_status(L.stream_handle()))
        eye = torch.eye(n, dtype=torch.float64, device="cuda")
        assert torch.isfinite(Q).all() and torch.isfinite(R).all(), fn
        assert torch.max(torch.abs(Q.T @ Q - eye)).item() < 1e-11, fn
        assert torch.max(torch.abs(Q @ R - A)).item() < 1e-5 * torch.max(torch.abs(A)).item(), fn
