"""Grouped contractions and the batched DMRG path on the GPU, against FP64 references."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from tnalg_gb300 import _lib as L  # noqa: E402


def _rand(*shape, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(*shape, generator=g, dtype=torch.float64).cuda()


def _problem(A, B, C, M, N, K, sA, sB, sC, nred=1, sAr=0, sBr=0, alpha=1.0, beta=0.0, accumulate=0, active=None):
    r = np.zeros(1, dtype=L.GEMM_PROBLEM_DTYPE)[0]
    r["M"], r["N"], r["K"], r["nred"] = M, N, K, nred
    r["A"], r["sAm"], r["sAk"], r["sAr"] = A.data_ptr(), sA[0], sA[1], sAr
    r["B"], r["sBk"], r["sBn"], r["sBr"] = B.data_ptr(), sB[0], sB[1], sBr
    r["C"], r["sCm"], r["sCn"] = C.data_ptr(), sC[0], sC[1]
    r["alpha"], r["beta"], r["accumulate"] = alpha, beta, accumulate
    r["active"] = 0 if active is None else active.data_ptr()
    return r


@pytest.mark.parametrize("precision", [L.PREC_FP64, L.PREC_TF32X3])
def test_grouped_gemm_uneven_problems(cuda_lib, precision):
    """Problems of uneven shapes (ragged edges, K not a multiple of the 32-wide K-block, a 1 x 1
    product), transposed operand views, a reduced sum over r, two problems adding into one output,
    alpha/beta and a problem switched off by its device flag, all in one grouped call."""
    if precision == L.PREC_TF32X3 and not L.tf32x3_available():
        pytest.skip("tf32x3 needs an sm_103 device")
    keep, recs, refs = [], [], []
    shapes = [(256, 128, 256), (130, 7, 70), (1, 1, 1), (64, 300, 33), (5, 129, 200)]
    for i, (M, N, K) in enumerate(shapes):
        A, B = _rand(M, K, seed=i), _rand(K, N, seed=100 + i)
        Cin = _rand(M, N, seed=200 + i)
        C = Cin.clone()
        keep += [A, B, C]
        recs.append(_problem(A, B, C, M, N, K, (K, 1), (N, 1), (N, 1), alpha=0.75, beta=-0.5))
        refs.append((C, 0.75 * (A @ B) - 0.5 * Cin))
    # transposed views: A stored (K, M), B stored (N, K)
    M, N, K = 96, 80, 40
    At, Bt = _rand(K, M, seed=7), _rand(N, K, seed=8)
    C = torch.zeros(M, N, dtype=torch.float64, device="cuda")
    keep += [At, Bt, C]
    recs.append(_problem(At, Bt, C, M, N, K, (1, M), (1, K), (N, 1)))
    refs.append((C, At.T @ Bt.T))
    # reduced sum over r = 0..2, and a second problem adding into the same output
    R, M, N, K = 3, 100, 60, 50
    Ar, Br = _rand(R, M, K, seed=9), _rand(R, K, N, seed=10)
    A2, B2 = _rand(M, 30, seed=11), _rand(30, N, seed=12)
    C = torch.zeros(M, N, dtype=torch.float64, device="cuda")
    keep += [Ar, Br, A2, B2, C]
    recs.append(_problem(Ar, Br, C, M, N, K, (K, 1), (N, 1), (N, 1), nred=R, sAr=M * K, sBr=K * N, accumulate=1))
    recs.append(_problem(A2, B2, C, M, N, 30, (30, 1), (N, 1), (N, 1), alpha=2.0, accumulate=1))
    refs.append((C, torch.einsum("rmk,rkn->mn", Ar, Br) + 2.0 * A2 @ B2))
    # switched off: its output must stay untouched
    off = torch.zeros(1, dtype=torch.int32, device="cuda")
    A3, B3 = _rand(40, 40, seed=13), _rand(40, 40, seed=14)
    C3 = torch.full((40, 40), 7.0, dtype=torch.float64, device="cuda")
    keep += [off, A3, B3, C3]
    recs.append(_problem(A3, B3, C3, 40, 40, 40, (40, 1), (40, 1), (40, 1), active=off))
    refs.append((C3, torch.full((40, 40), 7.0, dtype=torch.float64, device="cuda")))
    L.grouped_gemm(np.array(recs, dtype=L.GEMM_PROBLEM_DTYPE), precision=precision)
    L.check(L.load().tn_check_device_status(L.stream_handle()))
    torch.cuda.synchronize()
    for C, ref in refs:
        scale = max(torch.max(torch.abs(ref)).item(), 1.0)
        err = torch.max(torch.abs(C - ref)).item() / scale
        assert err < (1e-13 if precision == L.PREC_FP64 else 5e-6), err


def _sym_block(n, seed, shift=0.0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn(n, n, generator=g, dtype=torch.float64)
    return ((x + x.T) / 2 + shift * torch.eye(n, dtype=torch.float64)).cuda()


def _dense_heff(wl, wr, cl, d, cr):
    """H = WL (x) 1_cr + 1_cl (x) WR on psi[(a s) b] = psi[a (s b)]."""
    return torch.kron(wl, torch.eye(cr, dtype=torch.float64, device="cuda")) + \
        torch.kron(torch.eye(cl, dtype=torch.float64, device="cuda"), wr)


@pytest.mark.parametrize("precision", [L.PREC_FP64, L.PREC_TF32X3])
def test_batched_lanczos_matches_dense(cuda_lib, precision):
    """Jobs of uneven shapes (edge sites with chi_l = 1, interior sites up to chi = 40) solved in
    one batched call, against dense eigh: FP64 to 1e-10 in energy and eigenvector; split TF32 to
    its residual floor (its Rayleigh quotient to 1e-9, second order in the residual)."""
    if precision == L.PREC_TF32X3 and not L.tf32x3_available():
        pytest.skip("tf32x3 needs an sm_103 device")
    lib = L.load()
    shapes = [(1, 2, 2), (2, 2, 4), (8, 2, 16), (16, 2, 16), (40, 2, 24), (24, 2, 40), (32, 2, 32)]
    keep, jobs, dense = [], [], []
    for i, (cl, d, cr) in enumerate(shapes):
        wl = _sym_block(cl * d, 10 + i, shift=0.5)
        wr = _sym_block(d * cr, 50 + i)
        psi = _rand(cl * d * cr, seed=90 + i)
        out = torch.empty_like(psi)
        keep += [wl, wr, psi, out]
        j = L.BatchSolve()
        j.site = L.SiteDesc(cl, d, cr, wl.data_ptr(), wr.data_ptr(), 0, None, None)
        j.psi_in, j.psi_out = psi.data_ptr(), out.data_ptr()
        jobs.append(j)
        dense.append(_dense_heff(wl, wr, cl, d, cr))
    arr = (L.BatchSolve * len(jobs))(*jobs)
    opts = L.LanczosOpts(1e-12, 1e-4, 0.0, 2e-6, 40, 50, 3, precision, 0, 0)
    need = lib.tn_batched_lanczos_workspace_bytes(ctypes_ptr(arr), len(jobs), ctypes_ref(opts))
    ws = torch.empty(need + 1024, dtype=torch.uint8, device="cuda")
    res = (L.LanczosResult * len(jobs))()
    st = lib.tn_batched_lanczos(ctypes_ptr(arr), len(jobs), ctypes_ref(opts), ws.data_ptr(), ws.numel(),
                                ctypes_ptr(res), L.stream_handle())
    assert st == L.TN_OK, lib.tn_last_error()
    torch.cuda.synchronize()
    for i, H in enumerate(dense):
        w, v = torch.linalg.eigh(H)
        x = keep[4 * i + 3]
        scale = max(1.0, abs(w[0].item()))
        assert abs(torch.linalg.vector_norm(x).item() - 1.0) < 1e-12
        rq = (x @ (H @ x)).item()
        resid = torch.linalg.vector_norm(H @ x - rq * x).item()
        if precision == L.PREC_FP64:
            assert abs(res[i].energy - w[0].item()) < 1e-10 * scale, (i, res[i].energy, w[0].item())
            assert resid < 1e-7 * scale, (i, resid)
            assert abs(abs(torch.dot(x, v[:, 0]).item()) - 1.0) < 1e-10
        else:
            assert abs(rq - w[0].item()) < 1e-9 * scale, (i, rq, w[0].item())
            assert resid < 1e-4 * scale, (i, resid)
        assert res[i].converged == 1


def ctypes_ptr(arr):
    import ctypes
    return ctypes.cast(arr, ctypes.c_void_p)


def ctypes_ref(obj):
    import ctypes
    return ctypes.byref(obj)


@pytest.mark.parametrize("precision", [L.PREC_FP64, L.PREC_TF32X3])
def test_batched_lanczos_with_straddling_pairs(cuda_lib, precision):
    """Jobs whose effective Hamiltonian carries straddling pairs (ladder-like couplings across the
    site), mixed in one batch with jobs that have none."""
    if precision == L.PREC_TF32X3 and not L.tf32x3_available():
        pytest.skip("tf32x3 needs an sm_103 device")
    lib = L.load()
    specs = [(8, 2, 12, 2), (16, 2, 16, 0), (20, 2, 20, 3), (1, 2, 4, 0)]
    keep, jobs, dense = [], [], []
    for i, (cl, d, cr, ng) in enumerate(specs):
        wl = _sym_block(cl * d, 200 + i, shift=0.3)
        wr = _sym_block(d * cr, 300 + i)
        sl = torch.stack([_sym_block(cl, 400 + 7 * i + g) for g in range(ng)]) if ng else None
        sr = torch.stack([_sym_block(cr, 500 + 7 * i + g) for g in range(ng)]) if ng else None
        psi = _rand(cl * d * cr, seed=600 + i)
        out = torch.empty_like(psi)
        keep += [wl, wr, sl, sr, psi, out]
        j = L.BatchSolve()
        j.site = L.SiteDesc(cl, d, cr, wl.data_ptr(), wr.data_ptr(), ng, sl.data_ptr() if ng else None,
                            sr.data_ptr() if ng else None)
        j.psi_in, j.psi_out = psi.data_ptr(), out.data_ptr()
        jobs.append(j)
        H = _dense_heff(wl, wr, cl, d, cr)
        eye_d = torch.eye(d, dtype=torch.float64, device="cuda")
        for g in range(ng):
            H = H + torch.kron(sl[g], torch.kron(eye_d, sr[g]))
        dense.append(H)
    arr = (L.BatchSolve * len(jobs))(*jobs)
    opts = L.LanczosOpts(1e-12, 1e-4, 0.0, 2e-6, 30, 50, 3, precision, 0, 0)
    need = lib.tn_batched_lanczos_workspace_bytes(ctypes_ptr(arr), len(jobs), ctypes_ref(opts))
    ws = torch.empty(need + 1024, dtype=torch.uint8, device="cuda")
    res = (L.LanczosResult * len(jobs))()
    st = lib.tn_batched_lanczos(ctypes_ptr(arr), len(jobs), ctypes_ref(opts), ws.data_ptr(), ws.numel(),
                                ctypes_ptr(res), L.stream_handle())
    assert st == L.TN_OK, lib.tn_last_error()
    torch.cuda.synchronize()
    for i, H in enumerate(dense):
        w = torch.linalg.eigvalsh(H)
        x = keep[6 * i + 5]
        scale = max(1.0, abs(w[0].item()))
        rq = (x @ (H @ x)).item()
        tol = 1e-10 if precision == L.PREC_FP64 else 1e-9
        assert abs(rq - w[0].item()) < tol * scale, (i, rq, w[0].item())
        if precision == L.PREC_FP64:
            assert abs(res[i].energy - w[0].item()) < 1e-10 * scale
