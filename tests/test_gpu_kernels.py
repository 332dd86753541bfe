"""CUDA kernels through the C ABI against torch FP64 / numpy references (GPU only)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from tnalg_gb300 import _lib as L  # noqa: E402


def _dev():
    return torch.device("cuda")


def _rand(*shape, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(*shape, generator=g, dtype=torch.float64).to(_dev())


@pytest.mark.parametrize("M,N,K,batch,nred", [(64, 48, 80, 1, 1), (1024, 512, 1024, 1, 1), (7, 300, 5, 3, 1),
                                               (96, 40, 33, 2, 3), (16, 512, 1024, 1, 1), (1, 1, 1, 1, 1)])
def test_gemm_fp64_matches_torch(cuda_lib, M, N, K, batch, nred):
    A = _rand(batch, nred, K, M, seed=1)   # stored transposed: A(m,k) = A[b,r,k,m]
    B = _rand(batch, nred, K, N, seed=2)
    Cin = _rand(batch, M, N, seed=3)
    C = torch.empty_like(Cin)
    ws = L.Workspace(_dev())
    L.gemm(A, B, C, M, N, K, (1, M), (N, 1), (N, 1), Cin=Cin, batch=batch,
           bstrides=(nred * K * M, nred * K * N, M * N), nred=nred, rstrides=(K * M, K * N), alpha=0.75, beta=-0.5,
           ws=ws)
    ref = 0.75 * torch.einsum("brkm,brkn->bmn", A, B) - 0.5 * Cin
    torch.cuda.synchronize()
    assert torch.allclose(C, ref, rtol=1e-12, atol=1e-12 * K)


@pytest.mark.parametrize("m,n", [(1024, 512), (8, 16), (33, 17), (512, 1024), (2, 1), (96, 96)])
def test_qr_orthonormal_and_reconstructs(cuda_lib, m, n):
    lib = L.load()
    A = _rand(m, n, seed=m + n)
    k = min(m, n)
    Q = torch.empty((m, k), dtype=torch.float64, device=_dev())
    R = torch.empty((k, n), dtype=torch.float64, device=_dev())
    ws = L.Workspace(_dev())
    wp, wb = ws.args(lib.tn_qr_workspace_bytes(m, n))
    L.check(lib.tn_qr(m, n, L.ptr(A), n, 1, L.ptr(Q), k, 1, L.ptr(R), n, 1, wp, wb, L.stream_handle()))
    torch.cuda.synchronize()
    eye = torch.eye(k, dtype=torch.float64, device=_dev())
    assert torch.max(torch.abs(Q.T @ Q - eye)).item() < 1e-13 * max(1, m / 64)
    assert torch.max(torch.abs(Q @ R - A)).item() < 1e-12 * np.sqrt(m)
    assert torch.count_nonzero(torch.tril(R, -1)).item() == 0
    # LAPACK's reflector convention: |R| agrees with numpy's
    Rn = np.linalg.qr(A.cpu().numpy())[1]
    np.testing.assert_allclose(R.cpu().numpy(), Rn[:k], atol=1e-10 * np.sqrt(m))


def test_qr_strided_transpose_input(cuda_lib):
    lib = L.load()
    M = _rand(40, 2 * 24, seed=5)  # QR of M^T read through strides
    m, n = 48, 40
    Q = torch.empty((40, 48), dtype=torch.float64, device=_dev())  # written transposed
    R = torch.empty((40, 40), dtype=torch.float64, device=_dev())
    ws = L.Workspace(_dev())
    wp, wb = ws.args(lib.tn_qr_workspace_bytes(m, n))
    L.check(lib.tn_qr(m, n, L.ptr(M), 1, 48, L.ptr(Q), 1, 48, L.ptr(R), 40, 1, wp, wb, L.stream_handle()))
    torch.cuda.synchronize()
    assert torch.max(torch.abs(Q.T @ R - M.T)).item() < 1e-12


def _site(cl, d, cr, nstr, seed):
    wl = _rand(cl * d, cl * d, seed=seed)
    wl = wl + wl.T
    wr = _rand(d * cr, d * cr, seed=seed + 1)
    wr = wr + wr.T
    sl = _rand(max(nstr, 1), cl, cl, seed=seed + 2)
    sl = sl + sl.transpose(1, 2)
    sr = _rand(max(nstr, 1), cr, cr, seed=seed + 3)
    sr = sr + sr.transpose(1, 2)
    desc = L.SiteDesc(cl, d, cr, wl.data_ptr(), wr.data_ptr(), nstr, sl.data_ptr() if nstr else None,
                      sr.data_ptr() if nstr else None)
    dense = torch.kron(wl, torch.eye(cr, dtype=torch.float64, device=_dev()))
    dense = dense + torch.kron(torch.eye(cl, dtype=torch.float64, device=_dev()), wr)
    for k in range(nstr):
        dense = dense + torch.kron(torch.kron(sl[k], torch.eye(d, dtype=torch.float64, device=_dev())), sr[k])
    return desc, dense, (wl, wr, sl, sr)


@pytest.mark.parametrize("cl,d,cr,nstr", [(8, 2, 8, 0), (16, 2, 12, 2), (5, 3, 7, 1), (1, 2, 4, 0)])
def test_matvec_matches_dense(cuda_lib, cl, d, cr, nstr):
    lib = L.load()
    desc, dense, keep = _site(cl, d, cr, nstr, seed=cl * 7 + cr)
    psi = _rand(cl * d * cr, seed=11)
    y = torch.empty_like(psi)
    ws = L.Workspace(_dev())
    wp, wb = ws.args(lib.tn_matvec_workspace_bytes(ctypes.byref(desc), L.PREC_FP64))
    L.check(lib.tn_matvec(ctypes.byref(desc), L.ptr(psi), L.ptr(y), -1e-4, 1.0, L.PREC_FP64, wp, wb,
                          L.stream_handle()))
    torch.cuda.synchronize()
    ref = psi - 1e-4 * (dense @ psi)
    assert torch.max(torch.abs(y - ref)).item() < 1e-12


@pytest.mark.parametrize("cl,d,cr,nstr", [(16, 2, 16, 0), (24, 2, 20, 3), (6, 3, 9, 0), (1, 2, 2, 0)])
def test_lanczos_lowest_eigenpair(cuda_lib, cl, d, cr, nstr):
    lib = L.load()
    desc, dense, keep = _site(cl, d, cr, nstr, seed=3 * cl + cr)
    n = cl * d * cr
    psi = _rand(n, seed=21)
    opts = L.LanczosOpts(1e-14, 0.0, 1e-12, 0.0, 40, 200, 3, L.PREC_FP64, 1, 0)
    ws = L.Workspace(_dev())
    wp, wb = ws.args(lib.tn_lanczos_workspace_bytes(ctypes.byref(desc), ctypes.byref(opts)))
    res = L.LanczosResult()
    L.check(lib.tn_lanczos(ctypes.byref(desc), L.ptr(psi), ctypes.byref(opts), wp, wb, ctypes.byref(res),
                           L.stream_handle()))
    torch.cuda.synchronize()
    w = torch.linalg.eigvalsh(dense)
    scale = max(1.0, abs(w[0].item()))
    assert abs(res.energy - w[0].item()) < 1e-10 * scale
    assert abs(res.energy_fp64 - w[0].item()) < 1e-10 * scale
    r = dense @ psi - res.energy_fp64 * psi
    assert torch.linalg.vector_norm(r).item() < 1e-8 * scale
    assert abs(torch.linalg.vector_norm(psi).item() - 1.0) < 1e-13
    assert res.converged == 1


def test_singular_values_match_numpy(cuda_lib):
    lib = L.load()
    for k, n in ((12, 12), (33, 40), (64, 64), (5, 9)):
        X = _rand(k, n, seed=k)
        X[:, : k // 3] *= 1e-6  # spread the spectrum
        out = torch.empty(k, dtype=torch.float64, device=_dev())
        ws = L.Workspace(_dev())
        wp, wb = ws.args(lib.tn_singular_values_workspace_bytes(k, n))
        L.check(lib.tn_singular_values(k, n, L.ptr(X), n, 1, L.ptr(out), 1e-15, 60, wp, wb, L.stream_handle()))
        s = np.sort(out.cpu().numpy())[::-1]
        ref = np.linalg.svd(X.cpu().numpy(), compute_uv=False)
        np.testing.assert_allclose(s, ref, atol=1e-13 * ref[0], rtol=1e-11)


def test_singular_values_stop_on_rank_deficient_rows(cuda_lib):
    """More rows than columns (48 x 40): 8 rows end up numerically null and rounding noise keeps
    them from ever becoming orthogonal; the null-row test must let the sweeps stop well before
    max_sweeps (square cases of this size take 15-20 sweeps), so 25 sweeps return TN_OK. With one
    sweep allowed the call reports TN_ERR_NOCONV and still writes the values."""
    lib = L.load()
    k, n = 48, 40
    X = _rand(k, n, seed=11)
    out = torch.empty(k, dtype=torch.float64, device=_dev())
    ws = L.Workspace(_dev())
    wp, wb = ws.args(lib.tn_singular_values_workspace_bytes(k, n))
    st = lib.tn_singular_values(k, n, L.ptr(X), n, 1, L.ptr(out), 1e-15, 25, wp, wb, L.stream_handle())
    assert st == L.TN_OK, lib.tn_last_error()
    s = np.sort(out.cpu().numpy())[::-1]
    ref = np.linalg.svd(X.cpu().numpy(), compute_uv=False)
    np.testing.assert_allclose(s[:n], ref, atol=1e-13 * ref[0], rtol=1e-11)
    assert np.all(s[n:] <= 1e-12 * ref[0])
    st = lib.tn_singular_values(k, n, L.ptr(X), n, 1, L.ptr(out), 1e-15, 1, wp, wb, L.stream_handle())
    assert st == L.TN_ERR_NOCONV
    assert np.all(np.isfinite(out.cpu().numpy()))


def test_singular_values_batched_match_numpy(cuda_lib):
    """One batched call over matrices of different shapes (an odd row count, a transposed view,
    a 512 x 512 bond matrix), to 1e-13 of each matrix's largest value."""
    mats = []
    for k, n, seed in ((12, 12, 1), (33, 40, 2), (5, 9, 3), (512, 512, 4), (64, 64, 5)):
        X = _rand(k, n, seed=seed)
        X[:, : k // 3] *= 1e-4  # spread the spectrum
        mats.append(X)
    mats.append(_rand(40, 30, seed=6).T)  # 30 x 40 read through strides (1, 30)
    spectra = L.singular_values_batched(mats)
    L.check(L.load().tn_check_device_status(L.stream_handle()))
    tol = 1e-13
    for X, s in zip(mats, spectra):
        ref = np.linalg.svd(X.cpu().numpy(), compute_uv=False)
        np.testing.assert_allclose(s[: len(ref)], ref, atol=tol * ref[0], rtol=0)


def test_block_assembly_and_site_ops(cuda_lib):
    lib = L.load()
    chi, d = 6, 2
    env = _rand(3, chi, chi, seed=4)
    ops = _rand(4, d, d, seed=5)
    terms = [(0, -1, 1.0), (-1, 2, 0.3), (1, 3, -0.7), (2, 0, 1.5)]
    tt, nt = L.terms_tensor(terms, _dev())
    E, O = env.cpu().numpy(), ops.cpu().numpy()
    for side in (0, 1):
        W = torch.empty((chi * d, chi * d), dtype=torch.float64, device=_dev())
        L.check(lib.tn_assemble_block(side, chi, d, L.ptr(env), L.ptr(ops), L.ptr(tt), nt, L.ptr(W),
                                      L.stream_handle()))
        ref = np.zeros((chi * d, chi * d))
        for s, o, c in terms:
            e = np.eye(chi) if s < 0 else E[s]
            op = np.eye(d) if o < 0 else O[o]
            ref += c * (np.kron(e, op) if side == 0 else np.kron(op, e))
        np.testing.assert_allclose(W.cpu().numpy(), ref, atol=1e-14)
    out = torch.empty((2, chi, chi), dtype=torch.float64, device=_dev())
    ct, nc = L.terms_tensor([(0, 0, 2.0), (2, 0, -1.0), (1, 1, 0.5)], _dev())
    L.check(lib.tn_combine_slots(chi, L.ptr(env), L.ptr(ct), nc, 2, L.ptr(out), L.stream_handle()))
    np.testing.assert_allclose(out[0].cpu().numpy(), 2 * E[0] - E[2], atol=1e-14)
    np.testing.assert_allclose(out[1].cpu().numpy(), 0.5 * E[1], atol=1e-14)
    X = _rand(3, d, 5, seed=9)
    idx = torch.tensor([2, -1], dtype=torch.int32, device=_dev())
    Y = torch.empty((2, 3 * d * 5), dtype=torch.float64, device=_dev())
    L.check(lib.tn_apply_site_ops(3, d, 5, L.ptr(X), L.ptr(ops), L.ptr(idx), 2, L.ptr(Y), 3 * d * 5,
                                  L.stream_handle()))
    Xn = X.cpu().numpy()
    np.testing.assert_allclose(Y[0].cpu().numpy(), np.einsum("xs,asb->axb", O[2], Xn).ravel(), atol=1e-14)
    np.testing.assert_allclose(Y[1].cpu().numpy(), Xn.ravel(), atol=0)
    G = torch.zeros((d, d), dtype=torch.float64, device=_dev())
    T = _rand(3, d, 5, seed=10)
    L.check(lib.tn_pair_contract(3, d, 5, L.ptr(X), L.ptr(T), 1.0, L.ptr(G), L.stream_handle()))
    np.testing.assert_allclose(G.cpu().numpy(), np.einsum("xpz,xsz->ps", Xn, T.cpu().numpy()), atol=1e-13)


def test_errors_are_reported_not_raised(cuda_lib):
    lib = L.load()
    st = lib.tn_qr(0, 4, None, 1, 1, None, 1, 1, None, 1, 1, None, 0, L.stream_handle())
    assert st == L.TN_ERR_ARG and b"qr" in lib.tn_last_error()
    A = _rand(8, 4, seed=1)
    st = lib.tn_qr(8, 4, L.ptr(A), 4, 1, None, 1, 1, None, 1, 1, None, 0, L.stream_handle())
    assert st == L.TN_ERR_WORKSPACE


@pytest.mark.parametrize("k,n,chi", [(40, 60, 12), (96, 64, 30), (33, 33, 33)])
def test_svd_jacobi_truncation_matches_numpy(cuda_lib, k, n, chi):
    """tn_svd_jacobi with singular vectors: the rank-chi truncation U_r diag(s_r) Vt_r equals numpy's
    (the best rank-chi approximation), U and V have orthonormal columns / rows, and the singular
    values agree to 1e-13 of the largest."""
    X = _rand(k, n, seed=k + n)
    X[:, : n // 3] *= 1e-3   # spread the spectrum (distinct values, well separated at the cut)
    U, s, Vt = L.svd_truncated(X, chi)
    Xh = X.cpu().numpy()
    u, sv, vt = np.linalg.svd(Xh, full_matrices=False)
    r = min(chi, len(sv))
    np.testing.assert_allclose(s.cpu().numpy(), sv[:r], atol=1e-13 * sv[0], rtol=1e-11)
    approx = (U * s) @ Vt
    ref = (u[:, :r] * sv[:r]) @ vt[:r]
    assert np.max(np.abs(approx.cpu().numpy() - ref)) < 1e-11 * sv[0]
    eye = np.eye(r)
    assert np.max(np.abs((U.T @ U).cpu().numpy() - eye)) < 1e-12
    assert np.max(np.abs((Vt @ Vt.T).cpu().numpy() - eye)) < 1e-12


def test_bounded_wait_gives_up_and_the_context_stays_usable(cuda_lib):
    """A device wait that can never be satisfied (a grid barrier expecting one block more than
    launched) gives up after its limit and reports TN_ERR_TIMEOUT through the stream's error word;
    the next calls on the same stream run normally (a Jacobi SVD through the same barrier code)."""
    lib = L.load()
    ws = L.Workspace(_dev())
    buf = ws.get(4096)
    base = (buf.data_ptr() + 255) // 256 * 256
    st = lib.tn_selftest_wait_timeout(base, 1024, L.stream_handle())
    assert st == L.TN_ERR_TIMEOUT, lib.tn_last_error()
    assert b"gave up" in lib.tn_last_error()
    L.check(lib.tn_check_device_status(L.stream_handle()))   # the error word was read and cleared
    X = _rand(40, 64, seed=5)
    U, s, Vt = L.svd_truncated(X, 40, tol=1e-15)
    ref = np.linalg.svd(X.cpu().numpy(), compute_uv=False)
    np.testing.assert_allclose(np.sort(s.cpu().numpy())[::-1], ref, atol=1e-13 * ref[0], rtol=1e-11)
