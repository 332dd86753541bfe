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


def test_batched_qr_mixed_orthonormal_and_spanning(cuda_lib):
    """Many matrices of uneven shapes (2 x 2 up to 256 x 128 = the shared-memory limit, a transposed
    view, rank-deficient ones, widely scaled entries) in one call: Q^T Q = I to 1e-12, Q R = A to
    FP32 accuracy, R upper triangular, span(Q) = col(A)."""
    if not L.tf32x3_available():
        pytest.skip("needs an sm_103 device")
    lib = L.load()
    shapes = [(2, 2, 1.0), (8, 4, 1e-30), (64, 32, 1.0), (128, 64, 1e5), (256, 128, 1.0), (200, 100, 1.0),
              (96, 96, 1.0), (128, 128, 1.0)]
    keep, items, refs = [], [], []
    for i, (m, n, scale) in enumerate(shapes):
        A = _rand(m, n, seed=700 + i) * scale
        if i == 5:
            A[:, 50:] = A[:, :50] @ _rand(50, 50, seed=9)   # rank 50 of 100
        if i == 7:
            # columns 1e-21 below the rest: their FP32 squares are subnormal (no reflector from them)
            A[:, 32:] = A[:, :32] @ _rand(32, 96, seed=10) + 1e-21 * _rand(128, 96, seed=11)
        R = torch.zeros(n, n, dtype=torch.float64, device="cuda")
        keep += [A, R]
        refs.append(A.clone())
        items.append(_qr_item(A, m, n, (n, 1), R))
    At = _rand(48, 72, seed=800)          # A = At^T (72 x 48) read through strides; Q written back the same way
    Rt = torch.zeros(48, 48, dtype=torch.float64, device="cuda")
    keep += [At, Rt]
    refs.append(At.T.clone())
    items.append(_qr_item(At, 72, 48, (1, 72), Rt, flat=True))
    tab = np.concatenate(items)
    tp = ctypes_ptr_np(tab)
    ws = torch.empty(lib.tn_batched_qr_mixed_workspace_bytes(tp, len(items)) + 4096, dtype=torch.uint8,
                     device="cuda")
    L.check(lib.tn_batched_qr_mixed(tp, len(items), ws.data_ptr(), ws.numel(), L.stream_handle()))
    L.check(lib.tn_check_device_status(L.stream_handle()))
    torch.cuda.synchronize()
    for i, A0 in enumerate(refs):
        if i < len(shapes):
            Q, R = keep[2 * i], keep[2 * i + 1]
        else:
            Q, R = At.T, Rt
        m, n = A0.shape
        eye = torch.eye(n, dtype=torch.float64, device="cuda")
        assert torch.max(torch.abs(Q.T @ Q - eye)).item() < 1e-12, i
        scale = torch.max(torch.abs(A0)).item()
        assert torch.max(torch.abs(Q @ R - A0)).item() < 2e-6 * scale * np.sqrt(n), i
        assert torch.max(torch.abs(torch.tril(R, -1))).item() == 0.0
        # the part of A outside span(Q) is at FP32 level
        resid = A0 - Q @ (Q.T @ A0)
        assert torch.max(torch.abs(resid)).item() < 2e-6 * scale * np.sqrt(n), i


def _qr_item(A, m, n, sA, R, flat=False):
    r = np.zeros(1, dtype=L.QR_ITEM_DTYPE)
    r["m"], r["n"], r["a"], r["sAm"], r["sAn"] = m, n, A.data_ptr(), sA[0], sA[1]
    r["r"], r["sRm"], r["sRn"] = R.data_ptr(), n, 1
    return r


def ctypes_ptr_np(tab):
    import ctypes
    return ctypes.c_void_p(tab.ctypes.data)


def test_grouped_ops_match_the_single_kernels(cuda_lib):
    """Block assembly (both sides, strided environment stacks), slot combination and site
    operators of several jobs in one tn_grouped_ops launch, against tn_assemble_block /
    tn_combine_slots / tn_apply_site_ops one call at a time."""
    lib = L.load()
    d = 2
    ops = _rand(5, d, d, seed=1)
    terms = [(0, -1, 1.0), (1, 2, 0.5), (-1, 3, -0.25), (2, 1, 2.0)]
    tt, nt = L.terms_tensor(terms, torch.device("cuda"))
    gterms = [(1, 0, 1.0), (2, 0, -0.5), (0, 1, 3.0)]
    gt, ngt = L.terms_tensor(gterms, torch.device("cuda"))
    oi = torch.tensor([2, -1, 4], dtype=torch.int32, device="cuda")
    keep, items, checks = [], [], []
    for i, chi in enumerate([3, 16, 40]):
        env = _rand(3, chi, chi, seed=10 + i)
        for side in (0, 1):
            w = torch.empty((chi * d) ** 2, dtype=torch.float64, device="cuda")
            ref = torch.empty_like(w)
            L.check(lib.tn_assemble_block(side, chi, d, L.ptr(env), L.ptr(ops), L.ptr(tt), nt, L.ptr(ref),
                                          L.stream_handle()))
            items.append(_bop(side, chi, d, env, w, (chi * d) ** 2, terms=tt, nterms=nt, ops=ops, s_slot=chi * chi,
                              s_row=chi))
            keep += [w, ref]
            checks.append((w, ref))
        g = torch.empty(2, chi * chi, dtype=torch.float64, device="cuda")
        gref = torch.empty_like(g)
        L.check(lib.tn_combine_slots(chi, L.ptr(env), L.ptr(gt), ngt, 2, L.ptr(gref), L.stream_handle()))
        items.append(_bop(L.BOP_COMBINE, chi, d, env, g, 2 * chi * chi, terms=gt, nterms=ngt, s_slot=chi * chi,
                          s_row=chi, out_stride=chi * chi))
        checks.append((g, gref))
        x = _rand(chi, d, chi + 1, seed=20 + i)
        o = torch.empty(3, chi * d * (chi + 1), dtype=torch.float64, device="cuda")
        oref = torch.empty_like(o)
        L.check(lib.tn_apply_site_ops(chi, d, chi + 1, L.ptr(x), L.ptr(ops), L.ptr(oi), 3, L.ptr(oref),
                                      chi * d * (chi + 1), L.stream_handle()))
        items.append(_bop(L.BOP_SITE_OPS, chi, d, x, o, 3 * chi * d * (chi + 1), terms=oi, nterms=3, ops=ops,
                          chir=chi + 1, out_stride=chi * d * (chi + 1)))
        checks.append((o, oref))
        keep += [env, g, gref, x, o, oref]
    tab = np.concatenate(items)
    ws = torch.empty(lib.tn_grouped_ops_workspace_bytes(len(items)), dtype=torch.uint8, device="cuda")
    L.check(lib.tn_grouped_ops(ctypes_ptr_np(tab), len(items), ws.data_ptr(), ws.numel(), L.stream_handle()))
    torch.cuda.synchronize()
    for out, ref in checks:
        assert torch.max(torch.abs(out - ref)).item() < 1e-13


def _bop(kind, chi, d, src, out, total, terms=None, nterms=0, ops=None, s_slot=0, s_row=0, chir=0, out_stride=0):
    r = np.zeros(1, dtype=L.BATCH_OP_DTYPE)
    r["kind"], r["chi"], r["d"], r["chir"], r["nterms"] = kind, chi, d, chir, nterms
    r["src"], r["s_slot"], r["s_row"] = src.data_ptr(), s_slot, s_row
    r["ops"] = ops.data_ptr() if ops is not None else 0
    r["terms"] = terms.data_ptr() if terms is not None else 0
    r["out"], r["out_stride"], r["total"] = out.data_ptr(), out_stride, total
    return r


@pytest.mark.parametrize("precision", [L.PREC_FP64, L.PREC_TF32X3])
def test_grouped_gemm_batch_dimension(cuda_lib, precision):
    """batch > 1: C_z = A_z B_z at strides, with A shared by every z (stride 0) as in the closing
    contractions of an environment update."""
    if precision == L.PREC_TF32X3 and not L.tf32x3_available():
        pytest.skip("tf32x3 needs an sm_103 device")
    Z, M, N, K = 4, 72, 72, 144
    A = _rand(K, M, seed=1)          # used as A^T (strides (1, M))
    B = _rand(Z, K, N, seed=2)
    C = torch.zeros(Z, M, N, dtype=torch.float64, device="cuda")
    rec = _problem(A, B, C, M, N, K, (1, M), (N, 1), (N, 1))
    rec["batch"], rec["sAb"], rec["sBb"], rec["sCb"] = Z, 0, K * N, M * N
    L.grouped_gemm(np.array([rec], dtype=L.GEMM_PROBLEM_DTYPE), precision=precision)
    torch.cuda.synchronize()
    ref = torch.einsum("km,zkn->zmn", A, B)
    err = torch.max(torch.abs(C - ref)).item() / torch.max(torch.abs(ref)).item()
    assert err < (1e-13 if precision == L.PREC_FP64 else 5e-6), err


def test_grouped_engine_matches_the_per_job_engine(cuda_lib):
    """The batched engine's grouped path (job arenas, grouped launches, batched QR) against its
    per-job path on the same uneven jobs (XXZ chains and a ladder), split TF32: energies per site
    within 1e-8 (each path's trajectory carries its own split-TF32 rounding)."""
    if not L.tf32x3_available():
        pytest.skip("tf32x3 needs an sm_103 device")
    from tnalg_gb300 import batched, serving

    def jobs():
        out = []
        for k, (l, chi, jz, hz) in enumerate([(12, 16, 1.0, 0.0), (20, 32, 0.5, 0.3), (16, 64, 1.5, 0.1)]):
            out.append(batched.BatchJob(k, serving.chain_job_para(l, chi, jz=jz, hz=hz, sweeps=4), seed=50 + k))
        out.append(batched.BatchJob(3, serving.ladder_job_para(6, 32, j_rung=1.2, sweeps=4), seed=60))
        return out
    res = {}
    for grouped in (False, True):
        eng = batched.BatchEngine("cuda", "tf32x3", grouped=grouped)
        for j in jobs():
            eng.submit(j)
        res[grouped] = {j.job_id: j.result for j in eng.run()}
    for k in res[False]:
        assert abs(res[True][k]["e_per_site"] - res[False][k]["e_per_site"]) < 1e-8, k
        assert res[True][k]["solves"] == res[False][k]["solves"]


def test_batched_step_large_gauge_moves_side_by_side(cuda_lib):
    """Gauge moves above tn_batched_qr_mixed's shared-memory limit (chi = 256 and 512 sites, left and
    right moves, i.e. row-major and column-major layouts) in one tn_batched_step call run on side
    streams next to each other, small ones in the same call on the batched kernel: every Q and R
    equals tn_qr_mixed's on the same matrix, called alone."""
    if not L.tf32x3_available():
        pytest.skip("needs an sm_103 device")
    import ctypes
    lib = L.load()
    shapes = [(1024, 512, False), (512, 256, True), (1024, 512, True), (512, 256, False), (768, 384, False),
              (1024, 512, False), (512, 256, False), (1000, 500, True), (512, 512, False), (64, 32, False)]
    items, keep, ref = [], [], []
    for i, (m, n, colmajor) in enumerate(shapes):
        A = _rand(m, n, seed=900 + i) * (10.0 ** (i % 4 - 2))
        if i == 2:
            A[:, n // 4:] = A[:, :n // 4] @ _rand(n // 4, n - n // 4, seed=13)   # rank n/4 (a grown bond)
        store = A.T.contiguous() if colmajor else A.clone()   # column-major A: element (r, c) at store[c, r]
        sA = (1, m) if colmajor else (n, 1)
        R = torch.zeros(n, n, dtype=torch.float64, device="cuda")
        keep += [store, R]
        # the same move alone through tn_qr_mixed
        Qr = torch.empty_like(store)
        Rr = torch.zeros(n, n, dtype=torch.float64, device="cuda")
        ws = L.Workspace(torch.device("cuda"))
        wp, wb = ws.args(lib.tn_qr_mixed_workspace_bytes(m, n))
        L.check(lib.tn_qr_mixed(m, n, L.ptr(store), sA[0], sA[1], L.ptr(Qr), sA[0], sA[1], L.ptr(Rr), n, 1, wp, wb,
                                L.stream_handle()))
        ref.append((Qr, Rr, ws))
        r = np.zeros(1, dtype=L.QR_ITEM_DTYPE)
        r["m"], r["n"], r["a"], r["sAm"], r["sAn"] = m, n, store.data_ptr(), sA[0], sA[1]
        r["r"], r["sRm"], r["sRn"] = R.data_ptr(), n, 1
        items.append(r)
    torch.cuda.synchronize()
    tab = np.concatenate(items)
    d = L.BatchStepDesc()
    d.qr = tab.ctypes.data
    d.n_qr = len(items)
    d.precision = L.PREC_TF32X3
    opts = L.LanczosOpts(1e-12, 1e-4, 0.0, 2e-6, 24, 1, 3, L.PREC_TF32X3, 0, 0)
    need = lib.tn_batched_step_workspace_bytes(ctypes.byref(d), ctypes.byref(opts))
    wsb = L.Workspace(torch.device("cuda"))
    wp, wb = wsb.args(need)
    L.check(lib.tn_batched_step(ctypes.byref(d), ctypes.byref(opts), wp, wb, None, L.stream_handle()))
    L.check(lib.tn_check_device_status(L.stream_handle()))
    torch.cuda.synchronize()
    for i, (m, n, colmajor) in enumerate(shapes):
        store, R = keep[2 * i], keep[2 * i + 1]
        Qr, Rr, _ = ref[i]
        if m * n > 32768:
            # the same kernels on the same input: the same results
            assert torch.max(torch.abs(store - Qr)).item() <= 1e-14, i
            assert torch.max(torch.abs(R - Rr)).item() <= 1e-14 * max(1.0, torch.max(torch.abs(Rr)).item()), i
        Q = store.T if colmajor else store
        eye = torch.eye(n, dtype=torch.float64, device="cuda")
        assert torch.max(torch.abs(Q.T @ Q - eye)).item() < 1e-11, i
