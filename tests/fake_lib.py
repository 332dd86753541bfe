"""numpy test double of libtnalg_gb300's C ABI, operating on HOST pointers.

Used only by the CPU tests to exercise the host orchestration (layouts, strides,
environment bookkeeping, sweep logic) of tnalg_gb300 without a GPU. Each function
implements the documented semantics of the matching entry point in
include/tnalg_gb300.h with plain numpy; the CUDA kernels themselves are checked
on the GPU by the `gpu`-marked tests.
"""
import ctypes

import numpy as np
from scipy.sparse.linalg import LinearOperator, eigsh

OK, ERR_ARG, ERR_NOCONV = 0, 1, 4


def _addr(p):
    if p is None:
        return None
    if isinstance(p, ctypes.c_void_p):
        return p.value
    return int(p)


def _view(p, n, dtype=np.float64):
    a = _addr(p)
    if a is None or n <= 0:
        return np.zeros(0, dtype=dtype)
    ct = {np.float64: ctypes.c_double, np.int32: ctypes.c_int32}[dtype]
    return np.ctypeslib.as_array((ct * int(n)).from_address(a))


def _struct(ref):
    return ref._obj if hasattr(ref, "_obj") else ref


def _extent(*pairs):
    return 1 + sum((int(n) - 1) * abs(int(s)) for n, s in pairs if n > 0)


def _strided(p, shape, strides):
    n = _extent(*zip(shape, strides))
    base = _view(p, n)
    return np.lib.stride_tricks.as_strided(base, shape=shape, strides=[8 * s for s in strides])


def _terms(p, n):
    raw = _view(p, 2 * n) if n else np.zeros(0)
    out = []
    for k in range(n):
        slot_op = np.frombuffer(raw[2 * k:2 * k + 1].tobytes(), dtype=np.int32)
        out.append((int(slot_op[0]), int(slot_op[1]), float(raw[2 * k + 1])))
    return out


class FakeLib:
    def __init__(self):
        self.err = b""
        self.calls = {}
        self.tile_n = 0

    def tn_set_grouped_tile(self, tile_n):
        if tile_n not in (0, 64, 128):
            return ERR_ARG
        self.tile_n = int(tile_n)
        return OK

    def tn_get_grouped_tile(self):
        return self.tile_n or 128

    def _count(self, name):
        self.calls[name] = self.calls.get(name, 0) + 1

    def tn_last_error(self):
        return self.err

    def tn_version(self):
        return 100

    # -- GEMM ----------------------------------------------------------------------
    def tn_gemm_workspace_bytes(self, prec, M, N, K, batch, nred=1):
        return 0

    def tn_check_device_status(self, stream):
        return OK

    def tn_gemm(self, prec, M, N, K, A, sAm, sAk, B, sBk, sBn, C, sCm, sCn, Cin, batch, sAb, sBb, sCb, nred, sAr,
                sBr, alpha, beta, ws, wsb, stream):
        self._count("tn_gemm")
        M, N, K = int(M), int(N), int(K)
        if M == 0 or N == 0 or batch == 0:
            return OK
        Cv = _strided(C, (batch, M, N), (sCb, sCm, sCn))
        Ci = _strided(Cin, (batch, M, N), (sCb, sCm, sCn)).copy() if _addr(Cin) else Cv.copy()
        acc = np.zeros((batch, M, N))
        if K > 0 and nred > 0:
            Av = _strided(A, (batch, nred, M, K), (sAb, sAr, sAm, sAk))
            Bv = _strided(B, (batch, nred, K, N), (sBb, sBr, sBk, sBn))
            acc = np.einsum("brmk,brkn->bmn", Av, Bv)
        res = alpha * acc + (beta * Ci if beta != 0 else 0.0)
        Cv[...] = res
        return OK

    # -- building blocks -------------------------------------------------------------
    def tn_assemble_block(self, side, chi, d, env, ops, terms, nterms, w, stream):
        self._count("tn_assemble_block")
        chi, d = int(chi), int(d)
        tl = _terms(terms, int(nterms))
        nslot = 1 + max([s for s, _, _ in tl] + [0])
        E = _view(env, nslot * chi * chi).reshape(nslot, chi, chi)
        nop = 1 + max([o for _, o, _ in tl] + [0])
        O = _view(ops, nop * d * d).reshape(nop, d, d) if nop > 0 else None
        W = np.zeros((chi * d, chi * d))
        for slot, op, c in tl:
            e = np.eye(chi) if slot < 0 else E[slot]
            o = np.eye(d) if op < 0 else O[op]
            W += c * (np.kron(e, o) if side == 0 else np.kron(o, e))
        _view(w, W.size)[:] = W.reshape(-1)
        return OK

    def tn_combine_slots(self, chi, env, terms, nterms, ngroups, out, stream):
        self._count("tn_combine_slots")
        chi = int(chi)
        tl = _terms(terms, int(nterms))
        nslot = 1 + max([s for s, _, _ in tl] + [0])
        E = _view(env, nslot * chi * chi).reshape(nslot, chi, chi)
        res = np.zeros((int(ngroups), chi, chi))
        for slot, g, c in tl:
            res[g] += c * (np.eye(chi) if slot < 0 else E[slot])
        _view(out, res.size)[:] = res.reshape(-1)
        return OK

    def tn_apply_site_ops(self, chil, d, chir, inp, ops, opidx, nout, out, out_stride, stream):
        self._count("tn_apply_site_ops")
        chil, d, chir, nout = int(chil), int(d), int(chir), int(nout)
        idx = _view(opidx, nout, np.int32)
        nop = 1 + max(int(idx.max()), 0)
        O = _view(ops, nop * d * d).reshape(nop, d, d)
        X = _view(inp, chil * d * chir).reshape(chil, d, chir)
        o = _view(out, (nout - 1) * int(out_stride) + chil * d * chir)
        for k in range(nout):
            op = np.eye(d) if idx[k] < 0 else O[idx[k]]
            o[k * out_stride:k * out_stride + chil * d * chir] = np.einsum("xs,asb->axb", op, X).reshape(-1)
        return OK

    def tn_pair_contract(self, chil, d, chir, m, t, alpha, out, stream):
        self._count("tn_pair_contract")
        chil, d, chir = int(chil), int(d), int(chir)
        Mv = _view(m, chil * d * chir).reshape(chil, d, chir)
        Tv = _view(t, chil * d * chir).reshape(chil, d, chir)
        o = _view(out, d * d)
        o += alpha * np.einsum("xpz,xsz->ps", Mv, Tv).reshape(-1)
        return OK

    # -- matvec / Lanczos -------------------------------------------------------------
    def _heff(self, ds):
        cl, d, cr = int(ds.chil), int(ds.d), int(ds.chir)
        wl = _view(ds.wl, (cl * d) ** 2).reshape(cl * d, cl * d) if ds.wl else None
        wr = _view(ds.wr, (d * cr) ** 2).reshape(d * cr, d * cr) if ds.wr else None
        ns = int(ds.nstr)
        sl = _view(ds.sl, ns * cl * cl).reshape(ns, cl, cl) if ns else None
        sr = _view(ds.sr, ns * cr * cr).reshape(ns, cr, cr) if ns else None

        def mv(x):
            x = np.asarray(x).reshape(cl, d, cr)
            y = np.zeros_like(x)
            if wl is not None:
                y += (wl @ x.reshape(cl * d, cr)).reshape(cl, d, cr)
            if wr is not None:
                y += (x.reshape(cl, d * cr) @ wr.T).reshape(cl, d, cr)
            for k in range(ns):
                y += np.einsum("xa,asb,yb->xsy", sl[k], x, sr[k])
            return y.reshape(-1)
        return mv, cl * d * cr

    def tn_matvec_workspace_bytes(self, desc, prec):
        return 0

    def tn_matvec(self, desc, psi, y, alpha, beta, prec, ws, wsb, stream):
        self._count("tn_matvec")
        mv, n = self._heff(_struct(desc))
        x = _view(psi, n).copy()
        _view(y, n)[:] = beta * x + alpha * mv(x)
        return OK

    def tn_lanczos_workspace_bytes(self, desc, opts):
        return 0

    def tn_lanczos(self, desc, psi, opts, ws, wsb, res, stream):
        self._count("tn_lanczos")
        ds, o, r = _struct(desc), _struct(opts), _struct(res)
        mv, n = self._heff(ds)
        x0 = _view(psi, n).copy()
        calls = [0]

        def f(v):
            calls[0] += 1
            return mv(v)
        if n <= 2:
            H = np.stack([mv(e) for e in np.eye(n)], axis=1)
            w, v = np.linalg.eigh(H)
            e, vec = w[0], v[:, 0]
        else:
            w, v = eigsh(LinearOperator((n, n), matvec=f, dtype=float), k=1, which="SA", v0=x0, tol=1e-13)
            e, vec = w[0], v[:, 0]
        _view(psi, n)[:] = vec / np.linalg.norm(vec)
        r.energy = float(e)
        r.energy_fp64 = float(e)
        r.residual = float(np.linalg.norm(mv(vec) - e * vec))
        r.matvecs = calls[0]
        r.restarts = 0
        r.converged = 1
        return OK

    def tn_batched_lanczos_workspace_bytes(self, jobs, count, opts):
        return 0

    def tn_batched_lanczos(self, jobs, count, opts, ws, wsb, results, stream):
        """Every job of the batch through the single-job solver above (same documented result)."""
        self._count("tn_batched_lanczos")
        from tnalg_gb300 import _lib
        arr = ctypes.cast(jobs, ctypes.POINTER(_lib.BatchSolve))
        res = ctypes.cast(results, ctypes.POINTER(_lib.LanczosResult))
        for b in range(int(count)):
            j = arr[b]
            ds = j.site
            n = int(ds.chil * ds.d * ds.chir)
            if j.psi_out != j.psi_in:
                _view(j.psi_out, n)[:] = _view(j.psi_in, n)
            st = self.tn_lanczos(ctypes.byref(ds), j.psi_out, opts, None, 0, ctypes.byref(res[b]), stream)
            if st not in (OK, ERR_NOCONV):
                return st
        return OK

    def tn_batched_step_workspace_bytes(self, desc, opts):
        return 4096

    def tn_batched_step(self, desc, opts, ws, wsb, results, stream):
        """The phases of tn_batched_step in their documented order through the functions above."""
        self._count("tn_batched_step")
        from tnalg_gb300 import _lib
        d = _struct(desc)
        if isinstance(d, ctypes.c_void_p) or isinstance(d, int):
            d = ctypes.cast(d, ctypes.POINTER(_lib.BatchStepDesc))[0]
        if d.n_ops1:
            self.tn_grouped_ops(d.ops1, d.n_ops1, ws, wsb, stream)
        if d.n_qr:
            self.tn_batched_qr_mixed(d.qr, d.n_qr, ws, wsb, stream)
        if d.n_gemm1:
            self.tn_grouped_gemm(d.precision, d.gemm1, d.n_gemm1, ws, wsb, stream)
        if d.n_ops2:
            self.tn_grouped_ops(d.ops2, d.n_ops2, ws, wsb, stream)
        if d.n_gemm2:
            self.tn_grouped_gemm(d.precision, d.gemm2, d.n_gemm2, ws, wsb, stream)
        if d.n_ops3:
            self.tn_grouped_ops(d.ops3, d.n_ops3, ws, wsb, stream)
        if d.n_solves:
            return self.tn_batched_lanczos(d.solves, d.n_solves, opts, ws, wsb, results, stream)
        return OK

    def tn_svd_jacobi_workspace_bytes(self, k, n):
        return 0

    def tn_svd_jacobi(self, k, n, x, sXr, sXc, s_out, U, ldu, Vt, ldvt, tol, sweeps, ws, wsb, stream):
        self._count("tn_svd_jacobi")
        k, n = int(k), int(n)
        X = _strided(x, (k, n), (sXr, sXc)).copy()
        u, sv, vt = np.linalg.svd(X, full_matrices=False)
        r = len(sv)
        s = np.zeros(k)
        s[:r] = sv
        _view(s_out, k)[:] = s
        if _addr(U):
            Um = np.zeros((k, k))
            Um[:, :r] = u
            _strided(U, (k, k), (int(ldu), 1))[...] = Um
        if _addr(Vt):
            Vm = np.zeros((k, n))
            Vm[:r] = vt
            _strided(Vt, (k, n), (int(ldvt), 1))[...] = Vm
        return OK

    def tn_dot(self, n, x, y, out, ws, wsb, stream):
        n = int(n)
        _view(out, 1)[0] = float(np.dot(_view(x, n), _view(y, n)))
        return OK

    def tn_scale(self, n, x, alpha, nrm2, stream):
        n = int(n)
        f = alpha / np.sqrt(_view(nrm2, 1)[0]) if _addr(nrm2) else alpha
        _view(x, n)[:] *= f
        return OK

    # -- grouped contractions ----------------------------------------------------------------
    def tn_grouped_gemm_workspace_bytes(self, prec, problems, count):
        return 0

    def tn_grouped_gemm(self, prec, problems, count, ws, wsb, stream):
        self._count("tn_grouped_gemm")
        from tnalg_gb300 import _lib
        tab = np.ctypeslib.as_array((ctypes.c_uint8 * (int(count) * _lib.GEMM_PROBLEM_DTYPE.itemsize))
                                    .from_address(_addr(problems))).view(_lib.GEMM_PROBLEM_DTYPE)
        # every product is formed before any output is written (the device stages the operands in
        # a launch of their own first, so an output may alias an operand)
        results = []
        for q in tab:
            if q["active"] and _view(int(q["active"]), 1, np.int32)[0] == 0:
                continue
            M, N, K, R = int(q["M"]), int(q["N"]), int(q["K"]), int(q["nred"])
            for z in range(max(int(q["batch"]), 1)):
                acc = np.zeros((M, N))
                for r in range(R):
                    oa = 8 * (r * int(q["sAr"]) + z * int(q["sAb"]))
                    ob = 8 * (r * int(q["sBr"]) + z * int(q["sBb"]))
                    A = _strided(int(q["A"]) + oa, (M, K), (int(q["sAm"]), int(q["sAk"])))
                    B = _strided(int(q["B"]) + ob, (K, N), (int(q["sBk"]), int(q["sBn"])))
                    acc += A @ B
                results.append((q, z, acc))
        for q, z, acc in results:
            M, N = int(q["M"]), int(q["N"])
            C = _strided(int(q["C"]) + 8 * z * int(q["sCb"]), (M, N), (int(q["sCm"]), int(q["sCn"])))
            if q["accumulate"]:
                C += q["alpha"] * acc
            else:
                C[...] = q["alpha"] * acc + (q["beta"] * C if q["beta"] != 0 else 0.0)
        return OK

    def tn_grouped_ops_workspace_bytes(self, count):
        return 0

    def tn_grouped_ops(self, items, count, ws, wsb, stream):
        self._count("tn_grouped_ops")
        from tnalg_gb300 import _lib
        arr = ctypes.cast(items, ctypes.POINTER(_lib.BatchOp))
        for i in range(int(count)):
            it = arr[i]
            if it.active and _view(it.active, 1, np.int32)[0] == 0:
                continue
            chi, d, kind = int(it.chi), int(it.d), int(it.kind)
            if kind in (0, 1, 2):
                tl = _terms(it.terms, int(it.nterms))
                nslot = 1 + max([sl for sl, _, _ in tl] + [0])
                E = _strided(it.src, (nslot, chi, chi), (int(it.s_slot), int(it.s_row), 1))
            if kind in (0, 1):
                nop = 1 + max([o for _, o, _ in tl] + [0])
                O = _view(it.ops, nop * d * d).reshape(nop, d, d)
                W = np.zeros((chi * d, chi * d))
                for slot, op, c in tl:
                    e = np.eye(chi) if slot < 0 else E[slot]
                    o = np.eye(d) if op < 0 else O[op]
                    W += c * (np.kron(e, o) if kind == 0 else np.kron(o, e))
                _view(it.out, W.size)[:] = W.reshape(-1)
            elif kind == 2:
                ng = int(it.total) // (chi * chi)
                out = _strided(it.out, (ng, chi * chi), (int(it.out_stride), 1))
                res = np.zeros((ng, chi, chi))
                for slot, g, c in tl:
                    res[g] += c * (np.eye(chi) if slot < 0 else E[slot])
                out[...] = res.reshape(ng, -1)
            else:
                chir, nout = int(it.chir), int(it.nterms)
                idx = _view(it.terms, nout, np.int32)
                nop = 1 + max(int(idx.max()), 0)
                O = _view(it.ops, nop * d * d).reshape(nop, d, d)
                X = _view(it.src, chi * d * chir).reshape(chi, d, chir)
                out = _strided(it.out, (nout, chi * d * chir), (int(it.out_stride), 1))
                for k in range(nout):
                    op = np.eye(d) if idx[k] < 0 else O[idx[k]]
                    out[k] = np.einsum("xs,asb->axb", op, X).reshape(-1)
        return OK

    def tn_batched_qr_mixed_workspace_bytes(self, items, count):
        return 0

    def tn_batched_qr_mixed(self, items, count, ws, wsb, stream):
        """numpy QR with LAPACK's sign convention (the device's FP32 Householder agrees up to its
        rounding)."""
        self._count("tn_batched_qr_mixed")
        from tnalg_gb300 import _lib
        arr = ctypes.cast(items, ctypes.POINTER(_lib.QrItem))
        for i in range(int(count)):
            it = arr[i]
            if it.active and _view(it.active, 1, np.int32)[0] == 0:
                continue
            m, n = int(it.m), int(it.n)
            A = _strided(it.a, (m, n), (int(it.sAm), int(it.sAn)))
            Q, R = np.linalg.qr(A.copy())
            A[...] = Q
            _strided(it.r, (n, n), (int(it.sRm), int(it.sRn)))[...] = R
        return OK

    # -- decompositions -------------------------------------------------------------------
    def tn_qr_workspace_bytes(self, m, n):
        return 0

    def tn_qr(self, m, n, a, sAm, sAn, q, sQm, sQn, r, sRm, sRn, ws, wsb, stream):
        self._count("tn_qr")
        m, n = int(m), int(n)
        k = min(m, n)
        A = _strided(a, (m, n), (sAm, sAn)).copy()
        Q, R = np.linalg.qr(A)
        if _addr(q):
            _strided(q, (m, k), (sQm, sQn))[...] = Q[:, :k]
        if _addr(r):
            _strided(r, (k, n), (sRm, sRn))[...] = R[:k]
        return OK

    def tn_qr_mixed_workspace_bytes(self, m, n):
        return 0

    def tn_qr_mixed(self, m, n, a, sAm, sAn, q, sQm, sQn, r, sRm, sRn, ws, wsb, stream):
        """Same contract as tn_qr (Q orthonormal, A = Q R; the device version reaches it through an FP32
        factorisation re-orthogonalised in FP64); the double uses the FP64 factorisation."""
        self._count("tn_qr_mixed")
        return self.tn_qr(m, n, a, sAm, sAn, q, sQm, sQn, r, sRm, sRn, ws, wsb, stream)

    def tn_singular_values_workspace_bytes(self, k, n):
        return 0

    def tn_singular_values(self, k, n, x, sr, sc, out, tol, sweeps, ws, wsb, stream):
        self._count("tn_singular_values")
        X = _strided(x, (int(k), int(n)), (sr, sc)).copy()
        _view(out, int(k))[:] = np.linalg.svd(X, compute_uv=False)[: int(k)]
        return OK

    def tn_singular_values_batched_workspace_bytes(self, count, items):
        return 0

    def tn_singular_values_batched(self, count, items, tol, sweeps, ws, wsb, stream):
        self._count("tn_singular_values_batched")
        arr = ctypes.cast(items, ctypes.POINTER(ItemStruct()))
        for b in range(int(count)):
            it = arr[b]
            X = _strided(it.x, (int(it.k), int(it.n)), (it.sXr, it.sXc)).copy()
            _view(it.s_out, int(it.k))[:] = np.linalg.svd(X, compute_uv=False)[: int(it.k)]
        return OK


def ItemStruct():
    from tnalg_gb300 import _lib
    return _lib.SvItem


def install():
    """Route tnalg_gb300's C-ABI calls to a fresh FakeLib (host tensors accepted)."""
    from tnalg_gb300 import _lib
    fake = FakeLib()
    _lib.install_test_backend(fake)
    return fake


def uninstall():
    from tnalg_gb300 import _lib
    _lib.install_test_backend(None)
