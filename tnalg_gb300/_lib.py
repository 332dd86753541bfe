"""ctypes binding of libtnalg_gb300.so (the C ABI declared in include/tnalg_gb300.h).

The product path has no CPU fallback: every call requires CUDA FP64 tensors and
raises if the library is missing or a call fails.
"""
import ctypes
import os

import numpy as np
import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtnalg_gb300.so")

TN_OK, TN_ERR_ARG, TN_ERR_CUDA, TN_ERR_WORKSPACE, TN_ERR_NOCONV, TN_ERR_NUMERIC, TN_ERR_TIMEOUT = range(7)
PREC_FP64, PREC_TF32X3 = 0, 1
PRECISIONS = {"fp64": PREC_FP64, "tf32x3": PREC_TF32X3, "3xtf32": PREC_TF32X3, "mixed": PREC_TF32X3}

c_i64 = ctypes.c_int64
c_dbl = ctypes.c_double
c_vp = ctypes.c_void_p
c_int = ctypes.c_int
c_sz = ctypes.c_size_t


class TnError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("tnalg_gb300 error %d: %s" % (status, msg))
        self.status = status


class BlockTerm(ctypes.Structure):
    _fields_ = [("slot", ctypes.c_int32), ("op", ctypes.c_int32), ("coeff", ctypes.c_double)]


class SiteDesc(ctypes.Structure):
    _fields_ = [("chil", c_i64), ("d", c_i64), ("chir", c_i64), ("wl", c_vp), ("wr", c_vp),
                ("nstr", c_i64), ("sl", c_vp), ("sr", c_vp)]


class LanczosOpts(ctypes.Structure):
    _fields_ = [("eigs_tol", c_dbl), ("tau", c_dbl), ("tol_cap", c_dbl), ("mixed_floor", c_dbl),
                ("max_krylov", ctypes.c_int32), ("max_restarts", ctypes.c_int32), ("check_every", ctypes.c_int32),
                ("precision", ctypes.c_int32), ("refine", ctypes.c_int32), ("refine_cycles", ctypes.c_int32)]


class BatchSolve(ctypes.Structure):
    _fields_ = [("site", SiteDesc), ("psi_in", c_vp), ("psi_out", c_vp)]


class BatchStepDesc(ctypes.Structure):
    """tn_batch_step_desc: the phase tables of one local update of many jobs (HOST arrays)."""
    _fields_ = [("ops1", c_vp), ("qr", c_vp), ("gemm1", c_vp), ("ops2", c_vp), ("gemm2", c_vp), ("ops3", c_vp),
                ("solves", c_vp), ("n_ops1", ctypes.c_int32), ("n_qr", ctypes.c_int32), ("n_gemm1", ctypes.c_int32),
                ("n_ops2", ctypes.c_int32), ("n_gemm2", ctypes.c_int32), ("n_ops3", ctypes.c_int32),
                ("n_solves", ctypes.c_int32), ("precision", ctypes.c_int32)]


STEP_PHASES = ("ops1", "qr", "gemm1", "ops2", "gemm2", "ops3")


class BatchOp(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("chi", ctypes.c_int32), ("d", ctypes.c_int32), ("chir", ctypes.c_int32),
                ("nterms", ctypes.c_int32), ("reserved", ctypes.c_int32), ("src", c_vp), ("s_slot", c_i64),
                ("s_row", c_i64), ("ops", c_vp), ("terms", c_vp), ("out", c_vp), ("out_stride", c_i64),
                ("total", c_i64), ("active", c_vp)]


class QrItem(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int32), ("n", ctypes.c_int32), ("a", c_vp), ("sAm", c_i64), ("sAn", c_i64),
                ("r", c_vp), ("sRm", c_i64), ("sRn", c_i64), ("active", c_vp)]


BOP_BLOCK_LEFT, BOP_BLOCK_RIGHT, BOP_COMBINE, BOP_SITE_OPS = range(4)
BATCH_SOLVE_DTYPE = np.dtype([("chil", "<i8"), ("d", "<i8"), ("chir", "<i8"), ("wl", "<u8"), ("wr", "<u8"),
                              ("nstr", "<i8"), ("sl", "<u8"), ("sr", "<u8"), ("psi_in", "<u8"), ("psi_out", "<u8")],
                             align=True)
BATCH_OP_DTYPE = np.dtype([("kind", "<i4"), ("chi", "<i4"), ("d", "<i4"), ("chir", "<i4"), ("nterms", "<i4"),
                           ("reserved", "<i4"), ("src", "<u8"), ("s_slot", "<i8"), ("s_row", "<i8"), ("ops", "<u8"),
                           ("terms", "<u8"), ("out", "<u8"), ("out_stride", "<i8"), ("total", "<i8"),
                           ("active", "<u8")], align=True)
QR_ITEM_DTYPE = np.dtype([("m", "<i4"), ("n", "<i4"), ("a", "<u8"), ("sAm", "<i8"), ("sAn", "<i8"), ("r", "<u8"),
                          ("sRm", "<i8"), ("sRn", "<i8"), ("active", "<u8")], align=True)
assert BATCH_OP_DTYPE.itemsize == ctypes.sizeof(BatchOp) and QR_ITEM_DTYPE.itemsize == ctypes.sizeof(QrItem)
assert BATCH_SOLVE_DTYPE.itemsize == ctypes.sizeof(BatchSolve)


class SvItem(ctypes.Structure):
    _fields_ = [("k", c_i64), ("n", c_i64), ("x", c_vp), ("sXr", c_i64), ("sXc", c_i64), ("s_out", c_vp)]


class GroupedGemmProblem(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int32), ("N", ctypes.c_int32), ("K", ctypes.c_int32), ("nred", ctypes.c_int32),
                ("A", c_vp), ("sAm", c_i64), ("sAk", c_i64), ("sAr", c_i64),
                ("B", c_vp), ("sBk", c_i64), ("sBn", c_i64), ("sBr", c_i64),
                ("C", c_vp), ("sCm", c_i64), ("sCn", c_i64),
                ("alpha", c_dbl), ("beta", c_dbl), ("accumulate", ctypes.c_int32), ("batch", ctypes.c_int32),
                ("sAb", c_i64), ("sBb", c_i64), ("sCb", c_i64), ("active", c_vp)]


# the same record as a numpy dtype (C layout), for tables built with array operations
GEMM_PROBLEM_DTYPE = np.dtype([("M", "<i4"), ("N", "<i4"), ("K", "<i4"), ("nred", "<i4"),
                               ("A", "<u8"), ("sAm", "<i8"), ("sAk", "<i8"), ("sAr", "<i8"),
                               ("B", "<u8"), ("sBk", "<i8"), ("sBn", "<i8"), ("sBr", "<i8"),
                               ("C", "<u8"), ("sCm", "<i8"), ("sCn", "<i8"),
                               ("alpha", "<f8"), ("beta", "<f8"), ("accumulate", "<i4"), ("batch", "<i4"),
                               ("sAb", "<i8"), ("sBb", "<i8"), ("sCb", "<i8"), ("active", "<u8")], align=True)
assert GEMM_PROBLEM_DTYPE.itemsize == ctypes.sizeof(GroupedGemmProblem)


class LanczosResult(ctypes.Structure):
    _fields_ = [("energy", c_dbl), ("residual", c_dbl), ("energy_fp64", c_dbl), ("matvecs", ctypes.c_int32),
                ("restarts", ctypes.c_int32), ("converged", ctypes.c_int32), ("reserved", ctypes.c_int32)]


_SIGS = {
    "tn_last_error": (ctypes.c_char_p, []),
    "tn_version": (c_int, []),
    "tn_device_info": (c_int, [c_vp, c_vp, c_vp]),
    "tn_precision_available": (c_int, [c_int]),
    "tn_launch_count": (ctypes.c_ulonglong, []),
    "tn_gemm": (c_int, [c_int, c_i64, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_i64,
                        c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_i64, c_i64, c_dbl, c_dbl, c_vp, c_sz, c_vp]),
    "tn_gemm_workspace_bytes": (c_sz, [c_int, c_i64, c_i64, c_i64, c_i64, c_i64]),
    "tn_check_device_status": (c_int, [c_vp]),
    "tn_assemble_block": (c_int, [c_int, c_i64, c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_vp]),
    "tn_combine_slots": (c_int, [c_i64, c_vp, c_vp, c_i64, c_i64, c_vp, c_vp]),
    "tn_apply_site_ops": (c_int, [c_i64, c_i64, c_i64, c_vp, c_vp, c_vp, c_i64, c_vp, c_i64, c_vp]),
    "tn_pair_contract": (c_int, [c_i64, c_i64, c_i64, c_vp, c_vp, c_dbl, c_vp, c_vp]),
    "tn_matvec": (c_int, [c_vp, c_vp, c_vp, c_dbl, c_dbl, c_int, c_vp, c_sz, c_vp]),
    "tn_matvec_workspace_bytes": (c_sz, [c_vp, c_int]),
    "tn_lanczos": (c_int, [c_vp, c_vp, c_vp, c_vp, c_sz, c_vp, c_vp]),
    "tn_lanczos_workspace_bytes": (c_sz, [c_vp, c_vp]),
    "tn_qr": (c_int, [c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_sz, c_vp]),
    "tn_qr_workspace_bytes": (c_sz, [c_i64, c_i64]),
    "tn_qr_use_graphs": (c_int, [c_int]),
    "tn_qr_mixed": (c_int, [c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_sz,
                            c_vp]),
    "tn_qr_mixed_workspace_bytes": (c_sz, [c_i64, c_i64]),
    "tn_singular_values": (c_int, [c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_dbl, c_int, c_vp, c_sz, c_vp]),
    "tn_singular_values_workspace_bytes": (c_sz, [c_i64, c_i64]),
    "tn_singular_values_noalloc": (c_int, [c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_dbl, c_int, c_vp]),
    "tn_svd_jacobi": (c_int, [c_i64, c_i64, c_vp, c_i64, c_i64, c_vp, c_vp, c_i64, c_vp, c_i64, c_dbl, c_int, c_vp,
                              c_sz, c_vp]),
    "tn_svd_jacobi_workspace_bytes": (c_sz, [c_i64, c_i64]),
    "tn_selftest_wait_timeout": (c_int, [c_vp, c_sz, c_vp]),
    "tn_set_grouped_tile": (c_int, [c_int]),
    "tn_get_grouped_tile": (c_int, []),
    "tn_singular_values_batched": (c_int, [c_int, c_vp, c_dbl, c_int, c_vp, c_sz, c_vp]),
    "tn_singular_values_batched_workspace_bytes": (c_sz, [c_int, c_vp]),
    "tn_grouped_gemm": (c_int, [c_int, c_vp, c_int, c_vp, c_sz, c_vp]),
    "tn_grouped_gemm_workspace_bytes": (c_sz, [c_int, c_vp, c_int]),
    "tn_grouped_ops": (c_int, [c_vp, c_int, c_vp, c_sz, c_vp]),
    "tn_grouped_ops_workspace_bytes": (c_sz, [c_int]),
    "tn_batched_qr_mixed": (c_int, [c_vp, c_int, c_vp, c_sz, c_vp]),
    "tn_batched_qr_mixed_workspace_bytes": (c_sz, [c_vp, c_int]),
    "tn_batched_lanczos": (c_int, [c_vp, c_int, c_vp, c_vp, c_sz, c_vp, c_vp]),
    "tn_batched_lanczos_workspace_bytes": (c_sz, [c_vp, c_int, c_vp]),
    "tn_batched_step": (c_int, [c_vp, c_vp, c_vp, c_sz, c_vp, c_vp]),
    "tn_batched_step_workspace_bytes": (c_sz, [c_vp, c_vp]),
    "tn_profile_enable": (c_int, [c_int]),
    "tn_profile_reset": (c_int, []),
    "tn_profile_read": (c_int, [c_int, c_vp, c_vp, c_vp]),
    "tn_dot": (c_int, [c_i64, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "tn_scale": (c_int, [c_i64, c_vp, c_dbl, c_vp, c_vp]),
    "tn_set_identity": (c_int, [c_i64, c_vp, c_i64, c_vp]),
}

_lib = None
_host_test = False


def install_test_backend(fake):
    """Tests only: route calls to `fake` (an object with the tn_* functions) and accept CPU
    tensors. Never called by the library itself."""
    global _lib, _host_test
    _lib = fake
    _host_test = fake is not None


def load(path=None):
    """Load the library (once). Raises if it is missing: there is no fallback."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError("libtnalg_gb300.so not found at %s; run tnalg_gb300.build.build() first" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    # TNALG_QR_GRAPHS=0 launches the QR kernels one by one instead of replaying captured CUDA
    # graphs (same kernels; for per-kernel profilers and launch lists).
    if os.environ.get("TNALG_QR_GRAPHS", "1") == "0":
        lib.tn_qr_use_graphs(0)
    _lib = lib
    return lib


def exported_symbols():
    return sorted(_SIGS)


def check(status, what=""):
    if status != TN_OK:
        msg = load().tn_last_error().decode(errors="replace")
        raise TnError(status, (what + ": " if what else "") + msg)


def ptr(t):
    if t is None:
        return None
    if not t.is_cuda and not _host_test:
        raise TypeError("tnalg_gb300 requires CUDA tensors (got %s)" % t.device)
    return c_vp(t.data_ptr())


def stream_handle():
    if _host_test:
        return c_vp(0)
    return c_vp(torch.cuda.current_stream().cuda_stream)


class Workspace:
    """Grow-only device scratch buffer owned by one MPS (or engine)."""

    def __init__(self, device):
        self.device = device
        self.buf = None

    def get(self, nbytes):
        nbytes = int(max(nbytes, 256))
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(int(nbytes * 1.25) + 256, dtype=torch.uint8, device=self.device)
        return self.buf

    def args(self, nbytes):
        b = self.get(nbytes)
        return c_vp(b.data_ptr()), c_sz(b.numel())


def gemm(A, B, C, M, N, K, sA, sB, sC, *, Cin=None, batch=1, bstrides=(0, 0, 0), nred=1, rstrides=(0, 0),
         alpha=1.0, beta=0.0, precision=PREC_FP64, ws=None):
    """C = alpha * sum_r A.B + beta * Cin over flat CUDA buffers with explicit element strides.

    sA = (sAm, sAk), sB = (sBk, sBn), sC = (sCm, sCn); tensors may be views (their data_ptr is used).
    """
    lib = load()
    if ws is not None:
        need = lib.tn_gemm_workspace_bytes(precision, M, N, K, batch, nred)
        wp, wb = ws.args(need)
    else:
        wp, wb = None, 0
    check(lib.tn_gemm(precision, M, N, K, ptr(A), sA[0], sA[1], ptr(B), sB[0], sB[1], ptr(C), sC[0], sC[1],
                      ptr(Cin) if Cin is not None else None, batch, bstrides[0], bstrides[1], bstrides[2], nred,
                      rstrides[0], rstrides[1], alpha, beta, wp, wb, stream_handle()), "gemm")


def grouped_gemm(table, precision=PREC_TF32X3, ws=None, device=None):
    """Every problem of `table` (numpy array of GEMM_PROBLEM_DTYPE records) in one grouped call."""
    lib = load()
    n = int(table.shape[0])
    if n == 0:
        return
    table = np.ascontiguousarray(table, dtype=GEMM_PROBLEM_DTYPE)
    tp = c_vp(table.ctypes.data)
    need = lib.tn_grouped_gemm_workspace_bytes(precision, tp, n)
    ws = ws or Workspace(device or torch.device("cuda"))
    wp, wb = ws.args(need)
    check(lib.tn_grouped_gemm(precision, tp, n, wp, wb, stream_handle()), "grouped gemm")


def terms_tensor(terms, device):
    """list of (slot, op, coeff) -> device buffer of tn_block_term structs (16 bytes each)."""
    n = len(terms)
    arr = (BlockTerm * max(n, 1))()
    for i, (slot, op, c) in enumerate(terms):
        arr[i].slot = int(slot)
        arr[i].op = int(op)
        arr[i].coeff = float(c)
    raw = bytes(arr)[: 16 * max(n, 1)]
    host = torch.frombuffer(bytearray(raw), dtype=torch.uint8)
    return host.to(device), n


def singular_values_batched(mats, ws=None, tol=1e-15, max_sweeps=60):
    """Singular values (descending, numpy) of a list of 2-D CUDA tensors in one batched FP64 call."""
    if not mats:
        return []
    lib = load()
    outs = [torch.empty(int(M.shape[0]), dtype=torch.float64, device=M.device) for M in mats]
    items = (SvItem * len(mats))()
    for b, (M, o) in enumerate(zip(mats, outs)):
        items[b].k, items[b].n = int(M.shape[0]), int(M.shape[1])
        items[b].x = ptr(M).value
        items[b].sXr, items[b].sXc = int(M.stride(0)), int(M.stride(1))
        items[b].s_out = ptr(o).value
    table = ctypes.cast(items, c_vp)
    need = lib.tn_singular_values_batched_workspace_bytes(len(mats), table)
    ws = ws or Workspace(mats[0].device)
    buf = ws.get(need + 256)
    base = (buf.data_ptr() + 255) // 256 * 256
    st = lib.tn_singular_values_batched(len(mats), table, tol, max_sweeps, c_vp(base),
                                        c_sz(buf.numel() - (base - buf.data_ptr())), stream_handle())
    if st == TN_ERR_NOCONV:   # values written; the last Jacobi sweep still rotated some pair
        import warnings
        warnings.warn("singular values: Jacobi not converged after %d sweeps" % max_sweeps)
    else:
        check(st, "singular values")
    return [np.sort(o.cpu().numpy())[::-1] for o in outs]


def svd_truncated(X, chi, ws=None, tol=1e-15, max_sweeps=60):
    """Truncated SVD of a 2-D CUDA tensor X (k x n): (U (k x r), s (r,), Vt (r x n)) with the r =
    min(chi, k) largest singular values in descending order, from tn_svd_jacobi."""
    lib = load()
    k, n = int(X.shape[0]), int(X.shape[1])
    s = torch.empty(k, dtype=torch.float64, device=X.device)
    U = torch.empty(k, k, dtype=torch.float64, device=X.device)
    Vt = torch.empty(k, n, dtype=torch.float64, device=X.device)
    ws = ws or Workspace(X.device)
    buf = ws.get(lib.tn_svd_jacobi_workspace_bytes(k, n) + 256)
    base = (buf.data_ptr() + 255) // 256 * 256
    st = lib.tn_svd_jacobi(k, n, ptr(X), int(X.stride(0)), int(X.stride(1)), ptr(s), ptr(U), k, ptr(Vt), n, tol,
                           max_sweeps, c_vp(base), c_sz(buf.numel() - (base - buf.data_ptr())), stream_handle())
    if st != TN_ERR_NOCONV:
        check(st, "svd")
    # the k values are ordered on the host (the call has synchronised the stream already); a device
    # sort would load torch's sorting kernels on first use, which took seconds in a fresh process
    order = np.argsort(-s.cpu().numpy(), kind="stable")[: min(int(chi), k)]
    idx = torch.as_tensor(order, dtype=torch.long, device=X.device)
    return U[:, idx], s[idx], Vt[idx]


def tf32x3_available():
    return bool(load().tn_precision_available(PREC_TF32X3))


def launch_count():
    return int(load().tn_launch_count())


def profile_read(cls=0):
    """(total ms, launches, useful flops) of a profiled kernel class."""
    lib = load()
    ms, cnt, fl = ctypes.c_double(), ctypes.c_int64(), ctypes.c_double()
    check(lib.tn_profile_read(cls, ctypes.byref(ms), ctypes.byref(cnt), ctypes.byref(fl)), "profile")
    return ms.value, cnt.value, fl.value
