"""Small, self-contained launches of the hot kernels on synthetic inputs, for profilers.

    python -m tnalg_gb300.profile_case qr_mixed 1024 512 [--reps 5]
    python -m tnalg_gb300.profile_case matvec 512 2 512 [--reps 5]

qr_mixed: tn_qr_mixed of an m x n matrix with columns graded over eight decades (the gauge move of
a chi = n site with m = d * chi rows). matvec: tn_matvec of the split-TF32 effective Hamiltonian of a
(chil, d, chir) site with dense symmetric left/right blocks (the nearest-neighbour chain form).
Each case runs `reps` times after one untimed call and prints the mean time per call from CUDA
events on the launching stream.
"""
import argparse
import ctypes

import torch

from . import _lib as L


def _rand(*shape, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(*shape, generator=g, dtype=torch.float64).cuda()


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def qr_mixed(m, n, reps):
    lib = L.load()
    k = min(m, n)
    # random columns graded over eight decades (no torch.linalg: it may not load under profilers)
    A = _rand(m, n, seed=1) * torch.logspace(0, -8, n, dtype=torch.float64, device="cuda")
    Q = torch.empty((m, k), dtype=torch.float64, device="cuda")
    R = torch.empty((k, n), dtype=torch.float64, device="cuda")
    ws = L.Workspace(torch.device("cuda"))
    wp, wb = ws.args(lib.tn_qr_mixed_workspace_bytes(m, n))

    def call():
        L.check(lib.tn_qr_mixed(m, n, L.ptr(A), n, 1, L.ptr(Q), k, 1, L.ptr(R), n, 1, wp, wb, L.stream_handle()),
                "qr_mixed")

    ms = _time(call, reps)
    L.check(lib.tn_check_device_status(L.stream_handle()))
    return "tn_qr_mixed %d x %d: %.3f ms per call" % (m, n, ms)


def matvec(cl, d, cr, reps):
    lib = L.load()
    prec = L.PREC_TF32X3 if L.tf32x3_available() else L.PREC_FP64
    wl = _rand(cl * d, cl * d, seed=3)
    wl = wl + wl.T
    wr = _rand(d * cr, d * cr, seed=4)
    wr = wr + wr.T
    desc = L.SiteDesc(cl, d, cr, wl.data_ptr(), wr.data_ptr(), 0, None, None)
    psi = _rand(cl * d * cr, seed=5)
    y = torch.empty_like(psi)
    ws = L.Workspace(torch.device("cuda"))
    wp, wb = ws.args(lib.tn_matvec_workspace_bytes(ctypes.byref(desc), prec))

    def call():
        L.check(lib.tn_matvec(ctypes.byref(desc), L.ptr(psi), L.ptr(y), -1e-4, 1.0, prec, wp, wb,
                              L.stream_handle()), "matvec")

    ms = _time(call, reps)
    L.check(lib.tn_check_device_status(L.stream_handle()))
    return "tn_matvec (%d, %d, %d), precision %d: %.3f ms per call" % (cl, d, cr, prec, ms)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("case", choices=["qr_mixed", "matvec"])
    ap.add_argument("dims", type=int, nargs="+")
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    if a.case == "qr_mixed":
        print(qr_mixed(a.dims[0], a.dims[1], a.reps))
    else:
        print(matvec(a.dims[0], a.dims[1], a.dims[2], a.reps))


if __name__ == "__main__":
    main()
