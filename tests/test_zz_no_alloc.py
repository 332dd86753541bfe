"""The allocation-free singular-value entry point (GPU only; collected last on purpose).

tn_singular_values_noalloc serves hosts that cannot allocate device memory: its scratch is a
static device array instead of a caller workspace. These tests call it through the C ABI and
compare it with tn_singular_values (same algorithm, caller-provided workspace) on two calls in a
row, so a second call that inherits the shared array's contents must still be right.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

from tnalg_gb300 import _lib as L  # noqa: E402


def _with_workspace(lib, x, k, n, sr, sc):
    out = torch.empty(k, dtype=torch.float64, device="cuda")
    ws = torch.empty(lib.tn_singular_values_workspace_bytes(k, n), dtype=torch.uint8, device="cuda")
    L.check(lib.tn_singular_values(k, n, L.ptr(x), sr, sc, L.ptr(out), 1e-15, 60, L.ptr(ws), ws.numel(),
                                   L.stream_handle()))
    return np.sort(out.cpu().numpy())[::-1]


def _no_alloc(lib, x, k, n, sr, sc):
    out = torch.empty(k, dtype=torch.float64, device="cuda")
    L.check(lib.tn_singular_values_noalloc(k, n, L.ptr(x), sr, sc, L.ptr(out), 1e-15, 60, L.stream_handle()))
    return np.sort(out.cpu().numpy())[::-1]


def test_noalloc_matches_workspace_version_twice(cuda_lib):
    lib = L.load()
    g = torch.Generator(device="cpu").manual_seed(123)
    cases = []
    for k, n in ((48, 40), (33, 64), (256, 256)):
        x = torch.randn(k, n, generator=g, dtype=torch.float64)
        x[:, : max(1, k // 4)] *= 1e-5  # spread the spectrum
        cases.append((x.cuda(), k, n, n, 1))
    xt = torch.randn(40, 30, generator=g, dtype=torch.float64).cuda()
    cases.append((xt, 30, 40, 1, 30))  # rows read through strides (transpose of a 40 x 30 matrix)
    for x, k, n, sr, sc in cases:
        ref = _with_workspace(lib, x, k, n, sr, sc)
        first = _no_alloc(lib, x, k, n, sr, sc)
        second = _no_alloc(lib, x, k, n, sr, sc)
        np.testing.assert_allclose(first, ref, atol=1e-13 * ref[0], rtol=1e-11)
        np.testing.assert_allclose(second, ref, atol=1e-13 * ref[0], rtol=1e-11)
        # and against LAPACK on the host: the k x n matrix the strides describe
        xh = torch.as_strided(x, (k, n), (sr, sc)).cpu().numpy()
        lapack = np.linalg.svd(xh, compute_uv=False)
        np.testing.assert_allclose(second[: lapack.size], lapack, atol=1e-13 * lapack[0], rtol=1e-10)
        if k > lapack.size:   # k > n: the surplus rows of the rotated matrix carry zero norm
            assert np.all(second[lapack.size:] <= 1e-12 * lapack[0])


def test_noalloc_rejects_sizes_beyond_the_static_scratch(cuda_lib):
    lib = L.load()
    x = torch.zeros(300, 300, dtype=torch.float64, device="cuda")
    out = torch.empty(300, dtype=torch.float64, device="cuda")
    st = lib.tn_singular_values_noalloc(300, 300, L.ptr(x), 300, 1, L.ptr(out), 1e-15, 60, L.stream_handle())
    assert st == L.TN_ERR_ARG
    assert b"static scratch" in lib.tn_last_error()
