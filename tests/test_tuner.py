"""The tile-width autotuner's table lookup (CPU) and the grouped GEMM at both widths (GPU)."""
import numpy as np
import pytest

from tnalg_gb300 import tuner


def test_classes_and_choice():
    assert tuner.chi_class(16) == 32 and tuner.chi_class(64) == 64 and tuner.chi_class(100) == 128
    assert tuner.chi_class(4096) == tuner.CHI_CLASSES[-1]
    assert tuner.job_class(1) == 8 and tuner.job_class(100) == 64 and tuner.job_class(5000) == 512
    table = {tuner.key(32, 512): {"best": 64, "ms": {"64": 1.0, "128": 2.0}},
             tuner.key(128, 64): {"best": 128, "ms": {"64": 3.0, "128": 2.0}}}
    c = tuner.Choice(table)
    assert c.width(32, 400) == 64
    assert c.width(120, 50) == 128
    assert c.width(256, 8) == 0          # no class: the library default


def test_committed_table_is_well_formed():
    table = tuner.load()
    for k, v in table.items():
        assert k.startswith("chi") and v["best"] in tuner.CANDIDATES
        assert v["ms"][str(v["best"])] == min(v["ms"].values())


@pytest.mark.gpu
def test_grouped_gemm_same_results_at_both_tile_widths(cuda_lib):
    """The grouped split-TF32 GEMM at 64- and 128-column tiles: the same products summed in the same
    order, so the outputs agree to rounding, and both match FP64 to split-TF32 accuracy."""
    import torch
    from tnalg_gb300 import _lib as L
    if not L.tf32x3_available():
        pytest.skip("needs an sm_103 device")
    lib = L.load()
    outs = {}
    for w in (128, 64):
        table, keep = tuner.matvec_problems(48, 5, "cuda", seed=3)
        table2, keep2 = tuner.matvec_problems(96, 3, "cuda", seed=4)
        tab = np.concatenate([table, table2])
        L.check(lib.tn_set_grouped_tile(w))
        try:
            assert lib.tn_get_grouped_tile() == w
            L.grouped_gemm(tab, L.PREC_TF32X3)
        finally:
            lib.tn_set_grouped_tile(0)
        torch.cuda.synchronize()
        outs[w] = [t.clone() for t in (keep + keep2)[3::4]]
        # FP64 reference of the first job: y = WL x + x WR^T
        WL, WR, x, y = keep[0:4]
        chi, d = 48, 2
        ref = (WL @ x.view(chi * d, chi)).view(-1) + (x.view(chi, d * chi) @ WR.T).view(-1)
        assert torch.max(torch.abs(y - ref)).item() <= 1e-5 * torch.max(torch.abs(ref)).item()
    assert lib.tn_get_grouped_tile() == 128
    for a, b in zip(outs[128], outs[64]):
        assert torch.max(torch.abs(a - b)).item() <= 1e-12 * torch.max(torch.abs(a)).item()
