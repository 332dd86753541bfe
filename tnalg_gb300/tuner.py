"""Autotuner of the output tile width of the grouped split-TF32 GEMMs (batched engine).

The grouped tcgen05 kernel (csrc/grouped_gemm.cu) covers every problem of a step with 128-row
output tiles of 64 or 128 columns. Which width is faster depends on the batch: at small bond
dimension (chi = 32: the matvec products are 64 x 32 and 32 x 64) a 128-column tile wastes most of
its tensor-core work and a 64-column one doubles the tiles in flight; at chi = 128 with hundreds of
jobs the 128-column tile reads each A tile half as often. The tuner measures both widths on the
products of the batched matvec (WL . x and x . WR^T of every job, the shapes of tn_batched_lanczos)
for a grid of (chi, jobs) classes, with CUDA events over repeated grouped launches on identical
operands, and writes the winner of each class to a table. The engine picks the width of each step
from the table (the class of the batch's largest chi and its job count) and sets it for its own
thread with tn_set_grouped_tile.

    python -m tnalg_gb300.tuner [--out tnalg_gb300/tuning/grouped_tiles.json]

The committed table was measured on a GB300. The results of a step do not depend on the width beyond
rounding (the same products are summed in the same order), only its speed.
"""
import argparse
import json
import os
import time

import numpy as np

from . import _lib as L

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning", "grouped_tiles.json")
CANDIDATES = (128, 64)
CHI_CLASSES = (32, 64, 128, 256)
JOB_CLASSES = (8, 64, 512)


def chi_class(chi):
    """Smallest class >= chi (the largest class for anything above it)."""
    for c in CHI_CLASSES:
        if chi <= c:
            return c
    return CHI_CLASSES[-1]


def job_class(njobs):
    """Nearest class on a log scale."""
    return min(JOB_CLASSES, key=lambda c: abs(np.log2(max(njobs, 1)) - np.log2(c)))


def key(chi, njobs):
    return "chi%d_jobs%d" % (chi_class(chi), job_class(njobs))


def load(path=TABLE):
    """The tuned table ({} if there is none)."""
    try:
        with open(path) as f:
            return json.load(f).get("classes", {})
    except (OSError, ValueError):
        return {}


class Choice:
    """Tile width per step from a tuned table; 0 (the library default) for classes it lacks."""

    def __init__(self, table=None):
        self.table = load() if table is None else table

    def width(self, chi_max, njobs):
        hit = self.table.get(key(chi_max, njobs))
        return int(hit["best"]) if hit else 0


def matvec_problems(chi, njobs, device, seed=0):
    """The grouped products of one batched matvec step of `njobs` sites at bond dimension chi
    (d = 2): y = WL x (chi d x chi d times chi d x chi) and y += x WR^T (chi x chi d times chi d x chi d),
    with random operands; returns (table, keep-alive tensors)."""
    import torch
    d = 2
    g = torch.Generator(device=device).manual_seed(seed)
    keep, recs = [], []
    for _ in range(njobs):
        cl = cr = chi
        WL = torch.randn(cl * d, cl * d, generator=g, dtype=torch.float64, device=device)
        WR = torch.randn(d * cr, d * cr, generator=g, dtype=torch.float64, device=device)
        x = torch.randn(cl * d * cr, generator=g, dtype=torch.float64, device=device)
        y = torch.zeros(cl * d * cr, dtype=torch.float64, device=device)
        keep += [WL, WR, x, y]
        r = np.zeros(2, dtype=L.GEMM_PROBLEM_DTYPE)
        # WL (cl d x cl d) . x (cl d x cr) -> y (cl d x cr)
        r[0]["M"], r[0]["N"], r[0]["K"], r[0]["nred"] = cl * d, cr, cl * d, 1
        r[0]["A"], r[0]["sAm"], r[0]["sAk"] = WL.data_ptr(), cl * d, 1
        r[0]["B"], r[0]["sBk"], r[0]["sBn"] = x.data_ptr(), cr, 1
        r[0]["C"], r[0]["sCm"], r[0]["sCn"] = y.data_ptr(), cr, 1
        r[0]["alpha"], r[0]["accumulate"] = 1.0, 1
        # x (cl x d cr) . WR^T (d cr x d cr) -> y (cl x d cr)
        r[1]["M"], r[1]["N"], r[1]["K"], r[1]["nred"] = cl, d * cr, d * cr, 1
        r[1]["A"], r[1]["sAm"], r[1]["sAk"] = x.data_ptr(), d * cr, 1
        r[1]["B"], r[1]["sBk"], r[1]["sBn"] = WR.data_ptr(), 1, d * cr
        r[1]["C"], r[1]["sCm"], r[1]["sCn"] = y.data_ptr(), d * cr, 1
        r[1]["alpha"], r[1]["accumulate"] = 1.0, 1
        recs.append(r)
    return np.concatenate(recs), keep


def measure(table, width, device, reps=20, warmup=3):
    """Mean ms of one grouped launch of `table` at tile `width` (CUDA events on the stream)."""
    import torch
    lib = L.load()
    L.check(lib.tn_set_grouped_tile(int(width)), "tile width")
    ws = L.Workspace(torch.device(device))
    try:
        for _ in range(warmup):
            L.grouped_gemm(table, L.PREC_TF32X3, ws=ws, device=device)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            L.grouped_gemm(table, L.PREC_TF32X3, ws=ws, device=device)
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / reps
    finally:
        lib.tn_set_grouped_tile(0)


def tune(device="cuda", chis=CHI_CLASSES, jobs=JOB_CLASSES, reps=20):
    """Measure every candidate width on every (chi, jobs) class; returns the table's classes."""
    out = {}
    for chi in chis:
        for nj in jobs:
            # keep the operands of a class within ~1 GB
            if chi * chi * nj > 128 * 128 * 512:
                continue
            table, keep = matvec_problems(chi, nj, device)
            ms = {str(w): measure(table, w, device, reps=reps) for w in CANDIDATES}
            best = min(ms, key=ms.get)
            out[key(chi, nj)] = {"best": int(best), "ms": ms}
            del keep
    return out


def main(argv=None):
    import torch
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--device", default="cuda")
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args(argv)
    L.load()
    if not L.tf32x3_available():
        raise SystemExit("the split-TF32 grouped GEMM needs an sm_103 device")
    t0 = time.time()
    classes = tune(a.device, reps=a.reps)
    doc = {"kernel": "gg_tf32x3_kernel (grouped split-TF32 GEMM, tcgen05)",
           "device": torch.cuda.get_device_name(torch.device(a.device)),
           "workload": "batched matvec products WL.x and x.WR^T of `jobs` sites at bond chi, d = 2",
           "measure": "mean of %d grouped launches after 3 warm-up launches, CUDA events" % a.reps,
           "tuning_s": round(time.time() - t0, 1), "classes": classes}
    os.makedirs(os.path.dirname(a.out), exist_ok=True)
    with open(a.out, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
    print(json.dumps(doc))


if __name__ == "__main__":
    main()
