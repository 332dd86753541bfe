"""The N > 1 path of bench.py on CPU: replicas only (one independent DMRG job per rank), timed by the
slowest rank. Two gloo ranks on 127.0.0.1 check the max-over-ranks reduction and the whole-job
throughput, and run one small sweep each through the host orchestration (test double of the C
ABI) to show that ranks share nothing on the data path."""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, HERE)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import fake_lib
        from tnalg_gb300 import DMRG_anyH, Parameters as pm
        fake_lib.install()
        # each rank: its own small job with its own seed (a replica), no collective on the data path
        para = pm.generate_parameters_dmrg("chain")
        para.update(l=8, chi=4, sweep_time=2, dt_ob=1, device="cpu")
        para = pm.make_consistent_parameter_dmrg(para)
        np.random.seed(100 + rank)
        import contextlib, io
        with contextlib.redirect_stdout(io.StringIO()):
            ob, _, _, _ = DMRG_anyH.dmrg_finite_size(para)
        dist.barrier()
        ms = 100.0 + 50.0 * rank  # rank 1 is the slow replica
        mx = bench.max_over_ranks(ms, world, "cpu")
        out[rank] = (mx, bench.replica_throughput(world, 2, mx), float(ob["e_per_site"]))
    finally:
        dist.destroy_process_group()


def test_two_replicas_max_over_ranks_and_throughput():
    world = 2
    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    assert sorted(out.keys()) == [0, 1]
    for r in range(world):
        mx, thr, e = out[r]
        assert mx == 150.0  # both ranks see the slowest rank's time
        assert thr == pytest.approx(world * 2 / 0.150)
        assert np.isfinite(e) and e < -0.3  # each replica ran its own DMRG
