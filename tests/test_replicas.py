"""Multi-process replica aggregation on CPU (gloo, world size 2): every rank
runs its own circuit with the CPU baseline and the job's rate is all ranks'
updates over the slowest rank's time -- the same aggregation bench.py uses
across GPUs."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import sys

    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import ckt_oracle as O

    from legionorigins_gb300 import replicas

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    p = O.GenParams(4, 16, 64, 90, 100 + rank, L_offset=0.001)
    c = O.generate(p)
    secs = O.baseline_run(c, 1, 20 + 20 * rank, threads=1)
    updates = p.W * 10 * (20 + 20 * rank)
    total, tmax, n = replicas.aggregate(updates, secs)
    out[rank] = (updates, secs, total, tmax, n)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation_gloo():
    world, port = 2, _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True,
                       start_method="spawn")
    (u0, s0, t0, m0, n0), (u1, s1, t1, m1, n1) = out[0], out[1]
    assert n0 == n1 == 2
    assert t0 == t1 == pytest.approx(u0 + u1)
    assert m0 == m1 == pytest.approx(max(s0, s1))


def test_single_process_is_local():
    from legionorigins_gb300 import replicas

    assert replicas.aggregate(10.0, 2.0) == (10.0, 2.0, 1)
    assert replicas.rate(10.0, 2.0) == 5.0
