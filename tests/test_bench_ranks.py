"""The multi-rank path of bench.py on the CPU: two gloo ranks (127.0.0.1), as torchrun would
start them.  The path shards nothing (independent replicas), so its only host logic is the
reduction of the timings to the slowest rank and the whole-job rate; each rank reports
different timings and both must agree on the maxima."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_setup(None)
        mx = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 0.5 * rank])
        rate = bench.whole_job_rate(w, 50, mx[0])
        out[rank] = (w, r, local, mx, rate)
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest():
    world = 2
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    for rank in range(world):
        w, r, local, mx, rate = res[rank]
        assert (w, r, local) == (world, rank, rank)
        assert mx == [2.0, 10.0, 0.5]
        assert rate == pytest.approx(world * 50 / 2.0)


def test_single_process_is_the_identity():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert not torch.distributed.is_initialized()
    assert bench.max_over_ranks([3, 1.5]) == [3.0, 1.5]
    assert bench.whole_job_rate(1, 40, 2.0) == 20.0
