"""Multi-rank logic of bench.py (replicas, max-over-ranks time), run as two
gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, results):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch.distributed as dist
    import bench
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ws, r, local = bench.dist_env()
        local_ms = 100.0 + 25.0 * rank  # rank 1 is the slow one
        ms = bench.max_over_ranks(local_ms, "cpu")
        results[rank] = (ws, r, local, ms, bench.job_rate(40, ws, ms))
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_the_slowest_time():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        results = m.dict()
        mp.start_processes(_rank_main, args=(world, port, results), nprocs=world, join=True, start_method="spawn")
        res = dict(results)
    assert sorted(res) == [0, 1]
    for rank, (ws, r, local, ms, rate) in res.items():
        assert (ws, r, local) == (2, rank, rank)
        assert ms == 125.0                   # max over ranks
        assert rate == pytest.approx(2 * 40 / 0.125)  # both replicas' steps over the slowest time


def test_single_process_keeps_its_own_time():
    import bench
    assert bench.max_over_ranks(7.5, "cpu") == 7.5
    assert bench.job_rate(10, 1, 500.0) == pytest.approx(20.0)
