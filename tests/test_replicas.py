"""Multi-GPU bench path (replicas only): each rank solves its own copy and
the whole-job rate uses the slowest rank's time.  Two gloo ranks on CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        out[rank] = (ms, bench.replica_rate(1000, 20, ms, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_time_with_the_slowest_rank():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    # 2 ranks x 1000 cells x 20 steps in 15 ms
    assert abs(res[0][1] - 2 * 1000 * 20 / 0.015 / 1e6) < 1e-12


def test_single_rank_is_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.replica_rate(100, 10, 1.0, 1) == 1.0
