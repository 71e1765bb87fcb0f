"""The multi-rank path of bench.py on CPU: two gloo ranks (world size 2, 127.0.0.1) time their own
replica, meet at the barriers, and agree on the maximum of their times; the whole-job value counts
every rank's cells in that time (weak scaling, no collective on the data path)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        barrier, max_over_ranks = bench.rank_helpers(dist, torch.device("cpu"))
        barrier()
        seconds = [0.75, 1.5][rank]  # rank 1 is the slow one
        t = max_over_ranks(seconds)
        barrier()
        out[rank] = (t, bench.whole_job_mlups(world, 4_000_000, t))
    finally:
        dist.destroy_process_group()


def test_two_ranks_agree_on_the_slowest_time():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0][0] == out[1][0] == 1.5
    assert out[0][1] == out[1][1] == pytest.approx(2 * 4_000_000 / 1.5 / 1e6)


def test_single_rank_helpers_are_identity():
    import bench
    barrier, max_over_ranks = bench.rank_helpers(None, None)
    barrier()
    assert max_over_ranks(3.25) == 3.25
    assert bench.whole_job_mlups(1, 1e6, 0.5) == 2.0
