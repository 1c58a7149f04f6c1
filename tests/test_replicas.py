"""Replica mode of the benchmark.  The hot path does not shard: with N GPUs,
bench.py runs N independent replicas, one process per GPU, and only the
timing is shared.  Two gloo ranks on CPU check that host logic: every rank
learns the slowest rank's time, and the whole-job rate counts every
replica's rows over that time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out_dir):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(torch, times[rank], torch.device("cpu"))
        with open(os.path.join(out_dir, "rank%d" % rank), "w") as f:
            f.write(repr(ms))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("times", [(3.5, 7.25), (9.0, 1.0), (2.0, 2.0)])
def test_slowest_rank_time_on_every_rank(times, tmp_path):
    import torch.multiprocessing as mp
    world = len(times)
    mp.start_processes(_rank, args=(world, _free_port(), times, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    got = [float((tmp_path / ("rank%d" % r)).read_text()) for r in range(world)]
    assert got == [max(times)] * world


def test_whole_job_rate_counts_every_replica():
    sys.path.insert(0, ROOT)
    import bench
    rows = bench.N_FACT + bench.N_DIM
    one = bench.whole_job_rate(rows, 1, 2.0)
    assert one == rows / 2.0e-3
    # two replicas, the slower at 2.5 ms: twice the rows over the slower time
    assert bench.whole_job_rate(rows, 2, 2.5) == 2 * rows / 2.5e-3

