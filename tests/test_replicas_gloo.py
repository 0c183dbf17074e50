"""The multi-GPU path of bench.py on CPU: two gloo ranks.  The workload
shards by circuit (replicas, no collective on the data path), so the only
exchange is the max-over-ranks of the timed region; whole-job throughput is
every rank's circuits over the slowest rank's time, and each rank draws its
own circuits."""
import os
import socket

import pytest

import bench
from tnqvm_gb300 import circuits


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(100.0 + 50.0 * rank, dist, "cpu")
        seeds = [None] * world
        dist.all_gather_object(seeds, bench.replica_seed(rank))
        q.put((rank, ms, bench.job_throughput(1024, world, ms), seeds))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_max_time_and_job_throughput():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value, seeds in got:
        assert ms == pytest.approx(150.0)  # the slower rank's time on both
        assert value == pytest.approx(2 * 1024 / 0.150)
        assert len(set(seeds)) == 2


def test_rank_shards_are_distinct_circuits():
    a = circuits.vqe_batch(4, seed=bench.replica_seed(0))
    b = circuits.vqe_batch(4, seed=bench.replica_seed(1))
    assert [x["circuit"] for x in a] != [x["circuit"] for x in b]
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
