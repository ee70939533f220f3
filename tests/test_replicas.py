"""bench.py --gpus N runs N independent replicas ("replicas only": the path
has no exchange step): the slowest rank's time over the ranks, whole-job
throughput, and the reference arm run by rank 0 alone.  Two gloo ranks on the
CPU, rendezvous on 127.0.0.1."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (world, rank, rank)
        # each rank timed its own replica; every rank must report the slowest
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
        value = bench.replica_throughput(world, 1_000_000 * 20, ms)
        # the reference arm: rank 0 alone does the work, the others return
        ran = None
        if rank != 0:
            ran = bench.run_reference_arm(None)
        dist.barrier()
        out[rank] = (ms, value, ran)
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for rank in (0, 1):
        ms, value, ran = res[rank]
        assert ms == 15.0  # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 20_000_000 / 15e-3)
    assert res[1][2] is None  # rank 1 returned from the reference arm without work


def test_single_rank_is_the_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replica_throughput(1, 1e6, 1000.0) == 1e6
