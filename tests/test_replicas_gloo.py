"""N > 1 path of bench.py on the CPU: independent replicas, one per rank, combined by a
max-over-ranks reduction (gloo, world size 2).  No data-path collective exists: each rank
meshes its own molecule; only the step times are reduced."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env()[:2] == (world, rank)
        # each rank reports its own times; rank 1 is the slower one in the first value,
        # rank 0 in the second
        ms, e2e = bench.reduce_max([10.0 + 5.0 * rank, 30.0 - 4.0 * rank], world)
        value, e2e_value = bench.aggregate(world, 1e6, ms, e2e)
        out.put((rank, ms, e2e, value, e2e_value))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replica_times_are_max_over_ranks(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, e2e, value, e2e_value in res:
        assert ms == 15.0 and e2e == 30.0  # every rank sees the slowest rank's time
        assert value == pytest.approx(world * 1e6 / 15e-3)
        assert e2e_value == pytest.approx(world * 1e6 / 30e-3)


def test_single_rank_is_identity():
    assert bench.reduce_max([1.5, 2.5], 1) == [1.5, 2.5]
    assert bench.aggregate(1, 100.0, 10.0, 20.0) == pytest.approx((1e4, 5e3))
