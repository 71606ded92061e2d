"""The multi-GPU path of the benchmark on CPU: two gloo ranks shard the SNP
blocks (disjoint genotype seeds, weak scaling), exchange only the maximum of
their timings, and report all ranks' tests over the slowest rank's time."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    import torch
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seeds = bench.rank_block_seeds(rank, 4)
        local_seconds = 1.0 + rank  # rank 1 is the slower one
        slowest = bench.max_over_ranks(local_seconds, dist, torch.device("cpu"))
        value = bench.aggregate_throughput(world, 20, 16384, 100, slowest)
        q.put((rank, seeds, slowest, value))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_take_max_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    assert set(out[0][1]).isdisjoint(out[1][1])          # no block processed twice
    assert out[0][2] == out[1][2] == 2.0                 # both ranks see the slowest time
    assert out[0][3] == pytest.approx(2 * 20 * 16384 * 100 / 2.0)
