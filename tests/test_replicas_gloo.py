"""Multi-GPU runs are independent replicas (chains shard with no collective on
the data path): each rank samples its own chains (its own seeds) and the timed
region is the slowest rank's. Checked here as world-size-2 gloo process groups
on the CPU: both ranks agree on the maximum of their times, and the chain
seeds of one replica's whole run (a 2048-chain run of 600 steps) are disjoint
from the other's, so their pcg64 streams differ."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = 10.0 * (rank + 1) + 0.25
    got = bench.max_over_ranks(local_ms, world)
    # chain seeds of a long run (chain c of a step uses step_seed + c)
    chains, steps = 2048, 600
    seeds = [(bench.step_seed(rank, t, chains), chains) for t in (0, 1, steps - 1)]
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, got, seeds))


def test_replicas_take_the_slowest_rank_and_distinct_seeds():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, m0, s0), (_, m1, s1) = res
    assert m0 == m1 == 20.25
    # every chain seed of one replica lies outside the other replica's range
    lo0, hi0 = s0[0][0], s0[-1][0] + s0[-1][1]
    lo1, hi1 = s1[0][0], s1[-1][0] + s1[-1][1]
    assert hi0 <= lo1 or hi1 <= lo0, (lo0, hi0, lo1, hi1)
    assert all(a + c <= b for (a, c), (b, _) in zip(s0, s0[1:]))  # steps consecutive within a replica


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
