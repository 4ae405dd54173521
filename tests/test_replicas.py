"""bench.py's multi-GPU mode is replicas only (the solve does not shard):
N ranks each time the same workload, a barrier brackets the timed region
and rank 0 reports the whole-job value from the slowest rank.  These tests
run that plumbing as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, q):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": "2",
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, local, ws = bench.dist_init()
    bench.barrier(ws)
    slowest = bench.max_over_ranks(10.0 * (rank + 1), ws)      # each rank's "ms"
    bench.barrier(ws)
    q.put((r, ws, slowest))
    dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 20.0), (1, 2, 20.0)]
    # whole-job value: ws x steps / slowest time
    steps, ws, slowest_ms = 10, 2, 20.0
    assert ws * steps / (slowest_ms / 1e3) == 1000.0


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        m, n, steps, warmup = 100000, 500, 1, 0
    assert bench.run_reference(Args, 1, 2) is None


def test_batched_problems_shard_without_overlap():
    """bench.py --workload batched under N ranks: rank r solves problems
    [r P, (r + 1) P) of one seeded sequence, so the ranks' shares are
    disjoint, equal in count, and together the single-rank sequence."""
    sys.path.insert(0, ROOT)
    import bench
    P = 40
    whole = bench.batched_shapes(3 * P)
    parts = [bench.batched_shapes(P, rank=r, world=3) for r in range(3)]
    assert all(len(p) == P for p in parts)
    assert [x for p in parts for x in p] == whole
    assert all(m >= 8 * n and 1000 <= m <= 50000 and 16 <= n <= 256 for _, (m, n) in whole)
