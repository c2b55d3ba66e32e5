"""Replica (multi-GPU) host logic of bench.py on CPU ranks over gloo.

The decode path does not shard across GPUs (replicas only: every rank decodes
its own capture); the only cross-rank operations are the barrier around the
timed region and the max-over-ranks of the step time.  Two CPU processes
check both, and that the whole-job value sums the ranks' samples.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        ms = 10.0 + 5.0 * rank               # each rank's own step time
        slowest = bench.max_over_ranks(ms, world)
        samples = 1000000                    # per-rank capture (weak scaling)
        value = world * samples / (slowest / 1e3) / 1e6
        out.put((rank, slowest, value))
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_two_cpu_ranks_take_the_slowest_step_and_sum_the_work():
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
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == res[1][2] == pytest.approx(2 * 1000000 / 0.015 / 1e6)
