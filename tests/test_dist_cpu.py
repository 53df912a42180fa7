"""Multi-rank host logic of bench.py on CPU: two gloo ranks exchange their
timings (max over ranks) and ray counts (sum over ranks) the way the
replicas-only multi-GPU bench does; only rank 0 prints."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, REPO)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mx = bench._max_over_ranks(1.0 + rank, dist)
        sm = bench._sum_over_ranks(10.0 * (rank + 1), dist)
        bench._barrier(dist)
        out_q.put((rank, mx, sm))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_timings():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert res == [(0, 2.0, 30.0), (1, 2.0, 30.0)]


def test_reference_arm_non_zero_rank_exits_quietly(capsys):
    sys.path.insert(0, REPO)
    import argparse
    import bench
    args = argparse.Namespace(steps=1, warmup=3, impl="reference", workload="deforming")
    bench.run_reference(args, rank=1, ws=2, dist=None)
    assert capsys.readouterr().out == ""
