"""Multi-GPU layout: replicas only (independent fields, one per rank).

The only cross-rank step is the bench's timing reduction (maximum over ranks
for times, sum for launch counts); no data moves between ranks.  Two gloo
ranks on CPU exercise it here, and the reference arm's rule that ranks other
than 0 exit without work.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as D

    import bench
    D.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: times 1+r and 10-r, 3*(r+1) launches
        m, s = bench.reduce_over_ranks([1.0 + rank, 10.0 - rank], [3.0 * (rank + 1)], "cpu")
        e, none = bench.reduce_over_ranks([0.5 * (rank + 1)], [], "cpu")
        q.put((rank, m, s, e, none))
    finally:
        D.destroy_process_group()


def test_two_replicas_take_the_max_time_and_the_summed_launches():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        got = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
    assert [p.exitcode for p in procs] == [0, 0]
    for rank, m, s, e, none in got:
        assert m == [2.0, 10.0] and s == [9.0], rank
        assert e == [1.0] and none == [], rank


def test_reference_arm_runs_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup = 1, 0
    bench.run_reference(A, bench.WORKLOADS["c2"], rank=1, world=2)
    assert capsys.readouterr().out == ""
