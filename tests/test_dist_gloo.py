"""The replica path of bench.py on CPU: world size 2 over gloo (one process per rank, as torchrun
starts them).  Each rank times its own replica; the job's time is the max over ranks and the
throughput is the units of all ranks over it, with no data-path collective."""
import multiprocessing as mp
import os
import socket

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys

    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    try:
        d.barrier()
        t = d.max(1.0 + rank)           # per-rank chunk times -> the job's time
        n = d.sum(100.0 * (rank + 1))    # units of all ranks
        q.put((rank, d.world, d.local, t, n))
    finally:
        d.close()


def test_two_ranks_take_max_time_and_sum_units():
    pytest.importorskip("torch.distributed")
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in ps), [p.exitcode for p in ps]
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, world, local, t, n in out:
        assert world == 2 and local == rank
        assert t == 2.0 and n == 300.0


def test_reference_arm_runs_on_rank_zero_only():
    import sys

    sys.path.insert(0, ROOT)
    import bench

    class Rank1:
        rank, world, local = 1, 2, 1

    assert bench.run_reference_arm(None, Rank1()) is None  # returns before touching args or a GPU
