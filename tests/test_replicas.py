"""Replica runs of bench.py (--gpus N: one independent solve per rank, no
data-path collective): the step time is the max over ranks and the value the
whole-job total.  Two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, device="cpu")
    val = bench.replica_value(1e9, world, ms)
    q.put((rank, ms, val, bench.dist_env()))
    dist.destroy_process_group()


def test_two_replicas_max_time_and_total_value():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, val, env in out:
        assert ms == 15.0                      # slowest rank
        assert abs(val - 2 * 1e9 / 15e-3 / 1e9) < 1e-9
        assert env[0] == rank and env[1] == 2
