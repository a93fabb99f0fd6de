"""bench.py's multi-rank accounting on CPU: two gloo ranks reduce their
timings to the maximum (every rank sees the slowest), and the whole-job rate
counts the units of all replicas over that time. The replicas share no data:
the pixel path does not shard, one process per GPU runs its own image."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2")
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        out = bench.max_over_ranks([1.0 + rank, 5.0 - rank, 0.25 * (rank + 1)], 2, "cpu")
        q.put((rank, out, bench.dist_env()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_to_the_slowest():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict((r, (out, env)) for r, out, env in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        out, env = res[r]
        assert out == [2.0, 5.0, 0.5]
        assert env == (r, 2, 0)


def test_replica_rate_counts_all_ranks():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(1000, 4, 2.0) == 2000.0
    assert bench.max_over_ranks([3.0, 1.0], 1, "cpu") == [3.0, 1.0]
