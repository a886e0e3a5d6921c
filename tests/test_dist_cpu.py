"""The bench's multi-GPU contract on CPU: world_size-2 gloo ranks (one process each) reduce
their timings to the slowest rank and report the whole-job throughput of independent
replicas, with no collective on the data path."""
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench._dist() == (ws, rank, rank)
        ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        worst = bench.max_over_ranks(ms, ws, "cpu")
        q.put((rank, worst, bench.replica_throughput(ws, 1e9, 4, worst)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_replica_throughput_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port, ws = _free_port(), 2
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(ws))
    for rank, worst, value in got:
        assert worst == 15.0  # every rank reports the slowest rank's time
        assert value == pytest.approx(2 * 1e9 * 4 / 0.015)


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.replica_throughput(1, 48.3e9, 10, 300.0) == pytest.approx(48.3e9 * 10 / 0.3)
