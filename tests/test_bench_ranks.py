"""The multi-GPU path of bench.py (independent replicas, one per rank):
its only collective is the max-over-ranks timing reduction, checked here with
world_size 2 on the gloo backend (CPU), with the throughput arithmetic."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ms = bench.max_over_ranks(100.0 + 50.0 * rank, ws)      # rank 1 is the slowest
        q.put((rank, ms, bench.job_throughput(1000, ws, ms)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world_size_2():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in out:
        assert ms == 150.0
        assert value == pytest.approx(2 * 1000 / 0.150)


def test_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.job_throughput(4_000_000, 1, 200.0) == pytest.approx(2.0e7)
