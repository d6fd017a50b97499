"""The bench's replica aggregation over two gloo ranks on the CPU (torch.distributed)."""

import os

import pytest


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        q.put((rank, bench.aggregate_replicas(10.0 + 5.0 * rank, 4, world, dist, device="cpu")))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    import socket
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    out = dict(q.get(timeout=5) for _ in range(2))
    for r in (0, 1):
        max_ms, per_replica, whole = out[r]
        assert max_ms == pytest.approx(15.0)          # slowest rank
        assert per_replica == pytest.approx(15.0 / 4)
        assert whole == pytest.approx(15.0 / 8)       # both replicas' steps over the slowest time


def test_replica_aggregation_single():
    import bench
    assert bench.aggregate_replicas(8.0, 4, 1) == (8.0, 2.0, 2.0)
