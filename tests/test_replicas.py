"""Multi-GPU is replicas only: each rank indexes its own column and the
bench's job throughput is all ranks' rows over the slowest rank's time.  The
aggregation runs here on CPU as two gloo ranks (no GPU, no collective on any
data path)."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        elapsed = [40.0, 55.0][rank]  # rank 1 is the slowest
        q.put((rank,) + bench.replica_throughput(elapsed, 1000, 10, dist, "cpu"))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, max_ms, value in got:
        assert max_ms == 55.0
        assert value == pytest.approx(2 * 1000 * 10 / 0.055)


def test_replica_throughput_single_process():
    sys.path.insert(0, REPO)
    import bench
    max_ms, value = bench.replica_throughput(20.0, 500, 4)
    assert max_ms == 20.0 and value == pytest.approx(500 * 4 / 0.02)
