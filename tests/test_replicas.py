"""The bench's multi-GPU arithmetic on CPU: N independent replicas over a
gloo process group (world size 2, 127.0.0.1) — the job time is the slowest
replica's, the throughput counts every replica's steps."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank 0 ran its 10 steps in 20 ms, rank 1 in 30 ms
    value, ms = bench.replica_throughput(20.0 + 10.0 * rank, 10, world, device="cpu")
    q.put((rank, value, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms in res:
        assert ms == pytest.approx(3.0)            # the slower replica: 30 ms / 10 steps
        assert value == pytest.approx(2 * 10 / 0.030)  # both replicas' steps over that time


def test_replica_throughput_single():
    import bench
    value, ms = bench.replica_throughput(50.0, 100, 1, device="cpu")
    assert ms == pytest.approx(0.5) and value == pytest.approx(2000.0)
