"""The multi-GPU benchmark path on CPU: two gloo ranks run the same
aggregation the NCCL ranks run (sum of work, max of time) and the particle
sharding covers every particle exactly once."""

import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        pet = 1000 * (rank + 1)
        elapsed = 0.5 + rank  # rank 1 is the slow one
        total, t = bench.aggregate_over_ranks(pet, elapsed, torch.device("cpu"))
        q.put((rank, total, t))
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation():
    import socket

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
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, total, t in res:
        assert total == 3000.0
        assert t == 1.5


def test_shard_ranges_cover_all_particles():
    import bench

    for n, world in ((1_000_000, 8), (17, 4), (3, 5)):
        seen = []
        for r in range(world):
            a, b = bench.shard_range(n, r, world)
            seen.extend(range(a, b))
        assert seen == list(range(n))
