"""Multi-rank (replica) aggregation of the benchmark, on CPU with gloo: the
step time is the maximum over ranks and the rate counts every replica."""
import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench

        ms, value = bench.replica_rate(10.0 + rank, 1000, world, dist, "cpu")
        out.put((rank, ms, value))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_rate_two_ranks():
    world, port = 2, 29500 + os.getpid() % 1000
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in res:
        assert ms == 11.0  # the slower replica sets the step time
        assert value == pytest.approx(2 * 1000.0 * 1000.0 / 0.011)


def test_replica_rate_single():
    import bench

    ms, value = bench.replica_rate(5.0, 100, 1)
    assert ms == 5.0 and value == pytest.approx(1e4 / 0.005)
