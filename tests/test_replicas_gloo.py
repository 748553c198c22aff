"""The N > 1 path of bench.py is replicas only: each rank runs its own workload and the
step time is the max over ranks.  Checked with two gloo ranks on the CPU."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.aggregate_replicas(100.0 + 50.0 * rank, 64, world)
    q.put((rank, ms, value))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    for rank, ms, value in res:
        assert ms == 150.0
        assert abs(value - 2 * 64 / 0.150) < 1e-9
