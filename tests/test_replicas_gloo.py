"""The multi-GPU form of the bench is independent replicas: each rank times its own steps
and the job's time is the slowest rank's.  This runs that aggregation with two gloo ranks
on CPU (no GPU, no collective on the data path)."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank 0 took 30 ms for 10 steps, rank 1 took 50 ms
    ms_step, value = bench.replica_throughput(30.0 + 20.0 * rank, 10, world, "cpu")
    out.put((rank, ms_step, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, ms_step, value in res:
        assert ms_step == pytest.approx(5.0)
        assert value == pytest.approx(2 * 1000.0 / 5.0)


def test_replica_throughput_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(40.0, 8, 1, "cpu") == (5.0, 200.0)
