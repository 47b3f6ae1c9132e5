"""Multi-GPU runs are replicas (no data-path collective): each rank runs the
whole workload, the ranks exchange only their times, and rank 0 reports every
rank's bytes over the slowest rank's time. The exchange is exercised here on
CPU with two gloo ranks."""
import os
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    assert (r, w, local) == (rank, world, rank)
    my_time = 0.010 * (rank + 1)  # rank 1 is the slow replica
    t_max = bench.max_over_ranks(my_time, dist, "cpu")
    value = bench.replica_value(1e9, world, t_max)
    out.put((rank, t_max, value))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replicas_report_slowest_rank(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 2000
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, value in res:
        assert t_max == pytest.approx(0.020)
        assert value == pytest.approx(world * 1e9 / 0.020 / 1e9)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.5, None, "cpu") == 0.5
    assert bench.replica_value(2e9, 1, 0.5) == pytest.approx(4.0)
