"""The N>1 path of bench.py: replicas, no data-path collective.  Two gloo
ranks on CPU check the job-level aggregation (slowest rank's time, sum of the
ranks' work) and that the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [120.0, 150.0][rank]
    ms, units, value = bench.replica_aggregate(local_ms, 512 * 20, dist, "cpu")
    q.put((rank, ms, units, value))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, units, value in got:
        assert ms == 150.0
        assert units == 2 * 512 * 20
        assert value == pytest.approx(2 * 512 * 20 / 0.150)


def test_single_rank_aggregation():
    sys.path.insert(0, ROOT)
    import bench
    ms, units, value = bench.replica_aggregate(200.0, 1000, None)
    assert (ms, units) == (200.0, 1000)
    assert value == pytest.approx(5000.0)


def test_reference_arm_other_ranks_do_no_work():
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 0, 2
    assert bench.run_reference(A(), 1, 2) is None
