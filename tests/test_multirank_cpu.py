"""The bench's multi-process path on CPU: two ranks over gloo (replicas, no
data-path collective; the only exchange is the max of the timed regions)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    job = bench._job_ms(10.0 + 5.0 * rank, world)   # rank 1 is the slower one
    out[rank] = (job, bench._job_value(64, 5, world, job))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_take_the_max_time_and_count_all_units():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as manager:
        out = manager.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(180)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        res = dict(out)
    assert res[0] == res[1]
    job, value = res[0]
    assert job == 15.0
    assert value == pytest.approx(64 * 5 * 2 / 0.015)


def test_replica_ranks_get_their_own_instances(gastar):
    sys.path.insert(0, ROOT)
    import bench
    a = bench._instances(gastar, 0)
    b = bench._instances(gastar, 1)
    assert len(a) == len(b) == bench.WORKLOAD["instances"]
    assert any((x[0] != y[0]).any() for x, y in zip(a, b))
    # rank 0 keeps the single-GPU workload
    assert all((x[0] == y[0]).all() for x, y in zip(a, bench._instances(gastar)))
