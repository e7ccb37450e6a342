"""The multi-GPU path of bench.py is "replicas only": N ranks run independent
copies of the sweep and the job's step time is the slowest rank's.  This
checks the host side of that path with two gloo ranks on the CPU: the max over
ranks and the whole-job rate."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys

    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = [2.5, 4.0][rank]  # rank 1 is the slow one
    slowest = bench.max_over_ranks(ms)
    rate = bench.whole_job_rate(58.06, world, slowest)
    q.put((rank, slowest, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_and_rate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, rate in out:
        assert slowest == 4.0
        assert abs(rate - 2 * 58.06 / 4.0e-3) < 1e-6


def test_single_process_is_identity():
    import sys

    sys.path.insert(0, REPO)
    import bench

    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.whole_job_rate(10.0, 1, 2.0) == 5000.0
