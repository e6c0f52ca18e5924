"""The multi-GPU path of bench.py (replicas: no data-path collective, one
MAX over ranks of the elapsed time) on two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r "took" 1 + r seconds for 10 steps: the job is as slow as rank 1
    rate, slowest = bench.whole_job_rate(1.0 + rank, 10, world)
    q.put((rank, rate, slowest))
    dist.destroy_process_group()


def test_whole_job_rate_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, slowest in out:
        assert slowest == pytest.approx(2.0)
        assert rate == pytest.approx(2 * 10 / 2.0)


def test_whole_job_rate_single_rank():
    sys.path.insert(0, REPO)
    import bench
    assert bench.whole_job_rate(2.0, 10, 1) == (5.0, 2.0)
