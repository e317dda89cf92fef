"""Multi-GPU form (replicas): the throughput reduction over ranks, run as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from cityseer_gb300.replicas import job_throughput


def _free_port() -> int:
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r processed 1000 + r units in 2 + r seconds: the job is as slow as its slowest rank
        value, t_max = job_throughput(1000.0 + rank, 2.0 + rank)
        q.put((rank, value, t_max))
    finally:
        dist.destroy_process_group()


def test_single_process_no_group():
    assert job_throughput(500.0, 2.0) == (250.0, 2.0)


@pytest.mark.timeout(120)
def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(90)
        assert pr.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, t_max in got:
        assert t_max == 3.0
        assert value == pytest.approx((1000.0 + 1001.0) / 3.0)
