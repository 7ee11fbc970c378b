"""The multi-GPU bench path runs independent replicas with no collective on
the data path; its only cross-rank step is the throughput reduction (sum of
the flops all ranks processed over the slowest rank's time).  Exercised here
with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r processed (r + 1) TFLOP in (10 + r) ms
        v, ms = bench.world_throughput((rank + 1) * 1e12, 10.0 + rank, dist)
        q.put((rank, v, ms))
    finally:
        dist.destroy_process_group()


def test_world_throughput_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for _, v, ms in res:
        assert ms == pytest.approx(11.0)
        assert v == pytest.approx(3e12 / 11e-3 / 1e12)


def test_world_throughput_single_rank():
    v, ms = bench.world_throughput(2e12, 4.0)
    assert ms == 4.0 and v == pytest.approx(500.0)
