"""Replica aggregation across ranks (gloo, world size 2, CPU)."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from strawberryfields_gb300.replicas import job_throughput

    ups, mx = job_throughput(100.0 * (rank + 1), units_per_rank=10)
    out[rank] = (ups, mx)
    dist.destroy_process_group()


def test_job_throughput_max_over_ranks():
    import torch.multiprocessing as mp

    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    for r in range(2):
        ups, mx = out[r]
        assert mx == pytest.approx(200.0)
        assert ups == pytest.approx(2 * 10 / 0.2)


def test_single_process_fallback():
    from strawberryfields_gb300.replicas import job_throughput

    ups, mx = job_throughput(50.0, units_per_rank=5)
    assert ups == pytest.approx(100.0) and mx == 50.0
