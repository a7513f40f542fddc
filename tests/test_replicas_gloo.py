"""Replica mode over two processes (gloo on CPU): every rank sees the slowest rank's time and the whole-job
throughput."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from firepony_gb300.replicas import job_throughput
    ms = [100.0, 250.0][rank]
    t = [2.0, 1.5][rank]
    out[rank] = job_throughput(ms, t, 1_000_000, world, device="cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_job_throughput_two_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        value, e2e, ms, t = out[r]
        assert ms == 250.0 and t == 2.0
        assert value == pytest.approx(2_000_000 / 0.25)
        assert e2e == pytest.approx(2_000_000 / 2.0)
    assert torch is not None


def test_job_throughput_single():
    from firepony_gb300.replicas import job_throughput
    assert job_throughput(50.0, 0.5, 1000, 1) == (20000.0, 2000.0, 50.0, 0.5)
