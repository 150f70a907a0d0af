"""Multi-rank (gloo, CPU) test of the replica timing used by bench.py for N > 1."""
import os

import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from exadg_gb300.replicas import job_throughput, max_over_ranks

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 1.0 + rank  # rank 1 is the slow one
    m = max_over_ranks(ms)
    thr = job_throughput(1000, m * 1e-3, world)
    out[rank] = (m, thr)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_two_ranks():
    import random

    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = 29500 + random.randint(0, 2000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    m, thr = out[0]
    assert m == 2.0
    assert thr == pytest.approx(2 * 1000 / 2e-3)


def test_single_process_passthrough():
    from exadg_gb300.replicas import job_throughput, max_over_ranks

    assert max_over_ranks(3.5) == 3.5
    assert job_throughput(10, 2.0, 1) == 5.0
