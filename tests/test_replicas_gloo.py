"""Multi-GPU runs of bench.py are replicas: every rank renders its own frame,
ranks agree on the job time as the maximum over ranks, and only rank 0
reports. This checks that host-side reduction with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.job_time_ms(10.0 * (rank + 1), world, device="cpu")
    out[rank] = t
    dist.destroy_process_group()


def test_job_time_is_max_over_two_ranks():
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert out[0] == pytest.approx(20.0) and out[1] == pytest.approx(20.0)
