"""Multi-GPU runs are replicas (independent solves per rank, no collective on
the data path): the whole-job rate is all ranks' units over the slowest
rank's time.  Checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms_local = [40.0, 50.0][rank]  # rank 1 is the slow one
    rate, ms = bench.job_rate(1000, ms_local, world, "cpu")
    out[rank] = (rate, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_job_rate_is_all_units_over_the_slowest_rank():
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    for rank in (0, 1):
        rate, ms = out[rank]
        assert ms == 50.0
        assert rate == pytest.approx(2 * 1000 / 0.050)


def test_job_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    rate, ms = bench.job_rate(500, 25.0, 1, "cpu")
    assert ms == 25.0 and rate == pytest.approx(500 / 0.025)
