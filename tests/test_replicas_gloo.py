"""The replica path of bench.py on two CPU ranks (gloo): the whole-job rate is the sum
of all ranks' units over the slowest rank's time, and the reference arm runs on rank 0
only.  No GPU is involved."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = [3.0e6, 5.0e6][rank]
        ms = [40.0, 50.0][rank]
        rate, ms_max = bench.job_rate(units, ms)
        out[rank] = (rate, ms_max)

        class A:
            steps, warmup, solver, gpus = 1, 0, "hllc", world
        # the reference arm returns immediately on every rank but 0 (nothing to run)
        if rank != 0:
            bench.run_reference(A(), rank, world)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_job_rate_sums_units_over_the_slowest_rank():
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        rate, ms_max = res[r]
        assert ms_max == 50.0
        assert rate == pytest.approx((3.0e6 + 5.0e6) / 0.050)


def test_job_rate_single_process():
    rate, ms = bench.job_rate(1.0e6, 20.0)
    assert ms == 20.0 and rate == pytest.approx(5.0e7)
