"""The multi-rank logic of bench.py on CPU (gloo, world size 2): the barrier
and max-over-ranks timing every arm uses, the whole-job throughput formula,
and the reference arm, which only rank 0 runs and prints."""
from __future__ import annotations

import argparse
import contextlib
import io
import os
import socket
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        barrier, maxreduce = bench.sync_helpers(world, cuda=False)
        barrier()
        # the job's time is its slowest rank's
        assert maxreduce(10.0 + rank) == 10.0 + world - 1
        # every rank processes its own replica: throughput adds up over ranks
        assert bench.job_rate(world, 4_000_000, 2.0) == pytest.approx(world * 2.0)
        if rank > 0:
            args = argparse.Namespace(workload="spheres_cyl2048", radius=32.0, steps=1, warmup=0, cpu_seconds=1.0)
            out = io.StringIO()
            with contextlib.redirect_stdout(out):
                rc = bench.reference_arm(args, rank, world)
            assert rc == 0 and out.getvalue() == ""  # only rank 0 times the CPU path and prints
        barrier()
    finally:
        dist.destroy_process_group()


def test_bench_multi_rank_helpers():
    import torch.multiprocessing as mp
    mp.spawn(_rank, args=(2, _free_port()), nprocs=2, join=True)


def test_bench_single_rank_helpers():
    sys.path.insert(0, ROOT)
    import bench
    barrier, maxreduce = bench.sync_helpers(1, cuda=False)
    barrier()
    assert maxreduce(3.5) == 3.5
    assert bench.job_rate(1, 2_000_000, 4.0) == pytest.approx(0.5)
