"""The bench's multi-rank path on CPU (gloo, world size 2): process-group
set-up from the torchrun environment, the barrier, the max-over-ranks
timing and the reference arm running on rank 0 only.  Replicas share no
data-path collective; these are the only cross-rank operations."""
from __future__ import annotations

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import argparse

    import torch.distributed as dist

    import bench
    w, r, local = bench.dist_init(0)  # no GPUs: gloo
    try:
        assert (w, r, local) == (world, rank, rank)
        assert dist.get_backend() == "gloo"
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, w)
        dist.barrier()
        # reference arm: ranks other than 0 return without work
        ran = None
        if rank != 0:
            ran = bench.run_reference(argparse.Namespace(workload="box_3d", steps=1, warmup=0), w, r)
        q.put((rank, slowest, ran))
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 15.0, None), (1, 15.0, None)]
    del torch


def test_single_rank_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
