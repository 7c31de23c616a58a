"""Replicas: bench.py's multi-process helpers over gloo, world size 2, on CPU.

Independent solves exchange nothing, so N GPUs run N replicas; the only
cross-rank steps are the barrier around the timed region and the max over
ranks of the timed duration. This runs those helpers in two CPU processes.
"""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "MASTER_ADDR": "127.0.0.1",
                       "MASTER_PORT": str(port), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, str(ROOT))
    import argparse

    import bench
    args = argparse.Namespace(impl="reference")
    r, w = bench.dist_init(args)
    bench.barrier(w)
    v = bench.max_over_ranks(10.0 + r, w)
    # the reference arm does its work on rank 0 only; other ranks return at once
    if r != 0:
        bench.run_reference(argparse.Namespace(cases=4, steps=1, warmup=0, gpus=w), r, w)
    out.put((r, w, v))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_barrier_and_max_over_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 11.0), (1, 2, 11.0)]
