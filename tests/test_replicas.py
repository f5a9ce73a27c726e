"""The multi-GPU form of the benchmark is independent replicas: each rank
solves its own seeded batch, the ranks meet only at barriers, and the job's
time is the slowest rank's. This covers that host logic with two gloo ranks
on the CPU (bench.replica_seed, bench.max_over_ranks) and the reference arm's
rank-0-only output, without a GPU."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def replica_rank(rank, ws, port, q):
    import torch
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        ns, _ = bench.workload(batch=16, seed=bench.replica_seed(rank))
        # rank r "took" 1 + r seconds: every rank must see the slowest
        el = bench.max_over_ranks(torch, 1.0 + rank, ws, "cpu")
        dist.barrier()
        q.put((rank, el, ns.tolist()))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=replica_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = {}
    for _ in range(2):
        rank, el, ns = q.get(timeout=120)
        out[rank] = (el, ns)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 2.0
    assert out[0][1] != out[1][1]  # each replica has its own batch


def test_single_rank_needs_no_process_group():
    import torch

    import bench
    assert bench.max_over_ranks(torch, 3.5, 1, "cpu") == 3.5
    assert bench.replica_seed(0) == bench.SEED


def test_reference_arm_prints_on_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup = 1, 3

    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(Args())
    assert buf.getvalue() == ""
