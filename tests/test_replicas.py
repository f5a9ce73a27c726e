"""The benchmark's host logic, without a GPU. Its multi-GPU form is
independent replicas: each rank solves its own seeded batch, the ranks meet
only at barriers, and the job's time is the slowest rank's. Two gloo ranks on
the CPU cover bench.replica_seed and bench.max_over_ranks; the reference arm
(the CPU restatement on the host cores) is run end to end for its JSON line
and its rank-0-only output, and the LAPACK side baseline's child for its
JSON object."""
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


def test_reference_arm_json_line():
    # the reference arm runs on the host cores only: its JSON line carries
    # the contract's keys, with the CPU baseline describing this run
    import json
    import subprocess
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_lapack_side_baseline_child():
    import json
    import subprocess
    env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-lapack", "64"], capture_output=True,
                       text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["kind"] == "lapack" and out["value"] > 0 and out["cores"] >= 1


def test_roofline_figures():
    # the launch list's top kernels of the batched refined step are reported
    # with their algorithmic work over their time
    import bench
    r = bench.refine_roofline(70.0, 1750.0, 4096, {"frac": 0.1})
    assert r["kernel"] == "k_solve_refine" and r["bound"] == "tensor" and r["unit"] == "TFLOP/s"
    assert abs(r["frac"] - 0.04) < 1e-12 and r["fp32_pipe"]["frac"] == 0.1
    assert abs(r["traffic"] - 4 * bench.REFINE_DRAM_BYTES_PER_1024) < 1.0
    assert bench.refine_roofline(7.0, None, 4096, None)["frac"] is None


def test_launch_counts():
    # refined: one persistent kernel, (chase, replay) per pass and one
    # refinement over all matrices, the mark in a graph plan; other paths per
    # size bucket: tridiagonalisation, (chase, replay) per pass, the mark
    import bench
    assert bench.launches_per_step(8, 2, True, False) == 6
    assert bench.launches_per_step(8, bench.GRAPH_PASSES, True, True) == 11
    assert bench.launches_per_step(8, bench.GRAPH_PASSES, False, True) == 8 * 10
    assert bench.launches_per_step(8, 2, False, False) == 8 * 5
