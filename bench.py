"""Benchmark: batched self-adjoint eigensolver on GB300 (one JSON line).

Workload (batched configuration of the headline metric): 4096 real symmetric
GOE matrices A = (B + B')/2, B iid N(0, 1), orders n drawn uniform in
[8, 128] from numpy PCG64 seed 2; all eigenpairs (eigen!(Hermitian(A))).
A step = one solve of the whole batch. Synthetic data (the reference
publishes no benchmark dataset). The packed FP64 input arena is ~191 MB,
larger than the 129 MB L2, so every step streams it from HBM.

Paths timed: plain FP64 (the reference's arithmetic), plain FP32, and FP32 +
FP64 Ogita-Aishima refinement (the headline `value`, eigh/s, when it meets
residual and eigenvalue error <= 1e-13 ||A|| over every matrix of the batch).

The single-matrix half of the metric ("large"): n = 4096, FP64 GPU path vs
FP32 solve + refinement, on the prescribed-spectrum matrix Q diag(lam) Q'
(lam = +-logspace(-6, 0), cond 1e6, Haar Q, seed 3) and on a GOE matrix,
time per solve and accuracy of each result (best of 2 after a warm-up).

--impl reference times the reference algorithm on the host cores instead:
the CPU restatement of GenericLinearAlgebra.jl's eigen!(Hermitian)
(oracle/, one matrix per OpenMP thread) — Julia itself is not installed.
Multi-GPU: the batch shards per rank with no collective ("replicas only");
value = matrices solved by all ranks / max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "genericlinearalgebra.jl_gb300")
for _p in (ROOT, PKG, os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "eigh/s (batch n≤128) & n=4096 time at 1e-13 resid: FP32+refine vs FP64 GPU"
# DRAM bytes (read + write) of the refinement in one step of the 1024-matrix
# workload (ncu dram__bytes_read.sum + dram__bytes_write.sum)
REFINE_DRAM_BYTES_PER_1024 = 1233.8e6
BATCH = 4096
NLO, NHI = 8, 128
SEED = 2


def workload(batch=BATCH, seed=SEED):
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = rng.integers(NLO, NHI + 1, size=batch)
    mats = []
    for n in ns:
        B = rng.standard_normal((n, n))
        mats.append((B + B.T) / 2)
    return ns.astype(np.int64), mats


def pack_f(mats, dtype=np.float64):
    return np.concatenate([np.asarray(m, dtype=dtype).ravel(order="F") for m in mats])


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# A GLA_FLAG_GRAPH plan enqueues a fixed four chase passes (include/glagpu.h).
GRAPH_PASSES = 4


def launches_per_step(n_buckets, passes, refined, graph):
    """Kernels one batched execute launches. FP32 + refinement: the one
    persistent solve-and-refine kernel, then over all matrices at once a
    chase and a rotation replay per pass, the refinement (both finish only
    the matrices the persistent kernel leaves to the QL chase) and, in a
    graph plan, the kernel that marks matrices left unfinished. Other paths:
    per size bucket the tridiagonalisation, a chase and a rotation replay per
    pass, and the mark in a graph plan."""
    if refined:
        return 1 + 2 * passes + 1 + (1 if graph else 0)
    return n_buckets * (1 + 2 * passes + (1 if graph else 0))


def refine_roofline(achieved, peak, batch, fp32):
    """k_solve_refine, the persistent kernel that runs (almost) the whole
    batched refined step. Its tensor-core work: the refinement's three
    double-float products per iteration (A X, X'(A X), X'X), each 28 bf16
    slice products of 2 n^3 (the Ozaki scheme, seven slices per operand),
    i.e. 168 n^3 bf16 flops per matrix and iteration (the plan's refine_n3
    counter sums n^3 over matrices and iterations). achieved = those flops
    over the kernel's time (CUDA events on the execute's stream, the plan's
    "tridiag" phase); peak = MEASURED_PEAKS.json bf16 (burst). The kernel is
    latency-bound (per-column barriers of the FP32 reduction, the slicing),
    so the fraction is small by construction; fp32 gives its FP32-pipe work
    (reduction, Q, X = QY, X E) against the SGEMM FMA rate of this run.
    traffic: DRAM bytes of one launch over the first 1024 workload matrices
    (same order distribution), from an ncu capture, scaled by the matrix
    count; the algorithmic bytes are ~20 sum(n^2) = 0.48 GB per step, the
    rest is the per-matrix double-float scratch of the refinement (56 n^2
    bytes) and the products' slice scratch (224 KB per CTA, rewritten for
    every product), which do not stay in L2."""
    return {"kernel": "k_solve_refine", "bound": "tensor", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": (achieved / peak) if peak else None,
            "traffic": REFINE_DRAM_BYTES_PER_1024 * batch / 1024 if REFINE_DRAM_BYTES_PER_1024 else None,
            "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)", "fp32_pipe": fp32}


def replica_seed(rank):
    """Each rank solves its own seeded batch (replicas: no data exchange)."""
    return SEED + 1000 * rank


def max_over_ranks(torch, seconds, ws, dev):
    """The slowest rank's elapsed time: with independent replicas the job
    ends when the last one does (an all-reduce MAX when ws > 1)."""
    if ws <= 1:
        return seconds
    t = torch.tensor([seconds], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def start_clock_sampler():
    path = tempfile.mktemp(suffix=".csv")
    try:
        f = open(path, "w")
        p = subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
             "--format=csv,noheader,nounits", "-lms", "200"], stdout=f, stderr=subprocess.DEVNULL)
        return p, f, path
    except Exception:
        return None, None, path


def stop_clock_sampler(handle, gpu_index=0):
    p, f, path = handle
    if p is None:
        return None
    p.terminate()
    try:
        p.wait(timeout=5)
    except Exception:
        p.kill()
    f.close()
    sm, mx, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9 or parts[0] != str(gpu_index):
            continue
        try:
            sm.append(float(parts[1]))
            mx = max(mx, float(parts[2]))
        except ValueError:
            continue
        for nm, v in zip(names, parts[5:9]):
            if v.lower() in ("active", "1"):
                reasons.add(nm)
    os.unlink(path)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_dgemm_tflops(torch):
    """FP64 peak measured in this run: cuBLAS DGEMM 4096^3 (best of 3)."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * 4096 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


def measured_sgemm_tflops(torch):
    """FP32 pipe peak measured in this run: cuBLAS SGEMM 8192^3 with TF32 off (best of 3)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(8192, 8192, dtype=torch.float32, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float32, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2 * 8192 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b
    return best


def measured_peaks_file():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def oracle_values(ns, mats):
    """Eigenvalues of every workload matrix from the CPU oracle (the
    reference's eigvals! restated, FP64), all host threads; packed like w."""
    from oracle import oracle as O
    aoff = np.concatenate([[0], np.cumsum(ns * ns)[:-1]]).astype(np.int64)
    woff = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    A = pack_f(mats)
    w = np.zeros(int(ns.sum()))
    V = np.zeros(1)
    info = np.zeros(len(ns), np.int32)
    O.batched_raw("N", "L", np.ascontiguousarray(ns), aoff, A, w, woff, V, info, nthreads=os.cpu_count() or 1)
    return w


def check_all(ns, mats, w, V, woff, aoff, w_oracle):
    """Max residual ||AV - VW||/||A||, orthogonality ||V'V - I|| and eigenvalue
    error |w - w_oracle|/||A|| over EVERY matrix of the batch (2-norms,
    matrices of one order stacked)."""
    res = orth = ev = 0.0
    for n in np.unique(ns):
        idx = np.nonzero(ns == n)[0]
        n = int(n)
        A = np.stack([mats[b] for b in idx])
        Wb = np.stack([w[woff[b]: woff[b] + n] for b in idx]).astype(np.float64)
        Vb = np.stack([V[aoff[b]: aoff[b] + n * n].reshape(n, n, order="F") for b in idx]).astype(np.float64)
        Wo = np.stack([w_oracle[woff[b]: woff[b] + n] for b in idx])
        nA = np.linalg.norm(A, 2, axis=(1, 2))
        R = A @ Vb - Vb * Wb[:, None, :]
        res = max(res, float((np.linalg.norm(R, 2, axis=(1, 2)) / nA).max()))
        G = np.swapaxes(Vb, 1, 2) @ Vb - np.eye(n)
        orth = max(orth, float(np.linalg.norm(G, 2, axis=(1, 2)).max()))
        ev = max(ev, float((np.abs(Wb - Wo).max(axis=1) / nA).max()))
    return {"max_residual": res, "max_orthogonality": orth, "max_eig_err_vs_oracle": ev,
            "matrices_checked": int(len(ns))}


def run_ours(args):
    import torch

    import glagpu
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    ns, mats = workload(batch=args.batch, seed=replica_seed(rank))
    if args.nrange:  # profiling: keep one size range of the workload
        lo, hi = (int(x) for x in args.nrange.split(","))
        keep = [i for i in range(len(ns)) if lo <= ns[i] <= hi]
        ns, mats = ns[keep], [mats[i] for i in keep]
    aoff = np.concatenate([[0], np.cumsum(ns * ns)[:-1]]).astype(np.int64)
    woff = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    A64 = pack_f(mats)
    A32 = A64.astype(np.float32)
    nA = len(A64)
    nW = int(ns.sum())
    dA64 = torch.from_numpy(A64).to(dev)
    dA32 = torch.from_numpy(A32).to(dev)
    w_oracle = oracle_values(ns, mats)  # accuracy of every result is checked against these

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    results = {}
    tuned = {}
    for path in args.paths.split(","):
        # launch shapes per size bucket from the autotuner (measured at plan
        # creation on synthetic matrices, outside every timed region)
        plan = glagpu.Plan(ns, precision=path, timing=True, autotune=not args.no_autotune)
        tuned[path] = plan.bucket_configs()
        dt = torch.float32 if path == "f32" else torch.float64
        A = dA32 if path == "f32" else dA64
        w = torch.empty(nW, dtype=dt, device=dev)
        V = torch.empty(nA, dtype=dt, device=dev)
        info = torch.zeros(len(ns), dtype=torch.int32, device=dev)
        for _ in range(args.warmup):
            plan.execute(A, w, V, info)
        torch.cuda.synchronize()
        phases = {k: 0.0 for k in ("tridiag", "chase", "apply", "refine")}
        counters = None
        clk = start_clock_sampler() if path == "f32_refined" and rank == 0 else (None, None, "")
        barrier()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(args.steps):
            plan.execute(A, w, V, info)
            for k, v in plan.phase_times().items():
                phases[k] += v
        ev1.record()
        torch.cuda.synchronize()
        barrier()
        el = ev0.elapsed_time(ev1) * 1e-3
        clocks = stop_clock_sampler(clk, local) if clk[0] is not None else None
        el = max_over_ranks(torch, el, ws, dev)
        counters = plan.stats()
        wh = w.cpu().numpy()
        Vh = V.cpu().numpy()
        acc = check_all(ns, mats, wh, Vh, woff, aoff, w_oracle)
        n_bad = int((info.cpu().numpy() != 0).sum())
        results[path] = {
            "eigh_per_s": ws * len(ns) * args.steps / el,
            "ms_per_step": 1e3 * el / args.steps,
            "phase_ms_per_step": {k: v / args.steps for k, v in phases.items()},
            "counters": counters,
            "accuracy": acc,
            "info_nonzero": n_bad,
            "clocks": clocks,
            "launches_per_step": None,
        }
        results[path]["launches_per_step"] = launches_per_step(len(plan_buckets(ns)), counters["passes"],
                                                               path == "f32_refined", False)
        plan.close()
    if args.profile:  # profiling runs (under ncu) stop here: no e2e, CPU leg or JSON line
        return
    # ---- headline path captured in a CUDA graph and replayed
    graph_res = {}
    for path in ("f32_refined", "f64"):
        gplan = glagpu.Plan(ns, precision=path, graph=True, autotune=not args.no_autotune)
        w = torch.empty(nW, dtype=torch.float64, device=dev)
        V = torch.empty(nA, dtype=torch.float64, device=dev)
        info = torch.zeros(len(ns), dtype=torch.int32, device=dev)
        Ag = dA64.clone()
        g = gplan.capture(Ag, w, V, info)
        for _ in range(args.warmup):
            g.replay()
        torch.cuda.synchronize()
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(args.steps):
            g.replay()
        ev1.record()
        torch.cuda.synchronize()
        barrier()
        el = ev0.elapsed_time(ev1) * 1e-3
        el = max_over_ranks(torch, el, ws, dev)
        acc = check_all(ns, mats, w.cpu().numpy(), V.cpu().numpy(), woff, aoff, w_oracle)
        graph_res[path] = {"eigh_per_s": ws * len(ns) * args.steps / el, "ms_per_step": 1e3 * el / args.steps,
                           "accuracy": acc, "info_nonzero": int((info.cpu().numpy() != 0).sum()),
                           "launches_per_step": launches_per_step(len(plan_buckets(ns)), GRAPH_PASSES,
                                                                  path == "f32_refined", True)}
        del g
        gplan.close()
    # ---- end to end through the C ABI with host buffers (headline path)
    plan = glagpu.Plan(ns, precision="f32_refined", autotune=not args.no_autotune)
    hA = torch.from_numpy(A64).pin_memory()
    hw = torch.empty(nW, dtype=torch.float64).pin_memory()
    hV = torch.empty(nA, dtype=torch.float64).pin_memory()
    hinfo = torch.zeros(len(ns), dtype=torch.int32).pin_memory()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        plan.execute_host(hA.numpy(), hw.numpy(), hV.numpy(), hinfo.numpy(), stream)
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        plan.execute_host(hA.numpy(), hw.numpy(), hV.numpy(), hinfo.numpy(), stream)
    ev1.record()
    torch.cuda.synchronize()
    barrier()
    el_e2e = ev0.elapsed_time(ev1) * 1e-3
    # chunks the host execute overlapped its copies with (it also copies the
    # 24-byte chase state of every matrix out, to find the matrices finished
    # after their chunk's copy)
    e2e_chunks, e2e_pipelined = plan.host_pipeline()
    plan.close()
    el_e2e = max_over_ranks(torch, el_e2e, ws, dev)
    peak = measured_dgemm_tflops(torch) if rank == 0 else None
    cus = cusolver_batched(torch, ns, mats, dev) if rank == 0 else None
    large = run_large(torch, glagpu, dev) if (rank == 0 and not args.no_large) else None
    c4 = run_c4(torch, glagpu, dev) if (rank == 0 and not args.no_large) else None
    c1 = run_c1(torch, glagpu, dev) if rank == 0 else None
    c5 = run_c5(torch, glagpu, dev) if (rank == 0 and not args.no_large) else None

    if rank == 0:
        def meets(r):
            a = r["accuracy"]
            return r["info_nonzero"] == 0 and a["max_residual"] <= 1e-13 and a["max_eig_err_vs_oracle"] <= 1e-13
        hp = "f32_refined" if meets(results["f32_refined"]) and meets(graph_res["f32_refined"]) else "f64"
        H = results[hp]
        G = graph_res[hp]
        ph = H["phase_ms_per_step"]
        c = H["counters"]
        ns3 = float((ns.astype(np.float64) ** 3).sum())
        # Roofline of the refined step's dominant kernel, the persistent
        # k_solve_refine (its time is the plan's "tridiag" phase): bf16
        # tensor flops of the refinement's sliced products (refine_roofline),
        # and beside them its FP32-pipe flops: the reduction, Q and X = QY
        # ((4/3 + 4/3 + 2) n^3) and X E (2 n^3 per iteration) against the
        # SGEMM rate measured in this run.
        sg = measured_sgemm_tflops(torch)
        fused_ms = ph.get("tridiag", 0.0)
        sec = fused_ms * 1e-3
        tflops = 168.0 * c["refine_n3"] / sec / 1e12 if sec > 0 else 0.0
        f32_flops = (4.0 / 3.0 + 4.0 / 3.0 + 2.0) * ns3 + 2.0 * c["refine_n3"]
        f32_ach = f32_flops / sec / 1e12 if sec > 0 else 0.0
        mp = measured_peaks_file()
        bf16_peak = (mp or {}).get("bf16_tflops")
        fp32 = {"achieved": f32_ach, "peak": sg, "unit": "TFLOP/s", "frac": (f32_ach / sg) if sg else None,
                "peak_source": "measured in this run: cuBLAS SGEMM 8192^3"}
        cpu = cpu_baseline(ns, mats)
        lapack = lapack_baseline(ns, mats)
        line = {
            "metric": METRIC,
            "value": G["eigh_per_s"],
            "unit": "eigh/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": G["ms_per_step"],
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("f32 solve + refinement with double-float (f32 pair) accuracy: bf16-slice tensor-core "
                      "products (Ozaki), f32 SIMT elsewhere") if hp == "f32_refined" else "f64",
            "data": "synthetic (seeded GOE)",
            "config": {"workload": f"batched eigen!(Hermitian): {len(ns)} GOE matrices, n~U[{NLO},{NHI}], seed {SEED}",
                       "path": hp, "batch": len(ns), "sum_n": int(ns.sum()), "sum_n3": ns3,
                       "l2": "inputs larger than L2 (191 MB FP64 arena)", "parallelism": f"replicas x{ws}",
                       "timing": "CUDA-graph replay of the whole batched solve (plan with GLA_FLAG_GRAPH)"},
            "roofline": refine_roofline(tflops, bf16_peak, len(ns), fp32),
            "roofline_large": large_roofline(large, measured_peaks_file()),
            "fp64_dgemm_tflops_measured": peak,
            "cpu_baseline": cpu,
            "cpu_lapack": lapack,
            "e2e": {"value": ws * len(ns) * args.steps / el_e2e, "unit": "eigh/s",
                    "h2d_bytes_per_step": int(A64.nbytes),
                    "d2h_bytes_per_step": int(8 * nA + 8 * nW + 4 * len(ns) + (24 * len(ns) if e2e_pipelined else 0)),
                    "pipeline": {"chunks": e2e_chunks if e2e_pipelined else 0,
                                 "how": "copies of one chunk of matrices overlap the solve of another"
                                        if e2e_pipelined else "whole batch copied in, solved, copied out"}},
            "clocks": results["f32_refined"]["clocks"],
            "gpu_launches": int(G["launches_per_step"] * args.steps),  # the timed graph replays
            "paths": {k: {kk: vv for kk, vv in v.items() if kk != "clocks"} for k, v in results.items()},
            "graph": graph_res,
            "speedup_f32refined_vs_f64": graph_res["f32_refined"]["eigh_per_s"] / graph_res["f64"]["eigh_per_s"],
            "large": large,
            "c4_forward_adjoint": c4,
            "autotune": {"enabled": not args.no_autotune, "bucket_configs": tuned},
            "c1_single_n64": c1,
            "c5_mixed_forward_adjoint": c5,
            "cusolver_batched_f64": cus,
            "julia_probe": julia_probe(),
        }
        line["summary"] = summary(line)
        print(json.dumps(line), flush=True)
        for t in summary_lines(line["summary"]):
            print(t, flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def summary(line):
    """The figures a reader needs first, collected at the end of the JSON line
    (the batched headline, the single-matrix n = 2048 / 4096 results, C1, C4
    and C5)."""
    def g(d, *ks):
        for k in ks:
            if not isinstance(d, dict) or k not in d:
                return None
            d = d[k]
        return d
    out = {"c2_graph_eigh_per_s": {p: g(line, "graph", p, "eigh_per_s") for p in ("f32_refined", "f64")},
           "c2_speedup": line.get("speedup_f32refined_vs_f64"),
           "c2_refined_accuracy_all_matrices": g(line, "graph", "f32_refined", "accuracy"),
           "c2_e2e_eigh_per_s": g(line, "e2e", "value"),
           "c2_cpu_port_eigh_per_s": g(line, "cpu_baseline", "value")}
    large = line.get("large") or {}
    for key, r in large.items():
        acc = g(r, "f32_refined", "accuracy") or {}
        out[key] = {"f64_ms": g(r, "f64", "ms"), "refined_ms": g(r, "f32_refined", "ms"),
                    "speedup": r.get("speedup_f32refined_vs_f64"), "cusolver_f64_ms": g(r, "cusolver_f64", "ms"),
                    "refined_max_err": max([v for v in acc.values() if v is not None], default=None),
                    "refined_meets_1e13": r.get("refined_meets_1e13")}
    c1 = line.get("c1_single_n64") or {}
    out["c1_n64"] = {"gpu_us": c1.get("gpu_us_per_solve"), "cpu_1core_us": c1.get("cpu_oracle_us_per_solve_1core"),
                     "refined_route_us": g(c1, "refined_route", "us_per_solve")}
    c4 = line.get("c4_forward_adjoint") or {}
    if c4:
        out["c4_graph_speedup"] = (g(c4, "f32_refined", "graph_matrices_per_s") or 0) / max(
            g(c4, "f64", "graph_matrices_per_s") or 1e-30, 1e-30)
    c5 = line.get("c5_mixed_forward_adjoint") or {}
    if c5:
        out["c5_speedup"] = c5.get("speedup_f32refined_vs_f64")
    return out


def summary_lines(sm):
    """The summary as short plain-text lines printed after the JSON line."""
    lines = ["# summary: " + json.dumps({k: v for k, v in sm.items() if not k.startswith("n")})]
    for k, v in sm.items():
        if k.startswith("n") and isinstance(v, dict):
            lines.append(f"# {k}: " + json.dumps(v))
    return lines


def run_c4(torch, glagpu, dev, reps=3):
    """Differentiation workload: 1024 symmetric matrices, n ~ U{32..96}
    (seed 4), Q diag(lam) Q' with lam sorted on [-1, 1] and gaps >= 1e-3;
    one step = forward eigen-decomposition + adjoint with cotangents
    w, C ~ N(0, 1). Matrices per second, FP64 and FP32+refinement forward,
    run eagerly and as one captured CUDA graph (Plan.capture_step)."""
    from helpers import gapped_spectrum, prescribed
    rng = np.random.default_rng(4)
    ns = rng.integers(32, 97, size=1024)
    mats = [prescribed(gapped_spectrum(int(n), rng), int(rng.integers(1 << 30))) for n in ns]
    out = {}
    for path in ("f64", "f32_refined"):
        plan = glagpu.Plan(ns, precision=path)
        A = plan.pack(mats, device=dev)
        w = torch.empty(plan.w_elems, dtype=torch.float64, device=dev)
        V = torch.empty(plan.a_elems, dtype=torch.float64, device=dev)
        info = torch.zeros(len(ns), dtype=torch.int32, device=dev)
        wbar = torch.randn(plan.w_elems, dtype=torch.float64, device=dev)
        Vbar = torch.randn(plan.a_elems, dtype=torch.float64, device=dev)
        Abar = torch.empty_like(V)
        for _ in range(3):
            plan.execute(A, w, V, info)
            plan.adjoint(w, V, wbar, Vbar, Abar)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            plan.execute(A, w, V, info)
            plan.adjoint(w, V, wbar, Vbar, Abar)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        e0.record()
        for _ in range(reps):
            plan.adjoint(w, V, wbar, Vbar, Abar)
        e1.record()
        e1.synchronize()
        out[path] = {"matrices_per_s": len(ns) / (ms * 1e-3), "ms_per_step": ms,
                     "adjoint_ms": e0.elapsed_time(e1) / reps, "info_nonzero": int((info.cpu() != 0).sum())}
        plan.close()
        # the same step, forward plus adjoint, captured in one CUDA graph
        gplan = glagpu.Plan(ns, precision=path, graph=True)
        Ag = gplan.pack(mats, device=dev)
        wg, Vg, Abg = torch.empty_like(w), torch.empty_like(V), torch.empty_like(Abar)
        infog = torch.zeros_like(info)
        g = gplan.capture_step(Ag, wg, Vg, infog, wbar, Vbar, Abg)
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            g.replay()
        e1.record()
        e1.synchronize()
        gms = e0.elapsed_time(e1) / reps
        out[path].update({"graph_matrices_per_s": len(ns) / (gms * 1e-3), "graph_ms_per_step": gms,
                          "graph_info_nonzero": int((infog.cpu() != 0).sum()),
                          "graph_equals_eager": bool(torch.equal(wg, w) and torch.equal(Vg, V)
                                                     and torch.equal(Abg, Abar))})
        gplan.close()
    return out


def run_c1(torch, glagpu, dev, reps=200):
    """Single matrix: eigen!(Hermitian(A)) FP64, n = 64 GOE (seed 1), through
    gla_dsyev (device pointers; it synchronizes to return info: the
    reference's algorithm in FP64, whose QL chase is one serial FP64 chain)
    and through a one-matrix FP32 + refinement plan (FP64-accurate results).
    Latency per solve on the GPU beside one host core running the oracle
    port, and the error of both against the oracle and the 256-bit values."""
    import ctypes
    import glagpu._lib as L
    from helpers import goe, orth, residual
    from oracle import oracle as O
    lib = L.load()
    n = 64
    A0 = goe(n, 1)
    Ad = torch.tensor(A0.ravel(order="F"), device=dev)
    A = torch.empty_like(Ad)
    w = torch.empty(n, dtype=torch.float64, device=dev)
    info = ctypes.c_int(0)
    call = lambda: L.check(lib.gla_dsyev(b"V", b"L", n, ctypes.c_void_p(A.data_ptr()), n, ctypes.c_void_p(w.data_ptr()),
                                         ctypes.byref(info), None), "gla_dsyev")
    for _ in range(5):
        A.copy_(Ad)
        call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        A.copy_(Ad)
        call()
    torch.cuda.synchronize()
    gpu_us = (time.perf_counter() - t0) / reps * 1e6
    V = A.cpu().numpy().reshape(n, n).T
    wh = w.cpu().numpy()
    wo, _, _ = O.syev(A0)
    t0 = time.perf_counter()
    k = 0
    while time.perf_counter() - t0 < 1.0:
        O.syev(A0)
        k += 1
    cpu_us = (time.perf_counter() - t0) / k * 1e6
    # the same matrix through the FP32 + refinement route (FP64-accurate
    # results): a one-matrix plan, device buffers, info read back each call
    plan = glagpu.Plan([n], precision="f32_refined")
    wr = torch.empty(n, dtype=torch.float64, device=dev)
    Vr = torch.empty(n * n, dtype=torch.float64, device=dev)
    infor = torch.zeros(1, dtype=torch.int32, device=dev)
    for _ in range(5):
        plan.execute(Ad, wr, Vr, infor)
        int(infor.item())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        plan.execute(Ad, wr, Vr, infor)
        int(infor.item())
    ref_us = (time.perf_counter() - t0) / reps * 1e6
    Vh = Vr.cpu().numpy().reshape(n, n, order="F")
    wrh = wr.cpu().numpy()
    plan.close()
    out = {"n": n, "gpu_us_per_solve": gpu_us, "cpu_oracle_us_per_solve_1core": cpu_us,
           "timing": "host wall clock per gla_dsyev call (copy-in of A, solve, info read), mean of %d" % reps,
           "accuracy": {"residual": residual(A0, V, wh), "orthogonality": orth(V),
                        "eig_err_vs_oracle": float(np.abs(wh - wo).max())}, "info": int(info.value),
           "refined_route": {"us_per_solve": ref_us, "info": int(infor.item()),
                             "timing": "host wall clock per one-matrix FP32 + refinement plan execute "
                                       "(device buffers, info read back), mean of %d" % reps,
                             "accuracy": {"residual": residual(A0, Vh, wrh), "orthogonality": orth(Vh),
                                          "eig_err_vs_oracle": float(np.abs(wrh - wo).max())}}}
    try:  # the 256-bit eigenvalues of this exact input (tests/golden/golden_large.json)
        from helpers import golden_large
        A256, w256, _, _ = golden_large(n)
        if np.array_equal(A256, A0):
            out["eig_err_vs_256bit"] = float(np.abs(wh - w256).max())
            out["refined_route"]["eig_err_vs_256bit"] = float(np.abs(wrh - w256).max())
    except Exception:
        pass
    return out


def c5_workload():
    """Mixed workload: 256 symmetric matrices, n log-uniform in [16, 1024]
    (seed 5); even indices GOE, odd indices Q diag(lam) Q' with Q Haar and
    lam = +-logspace(-8, 0, n) with random signs (cond 1e8)."""
    from helpers import goe, prescribed
    rng = np.random.default_rng(5)
    ns = np.exp(rng.uniform(np.log(16), np.log(1024), size=256)).round().astype(np.int64)
    mats, lams = [], []
    for i, n in enumerate(ns):
        n = int(n)
        if i % 2 == 0:
            mats.append(goe(n, 5000 + i))
            lams.append(None)
        else:
            lam = np.logspace(-8, 0, n) * rng.choice([-1.0, 1.0], n)
            mats.append(prescribed(lam, 5000 + i))
            lams.append(np.sort(lam))
    return ns, mats, lams


def run_c5(torch, glagpu, dev, reps=2):
    """Mixed workload (c5_workload): one step = forward eigen-decomposition of
    all 256 matrices (one plan: orders <= 128 batched, larger ones by the
    blocked path) + adjoint with cotangents ~ N(0, 1). Matrices per second for
    FP64 and FP32 + refinement, accuracy over every matrix, and the HBM
    footprint of the step (device memory taken by the arenas and the plan's
    workspace, from cudaMemGetInfo). The step is not graph-captured: the
    blocked path reads convergence and cluster decisions on the host."""
    from helpers import orth, residual
    ns, mats, lams = c5_workload()
    out = {"workload": "256 symmetric matrices, n log-uniform [16, 1024] (seed 5), half GOE, half prescribed "
                       "spectrum +-logspace(-8, 0) (cond 1e8); forward + adjoint",
           "sum_n3": float((ns.astype(np.float64) ** 3).sum()), "orders_above_128": int((ns > 128).sum())}
    for path in ("f64", "f32_refined"):
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        free0 = torch.cuda.mem_get_info()[0]
        plan = glagpu.Plan(ns, precision=path)
        A = plan.pack(mats, device=dev)
        w = torch.empty(plan.w_elems, dtype=torch.float64, device=dev)
        V = torch.empty(plan.a_elems, dtype=torch.float64, device=dev)
        info = torch.zeros(len(ns), dtype=torch.int32, device=dev)
        g = torch.Generator(device="cpu").manual_seed(55)
        wbar = torch.randn(plan.w_elems, generator=g, dtype=torch.float64).to(dev)
        Vbar = torch.randn(plan.a_elems, generator=g, dtype=torch.float64).to(dev)
        Abar = torch.empty_like(V)
        plan.execute(A, w, V, info)
        plan.adjoint(w, V, wbar, Vbar, Abar)
        torch.cuda.synchronize()
        footprint = free0 - torch.cuda.mem_get_info()[0]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            plan.execute(A, w, V, info)
            plan.adjoint(w, V, wbar, Vbar, Abar)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        e0.record()
        plan.adjoint(w, V, wbar, Vbar, Abar)
        e1.record()
        e1.synchronize()
        adj_ms = e0.elapsed_time(e1)
        ws_, Vs_ = plan.unpack(w.cpu().numpy(), V.cpu().numpy())
        res = ort = eig = 0.0
        for Am, wg, Vg, lam in zip(mats, ws_, Vs_, lams):
            nA = max(np.linalg.norm(Am, 2), 1e-300)
            res = max(res, residual(Am, Vg, wg))
            ort = max(ort, orth(Vg))
            if lam is not None:
                eig = max(eig, float(np.abs(wg - lam).max()) / nA)
        out[path] = {"matrices_per_s": len(ns) / (ms * 1e-3), "ms_per_step": ms, "adjoint_ms": adj_ms,
                     "hbm_footprint_bytes": int(footprint), "info_nonzero": int((info.cpu() != 0).sum()),
                     "accuracy": {"max_residual": res, "max_orthogonality": ort,
                                  "max_eig_err_vs_prescribed": eig}}
        plan.close()
        del A, w, V, info, wbar, Vbar, Abar
    out["speedup_f32refined_vs_f64"] = out["f64"]["ms_per_step"] / out["f32_refined"]["ms_per_step"]
    return out


def large_roofline(large, peaks):
    """The tcgen05 Ozaki GEMM (double-float products of the n = 4096 refinement):
    bf16 tensor throughput against the measured bf16 peak (burst)."""
    if not large:
        return None
    oz = large.get("n4096_goe", {}).get("ozaki_gemm")
    if not oz:
        return None
    pk = peaks.get("bf16_tflops")
    src = "MEASURED_PEAKS.json bf16_tflops (burst)"
    if not pk:
        pk, src = 1900.0, "fallback 1.9 PFLOP/s bf16 (MEASURED_PEAKS.json absent)"
    return {"kernel": "oz::k_oz_gemm", "bound": "tensor", "achieved": oz["bf16_tflops"], "peak": pk,
            "unit": "TFLOP/s", "frac": oz["bf16_tflops"] / pk, "traffic": None, "peak_source": src,
            "fp64_equivalent_tflops": oz["fp64_equivalent_tflops"]}


def large_case(kind, n):
    """Single large matrix: 'c3' = Q diag(lam) Q', Q Haar (seed 3), lam = +-logspace(-6, 0, n)
    with random signs (cond 1e6); 'goe' = (B + B')/2, seed 4."""
    from helpers import goe, prescribed
    if kind == "c3":
        rng = np.random.default_rng(3)
        lam = np.logspace(-6, 0, n) * rng.choice([-1.0, 1.0], n)
        return prescribed(lam, 3), np.sort(lam)
    return goe(n, 4), None


def run_large(torch, glagpu, dev, reps=2):
    """Single-matrix solves (the large half of the headline metric): the
    precision workload at n = 2048 and n = 4096 and a GOE n = 4096, plain
    FP64 GPU path vs FP32 solve + refinement, time per solve (CUDA events;
    each execute synchronises), accuracy of every result."""
    out = {}
    for kind, n in (("c3", 2048), ("c3", 4096), ("goe", 4096)):
        A, lam = large_case(kind, n)
        nA = np.linalg.norm(A, 2) if lam is None else np.abs(lam).max()
        dA = torch.from_numpy(A.ravel(order="F").copy()).to(dev)
        res = {}
        wref = None
        for path in ("f64", "f32_refined"):
            plan = glagpu.Plan([n], precision=path, timing=True)
            w = torch.empty(n, dtype=torch.float64, device=dev)
            V = torch.empty(n * n, dtype=torch.float64, device=dev)
            info = torch.zeros(1, dtype=torch.int32, device=dev)
            plan.execute(dA, w, V, info)  # warm-up (first-touch of the plan)
            torch.cuda.synchronize()
            best = 1e30
            phases = None
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                plan.execute(dA, w, V, info)
                e1.record()
                e1.synchronize()
                t = e0.elapsed_time(e1)
                if t < best:
                    best, phases = t, plan.phase_times()
            iters = plan.stats()["refine_n3"] / float(n) ** 3
            wh = w.cpu().numpy()
            Vh = V.cpu().numpy().reshape(n, n, order="F")
            R = A @ Vh - Vh * wh
            acc = {"residual": float(np.linalg.norm(R, 2) / nA),
                   "orthogonality": float(np.linalg.norm(Vh.T @ Vh - np.eye(n), 2))}
            if lam is not None:
                acc["eig_err_vs_exact"] = float(np.abs(wh - lam).max() / nA)
            elif wref is not None:
                acc["eig_err_vs_f64_gpu"] = float(np.abs(wh - wref).max() / nA)
            if path == "f64":
                wref = wh
            res[path] = {"ms": best, "phases_ms": phases, "info": int(info.item()), "accuracy": acc,
                         "refine_iterations": iters}
            plan.close()
            del w, V
        res["speedup_f32refined_vs_f64"] = res["f64"]["ms"] / res["f32_refined"]["ms"]
        res["cusolver_f64"] = cusolver_single(torch, dA.view(n, n), lam, nA)
        # the tensor-core Ozaki GEMM of the refinement, timed alone on this order
        if kind == "goe":
            res["ozaki_gemm"] = time_ozaki(torch, glagpu, dev, n)
        ok = res["f32_refined"]["info"] == 0 and all(
            v <= 1e-13 for k, v in res["f32_refined"]["accuracy"].items() if k != "orthogonality")
        res["refined_meets_1e13"] = bool(ok)
        out[f"n{n}_{kind}"] = res
    return out


def cusolver_single(torch, A, lam, nA, reps=2):
    """Side comparator for the FP64 denominator, reported only: torch.linalg.eigh
    (NVIDIA cuSOLVER) on the same FP64 matrix, best of reps after a warm-up.
    The product never calls it."""
    try:
        At = A.t().contiguous()
        w, V = torch.linalg.eigh(At)
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            w, V = torch.linalg.eigh(At)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out = {"ms": best, "what": "torch.linalg.eigh FP64 (cuSOLVER), side comparator only"}
        if lam is not None:
            out["eig_err_vs_exact"] = float((w.cpu().numpy() - lam).__abs__().max() / nA)
        return out
    except Exception as e:  # a side number: report, never fail the benchmark
        return {"unavailable": f"{type(e).__name__}: {str(e)[:120]}"}


def cusolver_batched(torch, ns, mats, dev, reps=3):
    """Side comparator for the batched FP64 path, reported only: the workload
    grouped by order and solved with torch.linalg.eigh on stacked FP64 tensors
    (cuSOLVER's batched routines), inputs resident, CUDA events around all
    groups. The product never calls it."""
    try:
        groups = []
        for n in np.unique(ns):
            idx = np.nonzero(ns == n)[0]
            groups.append(torch.tensor(np.stack([mats[b] for b in idx]), dtype=torch.float64, device=dev))
        for g in groups:
            torch.linalg.eigh(g)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            for g in groups:
                torch.linalg.eigh(g)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        return {"eigh_per_s": len(ns) / (ms * 1e-3), "ms_per_step": ms, "launch_groups": len(groups),
                "what": "torch.linalg.eigh FP64 per order group (cuSOLVER), side comparator only"}
    except Exception as e:
        return {"unavailable": f"{type(e).__name__}: {str(e)[:120]}"}


def time_ozaki(torch, glagpu, dev, n, reps=5):
    """C = A X (n x n x n) to double-float accuracy through gla_gemm_df (the
    refinement's tcgen05 Ozaki GEMM): 28 bf16 slice products per multiply."""
    import glagpu._lib as L
    lib = L.load()
    g = torch.Generator(device="cpu").manual_seed(5)
    Ah = torch.randn(n, n, generator=g).to(dev)
    Al = (torch.randn(n, n, generator=g) * 2.0 ** -25).to(dev)
    Bh = torch.randn(n, n, generator=g).to(dev)
    Bl = (torch.randn(n, n, generator=g) * 2.0 ** -25).to(dev)
    Ch = torch.empty(n, n, device=dev)
    Cl = torch.empty(n, n, device=dev)
    ptr = lambda t: __import__("ctypes").c_void_p(t.data_ptr())
    call = lambda: L.check(lib.gla_gemm_df(n, n, n, ptr(Ah), ptr(Al), n, ptr(Bh), ptr(Bl), n, ptr(Ch), ptr(Cl), n,
                                           None), "gla_gemm_df")
    call()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    # each call: slicing kernels, then the GEMM kernel; the library records
    # stream events around both parts (gla_gemm_df_last_ms), so the kernel's
    # own average duration comes from the same timed calls
    import ctypes
    sl, gm = ctypes.c_float(0), ctypes.c_float(0)
    e0.record()
    kern = []
    for _ in range(reps):
        call()
        L.check(lib.gla_gemm_df_last_ms(ctypes.byref(sl), ctypes.byref(gm)), "gla_gemm_df_last_ms")
        kern.append(gm.value)
    e1.record()
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    kms = sum(kern) / len(kern)
    bf16_flops = 28 * 2.0 * n ** 3
    return {"ms_with_slicing": ms, "ms": kms, "bf16_tflops": bf16_flops / (kms * 1e-3) / 1e12,
            "fp64_equivalent_tflops": 2.0 * n ** 3 / (kms * 1e-3) / 1e12,
            "fp64_equivalent_tflops_with_slicing": 2.0 * n ** 3 / (ms * 1e-3) / 1e12,
            "timing": "k_oz_gemm alone: CUDA events around the kernel launch inside gla_gemm_df, mean of %d "
                      "calls on %d x %d float-pair operands" % (reps, n, n)}


def plan_buckets(ns):
    """Size buckets of width 16 that the plan creates (one stream each)."""
    return [i for i in range(8) if ((ns > 16 * i) & (ns <= 16 * (i + 1))).any()]


def cpu_baseline(ns, mats, budget_s=15.0):
    """The reference algorithm (CPU restatement, oracle/) on all host cores,
    one matrix per OpenMP thread, over a bounded sample of the workload."""
    from oracle import oracle as O
    nth = os.cpu_count() or 1
    # sample the first m matrices so that the run takes about budget_s
    m = min(len(ns), 256)
    t = time_oracle(ns[:m], mats[:m], nth)
    per = t / m
    m2 = int(min(len(ns), max(m, budget_s / max(per, 1e-9))))
    if m2 > m:
        t = time_oracle(ns[:m2], mats[:m2], nth)
        m = m2
    return {"value": m / t, "unit": "eigh/s", "cores": nth, "kind": "port",
            "sample": f"first {m} of the {len(ns)} workload matrices, eigen!(Hermitian) FP64, "
                      f"{nth} OpenMP threads (one matrix per thread)"}


def lapack_child(m):
    """Body of `bench.py --cpu-lapack M`, run in a fresh process whose
    environment pins BLAS to one thread: scipy.linalg.eigh (LAPACK dsyevr,
    the routine stdlib Julia's Float64 eigen(Hermitian) calls) over the first
    M workload matrices, one forked worker per core (this process holds no
    GPU context), wall time from a common start barrier to the last worker's
    end. Every wait is bounded. Prints one JSON object."""
    import multiprocessing as mp

    import scipy
    import scipy.linalg as sl
    ns, mats = workload()
    sample = mats[:m]
    nth = os.cpu_count() or 1
    ctx = mp.get_context("fork")
    barrier = ctx.Barrier(nth)
    q = ctx.Queue()

    def work(i):
        part = sample[i::nth]
        if part:
            sl.eigh(part[0], driver="evr", check_finite=False)  # load LAPACK before the clock starts
        barrier.wait(timeout=120)
        t0 = time.monotonic()
        for M in part:
            sl.eigh(M, driver="evr", check_finite=False)
        q.put((t0, time.monotonic()))

    procs = [ctx.Process(target=work, args=(i,), daemon=True) for i in range(nth)]
    for p in procs:
        p.start()
    try:
        spans = [q.get(timeout=240) for _ in procs]
    finally:
        for p in procs:
            p.join(timeout=5)
            if p.is_alive():
                p.terminate()
    wall = max(b for _, b in spans) - min(a for a, _ in spans)
    print(json.dumps({"value": m / wall, "unit": "eigh/s", "cores": nth, "kind": "lapack",
                      "sample": f"first {m} of the {len(ns)} workload matrices, scipy {scipy.__version__} "
                                f"linalg.eigh (LAPACK dsyevr, eigenvalues and vectors), {nth} processes x "
                                "1 BLAS thread"}), flush=True)


def lapack_baseline(ns, mats, budget_s=5.0):
    """LAPACK on the host cores (see lapack_child), in a subprocess with a
    time limit; a sample sized for about budget_s seconds of work. Returns
    the child's JSON object, or {"unavailable": reason}."""
    try:
        import scipy.linalg as sl
        nth = os.cpu_count() or 1
        k = min(len(mats), 64)
        t0 = time.perf_counter()
        for M in mats[:k]:
            sl.eigh(M, driver="evr", check_finite=False)
        per = (time.perf_counter() - t0) / max(k, 1)
        m = int(min(len(ns), max(k, budget_s * nth / max(per, 1e-9))))
        env = dict(os.environ, OPENBLAS_NUM_THREADS="1", OMP_NUM_THREADS="1", MKL_NUM_THREADS="1")
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-lapack", str(m)], env=env,
                           capture_output=True, text=True, timeout=300)
        if r.returncode != 0:
            return {"unavailable": f"LAPACK baseline process exited {r.returncode}: {r.stderr.strip()[-200:]}"}
        return json.loads(r.stdout.strip().splitlines()[-1])
    except Exception as e:  # a side baseline: report, never fail the benchmark
        return {"unavailable": f"LAPACK baseline failed: {type(e).__name__}"}


def time_oracle(ns, mats, nth):
    from oracle import oracle as O
    aoff = np.concatenate([[0], np.cumsum(ns * ns)[:-1]]).astype(np.int64)
    woff = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    A = pack_f(mats)
    w = np.zeros(int(ns.sum()))
    V = np.zeros(len(A))
    info = np.zeros(len(ns), np.int32)
    Ac = A.copy()
    O.batched_raw("V", "L", np.ascontiguousarray(ns), aoff, Ac, w, woff, V, info, nthreads=nth)  # warm
    Ac = A.copy()
    t0 = time.perf_counter()
    O.batched_raw("V", "L", np.ascontiguousarray(ns), aoff, Ac, w, woff, V, info, nthreads=nth)
    return time.perf_counter() - t0


def julia_probe():
    """Whether this host has Julia (the reference itself could then be timed);
    recorded in the JSON line."""
    import shutil
    exe = shutil.which("julia")
    if not exe:
        return {"julia": None, "note": "julia not on PATH: the reference arm is the CPU restatement"}
    try:
        r = subprocess.run([exe, "--version"], capture_output=True, text=True, timeout=60)
        return {"julia": exe, "version": r.stdout.strip()}
    except Exception as e:
        return {"julia": exe, "version": None, "error": type(e).__name__}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    ns, mats = workload()
    nth = os.cpu_count() or 1
    # each step: the whole 4096-matrix workload, one matrix per OpenMP thread
    m = len(ns)
    for _ in range(args.warmup):
        time_oracle(ns[:m], mats[:m], nth)
    tot = 0.0
    for _ in range(args.steps):
        tot += time_oracle(ns[:m], mats[:m], nth)
    val = m * args.steps / tot
    line = {
        "metric": METRIC, "value": val, "unit": "eigh/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded GOE)", "impl": "reference",
        "config": {"workload": f"batched eigen!(Hermitian): {len(ns)} GOE matrices, n~U[{NLO},{NHI}], seed {SEED}",
                   "path": "reference CPU", "batch": len(ns)},
        "cpu_baseline": {"value": val, "unit": "eigh/s", "cores": nth, "kind": "port",
                         "sample": f"all {m} matrices of the workload per step; CPU restatement of "
                                   "GenericLinearAlgebra.jl eigen!(Hermitian), "
                                   f"{nth} OpenMP threads (one matrix per thread)"},
        "e2e": {"value": val, "unit": "eigh/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "julia_probe": julia_probe(),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=BATCH, help="matrices in the batch (profiling: smaller cases)")
    ap.add_argument("--paths", default="f64,f32,f32_refined", help="paths to time (profiling)")
    ap.add_argument("--profile", action="store_true", help="profiling run: time the paths only, print nothing")
    ap.add_argument("--nrange", default="", help="profiling: keep matrices with lo <= n <= hi, as 'lo,hi'")
    ap.add_argument("--no-large", action="store_true", help="skip the n = 4096 single-matrix section")
    ap.add_argument("--no-autotune", action="store_true", help="fixed launch shapes instead of the autotuner's")
    ap.add_argument("--solve", type=int, default=0,
                    help="profiling: two solves of one GOE matrix of this order on the first of --paths")
    ap.add_argument("--c3-solve", type=int, default=0, metavar="N",
                    help="profiling: two FP32 + refinement solves of the cond-1e6 matrix of order N only")
    ap.add_argument("--c4", action="store_true",
                    help="only the differentiation workload (forward + adjoint, eager and one CUDA graph)")
    ap.add_argument("--cpu-lapack", type=int, default=0,
                    help="internal: the LAPACK CPU baseline over the first N workload matrices (one JSON object)")
    ap.add_argument("--ozaki", type=int, default=0,
                    help="profiling: time only the tensor-core double-float GEMM (gla_gemm_df) at this order")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.ozaki:
        import torch
        import glagpu
        print(json.dumps(time_ozaki(torch, glagpu, "cuda", args.ozaki)), flush=True)
        return
    if args.cpu_lapack:
        lapack_child(args.cpu_lapack)
        return
    if args.c4:
        import torch
        import glagpu
        print(json.dumps(run_c4(torch, glagpu, "cuda")), flush=True)
        return
    if args.solve:
        # profiling: two solves of one GOE matrix (seed 1) of order args.solve
        # on the first path of --paths
        import torch
        import glagpu
        from helpers import goe
        prec = args.paths.split(",")[0]
        n = args.solve
        plan = glagpu.Plan([n], precision=prec)
        dt = torch.float32 if prec == "f32" else torch.float64
        Ad = plan.pack([goe(n, 1)], device="cuda").to(dt)
        w = torch.empty(n, dtype=dt, device="cuda")
        V = torch.empty(n * n, dtype=dt, device="cuda")
        info = torch.zeros(1, dtype=torch.int32, device="cuda")
        for _ in range(2):
            plan.execute(Ad, w, V, info)
        torch.cuda.synchronize()
        print(json.dumps({"n": n, "path": prec, "info": int(info.item())}), flush=True)
        return
    if args.c3_solve:
        # profiling: two FP32 + refinement solves of the cond-1e6 matrix of order N
        import torch
        import glagpu
        N = args.c3_solve
        A, lam = large_case("c3", N)
        plan = glagpu.Plan([N], precision="f32_refined")
        Ad = plan.pack([A], device="cuda")
        w = torch.empty(N, dtype=torch.float64, device="cuda")
        V = torch.empty(N * N, dtype=torch.float64, device="cuda")
        info = torch.zeros(1, dtype=torch.int32, device="cuda")
        for _ in range(2):
            plan.execute(Ad, w, V, info)
        torch.cuda.synchronize()
        print(json.dumps({"info": int(info.item()), "eig_err": float(np.abs(w.cpu().numpy() - lam).max())}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
