#!/usr/bin/env python
"""Benchmark: sound-soft scattering solves/s on one GB300 (replicas per GPU).

Workload (default, `kite2048`): kite curve x(t) = (cos t + 0.65 cos 2t - 0.65,
1.5 sin t), N = 2048 piecewise constants equispaced in t, k = 100, plane wave
at the angle U[0, 2pi) drawn from numpy's default_rng(0), combined operator
1/2 I + D' - i k S (eta = k), QuadOption {L=3, N=5, sigma=0.15}.

One step = one SoundSoftScattering::Discretize() + Solve() through the C ABI
(bem2d_scattering_solve): FP64 assembly of A = Id + 2K and b, complex64 LU
with partial pivoting, FP64 iterative refinement to backward error 1e-12
(`mixed`).  The same step with a complex128 LU (`fp64`) is timed beside it
(the plain FP64 GPU path).  Synthetic input: the geometry is generated, no
dataset is read.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Under torchrun each rank runs an independent
replica (no collective on the data path) and value = total solves/s.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

QUAD = (3, 5, 0.15)


def workload(name):
    from bem2d_gb300 import geometry as G
    if name == "kite2048":
        th = float(np.random.default_rng(0).uniform(0, 2 * math.pi))
        g = G.kite(2048).add_poly_basis(0)
        return dict(g=g, k=100.0, eta=100.0, d=(math.cos(th), math.sin(th)),
                    desc="kite N=2048 equispaced, k=100, eta=k, plane wave angle "
                         "%.15g (rng seed 0), QuadOption{3,5,0.15}" % th)
    if name == "kite4096":
        th = float(np.random.default_rng(0).uniform(0, 2 * math.pi))
        g = G.kite(4096).add_poly_basis(0)
        return dict(g=g, k=100.0, eta=100.0, d=(math.cos(th), math.sin(th)),
                    desc="kite N=4096 equispaced, k=100, eta=k (profiling case)")
    if name == "disk160":
        g = G.curve_equispaced(G.CIRCLE, 160).add_poly_basis(0)
        return dict(g=g, k=10.0, eta=10.0, d=(1.0, 0.0),
                    desc="unit disk 160 equal-arc elements, k=10, d=(1,0)")
    raise SystemExit("unknown workload " + name)


def evals_per_matrix(n):
    """Kernel evaluations of one closed-curve P0 matrix with L=3, N=5:
    25 (N^2 - 3N) far + 225 * 2N neighbour + 450 * N self."""
    return 25 * (n * n - 3 * n) + 225 * 2 * n + 450 * n


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def clocks_start(path):
    try:
        f = open(path, "w")
        p = subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
            stdout=f, stderr=subprocess.DEVNULL)
        return p, f
    except (OSError, FileNotFoundError):
        return None, None


def clocks_stop(p, f, path, gpu_index):
    if p is None:
        return None
    p.terminate()
    try:
        p.wait(timeout=5)
    except subprocess.TimeoutExpired:
        p.kill()
    f.close()
    sm, smax, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9 or parts[0] != str(gpu_index):
            continue
        try:
            sm.append(float(parts[1]))
            smax = max(smax, float(parts[2]))
        except ValueError:
            continue
        for nm, v in zip(names, parts[5:9]):
            if v.lower() == "active":
                reasons.add(nm)
    if not sm:
        return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
            "samples": len(sm)}


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def cpu_reference(w, steps, warmup, threads):
    """The oracle (C restatement of the reference's assembly + LAPACK zgetrf /
    zgetrs through scipy) on the host cores: returns (seconds per solve list,
    x of the last solve)."""
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    from oracle import oracle as O
    from bem2d_gb300 import _build
    _build.build_oracle(with_reference=False)
    times, x = [], None
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        A, b = O.system(w["g"], w["k"], w["d"], w["eta"], QUAD, threads=threads)
        x = O.solve(A, b)
        t1 = time.perf_counter()
        if i >= warmup:
            times.append(t1 - t0)
    return times, x


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    w = workload(args.workload)
    threads = os.cpu_count() or 1
    times, _ = cpu_reference(w, args.steps, args.warmup, threads)
    v = len(times) / sum(times)
    print(json.dumps({
        "impl": "reference", "metric": "solves/s", "value": v, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w["desc"]},
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": "full assemble + LU solve per step (oracle restatement "
                                   "of the reference + scipy LAPACK zgetrf/zgetrs)"},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


def run_only(args):
    """Profiling driver: one phase only (assembly or solve), no JSON line."""
    import torch
    from bem2d_gb300 import capi
    w = workload(args.workload)
    n = w["g"].n_unknowns
    arrays = w["g"].arrays()
    ctx = capi.Context(0)
    ctx.enable_timers(True)
    A = torch.empty((n, n), dtype=torch.complex128, device="cuda")
    x = torch.zeros(n, dtype=torch.complex128, device="cuda")
    for _ in range(args.warmup + args.steps):
        if args.only == "assembly":
            ctx.discrete_kernel(arrays, "combined", w["k"], w["eta"], QUAD, 2.0, 1.0, out=A)
        else:
            ctx.scattering_solve(arrays, w["k"], w["d"], w["eta"], QUAD,
                                 precision=args.only, out=x)
    torch.cuda.synchronize()
    print(json.dumps({"only": args.only, "workload": args.workload,
                      "timers_ms": {k: v[0] / max(v[1], 1) for k, v in ctx.timers().items()}}))


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from bem2d_gb300 import capi
    w = workload(args.workload)
    g = w["g"]
    n = g.n_unknowns
    ctx = capi.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    x_dev = torch.zeros(n, dtype=torch.complex128, device="cuda")
    x_host = torch.zeros(n, dtype=torch.complex128).pin_memory()
    arrays = g.arrays()
    h2d = sum(a.nbytes for a in arrays.values())

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def timed(fn, k, warm):
        for _ in range(warm):
            fn()
        barrier()
        ms = []
        for _ in range(k):
            flush.zero_()  # L2 flush, outside the timed events
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record()
            fn()
            with torch.cuda.stream(stream):
                e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        barrier()
        return ms

    def step(prec, out):
        return lambda: ctx.scattering_solve(arrays, w["k"], w["d"], w["eta"], QUAD,
                                            precision=prec, out=out)

    # -- headline: mixed path, device-resident result -------------------------
    clk_path = os.path.join(ROOT, "gpurun_out" if os.path.isdir(os.path.join(ROOT, "gpurun_out"))
                            else "_build", "bench_clocks_%d.csv" % rank)
    os.makedirs(os.path.dirname(clk_path), exist_ok=True)
    cp, cf = clocks_start(clk_path)
    l0 = ctx.launches
    ms_mixed = timed(step("mixed", x_dev), args.steps, args.warmup)
    launches = (ctx.launches - l0) // (args.steps + args.warmup) * args.steps
    clocks = clocks_stop(cp, cf, clk_path, local)
    info_mixed = ctx.last_info
    # -- e2e: host result (device -> host copy inside the timed region) -------
    ms_e2e = timed(step("mixed", x_host.numpy()), args.steps, 1)
    # -- plain FP64 GPU path ---------------------------------------------------
    ms_fp64 = timed(step("fp64", x_dev), max(2, args.steps // 2), 1)
    # -- phase breakdown (events around each phase) ---------------------------
    ctx.enable_timers(True)
    step("mixed", x_dev)()
    ph_mixed = ctx.timers()
    ctx.enable_timers(True)
    step("fp64", x_dev)()
    ph_fp64 = ctx.timers()
    ctx.enable_timers(False)
    # -- roofline of the dominant kernel (FP64 far-field assembly) ------------
    ctx.enable_timers(True)
    A_dev = torch.empty((n, n), dtype=torch.complex128, device="cuda")
    for _ in range(3):
        ctx.discrete_kernel(arrays, "combined", w["k"], w["eta"], QUAD, 2.0, 1.0, out=A_dev)
    far_ms, far_n = ctx.timers()["far"]
    near_ms, near_n = ctx.timers()["near"]
    ctx.enable_timers(False)
    far_ms /= max(far_n, 1)
    near_ms /= max(near_n, 1)
    fp64_peak = capi.fma_peak("fp64")
    flops_far = 100.0 * 25 * (n * n - 3 * n)
    achieved = flops_far / (far_ms * 1e-3) / 1e12

    t_mixed = sum(ms_mixed) / len(ms_mixed)
    t_e2e = sum(ms_e2e) / len(ms_e2e)
    t_fp64 = sum(ms_fp64) / len(ms_fp64)
    per_rank = np.array([t_mixed, t_e2e, t_fp64])
    if ws > 1:
        t = torch.tensor(per_rank, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        per_rank = t.cpu().numpy()
    t_mixed, t_e2e, t_fp64 = per_rank
    if rank != 0:
        return
    res = {
        "metric": "solves/s", "value": ws * 1e3 / t_mixed, "unit": "solves/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_mixed,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 assembly + c64 LU + f64 refinement", "data": "synthetic",
        "config": {"workload": w["desc"], "n_unknowns": n, "precision": "mixed",
                   "l2": "256 MB write between timed steps, outside the step events",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": ws * 1e3 / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 16 * n},
        "gpu_launches": int(launches),
        "plain_fp64": {"value": ws * 1e3 / t_fp64, "unit": "solves/s", "ms_per_step": t_fp64},
        "mixed_over_fp64": t_fp64 / t_mixed,
        "galerkin_entries_per_s": n * n / ((far_ms + near_ms) * 1e-3),
        "refinement": {"iterations": info_mixed[1], "backward_error": info_mixed[2]},
        "phases_ms": {"mixed": {k: v[0] for k, v in ph_mixed.items()},
                      "fp64": {k: v[0] for k, v in ph_fp64.items()}},
        "roofline": {"bound": "fp64", "kernel": "far_fp64_kernel", "achieved": achieved,
                     "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                     "traffic": None,
                     "note": "100 flops per kernel evaluation (frozen convention), 25 (N^2-3N) "
                             "evaluations per launch; peak = FP64 FMA chain measured in this run "
                             "(MEASURED_PEAKS.json carries no FP64 figure)",
                     "far_ms": far_ms, "near_ms": near_ms},
    }
    if clocks:
        res["clocks"] = clocks
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        times, x_ref = cpu_reference(w, 1, 0, threads)
        v = 1.0 / times[0]
        res["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                               "sample": "one full assemble + LU solve (oracle restatement of "
                                         "the reference, OpenMP, + scipy LAPACK)"}
        x = x_dev.cpu().numpy()
        res["rel_err_vs_oracle"] = float(np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref))
    print(json.dumps(res))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="kite2048")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--only", choices=["assembly", "mixed", "fp64"],
                    help="profiling driver: run one phase, print its timers")
    args = ap.parse_args()
    if args.only:
        run_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
