#!/usr/bin/env python
"""Benchmark: sound-soft scattering solves/s on one GB300 (replicas per GPU).

Workloads (`--workload`):
  ellipse_sweep256 (default)  ellipse with semi-axes (2,1) (EllipseArc(2,1,0,2pi)),
      256 wavenumbers uniform in [20, 200], N_k = ceil(10 k P / 2pi)
      (309 ... 3084 unknowns, sum N_k^2 = 9.03e8 entries), elements equispaced in
      the parameter, plane wave d = (1, 0), eta = k.  One step = the whole sweep:
      256 independent Discretize() + Solve() problems through bem2d_sweep_solve.
  kite2048      kite curve, N = 2048 equispaced, k = 100, plane-wave angle from
      numpy default_rng(0).uniform(0, 2pi); one step = one solve.
  lshape16384   L-shaped domain (unit square minus [0.5,1]^2), corner grading
      (8 levels, ratio 0.15), N = 16384, k = 500, d = (1, 0); one solve.
  disk160       unit disk, 160 equal-arc elements, k = 10, d = (1, 0).
All use the combined operator 1/2 I + D' - i eta S, QuadOption {L=3, N=5,
sigma=0.15}.

A solve: FP64 near-field and small-argument assembly with a float-float
far field, complex64 LU with partial pivoting, FP64 iterative refinement to
backward error 1e-14 (`mixed`, the headline `value`).  Beside it the plain
FP64 GPU path (FP64 assembly + complex128 LU, one problem after another) is
timed (`plain_fp64`) and every mixed solution is compared with it.
Synthetic input: geometries are generated, no dataset is read.

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
# numerical range scan: both arms stop each angle at the same error
# estimate, 1e-11 of |H| (ten times below the 1e-10 accuracy bar)
NR_TOL = 1e-11
SWEEP_WORKERS = 16


def workload(name):
    """dict(problems=[(geometry, k, eta)], d, desc, cpu_sample=[indices])."""
    from bem2d_gb300 import geometry as G
    if name == "ellipse_sweep256":
        ks, ns = G.sweep_sizes(256, 20.0, 200.0)
        probs = [(G.ellipse_arc_closed(n).add_poly_basis(0), float(k), float(k))
                 for k, n in zip(ks, ns)]
        return dict(problems=probs, d=(1.0, 0.0), cpu_sample=list(range(16, 256, 32)),
                    ref_sample=[64, 192],
                    desc="ellipse (2,1) sweep: 256 k uniform in [20,200], N_k = "
                         "ceil(10 k P/2pi) = %d..%d, eta=k, d=(1,0), QuadOption{3,5,0.15}"
                         % (min(ns), max(ns)))
    if name in ("kite2048", "kite4096"):
        n = int(name[4:])
        th = float(np.random.default_rng(0).uniform(0, 2 * math.pi))
        return dict(problems=[(G.kite(n).add_poly_basis(0), 100.0, 100.0)],
                    d=(math.cos(th), math.sin(th)), cpu_sample=[0], ref_sample=[0],
                    desc="kite N=%d equispaced, k=100, eta=k, plane wave angle %.15g "
                         "(rng seed 0), QuadOption{3,5,0.15}" % (n, th))
    if name == "lshape16384":
        return dict(problems=[(G.lshape(4072, 8, 0.15).add_poly_basis(0), 500.0, 500.0)],
                    d=(1.0, 0.0), cpu_sample=None, ref_sample=None,
                    desc="L-shape, corner grading L=8 sigma=0.15, N=16384, k=500, eta=k, "
                         "d=(1,0), QuadOption{3,5,0.15}")
    if name == "disk160":
        g = G.curve_equispaced(G.CIRCLE, 160).add_poly_basis(0)
        return dict(problems=[(g, 10.0, 10.0)], d=(1.0, 0.0), cpu_sample=[0], ref_sample=[0],
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


def max_over_ranks(values, ws, device):
    """Element-wise maximum of per-rank step times over all ranks: the step
    time of a replica run is its slowest rank's.  One rank: unchanged."""
    vals = [float(v) for v in values]
    if ws <= 1:
        return vals
    import torch
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


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


def cpu_solves(w, idx, threads):
    """The oracle (C restatement of the reference's assembly, OpenMP, + scipy
    LAPACK zgetrf/zgetrs) on the host cores for the problems `idx`: returns
    (seconds, {index: x})."""
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    from oracle import oracle as O
    from bem2d_gb300 import _build
    _build.build_oracle(with_reference=False)
    xs = {}
    t0 = time.perf_counter()
    for i in idx:
        g, k, eta = w["problems"][i]
        A, b = O.system(g, k, w["d"], eta, QUAD, threads=threads)
        xs[i] = O.solve(A, b)
    return time.perf_counter() - t0, xs


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    w = workload(args.workload)
    if not w["ref_sample"]:
        print(json.dumps({"impl": "reference", "unavailable":
                          "the CPU restatement needs hours for this workload"}))
        return
    threads = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        t, _ = cpu_solves(w, w["ref_sample"], threads)
        if i >= args.warmup:
            times.append(t)
    v = len(w["ref_sample"]) * len(times) / sum(times)
    sample = ("problems %s of %d per step (assemble + LU solve each)"
              % (w["ref_sample"], len(w["problems"])))
    print(json.dumps({
        "impl": "reference", "metric": "solves/s", "value": v, "unit": "solves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w["desc"]},
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": sample + "; oracle restatement of the reference "
                                   "(OpenMP) + scipy LAPACK zgetrf/zgetrs"},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}))


AUX = {
    "square8192_normcond": "unit square, corner grading L=8 sigma=0.15, N=8192, k=200, eta=k: "
                           "||A||_2, ||A^-1||_2, cond(A) of ChangeBasis(A, Id)",
    "numrange2048": "unit square Polygon(pts, 512), N=2048, k=50, eta=k: numerical range of "
                    "ChangeBasis(A, Id), lambda_max of the Hermitian part at 360 angles",
}

# DRAM bytes (read + write) per launch of the far-field kernel, from an ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum) of the mixed assembly
# of the sweep's largest problem (ellipse, N = 3084); the file under
# profiles/ named traffic_far_ff_kernel_ellipse3084.txt holds the command.
TRAFFIC = {"far_ellipse3084": 1036800 + 167379456}


def measured_peaks():
    """HBM copy bandwidth and cuBLAS bf16 throughput measured on this GPU
    model (MEASURED_PEAKS.json beside this script), else the fallback figures
    of an earlier GB300 measurement."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        d["source"] = "measured"
        return d
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                "source": "fallback"}


def far_roofline(n, far_ms, fp32_peak, key=None):
    """The float-float far field against the FP32 FMA pipe: 100 flops per
    kernel evaluation (the frozen convention), 25 (N^2 - 3N) evaluations per
    assembly.  Algorithmic DRAM bytes: the complex128 entries written
    (16 N^2) plus their complex64 copy (8 N^2)."""
    flops = 100.0 * 25 * (n * n - 3 * n)
    ach = flops / (far_ms * 1e-3) / 1e12
    traffic = TRAFFIC.get(key) if key else None
    return {"bound": "fp32", "kernel": "far_ff_kernel + deferred_ff_kernel",
            "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ach / fp32_peak,
            "peak_source": "bem2d_fma_peak: FP32 FMA throughput measured in this run "
                           "(MEASURED_PEAKS.json has no FP32 figure)",
            "traffic": traffic,
            "algorithmic_bytes": 24.0 * n * n,
            "note": "N=%d; 25 (N^2-3N) evaluations x 100 flops per launch; %s"
                    % (n, "traffic = ncu dram bytes read+write per far-field launch at this N"
                       if traffic is not None else "traffic not captured at this N")}


def lu_roofline(n, lu_ms, peaks):
    """The complex64 LU against the TF32 tensor peak (half the measured bf16
    rate): 8N^3/3 real flops per factorisation (zgetrf's count).  The
    trailing update issues each product as three TF32 MMAs (hi*hi, hi*lo,
    lo*hi), so the tensor pipe executes about 3x the algorithmic flops."""
    flops = 8.0 * n ** 3 / 3.0
    ach = flops / (lu_ms * 1e-3) / 1e12
    peak = peaks["bf16_tflops"] / 2.0
    return {"bound": "tensor", "kernel": "complex64 LU (panels, trsm, tcgen05 trailing update)",
            "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
            "peak_source": "TF32 dense = bf16 burst / 2, bf16 %s (MEASURED_PEAKS.json)"
                           % peaks["source"],
            "traffic": None,
            "note": "N=%d; 8N^3/3 flops per factorisation; 3xTF32 split issues 3x" % n}


class Stepper:
    """Device-timed steps on the library's stream: a 256 MB L2 flush before
    each step (outside the events), then events around the host-synchronous
    call."""

    def __init__(self, ctx, ws=1):
        import torch
        self.torch = torch
        self.ws = ws
        self.stream = torch.cuda.ExternalStream(ctx.stream)
        self.flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier(self):
        self.torch.cuda.synchronize()
        if self.ws > 1:
            self.torch.distributed.barrier()

    def run(self, fn, k, warm):
        torch = self.torch
        if callable(warm):
            warm()
        else:
            for _ in range(warm):
                fn()
        self.barrier()
        ms = []
        for _ in range(k):
            self.flush.zero_()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(self.stream):
                e0.record()
            fn()
            with torch.cuda.stream(self.stream):
                e1.record()
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        self.barrier()
        return ms


def device_ms(fn):
    """Event time (ms) of one host-synchronous call."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    out = fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1), out


def aux_record(ctx, name, steps, warmup, check=True):
    """Norm / condition (graded square, N = 8192, k = 200) and numerical range
    (unit square, N = 2048, k = 50, 360 angles): one step = mixed assembly +
    ChangeBasis(A, Id) + the study, through the C ABI.  The plain FP64 study
    is timed beside it; results are checked once, untimed, against dense
    cuSOLVER spectra (torch.linalg)."""
    import torch
    from bem2d_gb300 import geometry as G
    if name == "square8192_normcond":
        g = G.graded_square(2032, 8, 0.15).add_poly_basis(0)
        k = 200.0
    else:
        g = G.polygon_uniform([(0, 0), (1, 0), (1, 1), (0, 1)], 512).add_poly_basis(0)
        k = 50.0
    arrays = g.arrays()
    n = g.n_unknowns
    dev = "cuda"
    A = torch.empty((n, n), dtype=torch.complex128, device=dev)   # column-major A = A.T view
    A32 = torch.empty((n, n), dtype=torch.complex64, device=dev)
    M = torch.zeros((n, n), dtype=torch.complex128, device=dev)
    B = torch.empty((n, n), dtype=torch.complex128, device=dev)
    bstart = np.arange(n + 1, dtype=np.int32)  # P0: 1 x 1 mass blocks
    thetas = 2 * np.pi * np.arange(360) / 360.0
    normcond = name == "square8192_normcond"

    def study(prec):
        if normcond:
            return ctx.norm_cond(B, precision=prec)
        return ctx.num_range_lmax(B, thetas, tol=NR_TOL, precision=prec)

    ph = {}

    def step():
        t = []
        for nm, fn in (
                ("assembly", lambda: ctx.discrete_kernel_mixed(arrays, "combined", k, k, QUAD,
                                                               2.0, 1.0, out=A, out32=A32)),
                ("change_basis", lambda: (ctx.eval_ident(arrays, QUAD, out=M),
                                          ctx.change_basis(A, M, bstart, out=B))),
                ("study", lambda: ph.__setitem__("out", study("mixed")))):
            t.append((nm, device_ms(fn)[0]))
        return t

    for _ in range(warmup):
        step()
    runs = [step() for _ in range(steps)]
    ms = [sum(v for _, v in r) for r in runs]
    phases = {nm: sum(r[i][1] for r in runs) / len(runs) for i, (nm, _) in enumerate(runs[0])}
    if normcond:  # where the mixed study's time goes (an untimed extra run)
        ctx.enable_timers(True)
        study("mixed")
        t = ctx.timers()
        ctx.enable_timers(False)
        ph["study_phases"] = {"factor_and_inverse_ms": t["lu"][0],
                              "products_with_inverse_ms": t["solve"][0],
                              "products": int(t["solve"][1])}
    study("fp64")  # warm the FP64 path's workspace
    t64, out64 = device_ms(lambda: study("fp64"))
    pre = phases["assembly"] + phases["change_basis"]
    res = {"metric": "norm-cond evaluations/s" if normcond else "numerical-range scans/s",
           "value": 1e3 * len(ms) / sum(ms), "unit": "1/s", "n_gpus": 1, "steps": steps,
           "warmup": warmup, "ms_per_step": sum(ms) / len(ms), "higher_is_better": True,
           "dtype": "mixed assembly; sigma_min by c64 Lanczos on complex64 LU solves, then "
                    "f64 Lanczos on refined solves from its Ritz vector" if normcond else
                    "mixed assembly; c64 Lanczos, then f64 Lanczos from its Ritz vectors",
           "data": "synthetic", "config": {"workload": AUX[name], "n_unknowns": n},
           "phases_ms": phases,
           "study_phases": ph.get("study_phases"),
           "plain_fp64": {"study_ms": t64, "value": 1e3 / (t64 + pre), "unit": "1/s",
                          "dtype": "f64 assembly products, complex128 LU / Lanczos"},
           "mixed_over_fp64_study": t64 / phases["study"]}
    Bt = B.T  # the column-major matrix as a torch view
    if normcond:
        nrm, cond = ph["out"]
        nrm64, cond64 = out64
        res["result"] = {"norm": nrm, "norm_inv": cond / nrm, "cond": cond}
        res["mixed_vs_fp64_rel_err"] = {"norm": abs(nrm - nrm64) / nrm64,
                                        "cond": abs(cond - cond64) / cond64}
        if check:
            # dense check: the extreme eigenvalues of B^H B (cuSOLVER zheevd)
            ev = torch.linalg.eigvalsh(Bt.conj().T @ Bt)
            smax, smin = float(ev[-1]) ** 0.5, float(ev[0]) ** 0.5
            res["rel_err_vs_dense_eig_BhB"] = {
                "norm": abs(nrm - smax) / smax, "norm_inv": abs(cond / nrm - 1 / smin) * smin,
                "cond": abs(cond - smax / smin) / (smax / smin),
                "note": "sigma = sqrt(eig(B^H B)): sigma_min to ~eps cond^2 relative, "
                        "so the sigma_min comparison is only as good as that"}
    else:
        lm, lm64 = ph["out"], out64
        res["mixed_vs_fp64_max_rel_err"] = float(np.max(np.abs(lm - lm64)) / np.max(np.abs(lm64)))
        res["result"] = {"lambda_max_min": float(np.min(lm)), "lambda_max_max": float(np.max(lm))}
        res["config"]["tol"] = NR_TOL
        if check:
            errs, errs64 = [], []
            for j in range(0, 360, 45):
                z = complex(np.cos(thetas[j]), np.sin(thetas[j]))
                H = 0.5 * (z * Bt + np.conj(z) * Bt.conj().T)
                ev = float(torch.linalg.eigvalsh(H)[-1])
                errs.append(abs(lm[j] - ev) / max(abs(ev), 1e-300))
                errs64.append(abs(lm64[j] - ev) / max(abs(ev), 1e-300))
            res["max_rel_err_vs_dense_eigvalsh"] = max(errs)
            res["plain_fp64"]["max_rel_err_vs_dense_eigvalsh"] = max(errs64)
            res["checked_angles"] = 8
    del A, A32, M, B
    torch.cuda.empty_cache()
    return res


def run_aux(args):
    from bem2d_gb300 import capi
    ctx = capi.Context(0)
    print(json.dumps(aux_record(ctx, args.workload, args.steps, args.warmup,
                                check=not args.no_check)))


def run_only(args):
    """Profiling driver: one phase only (assembly, mixed assembly or solve)
    of the largest problem of the workload, or the whole mixed sweep; no JSON
    bench line."""
    import torch
    from bem2d_gb300 import capi
    w = workload(args.workload)
    probs = w["problems"]
    g, k, eta = max(probs, key=lambda p: p[0].n_unknowns)
    n = g.n_unknowns
    arrays = g.arrays()
    ctx = capi.Context(0)
    ctx.enable_timers(args.only != "sweep")
    A = torch.empty((n, n), dtype=torch.complex128, device="cuda") \
        if args.only in ("assembly", "assembly_mixed") else None
    A32 = torch.empty((n, n), dtype=torch.complex64, device="cuda") \
        if args.only == "assembly_mixed" else None
    x = torch.zeros(n, dtype=torch.complex128, device="cuda")
    if args.only == "sweep":  # as the headline: geometry staged once, device results
        holds = [capi._GeomHold(p[0]) for p in probs]
        outs = [torch.zeros(h.n, dtype=torch.complex128, device="cuda") for h in holds]
    step_ms = []
    for it in range(args.warmup + args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        if args.only == "assembly":
            ctx.discrete_kernel(arrays, "combined", k, eta, QUAD, 2.0, 1.0, out=A)
        elif args.only == "assembly_mixed":
            ctx.discrete_kernel_mixed(arrays, "combined", k, eta, QUAD, 2.0, 1.0, out=A, out32=A32)
        elif args.only == "sweep":
            ctx.sweep_solve(holds, [p[1] for p in probs], w["d"], [p[2] for p in probs], QUAD,
                            "mixed", nworkers=args.workers, outs=outs)
        else:
            ctx.scattering_solve(arrays, k, w["d"], eta, QUAD, precision=args.only, out=x)
        e1.record()
        e1.synchronize()
        if it >= args.warmup:
            step_ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    print(json.dumps({"only": args.only, "workload": args.workload, "n": n,
                      "step_ms": step_ms, "workers": args.workers if args.only == "sweep" else None,
                      "timers_ms": {k: v[0] / max(v[1], 1) for k, v in ctx.timers().items()}}))


def lshape_cpu_leg(g, k, eta, threads, A_dev):
    """CPU baseline for the graded L-shape (N = 16384), where the oracle needs
    hours for a whole solve: 64 seeded rows of the oracle's assembly (timed,
    scaled by N/64, and compared with the GPU's rows) plus scipy's LAPACK
    zgetrf + zgetrs on a seeded random N/2 system (timed, scaled by 8 = the
    N^3 ratio)."""
    import scipy.linalg as sl
    from oracle import oracle as O
    from bem2d_gb300 import _build
    _build.build_oracle(with_reference=False)
    n = g.n_unknowns
    rows = np.sort(np.random.default_rng(0).choice(n, 64, replace=False))
    t0 = time.perf_counter()
    R = O.discrete_kernel_rows(g, rows, "combined", k, eta, QUAD, alpha=2.0, beta=1.0,
                               threads=threads)
    t_rows = time.perf_counter() - t0
    G = A_dev.T[rows.tolist()].cpu().numpy()  # rows of the column-major matrix
    row_err = float(np.linalg.norm(G - R) / np.linalg.norm(R))
    m = n // 2
    rng = np.random.default_rng(1)
    M = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    b = rng.standard_normal(m) + 0j
    t0 = time.perf_counter()
    lu = sl.lu_factor(M, overwrite_a=True, check_finite=False)
    sl.lu_solve(lu, b, check_finite=False)
    t_lu = time.perf_counter() - t0
    secs = t_rows * n / 64.0 + 8.0 * t_lu
    return {"value": 1.0 / secs, "unit": "solves/s", "cores": threads, "kind": "port",
            "sample": "64 seeded rows of the oracle's assembly (%.2f s, x N/64) + scipy "
                      "LAPACK zgetrf/zgetrs at N/2=%d (%.2f s, x 8): %.1f s per solve"
                      % (t_rows, m, t_lu, secs)}, row_err


def solve_record(ctx, args, wname, steps, warmup, ws=1, rank=0, sub=False):
    """Scattering solves of one workload through the C ABI: the mixed path
    device-resident (value), end to end with host results (e2e), the plain
    FP64 path, per-phase events of the largest problem and the rooflines.
    `sub`: a secondary record inside the headline line (fewer legs)."""
    import torch
    from bem2d_gb300 import capi
    w = workload(wname)
    probs = w["problems"]
    P = len(probs)
    st = Stepper(ctx, ws)
    holds = [capi._GeomHold(g.arrays()) for g, _, _ in probs]
    ks = [p[1] for p in probs]
    etas = [p[2] for p in probs]
    ns = [h.n for h in holds]
    x_dev = [torch.zeros(n, dtype=torch.complex128, device="cuda") for n in ns]
    x_pin = [torch.zeros(n, dtype=torch.complex128).pin_memory() for n in ns]
    x_host = [t.numpy() for t in x_pin]
    x_fp64 = [torch.zeros(n, dtype=torch.complex128, device="cuda") for n in ns]
    h2d = sum(a.nbytes for h in holds for a in h.arrays.values()) + 16 * P
    d2h = 16 * sum(ns)

    def mixed(outs):
        if P == 1:
            return lambda: ctx.scattering_solve(holds[0].arrays, ks[0], w["d"], etas[0], QUAD,
                                                precision="mixed", out=outs[0])
        return lambda: ctx.sweep_solve(holds, ks, w["d"], etas, QUAD, "mixed",
                                       nworkers=args.workers, outs=outs)

    def fp64_all():
        for i in range(P):
            ctx.scattering_solve(holds[i].arrays, ks[i], w["d"], etas[i], QUAD,
                                 precision="fp64", out=x_fp64[i])

    big = int(np.argmax(ns))

    def fp64_warm():  # workspace at its largest size; no full sweep
        ctx.scattering_solve(holds[big].arrays, ks[big], w["d"], etas[big], QUAD,
                             precision="fp64", out=x_fp64[big])

    # -- mixed path, device-resident results ----------------------------------
    clk_path = os.path.join(os.environ.get("BEM2D_CLOCKS_DIR", os.path.join(ROOT, "_build")),
                            "bench_clocks_%s_%d.csv" % (wname, rank))
    os.makedirs(os.path.dirname(clk_path), exist_ok=True)
    cp, cf = clocks_start(clk_path)
    l0 = ctx.launches
    ms_mixed = st.run(mixed(x_dev), steps, warmup)
    launches = (ctx.launches - l0) // (steps + warmup) * steps
    clocks = clocks_stop(cp, cf, clk_path, torch.cuda.current_device())
    infos = ctx.sweep_infos if P > 1 else [ctx.last_info]
    # -- e2e: host results (device -> host copies inside the timed region) ----
    ms_e2e = st.run(mixed(x_host), steps, 1)
    # -- plain FP64 GPU path, one problem after another -----------------------
    fp64_steps = 1 if P > 1 or ns[0] > 8192 else max(2, steps // 2)
    ms_fp64 = st.run(fp64_all, fp64_steps, fp64_warm)
    errs = [float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
            for a, b in zip(x_dev, x_fp64)]

    # -- phases of the largest problem (events around each phase) -------------
    def phases(prec):
        ctx.enable_timers(True)
        ctx.scattering_solve(holds[big].arrays, ks[big], w["d"], etas[big], QUAD,
                             precision=prec, out=x_fp64[big] if prec == "fp64" else x_dev[big])
        t = ctx.timers()
        ctx.enable_timers(False)
        return {k: v[0] for k, v in t.items()}

    ph_mixed = phases("mixed")
    ph_fp64 = phases("fp64") if ns[big] <= 8192 else None
    nb = ns[big]
    peaks = measured_peaks()
    fp32_peak = capi.fma_peak("mixed")
    key = "far_%s%d" % ("ellipse" if wname.startswith("ellipse") else wname.rstrip("0123456789"),
                        nb)
    roof_far = far_roofline(nb, ph_mixed["far"], fp32_peak, key)
    roof_lu = lu_roofline(nb, ph_mixed["lu"], peaks)

    t_mixed = sum(ms_mixed) / len(ms_mixed)
    t_e2e = sum(ms_e2e) / len(ms_e2e)
    t_fp64 = sum(ms_fp64) / len(ms_fp64)
    t_mixed, t_e2e, t_fp64 = max_over_ranks([t_mixed, t_e2e, t_fp64], ws, "cuda")
    entries = float(sum(n * n for n in ns))
    res = {
        "metric": "solves/s", "value": ws * P * 1e3 / t_mixed, "unit": "solves/s",
        "n_gpus": ws, "steps": steps, "warmup": warmup, "ms_per_step": t_mixed,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 LU + f64 refinement; float-float Bessel functions, f64 geometry",
        "data": "synthetic",
        "config": {"workload": w["desc"], "problems_per_step": P,
                   "n_unknowns": ns[0] if P == 1 else [min(ns), max(ns)],
                   "precision": "mixed", "lu_update": "3xTF32 (tcgen05 kind::tf32)",
                   "sweep_workers": args.workers if P > 1 else None,
                   "l2": "256 MB write between timed steps, outside the step events",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": ws * P * 1e3 / t_e2e, "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "plain_fp64": {"value": ws * P * 1e3 / t_fp64, "unit": "solves/s", "ms_per_step": t_fp64,
                       "steps": fp64_steps},
        "mixed_over_fp64": t_fp64 / t_mixed,
        "galerkin_entries_per_s": ws * entries * 1e3 / t_mixed,
        "mixed_vs_fp64_max_rel_err": max(errs),
        "refinement": {"max_iterations": max(i[1] for i in infos),
                       "max_backward_error": max(i[2] for i in infos)},
        "phases_ms_largest": {"n": nb, "mixed": ph_mixed, "fp64": ph_fp64},
        # the far field is the path's throughput-bound hot spot; the LU
        # (panels latency-bound, trailing update on the tensor cores) follows
        "roofline": dict(roof_far, phase="far"),
        "roofline_other": dict(roof_lu, phase="lu"),
    }
    if clocks:
        res["clocks"] = clocks
    if P == 1 and nb > 8192:
        # backward errors of both solutions against the FP64 system, on the device
        g, k, eta = probs[0]
        A = torch.empty((nb, nb), dtype=torch.complex128, device="cuda")
        A32 = torch.empty((nb, nb), dtype=torch.complex64, device="cuda")
        ctx.discrete_kernel_mixed(holds[0].arrays, "combined", k, eta, QUAD, 2.0, 1.0,
                                  out=A, out32=A32)
        del A32
        b = torch.from_numpy(ctx.rhs(holds[0].arrays, k, w["d"], eta, QUAD)).cuda()
        Am = A.T  # the column-major matrix
        nA = float(torch.linalg.matrix_norm(Am))
        nb_ = float(torch.linalg.vector_norm(b))

        def berr(x):
            return float(torch.linalg.vector_norm(b - Am @ x)) / (
                nA * float(torch.linalg.vector_norm(x)) + nb_)

        res["backward_error"] = {"mixed": berr(x_dev[0]), "fp64": berr(x_fp64[0]),
                                 "measure": "|b - A x| / (|A|_F |x| + |b|), FP64 A"}
        # the LU's trailing-update precision options on the same system: the
        # value above runs 3xTF32; 1xTF32 issues a third of the tensor work
        # and leaves more to the refinement
        x_t = torch.zeros(nb, dtype=torch.complex128, device="cuda")
        ms_t = st.run(lambda: ctx.scattering_solve(holds[0].arrays, k, w["d"], eta, QUAD,
                                                   precision="mixed_tf32", out=x_t),
                      steps, warmup)
        info_t = ctx.last_info
        ph_t = phases("mixed_tf32")
        t_t = max_over_ranks([sum(ms_t) / len(ms_t)], ws, "cuda")[0]
        res["update_options"] = {
            "ran": "3xTF32 (value, e2e)",
            "3xTF32": {"ms_per_step": t_mixed, "lu_ms": ph_mixed["lu"],
                       "solve_ms": ph_mixed["solve"], "iterations": infos[0][1],
                       "backward_error": res["backward_error"]["mixed"],
                       "rel_err_vs_fp64": errs[0]},
            "1xTF32": {"ms_per_step": t_t, "lu_ms": ph_t["lu"], "solve_ms": ph_t["solve"],
                       "iterations": info_t[1], "backward_error": berr(x_t),
                       "rel_err_vs_fp64": float(torch.linalg.vector_norm(x_t - x_fp64[0]) /
                                                torch.linalg.vector_norm(x_fp64[0]))}}
        del x_t
        if not args.no_cpu and rank == 0:
            threads = os.cpu_count() or 1
            res["cpu_baseline"], res["rows_rel_err_vs_oracle"] = lshape_cpu_leg(
                g, k, eta, threads, A)
        del A
    elif not args.no_cpu and w["cpu_sample"] and rank == 0:
        threads = os.cpu_count() or 1
        secs, xr = cpu_solves(w, w["cpu_sample"], threads)
        v = len(w["cpu_sample"]) / secs
        res["cpu_baseline"] = {"value": v, "unit": "solves/s", "cores": threads, "kind": "port",
                               "sample": "problems %s of %d (assemble + LU solve each; oracle "
                                         "restatement of the reference, OpenMP, + scipy LAPACK)"
                                         % (w["cpu_sample"], P)}
        rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
        res["rel_err_vs_oracle"] = {
            "mixed": max(rel(x_dev[i].cpu().numpy(), xr[i]) for i in xr),
            "fp64": max(rel(x_fp64[i].cpu().numpy(), xr[i]) for i in xr),
            "problems": sorted(xr)}
    del x_dev, x_fp64, x_pin, x_host
    torch.cuda.empty_cache()
    return res


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from bem2d_gb300 import capi
    ctx = capi.Context(local)
    res = solve_record(ctx, args, args.workload, args.steps, args.warmup, ws, rank)
    if ws == 1 and not args.no_sub and args.workload == "ellipse_sweep256":
        # the other single-GPU configurations of the path, each with its own
        # FP64 comparison and checks (not part of the headline value)
        sub = {}
        sub["lshape16384"] = solve_record(ctx, args, "lshape16384", args.sub_steps, 3, sub=True)
        for name in AUX:
            sub[name] = aux_record(ctx, name, args.sub_steps, 3)
        res["sub"] = sub
    if rank == 0:
        print(json.dumps(res))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ellipse_sweep256")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--workers", type=int, default=SWEEP_WORKERS,
                    help="concurrent problems (host workers, one stream each) of a sweep")
    ap.add_argument("--no-check", action="store_true",
                    help="norm/cond and numerical-range workloads: skip the dense cuSOLVER check")
    ap.add_argument("--no-sub", action="store_true",
                    help="headline workload only (skip the L-shape, norm/cond and "
                         "numerical-range records)")
    ap.add_argument("--sub-steps", type=int, default=3,
                    help="timed steps of each secondary record")
    ap.add_argument("--only", choices=["assembly", "assembly_mixed", "mixed", "fp64", "sweep"],
                    help="profiling driver: run one phase, print its timers")
    args = ap.parse_args()
    if args.workload in AUX:
        run_aux(args)
    elif args.only:
        run_only(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
