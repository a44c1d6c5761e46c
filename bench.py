#!/usr/bin/env python
"""Benchmark of the GPU numeric phase of the UCHOL direct solver.

Workload (default): 3D linear elasticity, Q1 hexahedra on 40 x 40 x 40 unit
elements (206,763 equations), E = 1, nu = 0.3, face z = 0 clamped with the
reference's LineCross semantics, the reference's default AMD ordering.
Right-hand side: consistent load of a unit body force plus uniform[-0.1, 0.1]
noise (seeded).  Synthetic data; no external dataset.

One step = numeric factorisation (mixed precision: BF16 tensor-core Schur
updates with FP32 accumulation, FP32 fronts and pivot blocks) + solve refined
with the FP64 residual product until ||b - Ax|| / ||b|| <= 1e-10.

metric value: the reference's FactorOperationCount divided by the time of
factorisation + refined solve (TFLOP/s), inputs resident in HBM.
e2e: the same through the public API (SymmetricUtduSolver refactorisation and
Solve) with host buffers: matrix values and b copied in, x copied out.
Inputs exceed L2 (factor 17.9 GB), so no L2 flush is needed between steps.

--impl reference: the reference's CPU algorithm (the C++ port in oracle/,
all host threads) on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "factor+solve s and TFLOP/s, mixed+refined vs FP64 GPU at relres≤1e-10"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--elements", type=int, nargs=3, default=[40, 40, 40])
    p.add_argument("--precision", default="BF16", choices=["BF16", "TF32", "FP64"])
    p.add_argument("--ordering", default="AMD", choices=["AMD", "Natural"])
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--fp64-compare", action="store_true", help="also time the plain FP64 factor+solve once")
    p.add_argument("--fp64-first", action="store_true",
                   help="time the FP64 arm's first factorisation (one-time graph capture included) instead of "
                        "a refactorisation after it: halves the FP64 arm's GPU time on the largest workloads")
    p.add_argument("--cpu-sample-elements", type=int, default=20)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--nrhs", type=int, default=1, help="right-hand sides per solve (the refactorisation "
                   "workload of 80x80x40 elements, natural ordering, takes 16)")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", "-lms", "200"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except FileNotFoundError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_workload(args):
    from magla_gb300 import generators as G
    ex, ey, ez = args.elements
    m, load = G.elasticity(ex, ey, ez)
    rng = np.random.default_rng(20260812)
    # n x nrhs block (column-major): unit body force plus uniform[-0.1, 0.1] noise per column
    b = np.asfortranarray(np.stack([load + rng.uniform(-0.1, 0.1, m.Size) for _ in range(args.nrhs)], axis=1))
    return m, (b[:, 0].copy() if args.nrhs == 1 else b)


def cpu_baseline(args, threads):
    """The oracle (C++ port of the reference's numeric phase) on a bounded sample:
    the same mesh family at --cpu-sample-elements^3, all host threads."""
    import oracle
    import magla_gb300 as mg
    from magla_gb300 import generators as G
    e = args.cpu_sample_elements
    m, load = G.elasticity(e, e, e)
    b = load + np.random.default_rng(20260812).uniform(-0.1, 0.1, m.Size)
    opts = mg.UtduSolverOptions(Ordering=mg.FillReducingOrdering[
        "ApproximateMinimumDegree" if args.ordering == "AMD" else "Natural"])
    sym = mg.UtduSymbolicFactorization.Analyze(m, opts)
    t = time.perf_counter()
    f = oracle.OracleFactor(sym, m.Values, workers=threads)
    x = f.Solve(b)
    dt = time.perf_counter() - t
    rr = oracle.residual_norm(m, b, x) / np.linalg.norm(b)
    return {"value": sym.FactorOperationCount / dt / 1e12, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": f"elasticity {e}^3 elements (n={m.Size}, FactorOperationCount={sym.FactorOperationCount:.3e}), "
                      f"factor+solve {dt:.2f} s, relres {rr:.1e}"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(args, threads)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.median(vals)) if vals else cb["value"]
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "impl": "reference",
            "config": {"workload": f"elasticity Q1 {args.cpu_sample_elements}^3 elements (bounded sample of "
                                   f"{args.elements[0]}x{args.elements[1]}x{args.elements[2]})",
                       "ordering": args.ordering},
            "dtype": "f64", "data": "synthetic", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import magla_gb300 as mg
    from magla_gb300 import _native
    from magla_gb300.replicas import max_over_ranks

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    m, b = make_workload(args)
    ordering = mg.FillReducingOrdering["ApproximateMinimumDegree" if args.ordering == "AMD" else "Natural"]
    prec = mg.Precision[args.precision]
    opts = mg.UtduSolverOptions(Ordering=ordering, Precision=prec, RefinementTolerance=args.tol,
                                RefinementMaxIterations=200)
    solver = mg.SymmetricUtduSolver(opts)
    t_sym = time.perf_counter()
    sym = solver.Analyze(m)
    t_sym = time.perf_counter() - t_sym
    stream = torch.cuda.current_stream()
    sym.SetStream(stream.cuda_stream)
    ops = sym.FactorOperationCount
    d_vals = torch.from_numpy(np.ascontiguousarray(m.Values)).cuda()
    nrhs = args.nrhs
    # column-major n x nrhs device blocks (a transposed contiguous tensor)
    d_b = torch.from_numpy(np.ascontiguousarray(b.T if nrhs > 1 else b)).cuda()
    d_x = torch.zeros_like(d_b)
    f = solver.Factorize(m, sym)
    lib = _native.gpu()

    def step():
        f.RefactorizeDevice(d_vals.data_ptr())
        return f.SolveRefinedDevice(d_b.data_ptr(), d_x.data_ptr(), nrhs, args.tol, 200)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = lib.uchol_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters = []
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            rs = step()
            iters.append(rs.iterations)
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = lib.uchol_kernel_launches() - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps)   # replicas: the slowest rank defines the step
    def worst_relres(fac, x_host):
        X = x_host.T if nrhs > 1 else x_host
        return float(np.max(fac.DeviceResidualNorms(b, X) / np.linalg.norm(b.reshape(m.Size, -1), axis=0)))

    relres = worst_relres(f, d_x.cpu().numpy())

    # end to end through the public API with host buffers
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f.Refactorize(m)
        x_host = f.Solve(b)
        torch.cuda.synchronize()
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e = float(np.mean(e2e_ms))
    e2e_relres = float(np.max(f.DeviceResidualNorms(b, x_host) / np.linalg.norm(b.reshape(m.Size, -1), axis=0)))

    # roofline of the dominant kernel: one instrumented factorisation after the timed steps
    lib.uchol_set_phase_timing(1)
    f.RefactorizeDevice(d_vals.data_ptr())
    lib.uchol_set_phase_timing(0)
    ph = f.PhaseTimes()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak_bf16 = peaks.get("bf16_tflops_sustained", 1700.0)
    peak = peak_bf16 if prec == mg.Precision.BF16 else peak_bf16 / 2.0
    achieved = ph["schur_tensor_flops"] / (ph["schur_tensor_ms"] * 1e-3) / 1e12 if ph["schur_tensor_ms"] > 0 else 0.0
    traffic = gemm_traffic(args, prec)
    fp64 = None
    if args.fp64_compare:
        f64s = mg.SymmetricUtduSolver(mg.UtduSolverOptions(Ordering=ordering, Precision=mg.Precision.FP64))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        del f
        if args.fp64_first:
            e0.record(stream)
            f64 = f64s.Factorize(m, sym)
        else:
            f64 = f64s.Factorize(m, sym)
            e0.record(stream)
            f64.RefactorizeDevice(d_vals.data_ptr())
        f64.SolveDevice(d_b.data_ptr(), d_x.data_ptr(), nrhs)
        e1.record(stream)
        torch.cuda.synchronize()
        s64 = e0.elapsed_time(e1) / 1e3
        rr64 = worst_relres(f64, d_x.cpu().numpy())
        fp64 = {"factor_solve_s": s64, "tflops": ops / s64 / 1e12, "relres": float(rr64),
                "speedup_mixed_vs_fp64": s64 / (ms / 1e3),
                "timed": "first factorisation + solve" if args.fp64_first else "refactorisation + solve"}
    if rank != 0:
        return
    cb = None if args.no_cpu_baseline else cpu_baseline(args, os.cpu_count() or 1)
    value = world * ops / (ms / 1e3) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16" if prec == mg.Precision.BF16 else ("tf32" if prec == mg.Precision.TF32 else "f64"),
        "data": "synthetic",
        "config": {"workload": f"elasticity Q1 {args.elements[0]}x{args.elements[1]}x{args.elements[2]} elements, "
                               f"n={m.Size}, nnz_upper={m.NonZeroCount}, {args.ordering} ordering",
                   "precision": f"{prec.name} Schur GEMMs (FP32 accumulation), FP32 fronts and pivot blocks, FP64-residual refinement",
                   "refine_tol": args.tol, "factor_ops": ops, "parallelism": f"replicas{world}", "nrhs": nrhs,
                   "l2": "inputs larger than L2 (no flush)"},
        "factor_solve_s": ms / 1e3, "refine_iterations": iters, "relres": float(relres),
        "symbolic_s": t_sym,
        "e2e": {"value": world * ops / (e2e / 1e3) / 1e12, "unit": "TFLOP/s", "ms_per_step": e2e,
                "h2d_bytes_per_step": int(m.NonZeroCount * 8 + m.Size * 8 * nrhs),
                "d2h_bytes_per_step": int(m.Size * 8 * nrhs),
                "relres": e2e_relres},
        "gpu_launches": int(launches),
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "kernel": "k_tc_gemm", "launches_per_step": ph["schur_tensor_launches"],
                     "note": "peak = bf16_tflops_sustained of MEASURED_PEAKS.json (half of it for TF32)"},
        "phases_ms": {k: ph[k] for k in ("pivot_block_ms", "panel_ms", "schur_ms", "extend_add_ms", "small_fronts_ms",
                                          "total_ms")},
        "clocks": clocks.summary(),
        "cpu_baseline": cb,
    }
    if fp64:
        line["fp64_gpu"] = fp64
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def gemm_traffic(args, prec):
    """DRAM bytes per k_tc_gemm launch (read + write) from the committed ncu capture of this
    workload (elasticity 40^3, BF16, AMD); None for any other configuration."""
    import magla_gb300 as mg
    f = ROOT / "profiles" / "k_tc_gemm_dram_elasticity40_bf16.txt"
    if list(args.elements) != [40, 40, 40] or prec != mg.Precision.BF16 or args.ordering != "AMD" or not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            return int(line.split(":")[1])
    return None


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        from magla_gb300 import build
        build.build_all()
        run_ours(args)


if __name__ == "__main__":
    main()
