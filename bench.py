#!/usr/bin/env python
"""Benchmark of the GPU numeric phase of the UCHOL direct solver.

Workload (default): the large refactorisation case.  3D linear elasticity,
Q1 hexahedra on 80 x 80 x 40 unit elements (807,003 equations), nu = 0.3,
face z = 0 clamped with the reference's LineCross semantics, natural
ordering (the reference's AMD ordering overflows its 32-bit factor layout
on this mesh).  Young's modulus per element is 1 x (1 + uniform[-0.05, 0.05]),
drawn afresh for each of 10 value sets with the sparsity pattern fixed; step
k refactorises value set k mod 10.  16 right-hand sides, each the consistent
load of a unit body force plus uniform[-0.1, 0.1] noise.  All seeded
synthetic data; no external dataset.

One step = numeric refactorisation (graph replay; TF32 tensor-core Schur
updates with FP32 accumulation, FP32 fronts) + the 16-column solve refined
with the FP64 residual product until every column has
||b - Ax|| / ||b|| <= 1e-10.

metric value: the reference's FactorOperationCount divided by the time of
factorisation + refined solve (TFLOP/s), inputs resident in HBM.
e2e: the same through the public API (SymmetricUtduSolver refactorisation and
Solve) with host buffers: matrix values and b copied in, x copied out.
fp64_gpu: the plain FP64 GPU factorisation + solve of value set 0 (its
device time, graph capture excluded), the mixed arm's speed-up over it, and
the forward error of the mixed solution of value set 0 against it.
Inputs exceed L2 (factor 67 GB), so no L2 flush is needed between steps.

--elements 40 40 40 --ordering AMD --precision BF16 --nrhs 1 --perturbations 0
gives the 206,763-equation elasticity case with E = 1.

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
    p.add_argument("--elements", type=int, nargs=3, default=[80, 80, 40])
    p.add_argument("--precision", default="TF32", choices=["BF16", "TF32", "FP64"])
    p.add_argument("--ordering", default="Natural", choices=["AMD", "Natural"])
    p.add_argument("--nrhs", type=int, default=16, help="right-hand sides per solve")
    p.add_argument("--perturbations", type=int, default=10,
                   help="value sets with E = 1 + uniform[-0.05, 0.05] per element (0: E = 1 throughout)")
    p.add_argument("--contrast", type=float, default=1.0,
                   help="> 1: Young's modulus log-uniform in [1, contrast] per element (seeded), the "
                        "stiffness-contrast elasticity case (1e4)")
    p.add_argument("--tol", type=float, default=1e-10)
    p.add_argument("--chain-merge-width", type=int, default=0,
                   help="widest device front grouped from a chain of supernodes (0: the library default, 2048)")
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 GPU arm")
    p.add_argument("--cpu-sample-elements", type=int, nargs=3, default=None,
                   help="mesh of the CPU baseline sample (default: 0.3 x the workload's mesh, at least 8)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def cpu_sample_elements(args):
    if args.cpu_sample_elements:
        return list(args.cpu_sample_elements)
    if args.ordering == "AMD":
        return [20, 20, 20]
    return [max(8, int(round(e * 0.3))) for e in args.elements]


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
    """Matrix (pattern of value set 0), the value sets, and the n x nrhs right-hand sides."""
    from magla_gb300 import generators as G
    ex, ey, ez = args.elements
    rng = np.random.default_rng(20260812)
    base = (G.log_uniform_youngs(ex * ey * ez, 1.0, args.contrast, np.random.default_rng(20260813))
            if args.contrast > 1.0 else np.ones(ex * ey * ez))
    sets = []
    if args.perturbations > 0:
        m = load = None
        for k in range(args.perturbations):
            E = base * (1.0 + rng.uniform(-0.05, 0.05, ex * ey * ez))
            mk, lk = G.elasticity(ex, ey, ez, youngs=E)
            if m is None:
                m, load = mk, lk
            elif mk.NonZeroCount != m.NonZeroCount or not np.array_equal(mk.ColumnIndices, m.ColumnIndices):
                raise RuntimeError("a value perturbation changed the sparsity pattern")
            sets.append(np.ascontiguousarray(mk.Values))
    else:
        m, load = G.elasticity(ex, ey, ez, youngs=base if args.contrast > 1.0 else None)
        sets.append(np.ascontiguousarray(m.Values))
    # n x nrhs block (column-major): unit body force plus uniform[-0.1, 0.1] noise per column
    b = np.asfortranarray(np.stack([load + rng.uniform(-0.1, 0.1, m.Size) for _ in range(args.nrhs)], axis=1))
    return m, sets, b


def cpu_baseline(args, threads):
    """The oracle (C++ port of the reference's numeric phase) on a bounded sample:
    the same mesh family and ordering on a smaller mesh, all host threads."""
    import oracle
    import magla_gb300 as mg
    from magla_gb300 import generators as G
    e = cpu_sample_elements(args)
    m, load = G.elasticity(*e)
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
            "sample": f"elasticity {e[0]}x{e[1]}x{e[2]} elements, {args.ordering} ordering (n={m.Size}, "
                      f"FactorOperationCount={sym.FactorOperationCount:.3e}), factor+solve of one right-hand "
                      f"side {dt:.2f} s, relres {rr:.1e}"}


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
    e = cpu_sample_elements(args)
    line = {"metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "impl": "reference",
            "config": {"workload": f"elasticity Q1 {e[0]}x{e[1]}x{e[2]} elements (bounded sample of "
                                   f"{args.elements[0]}x{args.elements[1]}x{args.elements[2]})",
                       "ordering": args.ordering},
            "dtype": "f64", "data": "synthetic", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _cols(b):
    return b.reshape(b.shape[0], -1)


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
    m, sets, b = make_workload(args)
    nrhs = args.nrhs
    ordering = mg.FillReducingOrdering["ApproximateMinimumDegree" if args.ordering == "AMD" else "Natural"]
    prec = mg.Precision[args.precision]
    opts = mg.UtduSolverOptions(Ordering=ordering, Precision=prec, RefinementTolerance=args.tol,
                                ChainMergeWidth=args.chain_merge_width,
                                RefinementMaxIterations=200)
    solver = mg.SymmetricUtduSolver(opts)
    t_sym = time.perf_counter()
    sym = solver.Analyze(m)
    t_sym = time.perf_counter() - t_sym
    stream = torch.cuda.current_stream()
    sym.SetStream(stream.cuda_stream)
    ops = sym.FactorOperationCount
    lib = _native.gpu()
    d_sets = [torch.from_numpy(v).cuda() for v in sets]
    # column-major n x nrhs device blocks (a transposed contiguous tensor)
    d_b = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    d_x = torch.zeros_like(d_b)
    bnorm = np.linalg.norm(_cols(b), axis=0)

    # ---- plain FP64 GPU arm: factorisation (device time; graph capture excluded) + one solve;
    # measured at N = 1 only (N > 1 runs replicas of the same step, and the arm holds every GPU
    # for minutes)
    fp64 = None
    x64 = None
    if not args.no_fp64 and prec != mg.Precision.FP64 and world == 1:
        s64 = mg.SymmetricUtduSolver(mg.UtduSolverOptions(Ordering=ordering, Precision=mg.Precision.FP64,
                                                          ChainMergeWidth=args.chain_merge_width))
        f64 = s64.FactorizeDevice(m, sym, d_sets[0].data_ptr())
        factor64_s = f64.FactorMilliseconds / 1e3
        f64.SolveDevice(d_b.data_ptr(), d_x.data_ptr(), nrhs)   # first call captures the solve graph
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        f64.SolveDevice(d_b.data_ptr(), d_x.data_ptr(), nrhs)
        e1.record(stream)
        torch.cuda.synchronize()
        solve64_s = e0.elapsed_time(e1) / 1e3
        x64 = d_x.cpu().numpy().T.copy()
        rr64 = float(np.max(f64.DeviceResidualNorms(b, x64) / bnorm))
        fp64 = {"factor_s": factor64_s, "solve_s": solve64_s, "factor_solve_s": factor64_s + solve64_s,
                "tflops": ops / (factor64_s + solve64_s) / 1e12, "relres": rr64,
                "timed": "factorisation (device time, capture excluded) + one solve of all right-hand sides"}
        del f64
        torch.cuda.synchronize()

    # ---- mixed arm
    f = solver.FactorizeDevice(m, sym, d_sets[0].data_ptr())

    def step(k):
        f.RefactorizeDevice(d_sets[k % len(d_sets)].data_ptr())
        return f.SolveRefinedDevice(d_b.data_ptr(), d_x.data_ptr(), nrhs, args.tol, 200)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches0 = lib.uchol_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    iters, relres_steps = [], []
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        # NVTX range of the timed steps: profilers select these launches with --nvtx-include "timed_steps/"
        torch.cuda.nvtx.range_push("timed_steps")
        ev0.record(stream)
        for k in range(args.steps):
            rs = step(k)
            iters.append(rs.iterations)
            relres_steps.append(rs.relative_residual)
        ev1.record(stream)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
    launches = lib.uchol_kernel_launches() - launches0
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps)   # replicas: the slowest rank defines the step
    # accuracy of value set 0: the library's FP64 residual, and the forward error against the FP64 arm
    step(0)
    torch.cuda.synchronize()
    x0 = d_x.cpu().numpy().T.copy()
    relres0 = float(np.max(f.DeviceResidualNorms(b, x0) / bnorm))
    fwd_err = None
    if x64 is not None:
        fwd_err = float(np.max(np.linalg.norm(_cols(x0 - x64), axis=0) / np.linalg.norm(_cols(x64), axis=0)))
        fp64["speedup_mixed_vs_fp64"] = fp64["factor_solve_s"] / (ms / 1e3)

    # ---- end to end through the public API with host buffers in page-locked memory (values
    # and b in, x out): the matrices' values, b and x live in pinned arrays filled before the
    # timed steps
    def pinned(shape):
        return torch.empty(shape[::-1], dtype=torch.float64, pin_memory=True).numpy().T   # column-major view
    mats = []
    for v in sets:
        pv = pinned((len(v),))
        pv[:] = v
        mats.append(_with_values(m, pv))
    b_host = pinned(b.shape)
    b_host[...] = b
    x_host = pinned(b.shape)
    e2e_ms, e2e_rr = [], []
    for k in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f.Refactorize(mats[k % len(mats)])
        f.Solve(b_host, out=x_host)
        torch.cuda.synchronize()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_rr.append(f.LastRefinement.relative_residual if f.LastRefinement is not None else None)
    e2e = float(np.mean(e2e_ms))

    # ---- roofline of the dominant kernel: one instrumented factorisation and solve after the timed steps
    lib.uchol_set_phase_timing(1)
    f.RefactorizeDevice(d_sets[0].data_ptr())
    f.SolveDevice(d_b.data_ptr(), d_x.data_ptr(), nrhs)
    lib.uchol_set_phase_timing(0)
    ph = f.PhaseTimes()
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak_bf16 = peaks.get("bf16_tflops_sustained", 1700.0)
    peak = peak_bf16 if prec == mg.Precision.BF16 else peak_bf16 / 2.0
    achieved = ph["schur_tensor_flops"] / (ph["schur_tensor_ms"] * 1e-3) / 1e12 if ph["schur_tensor_ms"] > 0 else 0.0
    traffic = gemm_traffic(args, prec)
    if rank != 0:
        return
    cb = None if (args.no_cpu_baseline or world > 1) else cpu_baseline(args, os.cpu_count() or 1)
    value = world * ops / (ms / 1e3) / 1e12
    entries = sym.FactorEntryCount
    apps = [it + 1 for it in iters]   # factor applications per refined solve (x0 plus one per step)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {mg.Precision.BF16: "bf16", mg.Precision.TF32: "tf32", mg.Precision.FP64: "f64"}[prec],
        "data": "synthetic",
        "config": {"workload": f"elasticity Q1 {args.elements[0]}x{args.elements[1]}x{args.elements[2]} elements, "
                               f"n={m.Size}, nnz_upper={m.NonZeroCount}, {args.ordering} ordering, {nrhs} right-hand "
                               f"sides, {max(1, args.perturbations)} value sets"
                               + (" (E x (1 + uniform[-0.05, 0.05]) per element)" if args.perturbations else "")
                               + (f", E log-uniform in [1, {args.contrast:g}] per element" if args.contrast > 1.0
                                  else ""),
                   "precision": (f"{prec.name} Schur GEMMs (FP32 accumulation), FP32 fronts, FP64-residual refinement"
                                 if prec != mg.Precision.FP64 else "FP64 throughout"),
                   "refine_tol": args.tol, "factor_ops": ops, "parallelism": f"replicas{world}", "nrhs": nrhs,
                   "l2": "inputs larger than L2 (no flush)"},
        "factor_solve_s": ms / 1e3, "refine_iterations": iters,
        "relres": float(max(relres_steps + [relres0])),
        "forward_error_vs_fp64_gpu": fwd_err,
        "flops_per_step": {"factor": ops,
                           "solves": float(sum(apps) / len(apps) * nrhs * (4.0 * (entries - m.Size) + m.Size)),
                           "refinement_spmv": float(sum(apps) / len(apps) * 2 * nrhs * 4.0 * m.NonZeroCount)},
        "symbolic_s": t_sym,
        "e2e": {"value": world * ops / (e2e / 1e3) / 1e12, "unit": "TFLOP/s", "ms_per_step": e2e,
                "h2d_bytes_per_step": int(m.NonZeroCount * 8 + m.Size * 8 * nrhs),
                "d2h_bytes_per_step": int(m.Size * 8 * nrhs),
                "relres": float(max(r for r in e2e_rr if r is not None)) if any(r is not None for r in e2e_rr) else None},
        "gpu_launches": int(launches),
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "kernel": "k_tc_gemm", "launches_per_step": ph["schur_tensor_launches"],
                     "note": "peak = bf16_tflops_sustained of MEASURED_PEAKS.json (half of it for TF32), of measured"},
        "phases_ms": {k: ph[k] for k in ("pivot_block_ms", "panel_ms", "schur_ms", "extend_add_ms", "small_fronts_ms",
                                          "total_ms")},
        "solve_phases_ms": {**{k: round(v, 3) for k, v in ph["solve_ms"].items()}, "total": ph["solve_total_ms"]},
        "clocks": clocks.summary(),
        "cpu_baseline": cb,
    }
    if fp64:
        line["fp64_gpu"] = fp64
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def _with_values(m, values):
    """A matrix of m's pattern holding the given values."""
    import copy
    mk = copy.copy(m)
    mk._val = np.ascontiguousarray(values, np.float64)
    return mk


def gemm_traffic(args, prec):
    """DRAM bytes per k_tc_gemm launch (read + write) from the committed ncu capture of the
    default workload (elasticity 80x80x40, TF32, natural order); None for any other one."""
    import magla_gb300 as mg
    f = ROOT / "profiles" / "k_tc_gemm_dram_elasticity80x80x40_tf32.txt"
    if list(args.elements) != [80, 80, 40] or prec != mg.Precision.TF32 or args.ordering != "Natural" \
            or args.chain_merge_width != 0 or not f.exists():
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
