"""Benchmark of the GB300 Krylov path (one JSON line on stdout).

Workload (default): 3D 7-point Poisson on a 128^3 grid (n = 2,097,152,
nnz = 14,581,760), b = A x_true with x_true ~ U[-1,1] (seed 2), x0 = 0,
CG + DiagonalPreconditioner to rtol 1e-10.  One step = one full solve.

  value     solves/s with A, b, x resident on the device (CUDA events on the
            library's stream around K solves)
  e2e       the same metric through the host-pointer API: each step copies b
            and x0 from pinned host memory to the device and x back
  roofline  the CSR product kernel (the dominant kernel): algorithmic bytes
            12*nnz + 4*(n+1) + 16*n per launch over its average CUDA-event
            duration across a loop of launches, against the measured HBM peak
  cpu_baseline  the oracle's CG + Jacobi on the host cores on a bounded
            sample (a fixed number of iterations, scaled to one solve)

``--impl reference`` times the reference's CPU path instead (the oracle
restatement of MTJ's CG; no JDK exists to run MTJ itself) on all host cores
as independent solves.  ``--gpus N`` runs N independent replicas (one
process per GPU; the path does not shard).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "matrix-toolkits-java_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
sys.path.insert(0, PKG)

import numpy as np  # noqa: E402

N_GRID = 128
SEED = 2
RTOL = 1e-10
MAX_ITER = 5000


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, val in zip(names, parts[2:]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU side
def _oracle_sample(args):
    """One process: the oracle's CG + Jacobi for `iters` iterations on C2."""
    iters, = args
    sys.path.insert(0, ORACLE_DIR)
    sys.path.insert(0, PKG)
    import oracle as O
    from mtjg import workloads
    n, rp, ci, v = workloads.poisson3d(N_GRID)
    A = O.Csr(n, n, rp, ci, v)
    b = O.mult(A, workloads.uniform(n, SEED))
    pc = O.Precond(O.PC_JACOBI, n)
    pc.set_matrix(A)
    t0 = time.perf_counter()
    _, res, _, _ = O.solve(O.CG, A, b, np.zeros(n), pc, max_iter=iters, rtol=RTOL, hist_cap=0)
    dt = time.perf_counter() - t0
    return dt, res.iterations


def cpu_baseline(iters_full: int, sample_iters: int, procs: int):
    """Solves/s of the oracle, from `procs` concurrent samples of
    `sample_iters` iterations, scaled by the full solve's iteration count."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        out = pool.map(_oracle_sample, [(sample_iters,)] * procs)
    per_iter = statistics.median(dt / max(1, it) for dt, it in out)
    t_solve = per_iter * iters_full
    return procs / t_solve, per_iter


# ------------------------------------------------------------- GPU side
def run_gpu(args):
    from mtjg import _lib as L
    from mtjg import sparse, workloads

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    lib = L.load()
    ctx = sparse.Context(local)
    n, rp, ci, v = workloads.poisson3d(args.grid)
    nnz = int(rp[-1])
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    xt = workloads.uniform(n, SEED)
    b = A.mult(xt)

    def ev(slot):
        if lib.mtjg_ctx_event_record(ctx.h, slot) != 0:
            raise RuntimeError(L.last_error())

    def elapsed(a, bb):
        ms = C.c_float()
        lib.mtjg_ctx_event_elapsed(ctx.h, a, bb, C.byref(ms))
        return ms.value

    # ---- device-resident buffers
    db, dx, dy = C.c_void_p(), C.c_void_p(), C.c_void_p()
    for p in (db, dx, dy):
        lib.mtjg_dev_alloc(ctx.h, 8 * n, C.byref(p))
    lib.mtjg_memcpy_h2d(ctx.h, db, b.ctypes.data_as(C.c_void_p), 8 * n)
    zeros = np.zeros(n)

    solver = sparse.CG(n, ctx=ctx)
    M = sparse.DiagonalPreconditioner(n, ctx)
    M.setMatrix(A)
    solver.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(MAX_ITER, RTOL, 1e-50, 1e5)
    solver.setIterationMonitor(mon)
    solver._sync_monitor()
    res = L.Result()

    def solve_dev():
        code = lib.mtjg_solver_solve_dev(solver.h, A.h, db, dx, C.byref(res))
        if code != 0:
            raise RuntimeError(f"solve failed: {code} {L.last_error()}")

    # x0 = 0 for every solve, copied before the events (not part of a solve)
    def reset_x():
        lib.mtjg_memcpy_h2d(ctx.h, dx, zeros.ctypes.data_as(C.c_void_p), 8 * n)

    for _ in range(args.warmup):
        reset_x()
        solve_dev()
    iters = res.iterations
    times = []
    launches0 = ctx.launchCount()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            reset_x()
            ev(0)
            solve_dev()
            ev(1)
            times.append(elapsed(0, 1))
    launches = ctx.launchCount() - launches0
    # residual check of the last solve
    xh = np.empty(n)
    lib.mtjg_memcpy_d2h(ctx.h, xh.ctypes.data_as(C.c_void_p), dx, 8 * n)
    rel_res = float(np.linalg.norm(b - A.mult(xh)) / np.linalg.norm(b))
    ms_solve = statistics.mean(times)

    # ---- end to end: host buffers through mtjg_solver_solve
    pin_b = np.empty(n)
    pin_x = np.empty(n)
    pin_b[:] = b
    e2e_times = []
    for i in range(args.warmup + args.steps):
        pin_x[:] = 0.0
        t0 = time.perf_counter()
        solver.solve(A, pin_b, pin_x)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append((t1 - t0) * 1e3)
    ms_e2e = statistics.mean(e2e_times)

    # ---- roofline: the CSR product kernel alone, many launches
    lib.mtjg_memcpy_h2d(ctx.h, dx, xt.ctypes.data_as(C.c_void_p), 8 * n)
    reps = args.spmv_reps
    for _ in range(5):
        lib.mtjg_csr_mult_dev(A.h, dx, dy)
    ev(2)
    for _ in range(reps):
        lib.mtjg_csr_mult_dev(A.h, dx, dy)
    ev(3)
    ms_spmv = elapsed(2, 3) / reps
    bytes_spmv = 12 * nnz + 4 * (n + 1) + 8 * n + 8 * n
    gbs = bytes_spmv / (ms_spmv * 1e-3) / 1e9
    peak, peak_kind = _peaks()

    # bytes per CG + Jacobi iteration (fused phases) for the solve-level fraction
    bytes_iter = bytes_spmv + 88 * n
    solve_gbs = bytes_iter * iters / (ms_solve * 1e-3) / 1e9

    out = {
        "rank": rank, "world": world, "ms_solve": ms_solve, "ms_e2e": ms_e2e, "iters": iters,
        "rel_res": rel_res, "launches": launches, "ms_spmv": ms_spmv, "gbs_spmv": gbs,
        "bytes_spmv": bytes_spmv, "solve_gbs": solve_gbs, "peak": peak, "peak_kind": peak_kind,
        "clocks": clk.summary(), "n": n, "nnz": nnz,
    }
    return out


def spmv_only(args):
    """CompRowMatrix.mult on the 3D Poisson matrix, `spmv_reps` launches."""
    from mtjg import _lib as L
    from mtjg import sparse, workloads

    lib = L.load()
    ctx = sparse.Context(0)
    n, rp, ci, v = workloads.poisson3d(args.grid)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    xt = workloads.uniform(n, SEED)
    dx, dy = C.c_void_p(), C.c_void_p()
    lib.mtjg_dev_alloc(ctx.h, 8 * n, C.byref(dx))
    lib.mtjg_dev_alloc(ctx.h, 8 * n, C.byref(dy))
    lib.mtjg_memcpy_h2d(ctx.h, dx, xt.ctypes.data_as(C.c_void_p), 8 * n)
    for _ in range(args.warmup):
        lib.mtjg_csr_mult_dev(A.h, dx, dy)
    lib.mtjg_ctx_event_record(ctx.h, 0)
    for _ in range(args.spmv_reps):
        lib.mtjg_csr_mult_dev(A.h, dx, dy)
    lib.mtjg_ctx_event_record(ctx.h, 1)
    ms = C.c_float()
    lib.mtjg_ctx_event_elapsed(ctx.h, 0, 1, C.byref(ms))
    us = 1e3 * ms.value / args.spmv_reps
    nnz = int(rp[-1])
    by = 12 * nnz + 4 * (n + 1) + 16 * n
    return {"workload": f"CSR product, 3D Poisson {args.grid}^3", "us": us, "bytes": by, "gbs": by / us / 1e3}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="mtjg", choices=["mtjg", "reference"])
    ap.add_argument("--grid", type=int, default=N_GRID)
    ap.add_argument("--spmv-reps", type=int, default=200)
    ap.add_argument("--cpu-sample-iters", type=int, default=40)
    ap.add_argument("--cpu-procs", type=int, default=0, help="0: all host cores")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only-spmv", action="store_true",
                    help="run only the CSR product loop (for profiling the product kernel)")
    args = ap.parse_args()
    if args.only_spmv:
        print(json.dumps(spmv_only(args)))
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    cfg = {"workload": f"CG + DiagonalPreconditioner, 3D 7-point Poisson {args.grid}^3, rtol 1e-10, x0 = 0",
           "n": args.grid ** 3, "rtol": RTOL, "seed": SEED,
           "l2": "inputs larger than L2 (CSR 190 MB + vectors)", "parallelism": f"replicas x{args.gpus}"}

    if args.impl == "reference":
        if rank != 0:
            return
        procs = args.cpu_procs or os.cpu_count() or 1
        # iteration count of the full solve, from one oracle solve on this grid
        iters_full = int(os.environ.get("MTJG_CG_ITERS", "0")) or _oracle_full_iters()
        times = []
        for _ in range(args.warmup + args.steps):
            v, per_iter = cpu_baseline(iters_full, args.cpu_sample_iters, procs)
            times.append(v)
        val = statistics.median(times[args.warmup:])
        line = {"impl": "reference", "metric": "solves/s", "value": val, "unit": "solves/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * procs / val, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
                "cpu_baseline": {"value": val, "unit": "solves/s", "cores": procs, "kind": "port",
                                 "sample": f"{procs} concurrent oracle CG+Jacobi runs of {args.cpu_sample_iters} "
                                           f"iterations each, scaled to the full solve's {iters_full} iterations"},
                "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    out = run_gpu(args)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        objs = [None] * world
        dist.all_gather_object(objs, out)
        dist.destroy_process_group()
    else:
        objs = [out]
    if rank != 0:
        return
    ms = max(o["ms_solve"] for o in objs)
    ms_e2e = max(o["ms_e2e"] for o in objs)
    value = world * 1e3 / ms
    o0 = objs[0]
    cpu = None
    if not args.no_cpu:
        procs = 1
        v, per_iter = cpu_baseline(o0["iters"], args.cpu_sample_iters, procs)
        cpu = {"value": v, "unit": "solves/s", "cores": procs, "kind": "port",
               "sample": f"oracle CG+Jacobi, {args.cpu_sample_iters} iterations on the full 128^3 system "
                         f"({per_iter * 1e3:.1f} ms/iteration), scaled to {o0['iters']} iterations"}
    line = {
        "metric": "solves/s", "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
        "iterations": o0["iters"], "final_rel_residual": o0["rel_res"],
        "spmv": {"gbs": o0["gbs_spmv"], "us": o0["ms_spmv"] * 1e3, "bytes": o0["bytes_spmv"],
                 "frac_of_hbm": o0["gbs_spmv"] / o0["peak"]},
        "solve_hbm_gbs": o0["solve_gbs"],
        "roofline": {"bound": "hbm", "achieved": o0["gbs_spmv"], "peak": o0["peak"], "unit": "GB/s",
                     "frac": o0["gbs_spmv"] / o0["peak"], "traffic": None,
                     "kernel": "k_spmv (CompRowMatrix.mult)", "peak_source": o0["peak_kind"]},
        "cpu_baseline": cpu,
        "e2e": {"value": world * 1e3 / ms_e2e, "unit": "solves/s", "h2d_bytes_per_step": 16 * o0["n"],
                "d2h_bytes_per_step": 8 * o0["n"]},
        "gpu_launches": o0["launches"],
        "clocks": o0["clocks"],
    }
    print(json.dumps(line))


def _oracle_full_iters():
    sys.path.insert(0, ORACLE_DIR)
    import oracle as O
    from mtjg import workloads
    n, rp, ci, v = workloads.poisson3d(N_GRID)
    A = O.Csr(n, n, rp, ci, v)
    b = O.mult(A, workloads.uniform(n, SEED))
    pc = O.Precond(O.PC_JACOBI, n)
    pc.set_matrix(A)
    _, res, _, _ = O.solve(O.CG, A, b, np.zeros(n), pc, max_iter=MAX_ITER, rtol=RTOL, hist_cap=0)
    return res.iterations


if __name__ == "__main__":
    main()
