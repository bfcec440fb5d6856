"""Benchmark of the GB300 Krylov path (one JSON line on stdout).

Workload (default, --workload serve): the served request stream.  Seeded
Poisson arrivals (2000 requests/s) draw 2D 5-point Poisson systems (grid
N ~ U{64..512}) or random SPD graph Laplacians (n log-uniform in [1k, 200k])
with equal odds; 70% reuse a matrix that is already resident with a new
right-hand side.  Every request is solved to rtol 1e-10 on its FP64 true
residual by mixed-precision CG + Jacobi in the continuous-batching server.
One step = serving the whole stream (1500 requests, 437 matrices).

  value     served solves/s: all matrices registered first, all requests
            submitted at once, CUDA events on the server's stream around
            submission .. drain
  e2e       the same stream through the host API as it arrives: matrices
            registered on first use, each request submitted at its arrival
            time; solves/s and p50/p99 latency (arrival -> x on the host)
  latency   p50/p99 at the stream's rate (above capacity), at a rate below
            capacity (300 requests/s), and at that rate with the resident
            matrices held to a 1.5 GiB budget (the stream's take about 6):
            idle matrices evicted least recently used, uploaded again on use
  plain_fp64  the plain FP64 drop-in (CG + DiagonalPreconditioner, one
            request at a time through the host API) on the same stream
  roofline  the CSR product kernel (CompRowMatrix.mult) on 3D 7-point Poisson
            128^3: algorithmic bytes 12*nnz + 4*(n+1) + 16*n per launch over
            its CUDA-event duration, against the measured HBM peak
  poisson3d_128  plain FP64 CG + Jacobi solves/s on that 3D Poisson system
  cpu_baseline  the oracle's FP64 CG + Jacobi on one host core: full solves
            of the stream's first requests for about 20 s

``--workload poisson3d`` makes the 3D Poisson CG solve the headline instead.
``--impl reference`` times the reference's CPU path (the oracle restatement
of MTJ's CG; no JDK exists to run MTJ itself) on all host cores.  ``--gpus N``
runs N independent replicas (one process per GPU; the path does not shard).
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
# DRAM bytes (read + write) of one k_spmv launch of CompRowMatrix.mult on the
# 3D Poisson 128^3 matrix, from one ncu capture (dram__bytes_read.sum +
# dram__bytes_write.sum); the algorithmic bytes of that launch are 216.92 MB
SPMV_TRAFFIC_128 = 211.75e6


def _traffic(grid):
    return SPMV_TRAFFIC_128 if grid == N_GRID else None


class Ranks:
    """The replicas of a --gpus N run (one process per GPU, launched by
    torch.distributed.run): a gloo group on the host for the barrier around
    the timed region and for gathering each rank's numbers.  The data path
    has no collective: every rank serves its own copy of the workload."""

    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def gather(self, obj):
        if not self.dist:
            return [obj]
        objs = [None] * self.world
        self.dist.all_gather_object(objs, obj)
        return objs

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None


def replica_rate(objs, units, key="sec"):
    """Whole-job rate of N replicas: all ranks' units over the slowest rank's time."""
    return len(objs) * units / max(o[key] for o in objs)


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


# ------------------------------------------------------------- serving (C5)
SERVE_SEED = 5
SERVE_RATE = 2000.0     # mean arrivals per second
SERVE_REUSE = 0.7       # share of requests that bring a new RHS for a resident matrix


def serve_stream(count: int, seed: int = SERVE_SEED, rate: float = SERVE_RATE, reuse: float = SERVE_REUSE):
    """The seeded request stream: Poisson arrivals; each request draws 2D
    5-point Poisson (grid N ~ U{64..512}) or a random SPD Laplacian (n
    log-uniform in [1k, 200k]) with equal odds, and reuses an already
    resident matrix of that kind with probability `reuse`.  Returns the
    matrix specs and requests (arrival s, matrix index, rhs seed, new?)."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    specs, reqs = [], []
    seen = {0: [], 1: []}
    for k in range(count):
        kind = int(rng.integers(0, 2))
        if seen[kind] and rng.random() < reuse:
            m, new = seen[kind][int(rng.integers(0, len(seen[kind])))], False
        else:
            if kind == 0:
                specs.append(("poisson2d", int(rng.integers(64, 513)), 0))
            else:
                n = int(np.exp(rng.uniform(np.log(1000.0), np.log(200000.0))))
                specs.append(("laplacian", n, 7000 + len(specs)))
            m, new = len(specs) - 1, True
            seen[kind].append(m)
        reqs.append((float(arrivals[k]), m, 100000 + k, new))
    return specs, reqs


def make_matrices(specs, threads: int = 16):
    """Generates the stream's matrices (host CSR) in parallel threads (the
    generators are C and release the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    from mtjg import workloads

    def one(spec):
        kind, n, s = spec
        return workloads.poisson2d(n) if kind == "poisson2d" else workloads.laplacian(n, s)

    with ThreadPoolExecutor(max(1, threads)) as ex:
        return list(ex.map(one, specs))


def _rhs(n, seed):
    from mtjg import workloads
    return workloads.uniform(n, seed)


def serve_backlog(ctx, mats, reqs, steps, warmup, max_systems, pool_rows, inner_rtol):
    """Server capacity: every matrix registered (resident) first, then per
    step all requests submitted at once and drained.  Returns per-step
    seconds, the results of the last step and the server's launch count."""
    from mtjg import serve
    srv = serve.Server(ctx, max_systems=max_systems, pool_rows=pool_rows, max_iter=100, rtol=RTOL,
                       inner_rtol=inner_rtol)
    ids = [srv.addMatrix(*m) for m in mats]
    rhs = [_rhs(mats[m][0], s) for _, m, s, _ in reqs]
    times, results = [], None
    launches = 0
    for step in range(warmup + steps):
        # CUDA events on the server's stream bracket the step; the stream is
        # idle before the first submission and after the drain
        srv.event(0)
        l0 = srv.launchCount()
        tickets = {srv.submit(ids[m], rhs[k]): k for k, (_, m, _, _) in enumerate(reqs)}
        srv.drain(600.0)
        srv.event(1)
        dt = srv.elapsed_ms(0, 1) * 1e-3
        got = {tickets[r.ticket]: r for r in srv.poll(cap=len(reqs) + 16)}
        if step >= warmup:
            times.append(dt)
            launches += srv.launchCount() - l0
        results = got
    stats = srv.stats()
    stats.update(srv.timing())
    srv.close()
    return times, results, rhs, stats, launches


def serve_open_loop(ctx, mats, reqs, max_systems, pool_rows, inner_rtol, rate=SERVE_RATE, budget=0, gmres_every=0,
                    gmres_mats=frozenset()):
    """The arrival stream end to end through the public API: a new matrix
    is registered when its first request arrives, each request is submitted
    at its arrival time (or as soon as the client is free), and latency runs
    from the scheduled arrival to the result being on the host.  `rate`
    rescales the stream's arrival times to that mean rate; `budget` is the
    server's matrix budget in bytes (0: every matrix stays resident);
    `gmres_every` = k sends every k-th request on a matrix in `gmres_mats` to
    the Krylov lane as GMRES."""
    from mtjg import serve
    srv = serve.Server(ctx, max_systems=max_systems, pool_rows=pool_rows, max_iter=100, rtol=RTOL,
                       inner_rtol=inner_rtol, matrix_budget=budget)
    scale = SERVE_RATE / rate
    reqs = [(ta * scale, m, s, new) for ta, m, s, new in reqs]
    rhs = [_rhs(mats[m][0], s) for _, m, s, _ in reqs]
    ids = {}
    arrival_of, lat, lat_g, gm = {}, [], [], set()
    h2d = d2h = 0
    t0 = time.perf_counter()

    def collect():
        now = time.perf_counter() - t0
        for r in srv.poll(cap=4096):
            (lat_g if r.ticket in gm else lat).append(now - arrival_of.pop(r.ticket))

    for k, (ta, m, _, _) in enumerate(reqs):
        while time.perf_counter() - t0 < ta:
            collect()
        if m not in ids:
            n, rp, ci, v = mats[m]
            ids[m] = srv.addMatrix(n, rp, ci, v)
            h2d += 4 * (n + 1) + 12 * len(ci)
        g = gmres_every > 0 and m in gmres_mats and k % gmres_every == gmres_every - 1
        t = srv.submit(ids[m], rhs[k], solver="gmres" if g else "cg")
        if g:
            gm.add(t)
        arrival_of[t] = ta
        h2d += 8 * mats[m][0]
        d2h += 8 * mats[m][0]
    while arrival_of:
        collect()
        time.sleep(0.0002)
    wall = time.perf_counter() - t0
    res = srv.residency()
    srv.close()
    lat = np.array(lat)
    out = {"wall_s": wall, "solves_s": len(reqs) / wall, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
           "p99_ms": 1e3 * float(np.percentile(lat, 99)), "h2d_bytes": h2d, "d2h_bytes": d2h,
           "offered_rate": rate, "uploads": res["uploads"], "evictions": res["evictions"],
           "matrix_budget": budget}
    if lat_g:
        out["gmres"] = {"requests": len(lat_g), "p50_ms": 1e3 * float(np.percentile(lat_g, 50)),
                        "p99_ms": 1e3 * float(np.percentile(lat_g, 99))}
    return out


def plain_fp64(ctx, mats, reqs, budget_s):
    """The plain FP64 drop-in, one request at a time through the host API:
    CG + DiagonalPreconditioner to rtol 1e-10 (the matrix uploaded and
    factored when first seen, as a caller of the drop-in would), on the
    stream's requests in order until `budget_s` has passed."""
    from mtjg import sparse
    dev = {}
    out = []
    t_start = time.perf_counter()
    for k, (_, m, s, _) in enumerate(reqs):
        if time.perf_counter() - t_start > budget_s and out:
            break
        n, rp, ci, v = mats[m]
        b = _rhs(n, s)
        t0 = time.perf_counter()
        if m not in dev:
            A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
            M = sparse.DiagonalPreconditioner(n, ctx)
            M.setMatrix(A)
            solver = sparse.CG(n, ctx=ctx)
            solver.setPreconditioner(M)
            solver.setIterationMonitor(sparse.DefaultIterationMonitor(100000, RTOL, 1e-50, 1e5))
            dev[m] = (A, M, solver)
        A, M, solver = dev[m]
        x = np.zeros(n)
        solver.solve(A, b, x)
        out.append((k, time.perf_counter() - t0, solver.getIterationMonitor().iterations()))
    return out


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
    ap.add_argument("--workload", default="serve",
                    choices=["serve", "poisson3d", "c4", "c4poisson", "c3mixed"] + sorted(CONFIGS),
                    help="serve: the served request stream (headline); poisson3d: one CG + Jacobi system; "
                         "c1/c2icc/c3gmres/c3bicg: the other single-system configurations; c4: the batch; c4poisson: a batch of 2D Poisson systems; c3mixed: FP64 vs mixed-precision GMRES / BiCGstab + ILU on 96^3")
    ap.add_argument("--batch-systems", type=int, default=4096)
    ap.add_argument("--serve-requests", type=int, default=1500)
    ap.add_argument("--serve-max-systems", type=int, default=512)
    ap.add_argument("--serve-pool-rows", type=int, default=1 << 26)
    ap.add_argument("--inner-rtol", type=float, default=1e-6)
    ap.add_argument("--inner-rtol-c3", type=float, default=1e-4,
                    help="inner residual decrease of the mixed GMRES / BiCGstab solves (c3mixed)")
    ap.add_argument("--serve-low-rate", type=float, default=300.0,
                    help="offered load (requests/s) of the below-capacity latency run")
    ap.add_argument("--serve-matrix-budget", type=float, default=1.5,
                    help="GiB of resident matrices in the budgeted run (the stream's matrices take about 6)")
    ap.add_argument("--plain-budget", type=float, default=8.0, help="seconds of plain FP64 one-at-a-time solves")
    ap.add_argument("--ref-seconds", type=float, default=6.0, help="reference arm: seconds of work per step")
    ap.add_argument("--ref-prepare", type=int, default=40,
                    help="reference arm: requests each process prepares (matrices built before the clock)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="cpu_baseline: seconds of oracle solves")
    args = ap.parse_args()
    if args.only_spmv:
        print(json.dumps(spmv_only(args)))
        return
    if args.workload == "serve":
        main_serve(args)
    elif args.workload == "poisson3d":
        main_poisson3d(args)
    elif args.workload in ("c4", "c4poisson"):
        run_batch(args)
    elif args.workload == "c3mixed":
        run_c3mixed(args)
    else:
        run_config(args)


def main_poisson3d(args):
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

    ranks = Ranks()
    ranks.barrier()
    out = run_gpu(args)
    ranks.barrier()
    objs = ranks.gather(out)
    ranks.close()
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
                     "frac": o0["gbs_spmv"] / o0["peak"], "traffic": _traffic(args.grid),
                     "kernel": "k_spmv (CompRowMatrix.mult)", "peak_source": o0["peak_kind"]},
        "cpu_baseline": cpu,
        "e2e": {"value": world * 1e3 / ms_e2e, "unit": "solves/s", "h2d_bytes_per_step": 16 * o0["n"],
                "d2h_bytes_per_step": 8 * o0["n"]},
        "gpu_launches": o0["launches"],
        "clocks": o0["clocks"],
    }
    print(json.dumps(line))


def _oracle_requests(specs, reqs, ks, seconds, limit=None):
    """The oracle's FP64 CG + Jacobi (MTJ's CPU path, restated) on requests
    ks of the stream, in order, until `seconds` of solving have passed (the
    request in progress at the deadline is finished and counted).  Matrices
    and their Jacobi diagonals are built before the clock starts, as the
    served `value` registers its matrices first.  Returns (solved, seconds)."""
    sys.path.insert(0, ORACLE_DIR)
    sys.path.insert(0, PKG)
    import oracle as O
    from mtjg import workloads
    ks = list(ks)[:limit] if limit else list(ks)
    cache = {}
    for k in ks:
        m = reqs[k][1]
        if m not in cache:
            kind, n, ms = specs[m]
            n, rp, ci, v = workloads.poisson2d(n) if kind == "poisson2d" else workloads.laplacian(n, ms)
            A = O.Csr(n, n, rp, ci, v)
            pc = O.Precond(O.PC_JACOBI, n)
            pc.set_matrix(A)
            cache[m] = (n, A, pc)
    rhs = {k: workloads.uniform(cache[reqs[k][1]][0], reqs[k][2]) for k in ks}
    done = 0
    t0 = time.perf_counter()
    for k in ks:
        if time.perf_counter() - t0 > seconds:
            break
        n, A, pc = cache[reqs[k][1]]
        O.solve(O.CG, A, rhs[k], np.zeros(n), pc, max_iter=100000, rtol=RTOL, hist_cap=0)
        done += 1
    return done, time.perf_counter() - t0


def _ref_worker(args):
    """Reference arm worker: requests w, w + P, ... of the stream (at most
    `cap` of them prepared) for `seconds` of solving."""
    w, procs, count, seconds, cap = args
    specs, reqs = serve_stream(count)
    return _oracle_requests(specs, reqs, range(w, len(reqs), procs), seconds, cap)


def _serve_config(args, nmat):
    return {"workload": "serving: seeded Poisson-arrival stream (2000 req/s) drawn 50/50 from 2D 5-point Poisson "
                        "(grid 64^2-512^2) and random SPD Laplacians (n 1k-200k), 70% new RHS on a resident "
                        "matrix; rtol 1e-10 on the FP64 true residual",
            "requests": args.serve_requests, "matrices": nmat, "seed": SERVE_SEED, "rtol": RTOL,
            "solver": "mixed-precision CG + Jacobi (FP32 inner, FP64 refinement)",
            "inner_rtol": args.inner_rtol, "max_systems": args.serve_max_systems,
            "pool_rows": args.serve_pool_rows,
            "l2": "inputs larger than L2 (resident matrices about 6 GB)",
            "parallelism": f"replicas x{args.gpus}"}


def reference_serve(args):
    """--impl reference on the serving workload: MTJ's CPU path (the oracle
    restatement; no JDK exists) solving the stream's requests one per host
    core, each step `ref_seconds` of work on every core."""
    procs = args.cpu_procs or os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    vals = []
    with ctx.Pool(procs) as pool:
        for _ in range(args.warmup + args.steps):
            out = pool.map(_ref_worker, [(w, procs, args.serve_requests, args.ref_seconds, args.ref_prepare)
                                         for w in range(procs)])
            vals.append(sum(d for d, _ in out) / max(t for _, t in out))
    val = statistics.median(vals[args.warmup:])
    specs, _ = serve_stream(args.serve_requests)
    line = {"impl": "reference", "metric": "served solves/s", "value": val, "unit": "solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * args.ref_seconds, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": _serve_config(args, len(specs)),
            "cpu_baseline": {"value": val, "unit": "solves/s", "cores": procs, "kind": "port",
                             "sample": f"{procs} processes, each solving every {procs}th request of the stream in "
                                       f"order (FP64 CG + Jacobi to rtol 1e-10, matrices built before the clock "
                                       f"starts) for {args.ref_seconds:.0f} s per step"},
            "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main_serve(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            reference_serve(args)
        return
    from mtjg import sparse

    specs, reqs = serve_stream(args.serve_requests)
    mats = make_matrices(specs)
    ctx = sparse.Context(local)
    # the single large system: plain FP64 CG + Jacobi and the CSR product roofline
    c2 = run_gpu(args)
    knobs = (args.serve_max_systems, args.serve_pool_rows, args.inner_rtol)
    ranks = Ranks()
    ranks.barrier()
    with ClockSampler(local) as clk:
        times, results, rhs, stats, launches = serve_backlog(ctx, mats, reqs, args.steps, args.warmup, *knobs)
    ranks.barrier()
    # every served result: status and the FP64 true residual b - A x
    import scipy.sparse as sp
    worst, failed = 0.0, 0
    for k, (_, m, _, _) in enumerate(reqs):
        r = results[k]
        n, rp, ci, v = mats[m]
        if r.status != 0:
            failed += 1
            continue
        A = sp.csr_matrix((v, ci, rp), shape=(n, n))
        worst = max(worst, float(np.linalg.norm(rhs[k] - A @ r.x) / np.linalg.norm(rhs[k])))
    inner = [results[k].inner_iterations for k in range(len(reqs))]
    outer = [results[k].iterations for k in range(len(reqs))]
    # FP32 inner iterations x rows, and x stored entries: the work of one step
    row_it = sum(float(mats[m][0]) * inner[k] for k, (_, m, _, _) in enumerate(reqs))
    nnz_it = sum(float(len(mats[m][2])) * inner[k] for k, (_, m, _, _) in enumerate(reqs))
    open_loop = serve_open_loop(ctx, mats, reqs, *knobs)
    low = serve_open_loop(ctx, mats, reqs, *knobs, rate=args.serve_low_rate)
    budget = int(args.serve_matrix_budget * (1 << 30))
    tight = serve_open_loop(ctx, mats, reqs, *knobs, rate=args.serve_low_rate, budget=budget)
    # GMRES(30) + Jacobi on the stream's Laplacians (the Poisson grids need
    # thousands of restarted iterations without a stronger preconditioner)
    lap = frozenset(i for i, sp in enumerate(specs) if sp[0] == "laplacian")
    with_gmres = serve_open_loop(ctx, mats, reqs, *knobs, rate=args.serve_low_rate, gmres_every=5, gmres_mats=lap)
    stream_bytes = sum(16 * len(mats[m][2]) + 8 * mats[m][0] for m in {m for _, m, _, _ in reqs})
    plain = plain_fp64(ctx, mats, reqs, args.plain_budget)
    sec = statistics.mean(times)
    value_rank = len(reqs) / sec
    plain_rate = len(plain) / sum(t for _, t, _ in plain)
    out = {"value": value_rank, "sec": sec, "e2e": open_loop["solves_s"], "plain": plain_rate, "c2": c2}
    objs = ranks.gather(out)
    ranks.close()
    if rank != 0:
        return
    sec_max = max(o["sec"] for o in objs)
    value = replica_rate(objs, len(reqs))
    e2e = sum(o["e2e"] for o in objs)
    cpu = None
    if not args.no_cpu:
        # the oracle on 1 core: full solves of the stream's first requests
        done, t_cpu = _oracle_requests(specs, reqs, range(len(reqs)), args.cpu_seconds, 80)
        cpu = {"value": done / t_cpu, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"oracle FP64 CG + Jacobi, full solves to rtol 1e-10 of the stream's first {done} "
                         f"requests in order ({t_cpu:.1f} s; matrices built before the clock starts)"}
    o0 = c2
    line = {
        "metric": "served solves/s", "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec_max, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": _serve_config(args, len(specs)),
        "timing": "CUDA events on the server's stream around each step (all requests submitted, then drained)",
        "served": {"failed": failed, "worst_rel_residual": worst, "mean_outer": float(np.mean(outer)),
                   "mean_inner": float(np.mean(inner)), "max_active": stats["max_active"],
                   "row_iterations_per_step": row_it, "nnz_iterations_per_step": nnz_it,
                   "inner_gbs": (8 * nnz_it + 56 * row_it) / sec / 1e9,
                   "inner_bytes": "8 per entry (FP32 value + column) + 56 per row (FP32 vectors) per inner iteration",
                   "scheduler_s": {k: stats[k] for k in ("gpu_s", "host_s", "wait_s")},
                   "mean_admitted_rows": stats["mean_rows"], "chunks": stats["chunks"]},
        "latency": {
            "p50_ms": open_loop["p50_ms"], "p99_ms": open_loop["p99_ms"], "arrival_rate": SERVE_RATE,
            "solves_s": open_loop["solves_s"],
            "below_capacity": {k: low[k] for k in ("offered_rate", "p50_ms", "p99_ms", "solves_s")},
            "matrix_budget": {**{k: tight[k] for k in ("offered_rate", "p50_ms", "p99_ms", "solves_s", "uploads",
                                                      "evictions")},
                              "budget_bytes": budget, "stream_matrix_bytes": stream_bytes,
                              "what": "below-capacity load with resident matrices held to the budget: idle "
                                      "matrices evicted LRU and uploaded again on their next request"},
            "with_gmres": {**{k: with_gmres[k] for k in ("offered_rate", "p50_ms", "p99_ms", "solves_s")},
                           "gmres": with_gmres.get("gmres"),
                           "what": "below-capacity load with every 5th request on a Laplacian a mixed-precision "
                                   "GMRES(30) + Jacobi solve on the Krylov lane; p50/p99 of the CG requests, and of "
                                   "the GMRES ones apart"}},
        "plain_fp64": {"solves_s": plain_rate, "requests": len(plain),
                       "mean_iterations": float(np.mean([it for _, _, it in plain])),
                       "what": "CG + DiagonalPreconditioner FP64, one request at a time through the host API"},
        "served_vs_plain": value / (world * plain_rate),
        "roofline": {"bound": "hbm", "achieved": o0["gbs_spmv"], "peak": o0["peak"], "unit": "GB/s",
                     "frac": o0["gbs_spmv"] / o0["peak"], "traffic": _traffic(args.grid),
                     "kernel": "k_spmv (CompRowMatrix.mult, 3D Poisson 128^3)", "peak_source": o0["peak_kind"]},
        "poisson3d_128": {"solves_s": 1e3 / o0["ms_solve"], "e2e_solves_s": 1e3 / o0["ms_e2e"],
                          "iterations": o0["iters"], "final_rel_residual": o0["rel_res"],
                          "spmv_us": o0["ms_spmv"] * 1e3, "spmv_gbs": o0["gbs_spmv"], "solve_hbm_gbs": o0["solve_gbs"],
                          "what": "plain FP64 CG + Jacobi on one 3D Poisson 128^3 system"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": open_loop["h2d_bytes"],
                "d2h_bytes_per_step": open_loop["d2h_bytes"],
                "what": "the arrival stream through the host API, matrices registered on first use"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


CONFIGS = {
    # name: (matrix, seed, solver, preconditioner, max iterations)
    "c1": (("poisson2d", 128), 1, "cg", "jacobi", 2000),
    "c2icc": (("poisson3d", 128), 2, "cg", "icc", MAX_ITER),
    "c3gmres": (("convdiff3d", 96), 3, "gmres", "ilu", MAX_ITER),
    "c3bicg": (("convdiff3d", 96), 3, "bicgstab", "ilu", MAX_ITER),
}


def run_config(args):
    """One of the other configurations: plain FP64 solves/s of one system,
    device-resident (CUDA events on the library's stream), plus the
    preconditioner's set-up time (setMatrix, host clock)."""
    from mtjg import _lib as L
    from mtjg import sparse, workloads

    (kind, N), seed, sname, pname, max_iter = CONFIGS[args.workload]
    lib = L.load()
    ctx = sparse.Context(int(os.environ.get("LOCAL_RANK", "0")))
    n, rp, ci, v = getattr(workloads, kind)(N)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    b = A.mult(workloads.uniform(n, seed))
    solver = {"cg": sparse.CG, "bicgstab": sparse.BiCGstab}[sname](n, ctx=ctx) if sname != "gmres" else \
        sparse.GMRES(n, restart=30, ctx=ctx)
    M = {"jacobi": lambda: sparse.DiagonalPreconditioner(n, ctx), "ilu": lambda: sparse.ILU(A),
         "icc": lambda: sparse.ICC(A)}[pname]()
    t0 = time.perf_counter()
    M.setMatrix(A)
    ctx.synchronize()
    setup_s = time.perf_counter() - t0
    solver.setPreconditioner(M)
    solver.setIterationMonitor(sparse.DefaultIterationMonitor(max_iter, RTOL, 1e-50, 1e5))
    solver._sync_monitor()
    db, dx = C.c_void_p(), C.c_void_p()
    lib.mtjg_dev_alloc(ctx.h, 8 * n, C.byref(db))
    lib.mtjg_dev_alloc(ctx.h, 8 * n, C.byref(dx))
    lib.mtjg_memcpy_h2d(ctx.h, db, b.ctypes.data_as(C.c_void_p), 8 * n)
    zeros = np.zeros(n)
    res = L.Result()
    times = []
    for i in range(args.warmup + args.steps):
        lib.mtjg_memcpy_h2d(ctx.h, dx, zeros.ctypes.data_as(C.c_void_p), 8 * n)
        lib.mtjg_ctx_event_record(ctx.h, 0)
        code = lib.mtjg_solver_solve_dev(solver.h, A.h, db, dx, C.byref(res))
        lib.mtjg_ctx_event_record(ctx.h, 1)
        ms = C.c_float()
        lib.mtjg_ctx_event_elapsed(ctx.h, 0, 1, C.byref(ms))
        if code != 0:
            raise RuntimeError(f"solve failed: {code} {L.last_error()}")
        if i >= args.warmup:
            times.append(ms.value)
    xh = np.empty(n)
    lib.mtjg_memcpy_d2h(ctx.h, xh.ctypes.data_as(C.c_void_p), dx, 8 * n)
    ms = statistics.mean(times)
    line = {"metric": "solves/s", "value": 1e3 / ms, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"{sname} + {pname}, {kind} {N}, rtol 1e-10, x0 = 0", "n": n, "nnz": len(ci),
                       "seed": seed},
            "iterations": res.iterations, "final_rel_residual": float(np.linalg.norm(b - A.mult(xh)) / np.linalg.norm(b)),
            "precond_setup_s": setup_s}
    print(json.dumps(line))


def _timed_solves(lib, ctx, solver, A, db, dx, n, steps, warmup):
    """Mean CUDA-event milliseconds of `steps` device-resident solves from
    x0 = 0 (after `warmup` untimed ones) and the last result."""
    from mtjg import _lib as L
    zeros = np.zeros(n)
    res = L.Result()
    times = []
    for i in range(warmup + steps):
        lib.mtjg_memcpy_h2d(ctx.h, dx, zeros.ctypes.data_as(C.c_void_p), 8 * n)
        lib.mtjg_ctx_event_record(ctx.h, 0)
        code = lib.mtjg_solver_solve_dev(solver.h, A.h, db, dx, C.byref(res))
        lib.mtjg_ctx_event_record(ctx.h, 1)
        ms = C.c_float()
        lib.mtjg_ctx_event_elapsed(ctx.h, 0, 1, C.byref(ms))
        if code != 0:
            raise RuntimeError(f"solve failed: {code} {L.last_error()}")
        if i >= warmup:
            times.append(ms.value)
    return statistics.mean(times), res


def run_c3mixed(args):
    """The precision form on 3D convection-diffusion 96^3: GMRES(30) + ILU(0)
    and BiCGstab + ILU(0), plain FP64 against mixed precision (FP32 inner
    solves with an FP32 ILU copy inside FP64 refinement), both to rtol 1e-10
    on the FP64 true residual; device-resident, CUDA events.  The oracle's
    FP64 GMRES(30) + ILU solve is the CPU baseline and the reference solution
    for the final error."""
    from mtjg import _lib as L
    from mtjg import sparse, workloads

    (kind, N), seed = ("convdiff3d", 96), 3
    lib = L.load()
    ctx = sparse.Context(int(os.environ.get("LOCAL_RANK", "0")))
    n, rp, ci, v = workloads.convdiff3d(N)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    b = A.mult(workloads.uniform(n, seed))
    M = sparse.ILU(A)
    M.setMatrix(A)
    db, dx = C.c_void_p(), C.c_void_p()
    lib.mtjg_dev_alloc(ctx.h, 8 * n, C.byref(db))
    lib.mtjg_dev_alloc(ctx.h, 8 * n, C.byref(dx))
    lib.mtjg_memcpy_h2d(ctx.h, db, b.ctypes.data_as(C.c_void_p), 8 * n)
    out, xs = {}, {}
    for sname in ("gmres", "bicgstab"):
        for mode in ("fp64", "mixed"):
            solver = sparse.GMRES(n, restart=30, ctx=ctx) if sname == "gmres" else sparse.BiCGstab(n, ctx=ctx)
            solver.setPreconditioner(M)
            solver.setIterationMonitor(sparse.DefaultIterationMonitor(MAX_ITER if mode == "fp64" else 100, RTOL,
                                                                      1e-50, 1e5))
            if mode == "mixed":
                solver.setMixedPrecision(True, args.inner_rtol_c3, 3000)
            solver._sync_monitor()
            ms, res = _timed_solves(lib, ctx, solver, A, db, dx, n, args.steps, args.warmup)
            xh = np.empty(n)
            lib.mtjg_memcpy_d2h(ctx.h, xh.ctypes.data_as(C.c_void_p), dx, 8 * n)
            xs[(sname, mode)] = xh
            out.setdefault(sname, {})[mode] = {
                "ms": ms, "solves_s": 1e3 / ms, "iterations": res.iterations,
                "inner_iterations": res.inner_iterations if mode == "mixed" else None,
                "final_rel_residual": float(np.linalg.norm(b - A.mult(xh)) / np.linalg.norm(b))}
        out[sname]["mixed_vs_fp64"] = out[sname]["fp64"]["ms"] / out[sname]["mixed"]["ms"]
        out[sname]["max_abs_diff_mixed_vs_fp64"] = float(np.max(np.abs(xs[(sname, "mixed")] - xs[(sname, "fp64")])))
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, ORACLE_DIR)
        import oracle as O
        Ao = O.Csr(n, n, rp, ci, v)
        pc = O.Precond(O.PC_ILU, n)
        t0 = time.perf_counter()
        pc.set_matrix(Ao)
        xo, ores, _, _ = O.solve(O.GMRES, Ao, b, np.zeros(n), pc, max_iter=MAX_ITER, rtol=RTOL, hist_cap=0)
        t_cpu = time.perf_counter() - t0
        cpu = {"value": 1.0 / t_cpu, "unit": "solves/s", "cores": 1, "kind": "port",
               "sample": f"one oracle FP64 GMRES(30) + ILU(0) solve of this system (factorisation included), "
                         f"{ores.iterations} iterations, {t_cpu:.1f} s"}
        scale = float(np.max(np.abs(xo)))
        for sname in ("gmres", "bicgstab"):
            for mode in ("fp64", "mixed"):
                out[sname][mode]["max_rel_error_vs_oracle"] = float(np.max(np.abs(xs[(sname, mode)] - xo)) / scale)
    g = out["gmres"]["mixed"]
    line = {"metric": "solves/s", "value": g["solves_s"], "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": g["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": f"mixed-precision GMRES(30) + ILU(0), {kind} {N}^3, rtol 1e-10 on the FP64 "
                                   f"true residual, x0 = 0 (BiCGstab + ILU(0) and the FP64 solves beside it)",
                       "n": n, "nnz": len(ci), "seed": seed, "inner_rtol": args.inner_rtol_c3},
            "solvers": out, "cpu_baseline": cpu}
    print(json.dumps(line))


def run_batch(args):
    """The batched configuration: 4096 random SPD Laplacians (n log-uniform
    in [500, 50000]) in one block-diagonal batch, CG + Jacobi per system to
    rtol 1e-10, FP64 and mixed precision; device-resident, CUDA events."""
    from concurrent.futures import ThreadPoolExecutor
    from mtjg import _lib as L
    from mtjg import sparse, workloads

    poisson = args.workload == "c4poisson"
    if poisson:
        # 2D Poisson grids N log-uniform in [32, 256]: hundreds of CG
        # iterations per system, where FP32 inner iterations pay
        count = args.batch_systems if args.batch_systems != 4096 else 1024
        grids = workloads.batch_sizes(count, 14, 32, 256)
        with ThreadPoolExecutor(16) as ex:
            systems = list(ex.map(lambda k: workloads.poisson2d(int(grids[k])), range(count)))
        what = f"batched: {count} 2D 5-point Poisson systems, grid N log-uniform [32, 256], CG + Jacobi, rtol 1e-10"
        seed = 14
    else:
        count = args.batch_systems
        sizes = workloads.batch_sizes(count, 4)
        with ThreadPoolExecutor(16) as ex:
            systems = list(ex.map(lambda k: workloads.laplacian(int(sizes[k]), 4 + k), range(count)))
        what = f"batched: {count} random SPD Laplacians, n log-uniform [500, 50000], CG + Jacobi, rtol 1e-10"
        seed = 4
    lib = L.load()
    ctx = sparse.Context(int(os.environ.get("LOCAL_RANK", "0")))
    A = sparse.BatchCompRowMatrix(systems, ctx)
    nt = A.numRows()
    b = np.concatenate([workloads.uniform(s[0], 100 + k) for k, s in enumerate(systems)])
    db, dx = C.c_void_p(), C.c_void_p()
    lib.mtjg_dev_alloc(ctx.h, 8 * nt, C.byref(db))
    lib.mtjg_dev_alloc(ctx.h, 8 * nt, C.byref(dx))
    lib.mtjg_memcpy_h2d(ctx.h, db, b.ctypes.data_as(C.c_void_p), 8 * nt)
    zeros = np.zeros(nt)
    out = {}
    for mode in ("fp64", "mixed"):
        solver = sparse.CG(nt, ctx=ctx)
        M = sparse.DiagonalPreconditioner(nt, ctx)
        M.setMatrix(A)
        solver.setPreconditioner(M)
        solver.setIterationMonitor(sparse.DefaultIterationMonitor(MAX_ITER if mode == "fp64" else 100, RTOL,
                                                                  1e-50, 1e5))
        if mode == "mixed":
            solver.setMixedPrecision(True, args.inner_rtol, 2000)
        solver._sync_monitor()
        res = L.Result()
        times = []
        for i in range(args.warmup + args.steps):
            lib.mtjg_memcpy_h2d(ctx.h, dx, zeros.ctypes.data_as(C.c_void_p), 8 * nt)
            lib.mtjg_ctx_event_record(ctx.h, 0)
            code = lib.mtjg_solver_solve_dev(solver.h, A.h, db, dx, C.byref(res))
            lib.mtjg_ctx_event_record(ctx.h, 1)
            ms = C.c_float()
            lib.mtjg_ctx_event_elapsed(ctx.h, 0, 1, C.byref(ms))
            if code not in (0, 1, 2, 3):
                raise RuntimeError(f"batch solve failed: {code} {L.last_error()}")
            if i >= args.warmup:
                times.append(ms.value)
        per = (L.Result * count)()
        lib.mtjg_solver_batch_results(solver.h, per, count)
        its = [per[k].iterations for k in range(count)]
        out[mode] = {"ms": statistics.mean(times), "solves_s": count * 1e3 / statistics.mean(times),
                     "converged": sum(1 for k in range(count) if per[k].status == 0),
                     "max_iterations": max(its), "mean_iterations": float(np.mean(its))}
    # the lanes per row the batch autotuner chose, per system class present
    tuned = {}
    for k, (n_k, rp_k, _, _) in enumerate(systems):
        lanes = C.c_int(0)
        lib.mtjg_batch_tuning(n_k, int(rp_k[-1]), C.byref(lanes))
        rows_band = int(np.searchsorted([2048, 8192, 32768, 131072], n_k, side="right"))
        per_band = int(np.searchsorted([6, 12, 24, 48], rp_k[-1] / max(1, n_k), side="right"))
        tuned[f"rows band {rows_band}, entries/row band {per_band}"] = lanes.value
    line = {"metric": "batched solves/s", "value": out["mixed"]["solves_s"], "unit": "solves/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["mixed"]["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": what, "rows": nt, "nnz": int(A.rowptr[-1]), "seed": seed},
            "fp64": out["fp64"], "mixed": out["mixed"], "mixed_vs_fp64": out["fp64"]["ms"] / out["mixed"]["ms"],
            "launch": "one persistent launch per solve (each CTA runs whole systems, largest first)",
            "tuned_lanes_per_row": dict(sorted(tuned.items()))}
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
