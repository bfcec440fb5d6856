"""Continuous-batching solve server (include/mtjg.h, mtjg_server_*).

    srv = Server(max_systems=256, pool_rows=1 << 24, matrix_budget=8 << 30)
    mid = srv.addMatrix(n, rowptr, colind, data)      # uploaded now or on first use
    t = srv.submit(mid, b)                            # returns a ticket
    for r in srv.poll(): ...                          # finished requests
    srv.drain(); srv.close()

Each request is solved by mixed-precision CG + Jacobi (FP64 refinement,
FP32 inner iterations) to `rtol` on the FP64 true residual; requests
submitted with solver="gmres" or "bicgstab" take a second lane
(mixed-precision GMRES(30) / BiCGstab + Jacobi, one at a time on its own
stream, concurrently with the CG batch).  With a
`matrix_budget` (bytes) the resident matrices are evicted least recently used
when idle and uploaded again on their next request.  No counterpart in the
reference.
"""
from __future__ import annotations

import ctypes as C
import sys
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .sparse import Context, _raise, default_context


@dataclass
class Finished:
    ticket: int
    matrix: int
    status: int
    iterations: int
    inner_iterations: int
    residual: float
    latency_s: float
    queue_s: float
    x: np.ndarray


class Server:
    def __init__(self, ctx: Context | None = None, max_systems=256, pool_rows=1 << 24, max_iter=100, rtol=1e-10,
                 atol=1e-50, dtol=1e5, inner_rtol=1e-6, inner_max_iter=2000, matrix_budget=0):
        self.ctx = ctx or default_context()
        self._lib = self.ctx._lib
        cfg = L.ServerConfig()
        self._lib.mtjg_server_config_defaults(C.byref(cfg))
        cfg.max_systems, cfg.pool_rows, cfg.max_iter = int(max_systems), int(pool_rows), int(max_iter)
        cfg.rtol, cfg.atol, cfg.dtol = float(rtol), float(atol), float(dtol)
        cfg.inner_rtol, cfg.inner_max_iter = float(inner_rtol), int(inner_max_iter)
        cfg.matrix_budget = int(matrix_budget)
        h = C.c_void_p()
        _raise(self._lib.mtjg_server_create(self.ctx.h, C.byref(cfg), C.byref(h)), "server_create")
        self.h = h
        self._out = {}   # ticket -> (x, b) kept alive until the request finishes
        self.sizes = {}

    def addMatrix(self, n, rowptr, colind, data) -> int:
        rp, ci, v = L.i32(rowptr), L.i32(colind), L.f64(data)
        mid = C.c_int()
        _raise(self._lib.mtjg_server_add_matrix(self.h, int(n), L.iptr(rp), L.iptr(ci), L.dptr(v), C.byref(mid)),
               "add_matrix")
        self.sizes[mid.value] = int(n)
        return mid.value

    def removeMatrix(self, mid: int):
        """Releases a registered matrix (freed once its requests are reported)."""
        _raise(self._lib.mtjg_server_remove_matrix(self.h, int(mid)), "remove_matrix")
        self.sizes.pop(mid, None)

    SOLVERS = {"cg": L.CG, "gmres": L.GMRES, "bicgstab": L.BICGSTAB}

    def submit(self, mid: int, b, x0=None, solver: str = "cg") -> int:
        """Queues a solve; solver "cg" joins the batched lane, "gmres" and
        "bicgstab" the Krylov lane (mtjg_server_submit_solver)."""
        n = self.sizes[mid]
        b = L.f64(b)
        if b.shape != (n,):
            raise ValueError("b has the wrong size")
        x = np.zeros(n)
        x0p = L.dptr(L.f64(x0)) if x0 is not None else None
        t = C.c_int64()
        _raise(self._lib.mtjg_server_submit_solver(self.h, mid, self.SOLVERS[solver], L.dptr(b), x0p, L.dptr(x),
                                                   C.byref(t)), "submit")
        self._out[t.value] = (x, b)
        return t.value

    def poll(self, cap=1024):
        out = (L.ServerResult * cap)()
        k = C.c_int()
        _raise(self._lib.mtjg_server_poll(self.h, out, cap, C.byref(k)), "poll")
        res = []
        for i in range(k.value):
            r = out[i]
            x, _ = self._out.pop(r.ticket)
            res.append(Finished(r.ticket, r.matrix, r.result.status, r.result.iterations, r.result.inner_iterations,
                                r.result.residual, r.latency_s, r.queue_s, x))
        return res

    def drain(self, timeout=600.0):
        _raise(self._lib.mtjg_server_drain(self.h, float(timeout)), "drain")

    def stats(self):
        c, a, m, t = C.c_int64(), C.c_int64(), C.c_int64(), C.c_double()
        _raise(self._lib.mtjg_server_stats(self.h, C.byref(c), C.byref(a), C.byref(m), C.byref(t)), "stats")
        return {"chunks": c.value, "admitted": a.value, "max_active": m.value, "clock_s": t.value}

    def residency(self):
        """Resident matrix bytes and count, uploads (registrations included), evictions."""
        v = [C.c_int64() for _ in range(4)]
        _raise(self._lib.mtjg_server_residency(self.h, *[C.byref(x) for x in v]), "residency")
        return dict(zip(("resident_bytes", "resident_matrices", "uploads", "evictions"), (x.value for x in v)))

    def timing(self):
        g, h, w, r = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        _raise(self._lib.mtjg_server_timing(self.h, C.byref(g), C.byref(h), C.byref(w), C.byref(r)), "timing")
        return {"gpu_s": g.value, "host_s": h.value, "wait_s": w.value, "mean_rows": r.value}

    def event(self, slot: int):
        """Records event `slot` on the server's stream."""
        _raise(self._lib.mtjg_ctx_event_record(self._ctx(), slot), "event_record")

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        _raise(self._lib.mtjg_ctx_event_elapsed(self._ctx(), a, b, C.byref(ms)), "event_elapsed")
        return ms.value

    def launchCount(self) -> int:
        """Kernels the server has launched so far."""
        return int(self._lib.mtjg_ctx_launch_count(self._ctx()))

    def _ctx(self):
        h = C.c_void_p()
        _raise(self._lib.mtjg_server_context(self.h, C.byref(h)), "server_context")
        return h

    def close(self):
        if getattr(self, "h", None):
            self._lib.mtjg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass
