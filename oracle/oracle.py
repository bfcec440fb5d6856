"""ctypes wrapper of the CPU restatement of MTJ's Krylov path (mtj_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker that the GPU library is compared
against.  Only tests, the smoke check and the CPU-baseline leg of the
benchmark import it; the product never does.

Parity pinning: the reference ships no golden vectors (its tests draw
unseeded Math.random inputs) and no JDK exists here to run it, so the oracle
is pinned by the properties the reference's own tests check (exact ILU/ICC
solves on tri/penta-diagonal systems, products against dense loops, solvers
recovering x within 1e-4) and by an independent pure-Python restatement on
small cases; see tests/test_oracle_*.py.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build", platform.machine())
SO = os.path.join(BUILD, "libmtj_oracle.so")
SRC = os.path.join(HERE, "mtj_oracle.c")

OK, NC_ITERATIONS, NC_DIVERGENCE, NC_BREAKDOWN = 0, 1, 2, 3
ERR_ILLEGAL_ARGUMENT, ERR_ZERO_PIVOT, ERR_ZERO_DIAGONAL, ERR_MISSING_DIAGONAL, ERR_SINGULAR = 10, 20, 21, 22, 23
ERR_UNSUPPORTED = 30
NORM_ONE, NORM_TWO, NORM_TWO_ROBUST, NORM_INFINITY = 0, 1, 2, 3
PC_IDENTITY, PC_JACOBI, PC_ILU, PC_ICC, PC_ICC_LITERAL, PC_SSOR, PC_ILUT = 0, 1, 2, 3, 4, 5, 6
CG, BICGSTAB, GMRES, BICG, CGS, QMR, CHEBYSHEV, IR = 0, 1, 2, 3, 4, 5, 6, 7
# breakdown detail: which quantity became zero
BD_RHO, BD_OMEGA, BD_XI, BD_DELTA, BD_EP, BD_BETA, BD_GAMMA = 1, 2, 3, 4, 5, 6, 7


def build() -> str:
    """Compiles the oracle with Java's rounding (no contraction of a*b+c)."""
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(SO) and os.path.getmtime(SO) >= max(os.path.getmtime(SRC),
                                                            os.path.getmtime(SRC[:-1] + "h")):
        return SO
    subprocess.run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
                    "-o", SO, SRC, "-lm"], check=True)
    return SO


class Monitor(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("rtol", C.c_double), ("atol", C.c_double),
                ("dtol", C.c_double), ("norm", C.c_int), ("matrix", C.c_int), ("normA", C.c_double),
                ("normb", C.c_double)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("residual", C.c_double),
                ("detail", C.c_int), ("history_len", C.c_int)]


_lib = None
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def lib():
    global _lib
    if _lib is None:
        l = C.CDLL(build())
        l.or_mult.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp]
        l.or_mult_add.argtypes = [C.c_int, _ip, _ip, _dp, C.c_double, _dp, _dp]
        l.or_trans_mult.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp]
        l.or_trans_mult_add.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, C.c_double, _dp, _dp]
        l.or_dot.argtypes = [C.c_int, _dp, _dp]
        l.or_dot.restype = C.c_double
        l.or_norm.argtypes = [C.c_int, _dp, C.c_int]
        l.or_norm.restype = C.c_double
        l.or_pc_new.argtypes = [C.c_int, C.c_int]
        l.or_pc_new.restype = C.c_void_p
        l.or_pc_free.argtypes = [C.c_void_p]
        l.or_pc_set_matrix.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _dp, _ip]
        l.or_pc_apply.argtypes = [C.c_void_p, _dp, _dp]
        l.or_pc_trans_apply.argtypes = [C.c_void_p, _dp, _dp]
        l.or_pc_values.argtypes = [C.c_void_p, _dp, C.c_int]
        l.or_pc_pattern.argtypes = [C.c_void_p, _ip, _ip, C.c_int]
        l.or_pc_diag.argtypes = [C.c_void_p, _ip]
        l.or_pc_set_params.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
        l.or_solve.restype = C.c_int
        l.or_solve.argtypes = [C.c_int, C.c_int, C.c_int, _ip, _ip, _dp, C.c_void_p, _dp, _dp,
                               C.POINTER(Monitor), C.POINTER(Result), _dp, _ip, C.c_int]
        l.or_solve_ex.restype = C.c_int
        l.or_solve_ex.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _ip, _ip, _dp, C.c_void_p,
                                  _dp, _dp, C.POINTER(Monitor), C.POINTER(Result), _dp, _ip, C.c_int]
        l.or_set_sum_order.argtypes = [C.c_int]
        _lib = l
    return _lib


class sum_order:
    """Context manager: run the oracle with dot products and norms summed in
    blocks of `block` entries combined pairwise, instead of MTJ's sequential
    sums, to measure how much a solver's history depends on the order of its
    reductions alone."""

    def __init__(self, block=256):
        self.mode = int(block)

    def __enter__(self):
        lib().or_set_sum_order(self.mode)

    def __exit__(self, *a):
        lib().or_set_sum_order(0)


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


class Csr:
    def __init__(self, n, m, rowptr, colind, val):
        self.n, self.m = int(n), int(m)
        self.rp = np.ascontiguousarray(rowptr, dtype=np.int32)
        self.ci = np.ascontiguousarray(colind, dtype=np.int32)
        self.v = np.ascontiguousarray(val, dtype=np.float64)
        if len(self.ci) == 0:
            self.ci = np.zeros(1, dtype=np.int32)
            self.v = np.zeros(1)


def mult(A: Csr, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(max(A.n, 1))
    lib().or_mult(A.n, _i(A.rp), _i(A.ci), _d(A.v), _d(x), _d(y))
    return y[: A.n]


def mult_add(A: Csr, alpha, x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.array(y, dtype=np.float64, copy=True)
    lib().or_mult_add(A.n, _i(A.rp), _i(A.ci), _d(A.v), alpha, _d(x), _d(y))
    return y


def trans_mult(A: Csr, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(max(A.m, 1))
    lib().or_trans_mult(A.n, A.m, _i(A.rp), _i(A.ci), _d(A.v), _d(x), _d(y))
    return y[: A.m]


def trans_mult_add(A: Csr, alpha, x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.array(y, dtype=np.float64, copy=True)
    lib().or_trans_mult_add(A.n, A.m, _i(A.rp), _i(A.ci), _d(A.v), alpha, _d(x), _d(y))
    return y


def dot(x, y):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    return lib().or_dot(len(x), _d(x), _d(y))


def norm(x, kind=NORM_TWO):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return lib().or_norm(len(x), _d(x), kind)


class Precond:
    def __init__(self, kind, n):
        self.kind, self.n = kind, n
        self.h = lib().or_pc_new(kind, n)
        self.status = None
        self.detail = 0

    def set_matrix(self, A: Csr):
        d = C.c_int(0)
        self.status = lib().or_pc_set_matrix(self.h, A.n, _i(A.rp), _i(A.ci), _d(A.v), C.byref(d))
        self.detail = d.value
        return self.status

    def set_params(self, a, b=0.0, c=0):
        """SSOR: (omegaF, omegaR, reverse); ILUT: (tau, unused, p)."""
        return lib().or_pc_set_params(self.h, float(a), float(b), int(c))

    def apply(self, b, x0=None):
        """M.apply(b, x); x0 is x's content before the call (SSOR starts its
        sweep from it; the others ignore it).  Default: zeros."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(max(self.n, 1))
        if x0 is not None:
            x[: self.n] = x0
        lib().or_pc_apply(self.h, _d(b), _d(x))
        return x[: self.n]

    def pattern(self):
        """(rowptr, colind, diag) of the factor (ILUT: its rows after the factor)."""
        nnz = lib().or_pc_pattern(self.h, None, None, 0)
        rp = np.empty(self.n + 1, dtype=np.int32)
        ci = np.empty(max(nnz, 1), dtype=np.int32)
        lib().or_pc_pattern(self.h, _i(rp), _i(ci), nnz)
        dg = np.empty(max(self.n, 1), dtype=np.int32)
        lib().or_pc_diag(self.h, _i(dg))
        return rp, ci[:nnz], dg[: self.n]

    def trans_apply(self, b, x0=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(max(self.n, 1))
        if x0 is not None:
            x[: self.n] = x0
        lib().or_pc_trans_apply(self.h, _d(b), _d(x))
        return x[: self.n]

    def values(self):
        n = lib().or_pc_values(self.h, None, 0)
        out = np.empty(max(n, 1))
        lib().or_pc_values(self.h, _d(out), n)
        return out[:n]

    def __del__(self):
        try:
            lib().or_pc_free(self.h)
        except Exception:
            pass


def solve(kind, A: Csr, b, x0, pc: Precond | None = None, max_iter=100000, rtol=1e-5, atol=1e-50, dtol=1e5,
          norm_type=NORM_TWO, restart=30, hist_cap=None, eigmin=0.0, eigmax=0.0, matrix_norms=None):
    """Runs the restated solver; returns (x, Result, hist_r, hist_it).
    eigmin / eigmax are Chebyshev's eigenvalue bounds; matrix_norms =
    (normA, normb) makes the monitor a MatrixIterationMonitor."""
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.array(x0, dtype=np.float64, copy=True)
    if hist_cap is None:
        hist_cap = 2 * max_iter + 64
    hr = np.empty(max(hist_cap, 1))
    hi = np.empty(max(hist_cap, 1), dtype=np.int32)
    mon = Monitor(max_iter, rtol, atol, dtol, norm_type)
    if matrix_norms is not None:
        mon.matrix = 1
        mon.normA, mon.normb = float(matrix_norms[0]), float(matrix_norms[1])
    res = Result()
    res.status = lib().or_solve_ex(kind, restart, eigmin, eigmax, A.n, _i(A.rp), _i(A.ci), _d(A.v),
                                   pc.h if pc else None, _d(b), _d(x) if len(x) else _d(np.zeros(1)), C.byref(mon),
                                   C.byref(res), _d(hr), _i(hi), hist_cap)
    k = min(res.history_len, hist_cap)
    return x, res, hr[:k].copy(), hi[:k].copy()
