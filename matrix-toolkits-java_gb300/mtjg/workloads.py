"""Seeded synthetic systems of the measured shapes (libmtjg_workloads.so).

  poisson2d(N)      2D 5-point Poisson on N x N (4 / -1)
  poisson3d(N)      3D 7-point Poisson on N^3 (6 / -1)
  convdiff3d(N)     3D upwind convection-diffusion, cell Peclet (0.5, 0.25, 0.125)
  laplacian(n, s)   random SPD graph Laplacian + 1e-2 I, 5..30 entries per row
  uniform(n, s)     U[lo, hi) vector from splitmix64(seed)
Each returns (n, rowptr, colind, data) as int32/int32/float64 numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import WORKLOADS_PATH

_w = None


def _lib():
    global _w
    if _w is None:
        if not os.path.exists(WORKLOADS_PATH):
            raise RuntimeError(f"{WORKLOADS_PATH} is missing: run matrix-toolkits-java_gb300/build.py")
        w = C.CDLL(WORKLOADS_PATH)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        w.mtjw_uniform.argtypes = [C.c_int64, C.c_uint64, C.c_double, C.c_double, dp]
        w.mtjw_uniform.restype = None
        w.mtjw_stencil_nnz.argtypes = [C.c_int, C.c_int]
        w.mtjw_stencil_nnz.restype = C.c_int64
        for f in ("mtjw_poisson2d", "mtjw_poisson3d", "mtjw_convdiff3d"):
            getattr(w, f).argtypes = [C.c_int, ip, ip, dp]
            getattr(w, f).restype = None
        w.mtjw_batch_sizes.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_int, ip]
        w.mtjw_batch_sizes.restype = None
        w.mtjw_laplacian.argtypes = [C.c_int, C.c_uint64, C.c_double, ip, ip, dp]
        w.mtjw_laplacian.restype = C.c_int64
        _w = w
    return _w


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def uniform(n: int, seed: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    out = np.empty(n)
    _lib().mtjw_uniform(n, seed, lo, hi, _p(out, C.c_double))
    return out


def _stencil(fn: str, dim: int, N: int):
    w = _lib()
    n = N ** dim
    nnz = w.mtjw_stencil_nnz(dim, N)
    rp = np.empty(n + 1, dtype=np.int32)
    ci = np.empty(nnz, dtype=np.int32)
    v = np.empty(nnz)
    getattr(w, fn)(N, _p(rp, C.c_int), _p(ci, C.c_int), _p(v, C.c_double))
    return n, rp, ci, v


def poisson2d(N: int):
    return _stencil("mtjw_poisson2d", 2, N)


def poisson3d(N: int):
    return _stencil("mtjw_poisson3d", 3, N)


def convdiff3d(N: int):
    return _stencil("mtjw_convdiff3d", 3, N)


def laplacian(n: int, seed: int, shift: float = 1e-2):
    w = _lib()
    nnz = w.mtjw_laplacian(n, seed, shift, None, None, None)
    rp = np.empty(n + 1, dtype=np.int32)
    ci = np.empty(nnz, dtype=np.int32)
    v = np.empty(nnz)
    w.mtjw_laplacian(n, seed, shift, _p(rp, C.c_int), _p(ci, C.c_int), _p(v, C.c_double))
    return n, rp, ci, v


def batch_sizes(count: int, seed: int, lo: int = 500, hi: int = 50000) -> np.ndarray:
    out = np.empty(count, dtype=np.int32)
    _lib().mtjw_batch_sizes(count, seed, lo, hi, _p(out, C.c_int))
    return out
