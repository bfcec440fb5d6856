"""Seeded test systems shaped like the reference's own tests.

The reference draws these with unseeded Math.random (T/Utilities.java:48-198,
TS/IterativeSolverTestAbstract.java:110-124); here a numpy Generator with a
fixed seed stands in, with the same shapes: up to `per_row` random entries
U[0,1) per row at uniform columns, a diagonal shift added until the
requested property holds.
"""
from __future__ import annotations

import numpy as np


def dense_to_csr(A, keep_diag=True):
    A = np.asarray(A, dtype=np.float64)
    n, m = A.shape
    rp = [0]
    ci, v = [], []
    for i in range(n):
        for j in range(m):
            if A[i, j] != 0 or (keep_diag and i == j):
                ci.append(j)
                v.append(A[i, j])
        rp.append(len(ci))
    return n, m, np.array(rp, dtype=np.int32), np.array(ci, dtype=np.int32), np.array(v, dtype=np.float64)


def row_populate(n, m, per_row, rng):
    """Utilities.rowPopulate: per_row draws of (column, value) per row."""
    A = np.zeros((n, m))
    for i in range(n):
        for _ in range(per_row):
            A[i, int(rng.random() * m)] = rng.random()
    return A


def symmetry_populate(n, per_band, rng):
    """Utilities.symmetryPopulate: per column j, per_band symmetric pairs."""
    A = np.zeros((n, n))
    for j in range(n):
        for _ in range(per_band):
            val = rng.random()
            k = int(rng.random() * n)
            A[k, j] = val
            A[j, k] = val
    return A


def nonsingular_system(n, b, rng, shift=100.0):
    """IterativeSolverTestAbstract.createMatrix: shift until nonsingular."""
    A = row_populate(n, n, b, rng)
    A[np.diag_indices(n)] += shift
    while abs(np.linalg.det(A)) < 1e-300 or np.linalg.cond(A) > 1e12:
        A[np.diag_indices(n)] += shift
    return A


def spd_system(n, b, rng, shift=100.0):
    """SPDIterativeSolverTestAbstract.createMatrix: shift until SPD."""
    A = symmetry_populate(n, b, rng)
    A[np.diag_indices(n)] += shift
    while n > 0 and np.linalg.eigvalsh(A)[0] <= 0:
        A[np.diag_indices(n)] += shift
    return A


def tridiagonal(n):
    A = np.zeros((n, n))
    for i in range(n):
        A[i, i] = 2
    for i in range(n - 1):
        A[i, i + 1] = A[i + 1, i] = -1
    return A


def pentadiagonal(n):
    A = np.zeros((n, n))
    for i in range(n):
        A[i, i] = 4
    for i in range(n - 1):
        A[i, i + 1] = A[i + 1, i] = -1
    for i in range(n - 2):
        A[i, i + 2] = A[i + 2, i] = -1
    return A
