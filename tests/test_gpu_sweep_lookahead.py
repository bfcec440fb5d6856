"""Triangular sweeps with and without lookahead give the same bits.

With lookahead a row whose dependency is still pending computes that
dependency's value itself, with the operations of the dependency's own row
in the same order; the stored results, and so every solve built on them,
must not change.  Each test runs with every mode looking ahead
(MTJG_SWEEP_LOOKAHEAD=7) and with none (0); the default set lies between.
Covered: ILU(0) L and U sweeps and the ICC transposed-gather and U sweeps
(FP64, both numerics), the FP32 ILU sweeps of a mixed-precision GMRES, and a
matrix whose rows exceed the lookahead's four entries (those rows wait
instead).  Parity of the sweeps
with the oracle is covered by the parity and config tests.
"""
import os

import numpy as np
import pytest

from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[0, 1], ids=["fast", "strict"])
def numerics(request, ctx):
    ctx.setNumerics(request.param)
    yield request.param
    ctx.setNumerics(0)


def _with_lookahead(on, fn):
    old = os.environ.get("MTJG_SWEEP_LOOKAHEAD")
    os.environ["MTJG_SWEEP_LOOKAHEAD"] = "7" if on else "0"
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["MTJG_SWEEP_LOOKAHEAD"]
        else:
            os.environ["MTJG_SWEEP_LOOKAHEAD"] = old


def _solve(ctx, mat, solver_cls, pc_cls, mixed=False, max_iter=400):
    n, rp, ci, v = mat
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    solver = solver_cls(n, ctx=ctx)
    M = pc_cls(A)
    M.setMatrix(A)
    solver.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(max_iter, 1e-10, 1e-50, 1e5)
    mon.setIterationReporter(sparse.IterationReporter(), history_cap=max_iter + 8)
    solver.setIterationMonitor(mon)
    if mixed:
        solver.setMixedPrecision(True, 1e-4, 1000)
    b = workloads.uniform(n, 17)
    x = np.zeros(n)
    solver.solve(A, b, x)
    gr, _ = solver.history
    return x, np.array(gr), mon.iterations()


def _apply(ctx, mat, pc_cls):
    n, rp, ci, v = mat
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    M = pc_cls(A)
    M.setMatrix(A)
    return M.apply(workloads.uniform(n, 23))


def _same(a, b):
    for u, w in zip(a, b):
        u, w = np.asarray(u), np.asarray(w)
        if u.dtype == np.float64:
            assert np.array_equal(u.view(np.int64), w.view(np.int64))
        else:
            assert np.array_equal(u, w)


@pytest.mark.parametrize("case", ["ilu_bicgstab", "icc_cg"])
def test_lookahead_solves_are_identical(ctx, numerics, case):
    if case == "ilu_bicgstab":
        mat, sc, pc = workloads.convdiff3d(20), sparse.BiCGstab, sparse.ILU
    else:
        mat, sc, pc = workloads.poisson3d(20), sparse.CG, sparse.ICC
    on = _with_lookahead(True, lambda: _solve(ctx, mat, sc, pc))
    off = _with_lookahead(False, lambda: _solve(ctx, mat, sc, pc))
    _same(on, off)
    assert on[2] > 5


@pytest.mark.parametrize("pc", ["ilu", "icc"])
def test_lookahead_applies_are_identical(ctx, numerics, pc):
    mat = workloads.poisson2d(60)
    cls = sparse.ILU if pc == "ilu" else sparse.ICC
    _same([_with_lookahead(True, lambda: _apply(ctx, mat, cls))], [_with_lookahead(False, lambda: _apply(ctx, mat, cls))])


def test_lookahead_fp32_sweeps_are_identical(ctx):
    mat = workloads.convdiff3d(20)
    on = _with_lookahead(True, lambda: _solve(ctx, mat, sparse.GMRES, sparse.ILU, mixed=True))
    off = _with_lookahead(False, lambda: _solve(ctx, mat, sparse.GMRES, sparse.ILU, mixed=True))
    _same(on, off)


def test_lookahead_wide_rows_are_identical(ctx, numerics):
    """Rows of up to ~20 entries each side of the diagonal: dependencies of
    more than four entries are waited for, the rest computed ahead."""
    rng = np.random.default_rng(9)
    n = 3000
    A = np.zeros((n, n))
    for i in range(n):
        for j in rng.integers(max(0, i - 60), min(n, i + 60), int(rng.integers(1, 12))):
            A[i, j] = A[j, i] = -rng.random()
    A[np.diag_indices(n)] = np.abs(A).sum(axis=1) + 1.0
    rp = np.zeros(n + 1, dtype=np.int32)
    ci, v = [], []
    for i in range(n):
        nz = np.nonzero(A[i])[0]
        ci.extend(nz)
        v.extend(A[i, nz])
        rp[i + 1] = len(ci)
    mat = (n, rp, np.array(ci, dtype=np.int32), np.array(v))
    on = _with_lookahead(True, lambda: _solve(ctx, mat, sparse.BiCGstab, sparse.ILU))
    off = _with_lookahead(False, lambda: _solve(ctx, mat, sparse.BiCGstab, sparse.ILU))
    _same(on, off)
