"""Skewed rows: an SPD arrow matrix whose first row and column hold every
column / row (200,000 entries), beside ordinary rows.  In FAST numerics a
row longer than a stage is summed ahead by many CTAs (fixed segments, then
the segments in order); the product, the transposed product and CG + Jacobi
(FP64 and mixed) must still match the oracle, and STRICT keeps MTJ's
sequential sum bit for bit."""
import numpy as np
import pytest

import oracle as O
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu

N = 200_000


def _arrow(n=N):
    """Row 0 and column 0 full (1e-3 off the diagonal), a -1/4/-1 band on the
    rest; diagonally dominant, so SPD."""
    import scipy.sparse as sp
    i = np.arange(1, n)
    rows = np.concatenate(([0], np.zeros(n - 1, dtype=np.int64), i, i, i[:-1], i[1:]))
    cols = np.concatenate(([0], i, np.zeros(n - 1, dtype=np.int64), i, i[1:], i[:-1]))
    vals = np.concatenate(([2.0 * n * 1e-3 + 10.0], np.full(n - 1, 1e-3), np.full(n - 1, 1e-3), np.full(n - 1, 4.0),
                           np.full(n - 2, -1.0), np.full(n - 2, -1.0)))
    A = sp.csr_array((vals, (rows, cols)), shape=(n, n))
    A.sort_indices()
    return n, A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64)


@pytest.fixture(scope="module")
def arrow():
    return _arrow()


def _scale(n, rp, ci, v, x):
    a = np.abs(v * x[ci])
    return np.add.reduceat(a, rp[:-1]) if len(a) else np.zeros(n)


@pytest.mark.parametrize("numerics", [0, 1], ids=["fast", "strict"])
def test_long_row_products(ctx, arrow, numerics):
    n, rp, ci, v = arrow
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    Ao = O.Csr(n, n, rp, ci, v)
    x = workloads.uniform(n, 31)
    ctx.setNumerics(numerics)
    try:
        y, yt = A.mult(x), A.transMult(x)
        y2 = A.mult(x)
    finally:
        ctx.setNumerics(0)
    yo, yto = O.mult(Ao, x), O.trans_mult(Ao, x)
    assert np.array_equal(y, y2)  # repeatable: fixed segments and orders
    if numerics == 1:
        assert np.array_equal(y, yo) and np.array_equal(yt, yto)
    else:
        assert np.all(np.abs(y - yo) <= 1e-13 * _scale(n, rp, ci, v, x) + 1e-300)
        import scipy.sparse as sp
        at = abs(sp.csr_array((v, ci, rp), shape=(n, n)).T.tocsr())
        assert np.all(np.abs(yt - yto) <= 1e-13 * (at @ np.abs(x)) + 1e-300)


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_long_row_cg(ctx, arrow, mixed):
    n, rp, ci, v = arrow
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    Ao = O.Csr(n, n, rp, ci, v)
    b = O.mult(Ao, workloads.uniform(n, 32))
    s = sparse.CG(n, ctx=ctx)
    M = sparse.DiagonalPreconditioner(n, ctx)
    M.setMatrix(A)
    s.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(500, 1e-10, 1e-50, 1e5)
    mon.setIterationReporter(None, history_cap=600)
    s.setIterationMonitor(mon)
    if mixed:
        s.setMixedPrecision(True, 1e-4, 500)
    x = np.zeros(n)
    s.solve(A, b, x)
    r = O.mult_add(Ao, -1.0, x, b)
    assert np.linalg.norm(r) < 1e-10 * np.linalg.norm(b)
    if not mixed:
        pc = O.Precond(O.PC_JACOBI, n)
        pc.set_matrix(Ao)
        xo, res, hr, hi = O.solve(O.CG, Ao, b, np.zeros(n), pc, max_iter=500, rtol=1e-10)
        assert res.status == 0 and abs(mon.iterations() - res.iterations) <= 2
        gr, gi = s.history
        k = min(len(gr), len(hr))
        assert np.max(np.abs(gr[:k] - hr[:k])) / hr[0] <= 1e-10


def _power_law(n=60_000, seed=3):
    """Rows of 3 to 900 entries (a heavy tail: 2 % of rows hold 64 or more),
    symmetrised and made diagonally dominant, so SPD."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    deg = np.minimum(900, np.maximum(3, (rng.pareto(1.2, n) * 3).astype(np.int64)))
    rows = np.repeat(np.arange(n), deg)
    cols = rng.integers(0, n, len(rows))
    A = sp.csr_array((np.full(len(rows), -0.5), (rows, cols)), shape=(n, n))
    A = A + A.T
    A.setdiag(0)
    A.eliminate_zeros()
    d = np.asarray(abs(A).sum(axis=1)).ravel() + 1.0
    A = (A + sp.diags_array(d)).tocsr()
    A.sum_duplicates()
    A.sort_indices()
    return n, A.indptr.astype(np.int32), A.indices.astype(np.int32), A.data.astype(np.float64)


@pytest.mark.parametrize("numerics", [0, 1], ids=["fast", "strict"])
def test_heavy_tailed_rows(ctx, numerics):
    """Rows of a few hundred entries among short ones get a warp each (their
    own tiles); products match the oracle and CG + Jacobi its history."""
    n, rp, ci, v = _power_law()
    lens = np.diff(rp)
    assert lens.max() >= 300 and (lens >= 64).sum() > 100 and np.median(lens) < 24
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    Ao = O.Csr(n, n, rp, ci, v)
    x = workloads.uniform(n, 41)
    ctx.setNumerics(numerics)
    try:
        y = A.mult(x)
        b = O.mult(Ao, workloads.uniform(n, 42))
        s = sparse.CG(n, ctx=ctx)
        M = sparse.DiagonalPreconditioner(n, ctx)
        M.setMatrix(A)
        s.setPreconditioner(M)
        mon = sparse.DefaultIterationMonitor(1000, 1e-10, 1e-50, 1e5)
        mon.setIterationReporter(None, history_cap=1000)
        s.setIterationMonitor(mon)
        xs = np.zeros(n)
        s.solve(A, b, xs)
    finally:
        ctx.setNumerics(0)
    yo = O.mult(Ao, x)
    if numerics == 1:
        assert np.array_equal(y, yo)
    else:
        assert np.all(np.abs(y - yo) <= 1e-13 * _scale(n, rp, ci, v, x) + 1e-300)
    pc = O.Precond(O.PC_JACOBI, n)
    pc.set_matrix(Ao)
    xo, res, hr, hi = O.solve(O.CG, Ao, b, np.zeros(n), pc, max_iter=1000, rtol=1e-10)
    assert res.status == 0 and abs(mon.iterations() - res.iterations) <= 2
    gr, gi = s.history
    k = min(len(gr), len(hr))
    assert np.max(np.abs(gr[:k] - hr[:k])) / hr[0] <= 1e-10
