"""new CompRowMatrix(A) for CompColMatrix and FlexCompRowMatrix inputs,
converted on the device (mtjg_csr_upload_csc, mtjg_csr_upload_rows): the
device CSR equals the CSR of A's stored entries (explicit zeros kept, rows
sorted), products then equal the oracle's CompRowMatrix products, a solve
on the converted matrix matches the oracle, and malformed input is
rejected with MTJ's IllegalArgumentException."""
import numpy as np
import pytest

import oracle as O
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu


def _random_sparse(rng, n, m, density):
    A = (rng.random((n, m)) < density) * rng.uniform(-2, 2, (n, m))
    A[rng.random((n, m)) < 0.02] = 0.0
    keep = (A != 0) | (rng.random((n, m)) < 0.01)  # a few stored zeros
    return A, keep


def _csr_of(A, keep):
    n, m = A.shape
    rp, ci, v = [0], [], []
    for i in range(n):
        cols = np.nonzero(keep[i])[0]
        ci += cols.tolist()
        v += A[i, cols].tolist()
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(v)


@pytest.mark.parametrize("shape", [(50, 50), (37, 61), (80, 20), (1, 1), (0, 5)])
def test_csc_conversion(ctx, shape):
    rng = np.random.default_rng(sum(shape))
    n, m = shape
    A, keep = _random_sparse(rng, n, m, 0.15)
    cp, ri, cv = [0], [], []
    for j in range(m):
        rows = np.nonzero(keep[:, j])[0]
        ri += rows.tolist()
        cv += A[rows, j].tolist()
        cp.append(len(ri))
    B = sparse.CompRowMatrix.fromCompColMatrix(n, m, np.array(cp), np.array(ri, dtype=np.int32), np.array(cv), ctx)
    rp, ci, v = _csr_of(A, keep)
    assert np.array_equal(B.getRowPointers(), rp) and np.array_equal(B.getColumnIndices(), ci)
    assert np.array_equal(B.getData(), v)
    if n and m:
        x = workloads.uniform(m, 5)
        ctx.setNumerics(1)
        try:
            assert np.array_equal(B.mult(x), O.mult(O.Csr(n, m, rp, ci, v), x))
        finally:
            ctx.setNumerics(0)


@pytest.mark.parametrize("slack", [0, 3])
def test_flex_rows_conversion_and_solve(ctx, slack):
    n, rp, ci, v = workloads.convdiff3d(8)
    rows = [(ci[rp[i]:rp[i + 1]], v[rp[i]:rp[i + 1]]) for i in range(n)]
    B = sparse.CompRowMatrix.fromFlexCompRowMatrix(n, rows, ctx, slack=slack)
    assert np.array_equal(B.getRowPointers(), rp) and np.array_equal(B.getColumnIndices(), ci)
    assert np.array_equal(B.getData(), v)
    Ao = O.Csr(n, n, rp, ci, v)
    b = O.mult(Ao, workloads.uniform(n, 2))
    solver = sparse.BiCGstab(n, ctx=ctx)
    M = sparse.ILU(B)
    M.setMatrix(B)
    solver.setPreconditioner(M)
    solver.setIterationMonitor(sparse.DefaultIterationMonitor(2000, 1e-10, 1e-50, 1e5))
    x = np.zeros(n)
    solver.solve(B, b, x)
    pc = O.Precond(O.PC_ILU, n)
    pc.set_matrix(Ao)
    xo, res, _, _ = O.solve(O.BICGSTAB, Ao, b, np.zeros(n), pc, max_iter=2000, rtol=1e-10)
    assert res.status == 0 and abs(solver.getIterationMonitor().iterations() - res.iterations) <= 2
    assert np.max(np.abs(x - xo)) <= 1e-8


def test_flex_rows_with_empty_rows_and_stored_zeros(ctx):
    rng = np.random.default_rng(9)
    A, keep = _random_sparse(rng, 40, 30, 0.1)
    keep[3] = False
    keep[17] = False
    rp, ci, v = _csr_of(A, keep)
    rows = [(ci[rp[i]:rp[i + 1]], v[rp[i]:rp[i + 1]]) for i in range(40)]
    B = sparse.CompRowMatrix.fromFlexCompRowMatrix(30, rows, ctx, slack=2)
    assert np.array_equal(B.getRowPointers(), rp) and np.array_equal(B.getColumnIndices(), ci)
    assert np.array_equal(B.getData(), v)


def test_malformed_inputs_are_rejected(ctx):
    with pytest.raises(sparse.IllegalArgumentException):  # row index out of range
        sparse.CompRowMatrix.fromCompColMatrix(2, 2, [0, 1, 2], [0, 2], [1.0, 1.0], ctx)
    with pytest.raises(sparse.IllegalArgumentException):  # unsorted column
        sparse.CompRowMatrix.fromCompColMatrix(3, 1, [0, 2], [2, 0], [1.0, 1.0], ctx)
    with pytest.raises(sparse.IllegalArgumentException):  # unsorted row
        sparse.CompRowMatrix.fromFlexCompRowMatrix(3, [(np.array([2, 0]), np.array([1.0, 1.0]))], ctx)
    with pytest.raises(sparse.IllegalArgumentException):  # column out of range
        sparse.CompRowMatrix.fromFlexCompRowMatrix(3, [(np.array([0, 3]), np.array([1.0, 1.0]))], ctx)
