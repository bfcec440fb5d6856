"""Matrix Market file -> device CSR (mtjg_csr_read_matrix_market) -> solve,
against the oracle: the symmetric lower triangle of 2D Poisson written as a
Matrix Market file reads back as the full matrix (S/CompRowMatrix.java:86-166
mirrors it), and CG + Jacobi on it matches the oracle's solve."""
import numpy as np
import pytest

import oracle as O
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu


def _write_lower(path, n, rp, ci, v, header=True):
    lines = ["%%MatrixMarket matrix coordinate real symmetric"] if header else []
    lines.append("% 2D 5-point Poisson, lower triangle")
    ent = [(i + 1, int(ci[k]) + 1, float(v[k])) for i in range(n) for k in range(rp[i], rp[i + 1]) if ci[k] <= i]
    lines.append(f"{n} {n} {len(ent)}")
    lines += [f"{a} {b} {x!r}" for a, b, x in ent]
    path.write_text("\n".join(lines) + "\n")


def test_file_to_device_csr_and_solve(ctx, tmp_path):
    n, rp, ci, v = workloads.poisson2d(40)
    p = tmp_path / "poisson.mtx"
    _write_lower(p, n, rp, ci, v)
    A = sparse.CompRowMatrix.fromMatrixMarket(str(p), ctx)
    assert (A.numRows(), A.numColumns()) == (n, n)
    assert np.array_equal(A.getRowPointers(), rp) and np.array_equal(A.getColumnIndices(), ci)
    assert np.array_equal(A.getData(), v)
    Ao = O.Csr(n, n, rp, ci, v)
    b = O.mult(Ao, workloads.uniform(n, 1))
    solver = sparse.CG(n, ctx=ctx)
    M = sparse.DiagonalPreconditioner(n, ctx)
    M.setMatrix(A)
    solver.setPreconditioner(M)
    solver.setIterationMonitor(sparse.DefaultIterationMonitor(2000, 1e-10, 1e-50, 1e5))
    x = np.zeros(n)
    solver.solve(A, b, x)
    pc = O.Precond(O.PC_JACOBI, n)
    pc.set_matrix(Ao)
    xo, res, _, _ = O.solve(O.CG, Ao, b, np.zeros(n), pc, max_iter=2000, rtol=1e-10)
    assert res.status == 0 and abs(solver.getIterationMonitor().iterations() - res.iterations) <= 2
    assert np.max(np.abs(x - xo)) <= 1e-8


def test_text_to_device_csr_products(ctx):
    text = (b"%%MatrixMarket matrix coordinate real skew-symmetric\n% c\n4 4 3\n2 1 1.5\n4 2 -2\n3 1 0.25\n")
    A = sparse.CompRowMatrix.fromMatrixMarket(text, ctx)
    n, m, rp, ci, v = sparse.parseMatrixMarket(text)
    assert np.array_equal(A.getRowPointers(), rp) and np.array_equal(A.getColumnIndices(), ci)
    x = workloads.uniform(4, 3)
    assert np.allclose(A.mult(x), O.mult(O.Csr(n, m, rp, ci, v), x), rtol=0, atol=1e-15)


def test_read_errors_leave_no_matrix(ctx, tmp_path):
    p = tmp_path / "bad.mtx"
    p.write_text("%%MatrixMarket matrix coordinate pattern general\n2 2 1\n1 1\n")
    with pytest.raises(sparse.UnsupportedOperationException):
        sparse.CompRowMatrix.fromMatrixMarket(str(p), ctx)
    with pytest.raises(IOError):
        sparse.CompRowMatrix.fromMatrixMarket(str(tmp_path / "missing.mtx"), ctx)
