"""Mixed precision: FP32 inner CG inside FP64 iterative refinement.

The monitor tests the FP64 true residual r = b - A x, so a converged solve
meets rtol on exactly the quantity MTJ's monitor would see; the final error
is compared with an FP64 oracle solve of the same system.
"""
import numpy as np
import pytest

import oracle as O
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu


def _mixed_solver(ctx, A, n, pc, rtol=1e-10, inner_rtol=1e-4):
    s = sparse.CG(n, ctx=ctx)
    if pc:
        M = sparse.DiagonalPreconditioner(n, ctx)
        M.setMatrix(A)
        s.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(200, rtol, 1e-50, 1e5)
    mon.setIterationReporter(None, history_cap=256)
    s.setIterationMonitor(mon)
    s.setMixedPrecision(True, inner_rtol, 2000)
    return s


@pytest.mark.parametrize("mat,N", [("poisson2d", 64), ("poisson3d", 20), ("laplacian", 6000)])
@pytest.mark.parametrize("pc", [False, True], ids=["identity", "jacobi"])
def test_mixed_reaches_fp64_tolerance(ctx, mat, N, pc):
    n, rp, ci, v = workloads.laplacian(N, 5) if mat == "laplacian" else getattr(workloads, mat)(N)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    Ao = O.Csr(n, n, rp, ci, v)
    xt = workloads.uniform(n, 3)
    b = O.mult(Ao, xt)
    s = _mixed_solver(ctx, A, n, pc)
    x = np.zeros(n)
    s.solve(A, b, x)
    # the monitor's test is on the FP64 residual of x itself
    r = O.mult_add(Ao, -1.0, x, b)
    assert np.linalg.norm(r) < 1e-10 * np.linalg.norm(b)
    hist, its = s.history
    assert np.array_equal(its, np.arange(len(its)))  # one test per refinement step
    assert abs(hist[0] - np.linalg.norm(b)) <= 1e-12 * np.linalg.norm(b)
    assert s.getIterationMonitor().iterations() <= 6
    assert s.innerIterations() > 0
    # the final error against an FP64 oracle solve of the same system
    pco = None
    if pc:
        pco = O.Precond(O.PC_JACOBI, n)
        pco.set_matrix(Ao)
    xo, res, _, _ = O.solve(O.CG, Ao, b, np.zeros(n), pco, max_iter=20000, rtol=1e-10)
    assert res.status == 0
    assert np.max(np.abs(x - xo)) <= 1e-6 * np.max(np.abs(xo))


def test_mixed_batch_equals_solo(ctx):
    systems = [workloads.poisson2d(40), workloads.laplacian(3000, 11), workloads.poisson3d(12),
               workloads.laplacian(800, 12)]
    bs = [O.mult(O.Csr(n, n, rp, ci, v), workloads.uniform(n, 20 + k)) for k, (n, rp, ci, v) in enumerate(systems)]
    A = sparse.BatchCompRowMatrix(systems, ctx)
    nt = A.numRows()
    s = _mixed_solver(ctx, A, nt, True)
    x = np.zeros(nt)
    res = s.solveBatch(A, np.concatenate(bs), x)
    for k, (n, rp, ci, v) in enumerate(systems):
        As = sparse.BatchCompRowMatrix([(n, rp, ci, v)], ctx)  # alone: a batch of one
        ss = _mixed_solver(ctx, As, n, True)
        xs = np.zeros(n)
        ss.solve(As, bs[k], xs)
        r0, r1 = A.systemRows(k)
        assert res[k][0] == 0 and res[k][1] == ss.getIterationMonitor().iterations()
        assert np.array_equal(x[r0:r1], xs)


def test_mixed_rejects_other_solvers(ctx):
    s = sparse.GMRES(10, ctx=ctx)
    with pytest.raises(sparse.UnsupportedOperationException):
        s.setMixedPrecision(True)
