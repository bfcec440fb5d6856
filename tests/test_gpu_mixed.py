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
    s = sparse.QMR(10, ctx=ctx)
    with pytest.raises(sparse.UnsupportedOperationException):
        s.setMixedPrecision(True)


def test_mixed_rejects_other_preconditioners(ctx):
    n, rp, ci, v = workloads.poisson2d(12)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    for make, M in ((sparse.CG, sparse.ILU(A)), (sparse.GMRES, sparse.ICC(A)), (sparse.BiCGstab, sparse.SSOR(A))):
        M.setMatrix(A)
        s = make(n, ctx=ctx)
        s.setPreconditioner(M)
        s.setMixedPrecision(True)
        with pytest.raises(sparse.UnsupportedOperationException):
            s.solve(A, np.ones(n), np.zeros(n))


def _krylov(ctx, kind, n, M, rtol=1e-10, inner_rtol=1e-4, max_iter=60):
    s = sparse.GMRES(n, ctx=ctx) if kind == "gmres" else sparse.BiCGstab(n, ctx=ctx)
    if M is not None:
        s.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(max_iter, rtol, 1e-50, 1e5)
    mon.setIterationReporter(None, history_cap=256)
    s.setIterationMonitor(mon)
    s.setMixedPrecision(True, inner_rtol, 3000)
    return s


_ORACLE_PC = {"identity": None, "jacobi": "PC_JACOBI", "ilu": "PC_ILU", "ilut": "PC_ILUT"}


@pytest.mark.parametrize("kind", ["gmres", "bicgstab"])
@pytest.mark.parametrize("pc,mat,N", [("ilu", "convdiff3d", 20), ("ilu", "convdiff3d", 32), ("ilut", "convdiff3d", 16),
                                      ("jacobi", "poisson2d", 48), ("identity", "convdiff3d", 12)])
def test_mixed_krylov_reaches_fp64_tolerance(ctx, kind, pc, mat, N):
    """Mixed GMRES(30) / BiCGstab: FP32 inner solves with an FP32 copy of the
    preconditioner inside FP64 refinement meet rtol 1e-10 on the FP64 true
    residual, with one monitor test per refinement step, and agree with an
    FP64 oracle solve of the same system."""
    n, rp, ci, v = getattr(workloads, mat)(N)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    Ao = O.Csr(n, n, rp, ci, v)
    b = O.mult(Ao, workloads.uniform(n, 4))
    M = None
    if pc != "identity":
        M = {"ilu": sparse.ILU, "ilut": sparse.ILUT, "jacobi": sparse.DiagonalPreconditioner}[pc](
            A if pc != "jacobi" else n, *(() if pc != "jacobi" else (ctx,)))
        M.setMatrix(A)
    s = _krylov(ctx, kind, n, M)
    x = np.zeros(n)
    s.solve(A, b, x)
    r = O.mult_add(Ao, -1.0, x, b)
    assert np.linalg.norm(r) < 1e-10 * np.linalg.norm(b)
    hist, its = s.history
    assert np.array_equal(its, np.arange(len(its)))
    assert abs(hist[0] - np.linalg.norm(b)) <= 1e-12 * np.linalg.norm(b)
    assert hist[-1] < 1e-10 * hist[0]
    assert s.getIterationMonitor().iterations() <= 8 and s.innerIterations() > 0
    pco = None
    if pc != "identity":
        pco = O.Precond(getattr(O, _ORACLE_PC[pc]), n)
        pco.set_matrix(Ao)
    xo, res, _, _ = O.solve(O.GMRES if kind == "gmres" else O.BICGSTAB, Ao, b, np.zeros(n), pco, max_iter=20000,
                            rtol=1e-10)
    assert res.status == 0
    assert np.max(np.abs(x - xo)) <= 1e-6 * np.max(np.abs(xo))


@pytest.mark.parametrize("kind", ["gmres", "bicgstab"])
def test_mixed_krylov_repeatable(ctx, kind):
    """Two solves from the same x0 give the same x bit for bit: every
    reduction runs in a fixed order."""
    n, rp, ci, v = workloads.convdiff3d(14)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    b = A.mult(workloads.uniform(n, 8))
    M = sparse.ILU(A)
    M.setMatrix(A)
    s = _krylov(ctx, kind, n, M)
    x1, x2 = np.zeros(n), np.zeros(n)
    s.solve(A, b, x1)
    it1, in1 = s.getIterationMonitor().iterations(), s.innerIterations()
    s.solve(A, b, x2)
    assert np.array_equal(x1, x2)
    assert s.getIterationMonitor().iterations() == it1 and s.innerIterations() == in1


def test_mixed_krylov_iteration_limit(ctx):
    """A refinement budget too small to reach rtol ends with Reason.Iterations."""
    n, rp, ci, v = workloads.convdiff3d(16)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    b = A.mult(workloads.uniform(n, 9))
    s = _krylov(ctx, "gmres", n, None, inner_rtol=0.5, max_iter=2)
    with pytest.raises(sparse.IterativeSolverNotConvergedException):
        s.solve(A, b, np.zeros(n))
    assert s.getIterationMonitor().iterations() == 2
