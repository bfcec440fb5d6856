"""Batched solves: many independent systems in the same launches.

Each system's iterate, iteration count and residual history must be
bit-identical to solving that system alone (as a batch of one), and
independent of the batch's
composition and order; and each must match the oracle (iterations +-2,
relative residual history within 1e-10 of r_0).
"""
import numpy as np
import pytest

import oracle as O
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu


def _systems():
    out = []
    for k in range(6):
        out.append(workloads.laplacian(500 + 700 * k, 40 + k))
    for N in (9, 17, 30, 41):
        out.append(workloads.poisson2d(N))
    for N in (5, 8, 11):
        out.append(workloads.poisson3d(N))
    out.append(workloads.convdiff3d(6))  # nonsymmetric: CG will not converge in 60 iterations
    return out


def _rhs(systems):
    bs = []
    for k, (n, rp, ci, v) in enumerate(systems):
        xt = workloads.uniform(n, 100 + k)
        bs.append(O.mult(O.Csr(n, n, rp, ci, v), xt))
    return bs


def _solo(ctx, n, rp, ci, v, b, pc, max_iter):
    # alone = a batch of one (a batch's systems take the batch grouping of
    # their reductions, which depends on the system only)
    A = sparse.BatchCompRowMatrix([(n, rp, ci, v)], ctx)
    s = sparse.CG(n, ctx=ctx)
    if pc:
        M = sparse.DiagonalPreconditioner(n, ctx)
        M.setMatrix(A)
        s.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(max_iter, 1e-10, 1e-50, 1e5)
    mon.setIterationReporter(sparse.IterationReporter(), history_cap=max_iter + 8)
    s.setIterationMonitor(mon)
    x = np.zeros(n)
    try:
        s.solve(A, b, x)
        st = 0
    except sparse.IterativeSolverNotConvergedException as e:
        st = e.getReason().value
    return x, st, mon.iterations(), s.history


@pytest.mark.parametrize("pc", [False, True], ids=["identity", "jacobi"])
def test_batch_equals_solo_bitwise(ctx, pc):
    systems = _systems()
    bs = _rhs(systems)
    max_iter = 400
    for order in (list(range(len(systems))), list(reversed(range(len(systems))))):
        sy = [systems[i] for i in order]
        A = sparse.BatchCompRowMatrix(sy, ctx)
        ntot = A.numRows()
        solver = sparse.CG(ntot, ctx=ctx)
        if pc:
            M = sparse.DiagonalPreconditioner(ntot, ctx)
            M.setMatrix(A)
            solver.setPreconditioner(M)
        mon = sparse.DefaultIterationMonitor(max_iter, 1e-10, 1e-50, 1e5)
        mon.setIterationReporter(None, history_cap=max_iter + 8)
        solver.setIterationMonitor(mon)
        b = np.concatenate([bs[i] for i in order])
        x = np.zeros(ntot)
        res = solver.solveBatch(A, b, x)
        for pos, i in enumerate(order):
            n, rp, ci, v = systems[i]
            r0, r1 = A.systemRows(pos)
            xs, st, it, hist = _solo(ctx, n, rp, ci, v, bs[i], pc, max_iter)
            assert res[pos][0] == st and res[pos][1] == it, (i, res[pos], st, it)
            assert np.array_equal(x[r0:r1], xs), i
            hb = solver.batchHistory(pos)
            assert np.array_equal(hb[0], hist[0]) and np.array_equal(hb[1], hist[1]), i


@pytest.mark.parametrize("pc", [False, True], ids=["identity", "jacobi"])
def test_batch_with_an_empty_system(ctx, pc):
    """A system of zero rows inside a batch converges at its first test, as it
    does alone, and leaves the other systems' results as they are alone."""
    empty = (0, np.zeros(1, dtype=np.int32), np.zeros(0, dtype=np.int32), np.zeros(0))
    systems = [workloads.poisson2d(9), empty, workloads.laplacian(700, 41), empty]
    bs = _rhs(systems)
    max_iter = 400
    A = sparse.BatchCompRowMatrix(systems, ctx)
    ntot = A.numRows()
    solver = sparse.CG(ntot, ctx=ctx)
    if pc:
        M = sparse.DiagonalPreconditioner(ntot, ctx)
        M.setMatrix(A)
        solver.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(max_iter, 1e-10, 1e-50, 1e5)
    mon.setIterationReporter(None, history_cap=max_iter + 8)
    solver.setIterationMonitor(mon)
    x = np.zeros(ntot)
    res = solver.solveBatch(A, np.concatenate(bs), x)
    for pos, (n, rp, ci, v) in enumerate(systems):
        r0, r1 = A.systemRows(pos)
        xs, st, it, hist = _solo(ctx, n, rp, ci, v, bs[pos], pc, max_iter)
        assert res[pos][0] == st == 0 and res[pos][1] == it, (pos, res[pos], st, it)
        if n == 0:
            assert it == 0 and r0 == r1
        assert np.array_equal(x[r0:r1], xs), pos
        hb = solver.batchHistory(pos)
        assert np.array_equal(hb[0], hist[0]) and np.array_equal(hb[1], hist[1]), pos


def test_batch_matches_oracle(ctx):
    systems = _systems()[:-1]
    bs = _rhs(systems)
    A = sparse.BatchCompRowMatrix(systems, ctx)
    ntot = A.numRows()
    solver = sparse.CG(ntot, ctx=ctx)
    M = sparse.DiagonalPreconditioner(ntot, ctx)
    M.setMatrix(A)
    solver.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(2000, 1e-10, 1e-50, 1e5)
    mon.setIterationReporter(None, history_cap=2100)
    solver.setIterationMonitor(mon)
    x = np.zeros(ntot)
    res = solver.solveBatch(A, np.concatenate(bs), x)
    for k, (n, rp, ci, v) in enumerate(systems):
        Ao = O.Csr(n, n, rp, ci, v)
        pco = O.Precond(O.PC_JACOBI, n)
        pco.set_matrix(Ao)
        xo, ro, hr, hi = O.solve(O.CG, Ao, bs[k], np.zeros(n), pco, max_iter=2000, rtol=1e-10)
        assert res[k][0] == 0 and ro.status == 0
        assert abs(res[k][1] - ro.iterations) <= 2
        gr, gi = solver.batchHistory(k)
        m = min(len(gr), len(hr))
        assert np.array_equal(gi[:m], hi[:m])
        assert np.max(np.abs(gr[:m] - hr[:m])) / hr[0] <= 1e-10
        r0, r1 = A.systemRows(k)
        assert np.max(np.abs(x[r0:r1] - xo)) <= 1e-8 * max(1.0, np.max(np.abs(xo)))


def test_batch_rejects_coupled_systems(ctx):
    # system 0 references a column of system 1
    rp = np.array([0, 2, 3], dtype=np.int32)
    ci = np.array([0, 1, 1], dtype=np.int32)
    v = np.array([2.0, -1.0, 2.0])
    lib = ctx._lib
    import ctypes as C
    from mtjg import _lib as L
    h = C.c_void_p()
    sys_rows = np.array([0, 1, 2], dtype=np.int32)
    code = lib.mtjg_batch_upload(ctx.h, 2, L.iptr(sys_rows), L.iptr(rp), L.iptr(ci), L.dptr(v), C.byref(h))
    assert code == L.ERR_ILLEGAL_ARGUMENT


def test_autotuner_records_a_choice_per_class(ctx):
    # the persistent batched CG tunes lanes per row per system class on the
    # first batch holding the class; the choice is one of the candidates and
    # stays fixed for the process, so a second solve is bit-identical
    import ctypes as C
    systems = [workloads.laplacian(3000 + 500 * k, 70 + k) for k in range(5)]
    A = sparse.BatchCompRowMatrix(systems, ctx)
    s = sparse.CG(A.numRows(), ctx=ctx)
    M = sparse.DiagonalPreconditioner(A.numRows(), ctx)
    M.setMatrix(A)
    s.setPreconditioner(M)
    s.setIterationMonitor(sparse.DefaultIterationMonitor(500, 1e-10, 1e-50, 1e5))
    b = np.concatenate(_rhs(systems))
    x1 = np.zeros(A.numRows())
    out1 = s.solveBatch(A, b, x1)
    lanes = C.c_int(-1)
    n, rp, ci, v = systems[0]
    assert ctx._lib.mtjg_batch_tuning(n, int(rp[-1]), C.byref(lanes)) == 0
    assert lanes.value in (1, 2, 4, 8, 32)
    x2 = np.zeros(A.numRows())
    out2 = s.solveBatch(A, b, x2)
    assert out1 == out2 and np.array_equal(x1, x2)
    assert all(st == 0 for st, _, _ in out1)
