"""MatrixIterationMonitor on the GPU against the oracle.

S/MatrixIterationMonitor.java: every test converges iff
r < max(rtol (normA |x| + normb), atol), |x| the iterate's norm at that
moment (formed on the device before each test).  Bars as for the default
monitor: the oracle's status, its iteration count within 2, the relative
residual history r_k / r_0 within 1e-10 over the common prefix (the
Lanczos-type solvers: four times the oracle's own summation-order envelope
when that is larger), x within 1e-8.  GMRES stops with
UnsupportedOperationException at its first inner test (converged(double)),
after recording it, as in MTJ.  The batched and mixed-precision forms
refuse the monitor.
"""
import numpy as np
import pytest

import oracle as O
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu

KIND = {"cg": (O.CG, sparse.CG), "bicgstab": (O.BICGSTAB, sparse.BiCGstab), "bicg": (O.BICG, sparse.BiCG),
        "cgs": (O.CGS, sparse.CGS), "qmr": (O.QMR, sparse.QMR), "ir": (O.IR, sparse.IR),
        "chebyshev": (O.CHEBYSHEV, None), "gmres": (O.GMRES, sparse.GMRES)}
PCS = {"identity": (None, None), "jacobi": (sparse.DiagonalPreconditioner, O.PC_JACOBI),
       "ilu": (sparse.ILU, O.PC_ILU), "icc": (sparse.ICC, O.PC_ICC)}
LANCZOS = ("bicgstab", "bicg", "cgs", "qmr")


@pytest.fixture(params=[0, 1], ids=["fast", "strict"])
def numerics(request, ctx):
    ctx.setNumerics(request.param)
    yield request.param
    ctx.setNumerics(0)


def _system(name):
    if name == "chebyshev":
        return workloads.poisson2d(16)
    if name == "cg":
        return workloads.poisson2d(24)
    return workloads.convdiff3d(10)


def _eig(n, rp, ci, v):
    """The extreme eigenvalues of A (Chebyshev without a preconditioner)."""
    Ad = np.zeros((n, n))
    for i in range(n):
        Ad[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    ev = np.linalg.eigvalsh(Ad)
    return float(ev[0]), float(ev[-1])


def _norms(n, rp, v, b):
    normA = max(float(np.abs(v[rp[i]:rp[i + 1]]).sum()) for i in range(n))  # |A|_inf
    return normA, float(np.linalg.norm(b))


def _solver(name, n, ctx, eig):
    if name == "chebyshev":
        return sparse.Chebyshev(n, eig[0], eig[1], ctx=ctx)
    if name == "gmres":
        return sparse.GMRES(n, restart=30, ctx=ctx)
    return KIND[name][1](n, ctx=ctx)


def _both(ctx, name, pname, norm=sparse.Norm.Two, max_iter=2000, rtol=1e-9):
    n, rp, ci, v = _system(name)
    b = workloads.uniform(n, 7)
    normA, normb = _norms(n, rp, v, b)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    Ao = O.Csr(n, n, rp, ci, v)
    eig = _eig(n, rp, ci, v) if name == "chebyshev" else (0.0, 0.0)
    solver = _solver(name, n, ctx, eig)
    pcls, pk = PCS[pname]
    pco = None
    if pcls is not None:
        M = pcls(n, ctx) if pcls is sparse.DiagonalPreconditioner else pcls(A)
        M.setMatrix(A)
        solver.setPreconditioner(M)
        pco = O.Precond(pk, n)
        assert pco.set_matrix(Ao) == 0
    mon = sparse.MatrixIterationMonitor(normA, normb, max_iter, rtol, 1e-50, 1e5)
    mon.setNormType(norm)
    mon.setIterationReporter(sparse.IterationReporter(), history_cap=4 * max_iter + 64)
    solver.setIterationMonitor(mon)
    x = np.zeros(n)
    exc = None
    try:
        solver.solve(A, b, x)
    except (sparse.IterativeSolverNotConvergedException, sparse.UnsupportedOperationException) as e:
        exc = e
    xo, res, hr, hi = O.solve(KIND[name][0], Ao, b, np.zeros(n), pco, max_iter=max_iter, rtol=rtol,
                              norm_type=int(norm), eigmin=eig[0], eigmax=eig[1], matrix_norms=(normA, normb))
    return x, exc, solver, mon, xo, res, hr, hi, (Ao, pco, b, eig, max_iter, rtol, normA, normb)


def _envelope(name, ctx_args, h_seq, it_seq):
    """How far the oracle's own history (relative to r_0) and iteration count
    move when only its dot products and norms are summed in another order."""
    Ao, pco, b, eig, max_iter, rtol, normA, normb = ctx_args
    env, it_env = 0.0, 0
    for block in (16, 64, 256, 1024):
        with O.sum_order(block):
            _, r, h_blk, _ = O.solve(KIND[name][0], Ao, b, np.zeros(Ao.n), pco, max_iter=max_iter, rtol=rtol,
                                     eigmin=eig[0], eigmax=eig[1], matrix_norms=(normA, normb))
        k = min(len(h_seq), len(h_blk))
        env = max(env, float(np.max(np.abs(h_seq[:k] - h_blk[:k])) / h_seq[0]))
        it_env = max(it_env, abs(r.iterations - it_seq))
    return env, it_env


CASES = [("cg", "jacobi"), ("cg", "icc"), ("cg", "identity"), ("bicgstab", "ilu"), ("bicgstab", "jacobi"),
         ("bicg", "ilu"), ("cgs", "ilu"), ("qmr", "ilu"), ("ir", "ilu"), ("chebyshev", "identity")]


def _status(exc):
    if exc is None:
        return O.OK
    if isinstance(exc, sparse.UnsupportedOperationException):
        return O.ERR_UNSUPPORTED
    return exc.getReason().value


@pytest.mark.parametrize("case", CASES, ids=["-".join(c) for c in CASES])
def test_matrix_monitor_matches_oracle(ctx, numerics, case):
    name, pname = case
    x, exc, solver, mon, xo, res, hr, hi, args = _both(ctx, name, pname)
    assert _status(exc) == res.status, (exc, res.status)
    if name != "chebyshev":
        assert res.status == O.OK
    env, it_env = _envelope(name, args, hr, res.iterations) if name in LANCZOS else (0.0, 0)
    assert abs(mon.iterations() - res.iterations) <= 2 + it_env, (mon.iterations(), res.iterations, it_env)
    gr, gi = solver.history
    k = min(len(gr), len(hr))
    assert k > 0 and np.array_equal(gi[:k], hi[:k])
    rel = float(np.max(np.abs(gr[:k] - hr[:k])) / hr[0])
    assert rel <= max(1e-10, 4.0 * env), (rel, env)
    if res.status == O.OK:
        assert np.max(np.abs(x - xo)) <= 1e-8 * max(1.0, np.max(np.abs(xo)))


@pytest.mark.parametrize("norm", [sparse.Norm.One, sparse.Norm.TwoRobust, sparse.Norm.Infinity])
def test_matrix_monitor_norms(ctx, norm):
    x, exc, solver, mon, xo, res, hr, hi, _ = _both(ctx, "cg", "jacobi", norm=norm)
    assert exc is None and res.status == O.OK
    assert abs(mon.iterations() - res.iterations) <= 2
    gr, _ = solver.history
    k = min(len(gr), len(hr))
    assert float(np.max(np.abs(gr[:k] - hr[:k])) / hr[0]) <= 1e-10


def test_matrix_monitor_differs_from_default(ctx):
    """The criterion is the matrix one: a default monitor with the same rtol
    stops at another iteration."""
    _, _, _, mon, _, res, _, _, _ = _both(ctx, "cg", "jacobi")
    n, rp, ci, v = _system("cg")
    b = workloads.uniform(n, 7)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    s = sparse.CG(n, ctx=ctx)
    M = sparse.DiagonalPreconditioner(n, ctx)
    M.setMatrix(A)
    s.setPreconditioner(M)
    dmon = sparse.DefaultIterationMonitor(2000, 1e-9, 1e-50, 1e5)
    s.setIterationMonitor(dmon)
    s.solve(A, b, np.zeros(n))
    assert dmon.iterations() != mon.iterations()


def test_matrix_monitor_iteration_limit(ctx, numerics):
    x, exc, solver, mon, xo, res, hr, hi, _ = _both(ctx, "cg", "jacobi", max_iter=5)
    assert res.status == O.NC_ITERATIONS
    assert isinstance(exc, sparse.IterativeSolverNotConvergedException)
    assert mon.iterations() == 5
    gr, gi = solver.history
    assert np.array_equal(gi, hi) and float(np.max(np.abs(gr - hr)) / hr[0]) <= 1e-12


def test_gmres_inner_test_is_unsupported(ctx, numerics):
    x, exc, solver, mon, xo, res, hr, hi, _ = _both(ctx, "gmres", "ilu")
    assert res.status == O.ERR_UNSUPPORTED
    assert isinstance(exc, sparse.UnsupportedOperationException)
    gr, gi = solver.history
    assert list(gi) == [0, 0] and list(hi) == [0, 0]
    assert float(np.max(np.abs(gr - hr)) / hr[0]) <= 1e-12


def test_matrix_monitor_refused_by_mixed_and_batched(ctx):
    n, rp, ci, v = _system("cg")
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    b = workloads.uniform(n, 7)
    s = sparse.CG(n, ctx=ctx)
    s.setIterationMonitor(sparse.MatrixIterationMonitor(8.0, float(np.linalg.norm(b)), 2000, 1e-9))
    s.setMixedPrecision(True)
    with pytest.raises(sparse.UnsupportedOperationException):
        s.solve(A, b, np.zeros(n))


def test_matrix_monitor_refused_by_a_batch_of_one(ctx):
    """A batch upload (even of one system) runs the batched kernels, which
    keep only the default monitor."""
    n, rp, ci, v = workloads.poisson2d(12)
    B = sparse.BatchCompRowMatrix([(n, rp, ci, v)], ctx)
    b = workloads.uniform(n, 3)
    s = sparse.CG(n, ctx=ctx)
    s.setIterationMonitor(sparse.MatrixIterationMonitor(8.0, float(np.linalg.norm(b)), 2000, 1e-9))
    with pytest.raises(sparse.UnsupportedOperationException):
        s.solveBatch(B, b, np.zeros(n))


def test_custom_monitor_is_refused(ctx):
    """Only MTJ's two monitors run on the device; any other is refused
    (no CPU fallback)."""

    class Custom:
        pass

    s = sparse.CG(10, ctx=ctx)
    with pytest.raises(sparse.UnsupportedOperationException):
        s.setIterationMonitor(Custom())
