"""The oracle's MatrixIterationMonitor (S/MatrixIterationMonitor.java:101-129).

Its convergence test is r < max(rtol (normA |x| + normb), atol) on the
iterate of the moment; divergence, iteration and NaN tests are those of
DefaultIterationMonitor, and converged(double) -- GMRES's inner test --
is unsupported.  Pinned here: with normA = 0 and normb = |r_0| the test is
DefaultIterationMonitor's exactly, so every solver must reproduce its
default run bit for bit; a run that converges satisfies the criterion on
its returned x and its previous test did not; GMRES stops with the
unsupported status after recording the inner residual, unless its first
test converges.
"""
import numpy as np
import pytest

import oracle as O
from mtjg import workloads

KINDS = {"cg": O.CG, "bicgstab": O.BICGSTAB, "bicg": O.BICG, "cgs": O.CGS, "qmr": O.QMR, "ir": O.IR,
         "chebyshev": O.CHEBYSHEV}


def _system(kind):
    if kind in ("cg", "chebyshev"):
        n, rp, ci, v = workloads.poisson2d(12)
    else:
        n, rp, ci, v = workloads.convdiff3d(6)
    A = O.Csr(n, n, rp, ci, v)
    pc = O.Precond(O.PC_JACOBI, n)
    assert pc.set_matrix(A) == 0
    return n, rp, ci, v, A, pc, workloads.uniform(n, 31)


def _eig(kind):
    return (0.05, 2.0) if kind == "chebyshev" else (0.0, 0.0)


@pytest.mark.parametrize("name", sorted(KINDS))
def test_zero_matrix_norm_is_the_default_monitor(name):
    n, rp, ci, v, A, pc, b = _system(name)
    emin, emax = _eig(name)
    x0 = np.zeros(n)
    xd, rd, hd, id_ = O.solve(KINDS[name], A, b, x0, pc, max_iter=400, rtol=1e-8, eigmin=emin, eigmax=emax)
    # DefaultIterationMonitor tests against initR, set at every test while
    # isFirst(): BiCGstab's mid-step test on s in iteration 0 replaces r_0
    # by |s_0| (S/BiCGstab.java:103), so there |s_0| is the equivalent normb
    r0 = hd[1] if name == "bicgstab" else hd[0]
    xm, rm, hm, im = O.solve(KINDS[name], A, b, x0, pc, max_iter=400, rtol=1e-8, eigmin=emin, eigmax=emax,
                             matrix_norms=(0.0, r0))
    assert (rd.status, rd.iterations, rd.history_len) == (rm.status, rm.iterations, rm.history_len)
    assert np.array_equal(hd, hm) and np.array_equal(id_, im)
    assert np.array_equal(xd, xm)


@pytest.mark.parametrize("norm", [O.NORM_ONE, O.NORM_TWO, O.NORM_INFINITY])
def test_converged_run_meets_the_matrix_criterion(norm):
    n, rp, ci, v, A, pc, b = _system("cg")
    normA, normb = 8.0, float(np.linalg.norm(b))
    rtol = 1e-9
    x, res, hr, hi = O.solve(O.CG, A, b, np.zeros(n), pc, max_iter=400, rtol=rtol, norm_type=norm,
                             matrix_norms=(normA, normb))
    assert res.status == O.OK
    xn = {O.NORM_ONE: np.abs(x).sum(), O.NORM_TWO: np.linalg.norm(x), O.NORM_INFINITY: np.abs(x).max()}[norm]
    assert hr[-1] < rtol * (normA * xn + normb)
    # the default monitor's relative test is a different criterion: it stops elsewhere
    _, rd, _, _ = O.solve(O.CG, A, b, np.zeros(n), pc, max_iter=400, rtol=rtol, norm_type=norm)
    assert rd.status == O.OK and rd.iterations != res.iterations


def test_gmres_inner_test_is_unsupported():
    n, rp, ci, v, A, pc, b = _system("gmres")
    x, res, hr, hi = O.solve(O.GMRES, A, b, np.zeros(n), pc, max_iter=400, rtol=1e-8,
                             matrix_norms=(8.0, float(np.linalg.norm(b))))
    assert res.status == O.ERR_UNSUPPORTED
    # the outer test at iteration 0, then the first inner test records |s_0| and stops
    assert res.history_len == 2 and list(hi) == [0, 0] and hr[0] == hr[1]


def test_gmres_converged_at_the_first_test():
    n, rp, ci, v, A, pc, b = _system("gmres")
    x, res, hr, hi = O.solve(O.GMRES, A, b, np.zeros(n), pc, max_iter=400, rtol=1e-8,
                             matrix_norms=(0.0, 1e12))
    assert res.status == O.OK and res.history_len == 1
