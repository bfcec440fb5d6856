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


# ------------------------------------- against the independent Python restatement
def _random_system(seed, spd):
    from helpers import dense_to_csr, nonsingular_system, spd_system
    rng = np.random.default_rng(900 + seed)
    n = int(rng.integers(5, 60))
    bw = int(rng.integers(1, min(6, n) + 1))
    Ad = spd_system(n, bw, rng) if spd else nonsingular_system(n, bw, rng)
    n, _, rp, ci, v = dense_to_csr(Ad)
    b = list(rng.standard_normal(n))
    return n, rp, ci, v, b


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("name", ["cg", "bicgstab", "gmres"])
def test_oracle_matches_pyref_with_matrix_monitor(seed, name):
    """Oracle and tests/pyref.py, both restating MTJ in plain IEEE double
    arithmetic, agree bit for bit under a MatrixIterationMonitor: status,
    iteration count, every recorded residual and x."""
    import pyref
    n, rp, ci, v, b = _random_system(seed, name == "cg")
    A = O.Csr(n, n, rp, ci, v)
    pc = O.Precond(O.PC_JACOBI, n)
    assert pc.set_matrix(A) == 0
    M = pyref.jacobi(list(rp), list(ci), list(v))
    normA = max(float(np.abs(v[rp[i]:rp[i + 1]]).sum()) for i in range(n))
    normb = float(np.linalg.norm(b))
    mon = pyref.MatrixMonitor(normA, normb, 300, 1e-10)
    kind = {"cg": O.CG, "bicgstab": O.BICGSTAB, "gmres": O.GMRES}[name]
    x0 = [0.0] * n
    code, xp = 0, None
    try:
        if name == "gmres":
            xp = pyref.gmres(list(rp), list(ci), list(v), b, x0, M, mon, 4)
        else:
            xp = {"cg": pyref.cg, "bicgstab": pyref.bicgstab}[name](list(rp), list(ci), list(v), b, x0, M, mon)
    except pyref.NotConverged as e:
        code = e.code
    except pyref.Unsupported:
        code = O.ERR_UNSUPPORTED
    xo, res, hr, hi = O.solve(kind, A, np.array(b), np.zeros(n), pc, max_iter=300, rtol=1e-10, restart=4,
                              matrix_norms=(normA, normb))
    assert res.status == code
    assert res.iterations == mon.iter
    assert np.array_equal(hr, np.array([h[0] for h in mon.hist]))
    assert np.array_equal(hi, np.array([h[1] for h in mon.hist]))
    if code == 0:
        assert np.array_equal(xo, np.array(xp))
