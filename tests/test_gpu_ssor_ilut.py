"""SSOR and ILUT on the GPU against the oracle (S/SSOR.java, S/ILUT.java).

The ILUT factor (host) equals the oracle's bit for bit: pattern, diagonal
positions and values.  In STRICT numerics SSOR's sweeps (which start from
x's content) and ILUT's solves equal the oracle bit for bit; FAST within
1e-12.  Solvers with either preconditioner meet the usual parity bars, and
the reference's tests for them (TS/ILUTTest, TS/CGSSORTest,
TS/ChebyshevSSORTest, TS/*ILUTTest) hold."""
import numpy as np
import pytest

import oracle as O
from helpers import dense_to_csr, nonsingular_system, pentadiagonal, spd_system, tridiagonal
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[0, 1], ids=["fast", "strict"])
def numerics(request, ctx):
    ctx.setNumerics(request.param)
    yield request.param
    ctx.setNumerics(0)


def _close(a, b, strict):
    if strict:
        return np.array_equal(a, b)
    return np.allclose(a, b, rtol=1e-12, atol=1e-14)


MATS = {"poisson2d_16": lambda: workloads.poisson2d(16), "convdiff3d_8": lambda: workloads.convdiff3d(8),
        "laplacian_2000": lambda: workloads.laplacian(2000, 5)}


@pytest.mark.parametrize("mat", sorted(MATS))
@pytest.mark.parametrize("omega,reverse", [((1.0, 1.0), True), ((1.4, 0.8), True), ((0.6, 1.0), False)])
def test_ssor_apply(ctx, numerics, mat, omega, reverse):
    n, rp, ci, v = MATS[mat]()
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    M = sparse.SSOR(A, reverse, omega[0], omega[1])
    M.setMatrix(A)
    Mo = O.Precond(O.PC_SSOR, n)
    Mo.set_params(omega[0], omega[1], 1 if reverse else 0)
    assert Mo.set_matrix(O.Csr(n, n, rp, ci, v)) == 0
    b = workloads.uniform(n, 31)
    x0 = workloads.uniform(n, 32)
    assert _close(M.apply(b, x0.copy()), Mo.apply(b, x0), numerics)
    assert _close(M.transApply(b, x0.copy()), Mo.trans_apply(b, x0), numerics)


def test_ssor_errors(ctx):
    n, _, rp, ci, v = dense_to_csr(np.array([[1.0, 2.0], [3.0, 0.0]]), keep_diag=False)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    with pytest.raises(sparse.IllegalArgumentException):
        sparse.SSOR(A, True, 2.5, 1.0)
    M = sparse.SSOR(A)
    with pytest.raises(RuntimeError, match="Missing diagonal on row 2"):
        M.setMatrix(A)


ILUT_CASES = [("convdiff3d_8", 1e-6, 25), ("convdiff3d_8", 0.05, 2), ("poisson2d_16", 1e-3, 0),
              ("laplacian_2000", 1e-6, 25)]


@pytest.mark.parametrize("case", ILUT_CASES, ids=[f"{c[0]}-{c[1]}-{c[2]}" for c in ILUT_CASES])
def test_ilut_factor_and_apply(ctx, numerics, case):
    mat, tau, p = case
    n, rp, ci, v = MATS[mat]()
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    M = sparse.ILUT(A, tau, p)
    M.setMatrix(A)
    Mo = O.Precond(O.PC_ILUT, n)
    Mo.set_params(tau, 0.0, p)
    assert Mo.set_matrix(O.Csr(n, n, rp, ci, v)) == 0
    grp, gci, gdg = M.pattern()
    orp, oci, odg = Mo.pattern()
    assert np.array_equal(grp, orp) and np.array_equal(gci, oci) and np.array_equal(gdg, odg)
    assert np.array_equal(M.values(), Mo.values())
    b = workloads.uniform(n, 41)
    assert _close(M.apply(b), Mo.apply(b), numerics)
    assert _close(M.transApply(b), Mo.trans_apply(b), numerics)


@pytest.mark.parametrize("seed", range(10))
def test_ilut_random_systems_factor(ctx, seed):
    rng = np.random.default_rng(800 + seed)
    n = int(rng.integers(2, 60))
    Ad = nonsingular_system(n, int(rng.integers(1, min(10, n) + 1)), rng)
    n, _, rp, ci, v = dense_to_csr(Ad)
    tau, p = [(1e-6, 25), (0.1, 1), (0.0, 0)][seed % 3]
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    M = sparse.ILUT(A, tau, p)
    Mo = O.Precond(O.PC_ILUT, n)
    Mo.set_params(tau, 0.0, p)
    st = Mo.set_matrix(O.Csr(n, n, rp, ci, v))
    if st != 0:
        with pytest.raises(Exception):
            M.setMatrix(A)
        return
    M.setMatrix(A)
    assert np.array_equal(M.values(), Mo.values())
    assert all(np.array_equal(a, b) for a, b in zip(M.pattern(), Mo.pattern()))


@pytest.mark.parametrize("n", range(1, 11))
@pytest.mark.parametrize("shape", ["tri", "penta"])
def test_ilut_exact_on_banded(ctx, n, shape):
    # TS/ILUTTest with TS/IncompleteFactorizationTestAbstract.java:31-69
    Ad = tridiagonal(n) if shape == "tri" else pentadiagonal(n)
    n, _, rp, ci, v = dense_to_csr(Ad)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    M = sparse.ILUT(A)
    M.setMatrix(A)
    b = A.mult(np.ones(n))
    x = M.apply(b)
    assert np.linalg.norm(A.multAdd(-1, x, b.copy())) <= 1e-5


# SSOR starts each apply from the solver's previous vector (MTJ's z), so
# inside CG and Chebyshev it is no fixed preconditioner: on 2D Poisson MTJ's
# CG + SSOR stalls and Chebyshev + SSOR diverges.  The GPU must do the same:
# the oracle's status, iterations and history, converged or not.
SOLVES = [("cg", "ssor", "poisson2d", 24), ("chebyshev", "ssor", "poisson2d", 16), ("ir", "ssor", "poisson2d", 16),
          ("bicgstab", "ilut", "convdiff3d", 10), ("gmres", "ilut", "convdiff3d", 10),
          ("qmr", "ilut", "convdiff3d", 10), ("cg", "ilut", "poisson2d", 24)]
KIND = {"cg": O.CG, "chebyshev": O.CHEBYSHEV, "ir": O.IR, "bicgstab": O.BICGSTAB, "gmres": O.GMRES, "qmr": O.QMR}


@pytest.mark.parametrize("case", SOLVES, ids=["-".join(map(str, c)) for c in SOLVES])
def test_solvers_with_ssor_ilut_match_oracle(ctx, numerics, case):
    name, pname, mat, N = case
    n, rp, ci, v = getattr(workloads, mat)(N)
    Ao = O.Csr(n, n, rp, ci, v)
    b = O.mult(Ao, workloads.uniform(n, 1))
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    pk = O.PC_SSOR if pname == "ssor" else O.PC_ILUT
    M = sparse.SSOR(A) if pname == "ssor" else sparse.ILUT(A)
    M.setMatrix(A)
    Mo = O.Precond(pk, n)
    assert Mo.set_matrix(Ao) == 0
    eig = (0.0, 0.0)
    if name == "chebyshev":
        Ad = np.zeros((n, n))
        for i in range(n):
            Ad[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
        # SSOR from a zero start is a fixed symmetric operator: the spectrum of M^-1 A
        Minv = np.column_stack([Mo.apply(e) for e in np.eye(n)])
        ev = np.sort(np.linalg.eigvals(Minv @ Ad).real)
        eig = (float(ev[0]), float(ev[-1]))
        Mo = O.Precond(pk, n)
        Mo.set_matrix(Ao)
    solver = {"cg": lambda: sparse.CG(n, ctx=ctx), "chebyshev": lambda: sparse.Chebyshev(n, eig[0], eig[1], ctx=ctx),
              "ir": lambda: sparse.IR(n, ctx=ctx), "bicgstab": lambda: sparse.BiCGstab(n, ctx=ctx),
              "gmres": lambda: sparse.GMRES(n, ctx=ctx), "qmr": lambda: sparse.QMR(n, ctx=ctx)}[name]()
    solver.setPreconditioner(M)
    max_iter = 400
    mon = sparse.DefaultIterationMonitor(max_iter, 1e-10, 1e-50, 1e5)
    mon.setIterationReporter(sparse.IterationReporter(), history_cap=2 * max_iter + 64)
    solver.setIterationMonitor(mon)
    x = np.zeros(n)
    status = 0
    try:
        solver.solve(A, b, x)
    except sparse.IterativeSolverNotConvergedException as e:
        status = e.getReason().value
    xo, res, hr, hi = O.solve(KIND[name], Ao, b, np.zeros(n), Mo, max_iter=max_iter, rtol=1e-10, eigmin=eig[0],
                              eigmax=eig[1])
    assert status == res.status
    assert abs(mon.iterations() - res.iterations) <= 2
    gr, gi = solver.history
    k = min(len(gr), len(hr))
    assert np.array_equal(gi[:k], hi[:k])
    # a history that diverges is compared up to the oracle's divergence test
    fin = np.isfinite(gr[:k]) & np.isfinite(hr[:k]) & (hr[:k] < 1e3 * hr[0])
    bar = 1e-10
    if name == "qmr":
        # QMR's history moves by more than that under a mere change of the
        # order of the oracle's own dot products: four times that envelope
        for block in (16, 64, 256, 1024):
            Mb = O.Precond(pk, n)
            Mb.set_matrix(Ao)
            with O.sum_order(block):
                _, _, hb, _ = O.solve(KIND[name], Ao, b, np.zeros(n), Mb, max_iter=max_iter, rtol=1e-10)
            kb = min(len(hb), len(hr))
            bar = max(bar, 4 * float(np.max(np.abs(hb[:kb] - hr[:kb])) / hr[0]))
    assert float(np.max(np.abs(gr[:k][fin] - hr[:k][fin])) / hr[0]) <= bar
    if res.status == 0:
        assert np.max(np.abs(x - xo)) <= 1e-8 * max(1.0, np.max(np.abs(xo)))


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("name", ["bicgstab", "gmres", "bicg", "qmr", "cgs"])
def test_reference_style_ilut_solves(ctx, seed, name):
    # TS/BiCGstabILUTTest, GMRESILUTTest, BiCG / QMR / CGSILUTTest shapes
    rng = np.random.default_rng(6100 + seed)
    n = int(rng.integers(2, 51))
    Ad = nonsingular_system(n, int(rng.integers(1, min(10, n) + 1)), rng)
    n, _, rp, ci, v = dense_to_csr(Ad)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    M = sparse.ILUT(A)
    M.setMatrix(A)
    solver = {"bicgstab": sparse.BiCGstab, "gmres": sparse.GMRES, "bicg": sparse.BiCG, "qmr": sparse.QMR,
              "cgs": sparse.CGS}[name](n, ctx=ctx)
    solver.setPreconditioner(M)
    for _ in range(3):
        xt = rng.random(n)
        x = rng.random(n)
        solver.solve(A, Ad @ xt, x)
        assert np.max(np.abs(x - xt)) <= 1e-4


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("name", ["cg", "chebyshev"])
def test_reference_style_ssor_solves(ctx, seed, name):
    # TS/CGSSORTest, TS/ChebyshevSSORTest (SPD shapes)
    rng = np.random.default_rng(6200 + seed)
    n = int(rng.integers(2, 51))
    Ad = spd_system(n, int(rng.integers(1, min(10, n) + 1)), rng)
    n, _, rp, ci, v = dense_to_csr(Ad)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    M = sparse.SSOR(A)
    M.setMatrix(A)
    if name == "cg":
        solver = sparse.CG(n, ctx=ctx)
    else:
        Mo = O.Precond(O.PC_SSOR, n)
        Mo.set_matrix(O.Csr(n, n, rp, ci, v))
        ev = np.sort(np.linalg.eigvals(np.column_stack([Mo.apply(e) for e in np.eye(n)]) @ Ad).real)
        solver = sparse.Chebyshev(n, float(ev[0]), float(ev[-1]), ctx=ctx)
    solver.setPreconditioner(M)
    xt = rng.random(n)
    x = rng.random(n)
    solver.solve(A, Ad @ xt, x)
    assert np.max(np.abs(x - xt)) <= 1e-4
