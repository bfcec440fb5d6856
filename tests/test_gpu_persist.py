"""The one-launch CG (persist.cuh) against the graph-captured phase launches.

CG with the identity or Jacobi preconditioner on a system of at most 512
product tiles runs its whole loop in one cooperative launch.  It must give
the graph path's results bit for bit -- x, status, iteration count and every
recorded residual -- under both numerics, every norm and every lanes-per-row
class, and it must actually be the path taken (one launch for the loop).
Parity of the graph path with the oracle is covered by the parity and config
tests; C1 (2D Poisson 128^2) now runs through this path there as well.
"""
import numpy as np
import pytest

from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu

FAST, STRICT = 0, 1


def wide_spd(n, seed):
    """A graph Laplacian (+1e-2 I) whose rows span the three lanes-per-row
    classes: most rows about 20 entries, every 40th row a hub of about 150."""
    rng = np.random.default_rng(seed)
    rows, cols, w = [], [], []
    for i in range(n):
        k = 150 if i % 40 == 0 else 9
        js = rng.integers(0, n, k)
        for j in js:
            if j != i:
                rows.append(i)
                cols.append(int(j))
                w.append(rng.random() + 0.1)
    rows, cols, w = np.array(rows), np.array(cols), np.array(w)
    W = {}
    for i, j, x in zip(rows, cols, w):
        a, b = (i, j) if i < j else (j, i)
        W[(a, b)] = W.get((a, b), 0.0) + x
    adj = [dict() for _ in range(n)]
    for (a, b), x in W.items():
        adj[a][b] = -x
        adj[b][a] = -x
    rp, ci, v = [0], [], []
    for i in range(n):
        d = -sum(adj[i].values()) + 1e-2
        ent = dict(adj[i])
        ent[i] = d
        for j in sorted(ent):
            ci.append(j)
            v.append(ent[j])
        rp.append(len(ci))
    return n, np.array(rp, dtype=np.int32), np.array(ci, dtype=np.int32), np.array(v)


def arrow(n, width):
    """SPD arrow matrix: row 0 holds `width` entries (longer than a tile)."""
    rp, ci, v = [0], [], []
    cols0 = list(range(0, width))
    for i in range(n):
        if i == 0:
            ci += cols0
            v += [float(width)] + [-0.5 / width] * (width - 1)
        elif i < width:
            ci += [0, i]
            v += [-0.5 / width, 2.0]
        else:
            ci += [i]
            v += [2.0]
        rp.append(len(ci))
    return n, np.array(rp, dtype=np.int32), np.array(ci, dtype=np.int32), np.array(v)


MATS = {
    "poisson2d_128": workloads.poisson2d(128),
    "poisson3d_16": workloads.poisson3d(16),
    "laplacian_6000": workloads.laplacian(6000, 3),
    "wide_spd_3000": wide_spd(3000, 5),
}


@pytest.fixture(params=[FAST, STRICT], ids=["fast", "strict"])
def numerics(request, ctx):
    ctx.setNumerics(request.param)
    yield request.param
    ctx.setNumerics(FAST)


def _solve(ctx, mat, pc, graph, b=None, x0=None, max_iter=3000, rtol=1e-10, norm=sparse.Norm.Two):
    n, rp, ci, v = mat
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    solver = sparse.CG(n, ctx=ctx)
    if pc == "jacobi":
        M = sparse.DiagonalPreconditioner(n, ctx)
        M.setMatrix(A)
        solver.setPreconditioner(M)
    mon = sparse.DefaultIterationMonitor(max_iter, rtol, 1e-50, 1e5)
    mon.setNormType(norm)
    mon.setIterationReporter(sparse.IterationReporter(), history_cap=max_iter + 8)
    solver.setIterationMonitor(mon)
    if graph:
        solver.setGraphLaunch(True)
    b = workloads.uniform(n, 41) if b is None else b
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    before = ctx.launchCount()
    exc = None
    try:
        solver.solve(A, b, x)
    except sparse.IterativeSolverNotConvergedException as e:
        exc = type(e).__name__ + ":" + str(e)
    launches = ctx.launchCount() - before
    gr, gi = solver.history
    return x, exc, mon.iterations(), np.array(gr), np.array(gi), launches


def _same(a, b):
    xa, ea, ia, ra, ha, _ = a
    xb, eb, ib, rb, hb, _ = b
    assert ea == eb
    assert ia == ib
    assert np.array_equal(ha, hb)
    assert np.array_equal(ra.view(np.int64), rb.view(np.int64))
    assert np.array_equal(xa.view(np.int64), xb.view(np.int64))


@pytest.mark.parametrize("pc", ["identity", "jacobi"])
@pytest.mark.parametrize("name", sorted(MATS))
def test_one_launch_equals_graph(ctx, numerics, pc, name):
    one = _solve(ctx, MATS[name], pc, graph=False)
    many = _solve(ctx, MATS[name], pc, graph=True)
    _same(one, many)
    assert one[1] is None and one[2] > 5
    # cg_init (one product launch per lanes-per-row class and its finalize)
    # plus the loop's one launch, against five launches per iteration
    assert one[5] <= 5, one[5]
    assert many[5] >= 5 * one[2]


@pytest.mark.parametrize("norm", [sparse.Norm.One, sparse.Norm.TwoRobust, sparse.Norm.Infinity])
def test_one_launch_norms(ctx, numerics, norm):
    mat = MATS["laplacian_6000"]
    _same(_solve(ctx, mat, "jacobi", graph=False, norm=norm), _solve(ctx, mat, "jacobi", graph=True, norm=norm))


def test_one_launch_iteration_limit(ctx, numerics):
    mat = MATS["poisson2d_128"]
    one = _solve(ctx, mat, "jacobi", graph=False, max_iter=7)
    many = _solve(ctx, mat, "jacobi", graph=True, max_iter=7)
    _same(one, many)
    assert one[1] is not None and "Iterations" in one[1]
    assert one[2] == 7 and len(one[3]) == 8


def test_one_launch_converged_at_start(ctx):
    """x0 solves the system exactly (integer data): cg_init's test stops the
    solve and the loop's launch has nothing to do."""
    n, rp, ci, v = MATS["poisson2d_128"]
    x0 = np.arange(n, dtype=np.float64) % 7
    b = np.zeros(n)
    for i in range(n):
        b[i] = np.dot(v[rp[i]:rp[i + 1]], x0[ci[rp[i]:rp[i + 1]]])
    one = _solve(ctx, MATS["poisson2d_128"], "jacobi", graph=False, b=b, x0=x0)
    many = _solve(ctx, MATS["poisson2d_128"], "jacobi", graph=True, b=b, x0=x0)
    _same(one, many)
    assert one[1] is None and one[2] == 0
    assert np.array_equal(one[0], x0)


def test_one_launch_repeatable_and_reused(ctx):
    """Solves back to back on one solver (buffers reused) give identical
    results, and a nonzero x0 is honoured."""
    n, rp, ci, v = MATS["poisson3d_16"]
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    solver = sparse.CG(n, ctx=ctx)
    solver.setIterationMonitor(sparse.DefaultIterationMonitor(2000, 1e-10, 1e-50, 1e5))
    b = workloads.uniform(n, 5)
    xs = []
    for _ in range(3):
        x = workloads.uniform(n, 6)
        solver.solve(A, b, x)
        xs.append(x)
    assert all(np.array_equal(xs[0], x) for x in xs[1:])
    r = b - np.array([np.dot(v[rp[i]:rp[i + 1]], xs[0][ci[rp[i]:rp[i + 1]]]) for i in range(n)])
    assert np.linalg.norm(r) < 1e-9 * np.linalg.norm(b)


def test_large_system_takes_the_graph(ctx):
    """A system of more than 512 product tiles keeps the graph path."""
    mat = workloads.poisson3d(48)
    one = _solve(ctx, mat, "jacobi", graph=False)
    many = _solve(ctx, mat, "jacobi", graph=True)
    _same(one, many)
    assert one[5] > 5 * one[2]


def test_long_row_takes_the_graph(ctx):
    """A row longer than a tile (1152 entries) keeps the graph path."""
    mat = arrow(3000, 1500)
    one = _solve(ctx, mat, "jacobi", graph=False)
    many = _solve(ctx, mat, "jacobi", graph=True)
    _same(one, many)
    assert one[5] > 3
