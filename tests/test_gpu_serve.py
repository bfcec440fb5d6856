"""Continuous-batching server: results alone equal results in a mix, every
request meets rtol on its FP64 true residual, admission honours the vector
pool, and requests join a batch that is already running."""
import time

import numpy as np
import pytest

import oracle as O
from mtjg import serve, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture
def servers(ctx):
    made = []

    def make(**kw):
        made.append(serve.Server(ctx, **kw))
        return made[-1]

    yield make
    for s in made:  # also when a test fails: no scheduler thread outlives its test
        s.close()


def _library():
    return [workloads.poisson2d(40), workloads.poisson2d(97), workloads.laplacian(1500, 3),
            workloads.laplacian(12000, 4), workloads.poisson3d(14), workloads.laplacian(4000, 5)]


def _rhs(mats, count, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for k in range(count):
        m = int(rng.integers(0, len(mats)))
        n = mats[m][0]
        reqs.append((m, workloads.uniform(n, 1000 + k)))
    return reqs


def _solve_all(srv, mids, reqs, one_at_a_time):
    out = {}
    tickets = {}
    for k, (m, b) in enumerate(reqs):
        t = srv.submit(mids[m], b)
        tickets[t] = k
        if one_at_a_time:
            srv.drain(120.0)
            for r in srv.poll():
                out[tickets[r.ticket]] = r
    srv.drain(120.0)
    for r in srv.poll():
        out[tickets[r.ticket]] = r
    return out


def test_alone_equals_mix_and_converges(servers):
    mats = _library()
    reqs = _rhs(mats, 30, 7)
    srv = servers(max_systems=64, pool_rows=1 << 20)
    mids = [srv.addMatrix(*m) for m in mats]
    alone = _solve_all(srv, mids, reqs, True)
    mix = _solve_all(srv, mids, reqs, False)
    st = srv.stats()
    assert len(alone) == len(mix) == len(reqs)
    assert st["max_active"] > 1  # the mix really ran together
    for k, (m, b) in enumerate(reqs):
        a, x = alone[k], mix[k]
        assert a.status == 0 and x.status == 0
        assert a.iterations == x.iterations and a.inner_iterations == x.inner_iterations
        assert np.array_equal(a.x, x.x), k
        n, rp, ci, v = mats[m]
        r = O.mult_add(O.Csr(n, n, rp, ci, v), -1.0, x.x, b)
        assert np.linalg.norm(r) < 1e-10 * np.linalg.norm(b)


def test_admission_by_pool_footprint(servers):
    mats = [workloads.laplacian(20000, 8), workloads.laplacian(20000, 9)]
    srv = servers(max_systems=16, pool_rows=30000)  # room for one system at a time
    mids = [srv.addMatrix(*m) for m in mats]
    reqs = [(k % 2, workloads.uniform(20000, 50 + k)) for k in range(6)]
    out = _solve_all(srv, mids, reqs, False)
    st = srv.stats()
    assert st["max_active"] == 1
    assert all(out[k].status == 0 for k in range(6))


def test_requests_join_a_running_batch(servers):
    mats = [workloads.poisson2d(600), workloads.laplacian(3000, 2)]
    srv = servers(max_systems=32, pool_rows=1 << 20)
    mids = [srv.addMatrix(*m) for m in mats]
    big = srv.submit(mids[0], workloads.uniform(360000, 1))
    time.sleep(0.02)
    assert srv.poll() == []  # the large solve (thousands of inner iterations) is still running
    small = [srv.submit(mids[1], workloads.uniform(3000, 10 + k)) for k in range(8)]
    srv.drain(120.0)
    res = {r.ticket: r for r in srv.poll()}
    st = srv.stats()
    assert st["max_active"] >= 2
    # the small requests were admitted while the large one was running and
    # finished before it
    assert all(res[t].latency_s < res[big].latency_s for t in small)
    assert all(res[t].status == 0 for t in small + [big])


def test_unknown_matrix_is_rejected(servers):
    srv = servers(max_systems=4, pool_rows=1000)
    with pytest.raises(KeyError):
        srv.submit(5, np.zeros(3))


def test_remove_matrix_while_its_requests_run(servers):
    from mtjg import sparse
    mats = [workloads.poisson2d(150), workloads.laplacian(2000, 6)]
    srv = servers(max_systems=8, pool_rows=1 << 18)
    mids = [srv.addMatrix(*m) for m in mats]
    t = [srv.submit(mids[0], workloads.uniform(22500, 70 + k)) for k in range(3)]
    srv.removeMatrix(mids[0])  # its three requests still finish
    with pytest.raises(KeyError):
        srv.submit(mids[0], workloads.uniform(22500, 1))
    with pytest.raises(sparse.IllegalArgumentException):  # removed twice
        srv.removeMatrix(mids[0])
    u = srv.submit(mids[1], workloads.uniform(2000, 5))
    srv.drain(120.0)
    res = {r.ticket: r for r in srv.poll()}
    assert all(res[k].status == 0 for k in t + [u])
    srv.removeMatrix(mids[1])  # nothing outstanding: freed at once


def test_zero_rhs_and_iteration_limit(servers):
    """b = 0 converges at the first test with x = 0; a server whose refinement
    budget cannot reach rtol reports the iteration limit; a normal request
    beside either is unaffected."""
    mats = [workloads.poisson2d(60), workloads.poisson2d(200)]
    srv = servers(max_systems=8, pool_rows=1 << 18)
    mids = [srv.addMatrix(*m) for m in mats]
    zero = srv.submit(mids[0], np.zeros(3600))
    ok = srv.submit(mids[1], workloads.uniform(40000, 3))
    srv.drain(120.0)
    res = {r.ticket: r for r in srv.poll()}
    assert res[zero].status == 0 and res[zero].iterations == 0
    assert not np.any(res[zero].x)
    assert res[ok].status == 0
    tight = servers(max_systems=8, pool_rows=1 << 18, max_iter=2, inner_max_iter=5)
    tids = [tight.addMatrix(*m) for m in mats]
    lim = tight.submit(tids[1], workloads.uniform(40000, 3))
    tight.drain(120.0)
    res = {r.ticket: r for r in tight.poll()}
    assert res[lim].status == 1  # IterativeSolverNotConvergedException, Reason.Iterations
    assert res[lim].iterations <= 2


def _sizes(servers, mats):
    """Device bytes of each matrix, read from an unlimited server's residency."""
    srv = servers(max_systems=4, pool_rows=1 << 20)
    out, prev = [], 0
    for m in mats:
        srv.addMatrix(*m)
        now = srv.residency()["resident_bytes"]
        out.append(now - prev)
        prev = now
    srv.close()
    return out


def test_matrix_budget_evicts_and_results_do_not_change(servers):
    """A budget that holds about two of the six matrices: idle matrices are
    evicted and uploaded again on demand, the resident bytes never exceed
    the budget, and every result equals the one from a server that keeps
    all six resident."""
    mats = _library()
    sizes = _sizes(servers, mats)
    budget = sorted(sizes)[-1] + sorted(sizes)[-2]
    reqs = _rhs(mats, 40, 11)
    ref = servers(max_systems=64, pool_rows=1 << 20)
    rids = [ref.addMatrix(*m) for m in mats]
    want = _solve_all(ref, rids, reqs, False)
    srv = servers(max_systems=64, pool_rows=1 << 20, matrix_budget=budget)
    mids = [srv.addMatrix(*m) for m in mats]
    reg = srv.residency()
    assert reg["resident_bytes"] <= budget and reg["evictions"] == 0  # registration never evicts
    assert reg["resident_matrices"] < len(mats)
    got = _solve_all(srv, mids, reqs, False)
    res = srv.residency()
    assert res["evictions"] > 0 and res["uploads"] > len(mats)
    assert res["resident_bytes"] <= budget
    for k in range(len(reqs)):
        assert got[k].status == 0
        assert got[k].iterations == want[k].iterations
        assert np.array_equal(got[k].x, want[k].x), k


def test_lru_order_of_evictions(servers):
    """With room for two of three equal matrices, using A, B, A, C evicts B
    (least recently used), not A; a request for B then uploads it again."""
    mats = [workloads.laplacian(5000, 20 + k) for k in range(3)]
    sizes = _sizes(servers, mats)
    srv = servers(max_systems=8, pool_rows=1 << 18, matrix_budget=max(sizes) * 2 + 1024)
    A, B, C = [srv.addMatrix(*m) for m in mats]
    assert srv.residency()["resident_matrices"] == 2  # C waits for its first request
    for mid in (A, B, A):
        srv.submit(mid, workloads.uniform(5000, mid))
        srv.drain(60.0)
    assert srv.residency()["evictions"] == 0
    srv.submit(C, workloads.uniform(5000, 9))
    srv.drain(60.0)
    r = srv.residency()
    assert r["evictions"] == 1 and r["uploads"] == 3
    srv.submit(A, workloads.uniform(5000, 10))  # A stayed: no upload
    srv.drain(60.0)
    assert srv.residency()["uploads"] == 3
    srv.submit(B, workloads.uniform(5000, 11))  # B was the one evicted
    srv.drain(60.0)
    r = srv.residency()
    assert r["uploads"] == 4 and r["evictions"] == 2
    assert all(f.status == 0 for f in srv.poll())


def test_budget_held_by_busy_matrices_makes_requests_wait(servers):
    """Room for one matrix: requests for two matrices alternate, so the
    second matrix's request waits until the first one's systems are
    delivered; everything still finishes."""
    mats = [workloads.poisson2d(120), workloads.poisson2d(121)]
    sizes = _sizes(servers, mats)
    srv = servers(max_systems=8, pool_rows=1 << 18, matrix_budget=max(sizes) + 1024)
    mids = [srv.addMatrix(*m) for m in mats]
    reqs = [(k % 2, workloads.uniform(mats[k % 2][0], 300 + k)) for k in range(6)]
    out = _solve_all(srv, mids, reqs, False)
    assert all(out[k].status == 0 for k in range(6))
    r = srv.residency()
    assert r["resident_matrices"] == 1 and r["evictions"] >= 5


def test_registration_checks(servers):
    from mtjg import sparse
    n, rp, ci, v = workloads.poisson2d(30)
    sizes = _sizes(servers, [(n, rp, ci, v)])
    srv = servers(max_systems=4, pool_rows=1 << 16, matrix_budget=sizes[0] - 1)
    with pytest.raises(sparse.IllegalArgumentException):  # larger than the whole budget
        srv.addMatrix(n, rp, ci, v)
    v0 = v.copy()
    v0[rp[7] + list(ci[rp[7]:rp[8]]).index(7)] = 0.0
    srv2 = servers(max_systems=4, pool_rows=1 << 16)
    with pytest.raises(RuntimeError, match="Zero diagonal on row 8"):
        srv2.addMatrix(n, rp, ci, v0)
    with pytest.raises(sparse.IllegalArgumentException):  # unsorted columns
        bad = ci.copy()
        bad[rp[3]], bad[rp[3] + 1] = bad[rp[3] + 1], bad[rp[3]]
        srv2.addMatrix(n, rp, bad, v)


def _direct_krylov(ctx, kind, mat, b):
    """What a lone mtjg_solver_solve gives with the server's default settings:
    mixed-precision GMRES(30) / BiCGstab + Jacobi, 100 refinements, rtol 1e-10,
    inner_rtol 1e-6, 2000 inner iterations."""
    from mtjg import sparse
    n, rp, ci, v = mat
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx)
    s = sparse.GMRES(n, restart=30, ctx=ctx) if kind == "gmres" else sparse.BiCGstab(n, ctx=ctx)
    M = sparse.DiagonalPreconditioner(n, ctx)
    M.setMatrix(A)
    s.setPreconditioner(M)
    s.setIterationMonitor(sparse.DefaultIterationMonitor(100, 1e-10, 1e-50, 1e5))
    s.setMixedPrecision(True, 1e-6, 2000)
    x = np.zeros(n)
    s.solve(A, b, x)
    return x, s.getIterationMonitor().iterations()


def test_krylov_lane_in_the_mix(servers, ctx):
    """GMRES and BiCGstab requests beside CG requests: each Krylov-lane result
    equals a lone solver call with the same settings and the same request
    served alone, bit for bit, and meets rtol on its FP64 residual; the CG
    results equal their alone results too."""
    mats = _library()
    rng = np.random.default_rng(21)
    reqs = []
    for k in range(24):
        m = int(rng.integers(0, len(mats)))
        reqs.append((m, workloads.uniform(mats[m][0], 500 + k), ("cg", "gmres", "bicgstab")[k % 3]))
    srv = servers(max_systems=64, pool_rows=1 << 20)
    mids = [srv.addMatrix(*m) for m in mats]

    def run(batch):
        tickets = {srv.submit(mids[m], b, solver=kind): k for k, (m, b, kind) in batch}
        srv.drain(300.0)
        return {tickets[r.ticket]: r for r in srv.poll()}

    mix = run(list(enumerate(reqs)))
    assert len(mix) == len(reqs)
    for k, (m, b, kind) in enumerate(reqs):
        alone = run([(k, (m, b, kind))])[k]
        got = mix[k]
        assert got.status == 0 and alone.status == 0
        assert np.array_equal(got.x, alone.x), (k, kind)
        n, rp, ci, v = mats[m]
        r = O.mult_add(O.Csr(n, n, rp, ci, v), -1.0, got.x, b)
        assert np.linalg.norm(r) < 1e-10 * np.linalg.norm(b)
        if kind != "cg" and k < 9:
            xd, it = _direct_krylov(ctx, kind, mats[m], b)
            assert np.array_equal(got.x, xd) and got.iterations == it


def test_krylov_lane_under_a_matrix_budget(servers):
    """GMRES requests on six matrices with room for two: matrices are evicted
    and uploaded again, and the results equal those of an unlimited server."""
    mats = _library()
    sizes = _sizes(servers, mats)
    reqs = [(k % len(mats), workloads.uniform(mats[k % len(mats)][0], 900 + k)) for k in range(12)]
    out = []
    for budget in (0, sorted(sizes)[-1] + sorted(sizes)[-2]):
        srv = servers(max_systems=16, pool_rows=1 << 20, matrix_budget=budget)
        mids = [srv.addMatrix(*m) for m in mats]
        tickets = {srv.submit(mids[m], b, solver="gmres"): k for k, (m, b) in enumerate(reqs)}
        srv.drain(300.0)
        out.append(({tickets[r.ticket]: r for r in srv.poll()}, srv.residency()))
    (free, _), (tight, res) = out
    assert res["evictions"] > 0 and res["resident_bytes"] <= sorted(sizes)[-1] + sorted(sizes)[-2]
    for k in range(len(reqs)):
        assert free[k].status == 0 and np.array_equal(free[k].x, tight[k].x)


def test_server_rejects_other_solvers(servers):
    import ctypes as C
    from mtjg import _lib as L
    srv = servers(max_systems=4, pool_rows=1 << 14)
    n, rp, ci, v = workloads.poisson2d(10)
    mid = srv.addMatrix(n, rp, ci, v)
    b, x = np.ones(n), np.zeros(n)
    t = C.c_int64()
    code = srv._lib.mtjg_server_submit_solver(srv.h, mid, L.QMR, L.dptr(b), None, L.dptr(x), C.byref(t))
    assert code == L.ERR_UNSUPPORTED
