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
