"""The server under concurrent callers: four threads submit CG, GMRES and
BiCGstab requests at once to a server whose matrix budget holds about two
of its six matrices (so both lanes evict and upload while others run), and
a fifth thread registers a matrix, submits to it and removes it while its
requests run.  Every result must equal, bit for bit, the result of the same
request on a quiet unlimited server, since a request's arithmetic does not
depend on what runs beside it."""
import threading

import numpy as np
import pytest

from mtjg import serve, workloads

pytestmark = pytest.mark.gpu

KINDS = ("cg", "gmres", "bicgstab")


def _library():
    return [workloads.poisson2d(40), workloads.laplacian(1500, 3), workloads.laplacian(6000, 4),
            workloads.poisson2d(70), workloads.laplacian(3000, 5), workloads.poisson3d(12)]


def _requests(mats, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        m = int(rng.integers(0, len(mats)))
        out.append((m, KINDS[int(rng.integers(0, 3))], workloads.uniform(mats[m][0], seed * 1000 + k)))
    return out


def test_concurrent_callers_under_a_budget(ctx):
    mats = _library()
    extra = workloads.laplacian(2500, 9)
    per_thread = [_requests(mats, 12, 50 + t) for t in range(4)]
    extra_reqs = [(KINDS[k % 3], workloads.uniform(extra[0], 7000 + k)) for k in range(3)]

    # reference: a quiet server with every matrix resident, one request at a time
    ref = serve.Server(ctx, max_systems=16, pool_rows=1 << 20)
    try:
        ids = [ref.addMatrix(*m) for m in mats]
        xid = ref.addMatrix(*extra)
        want = {}
        for t, reqs in enumerate(per_thread):
            for k, (m, kind, b) in enumerate(reqs):
                ref.submit(ids[m], b, solver=kind)
                ref.drain(120.0)
                want[(t, k)] = ref.poll()[0].x
        for k, (kind, b) in enumerate(extra_reqs):
            ref.submit(xid, b, solver=kind)
            ref.drain(120.0)
            want[("x", k)] = ref.poll()[0].x
        sizes = []
        for m in mats:
            probe = serve.Server(ctx, max_systems=2, pool_rows=1 << 16)
            probe.addMatrix(*m)
            sizes.append(probe.residency()["resident_bytes"])
            probe.close()
    finally:
        ref.close()

    budget = sorted(sizes)[-1] + sorted(sizes)[-2]
    srv = serve.Server(ctx, max_systems=16, pool_rows=1 << 20, matrix_budget=budget)
    try:
        ids = [srv.addMatrix(*m) for m in mats]
        tickets, lock, errors = {}, threading.Lock(), []

        def caller(t):
            try:
                for k, (m, kind, b) in enumerate(per_thread[t]):
                    tk = srv.submit(ids[m], b, solver=kind)
                    with lock:
                        tickets[tk] = (t, k)
            except Exception as e:  # pragma: no cover - reported below
                errors.append(repr(e))

        def register_submit_remove():
            try:
                xid = srv.addMatrix(*extra)
                for k, (kind, b) in enumerate(extra_reqs):
                    tk = srv.submit(xid, b, solver=kind)
                    with lock:
                        tickets[tk] = ("x", k)
                srv.removeMatrix(xid)  # its requests still finish
            except Exception as e:  # pragma: no cover
                errors.append(repr(e))

        threads = [threading.Thread(target=caller, args=(t,)) for t in range(4)]
        threads.append(threading.Thread(target=register_submit_remove))
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        assert not errors, errors
        srv.drain(300.0)
        got = {tickets[r.ticket]: r for r in srv.poll(cap=4096)}
        assert len(got) == len(want)
        for key, x in want.items():
            assert got[key].status == 0, key
            assert np.array_equal(got[key].x, x), key
        res = srv.residency()
        assert res["evictions"] > 0 and res["resident_bytes"] <= budget
    finally:
        srv.close()
