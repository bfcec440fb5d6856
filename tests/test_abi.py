"""The C-ABI library loads and exports every symbol include/mtjg.h declares
(no compute call: runs without a GPU), and the host-only workload
generators produce the documented shapes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mtjg import _lib as L
from mtjg import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "mtjg.h")).read()
    return sorted(set(re.findall(r"MTJG_API\s+[^;(]*?\**\s*(mtjg_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = L.load()
    names = _declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    assert set(_declared()) == set(L.PROTOTYPES)


def test_header_numbering_matches_binding_and_oracle():
    import oracle as O
    text = open(os.path.join(ROOT, "include", "mtjg.h")).read()
    for name, val in (("MTJG_NOT_CONVERGED_ITERATIONS", 1), ("MTJG_NOT_CONVERGED_BREAKDOWN", 3),
                      ("MTJG_ERR_ZERO_PIVOT", 20), ("MTJG_ERR_MISSING_DIAGONAL", 22), ("MTJG_ERR_SINGULAR", 23)):
        assert re.search(rf"{name} = {val}\b", text)
    assert (L.ERR_ZERO_PIVOT, L.ERR_SINGULAR) == (O.ERR_ZERO_PIVOT, O.ERR_SINGULAR)


def test_monitor_defaults_without_gpu():
    lib = L.load()
    m = L.Monitor()
    lib.mtjg_monitor_defaults(C.byref(m))
    assert (m.max_iter, m.rtol, m.atol, m.dtol, m.norm) == (100000, 1e-5, 1e-50, 1e5, L.NORM_TWO)


@pytest.mark.parametrize("dim,N", [(2, 1), (2, 7), (3, 1), (3, 5)])
def test_stencil_shapes(dim, N):
    gen = workloads.poisson2d if dim == 2 else workloads.poisson3d
    n, rp, ci, v = gen(N)
    assert n == N ** dim
    assert rp[-1] == n + 2 * dim * (N - 1) * N ** (dim - 1)
    for i in range(n):
        cols = ci[rp[i]:rp[i + 1]]
        assert np.all(np.diff(cols) > 0)
        assert i in cols
    # symmetric
    A = np.zeros((n, n))
    for i in range(n):
        A[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    assert np.array_equal(A, A.T)
    assert np.all(np.diag(A) == 2 * dim)


def test_convdiff_rows_sum_to_zero_inside():
    n, rp, ci, v = workloads.convdiff3d(6)
    sums = np.array([v[rp[i]:rp[i + 1]].sum() for i in range(n)])
    full = np.array([rp[i + 1] - rp[i] == 7 for i in range(n)])
    assert np.allclose(sums[full], 0.0)
    assert np.all(sums[~full] > 0)


def test_laplacian_shape_and_determinism():
    n, rp, ci, v = workloads.laplacian(5000, 9)
    lens = np.diff(rp)
    assert lens.min() >= 5 and lens.max() <= 30
    assert 15 < lens.mean() < 23
    n2, rp2, ci2, v2 = workloads.laplacian(5000, 9)
    assert np.array_equal(rp, rp2) and np.array_equal(ci, ci2) and np.array_equal(v, v2)
    A = np.zeros((n, n))
    for i in range(n):
        A[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    assert np.array_equal(A, A.T)
    off = A - np.diag(np.diag(A))
    assert np.allclose(np.diag(A), -off.sum(axis=1) + 1e-2)


def test_batch_sizes_log_uniform():
    s = workloads.batch_sizes(4096, 4)
    assert s.min() >= 500 and s.max() <= 50000
    # log-uniform: the median is near sqrt(500 * 50000) = 5000
    assert 3500 < np.median(s) < 7000
    assert np.array_equal(s, workloads.batch_sizes(4096, 4))


def test_uniform_is_seeded():
    a = workloads.uniform(1000, 1)
    assert np.array_equal(a, workloads.uniform(1000, 1))
    assert a.min() >= -1 and a.max() < 1
    assert not np.array_equal(a, workloads.uniform(1000, 2))
