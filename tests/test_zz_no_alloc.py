"""mtjg_csr_mult_add_norm_noalloc (y = alpha A x + y and the two-norm of the
new y, on the library's fixed device scratch) against the allocating path:
mtjg_csr_mult_add_dev for y and a host norm of that y.

Kept last in collection order; it passes alone in a fresh process too
(``pytest tests/test_zz_no_alloc.py -m gpu``)."""
import ctypes as C

import numpy as np
import pytest

from mtjg import _lib as L
from mtjg import sparse, workloads

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


def _fn(lib):
    f = lib.mtjg_csr_mult_add_norm_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


class DevVec:
    def __init__(self, ctx, n):
        self.lib, self.ctx, self.n = ctx._lib, ctx, int(n)
        p = C.c_void_p()
        assert self.lib.mtjg_dev_alloc(ctx.h, 8 * max(1, self.n), C.byref(p)) == 0, L.last_error()
        self.p = p

    def put(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == self.n
        assert self.lib.mtjg_memcpy_h2d(self.ctx.h, self.p, a.ctypes.data_as(C.c_void_p), 8 * self.n) == 0

    def get(self):
        out = np.empty(self.n)
        assert self.lib.mtjg_memcpy_d2h(self.ctx.h, out.ctypes.data_as(C.c_void_p), self.p, 8 * self.n) == 0
        return out

    def free(self):
        self.lib.mtjg_dev_free(self.ctx.h, self.p)


def _compare(ctx, A, nsys, sys_rows, alpha, calls):
    lib = ctx._lib
    f = _fn(lib)
    n = A.n
    dx, dy1, dy2, dnorm = DevVec(ctx, n), DevVec(ctx, n), DevVec(ctx, n), DevVec(ctx, nsys)
    try:
        for call in range(calls):  # consecutive calls reuse the same scratch
            x = workloads.uniform(n, 11 + call)
            y0 = workloads.uniform(n, 97 + call)
            dx.put(x)
            dy1.put(y0)
            dy2.put(y0)
            assert lib.mtjg_csr_mult_add_dev(A.h, alpha, dx.p, dy1.p) == 0, L.last_error()
            assert f(A.h, alpha, dx.p, dy2.p, dnorm.p) == 0, L.last_error()
            ctx.synchronize()
            y_ref, y_new, norms = dy1.get(), dy2.get(), dnorm.get()
            np.testing.assert_allclose(y_new, y_ref, rtol=1e-13, atol=1e-300)
            for s in range(nsys):
                seg = y_ref[sys_rows[s]:sys_rows[s + 1]]
                ref = float(np.sqrt(np.sum(seg * seg)))
                assert abs(norms[s] - ref) <= 1e-12 * max(ref, 1e-300), (call, s, norms[s], ref)
    finally:
        for v in (dx, dy1, dy2, dnorm):
            v.free()


def test_matches_mult_add_and_host_norm(ctx):
    n, rp, ci, v = workloads.poisson3d(40)
    A = sparse.CompRowMatrix(n, n, rp, ci, v, ctx=ctx)
    _compare(ctx, A, 1, [0, n], -1.0, calls=2)
    n2, rp2, ci2, v2 = workloads.laplacian(50000, 3)
    B = sparse.CompRowMatrix(n2, n2, rp2, ci2, v2, ctx=ctx)
    _compare(ctx, B, 1, [0, n2], 0.75, calls=2)


def test_batch_gives_one_norm_per_system(ctx):
    systems = [workloads.laplacian(int(k), 20 + i) for i, k in enumerate([700, 3000, 128, 9000])]
    A = sparse.BatchCompRowMatrix(systems, ctx=ctx)
    _compare(ctx, A, A.numSystems(), [int(r) for r in A.sys_rows], -1.0, calls=2)


def test_rejects_more_groups_than_the_scratch_holds(ctx):
    one = (2, np.array([0, 1, 2]), np.array([0, 1]), np.array([2.0, 3.0]))
    A = sparse.BatchCompRowMatrix([one] * 16385, ctx=ctx)
    f = _fn(ctx._lib)
    dx, dy, dnorm = DevVec(ctx, A.n), DevVec(ctx, A.n), DevVec(ctx, 16385)
    try:
        assert f(A.h, 1.0, dx.p, dy.p, dnorm.p) == L.ERR_ILLEGAL_ARGUMENT
        assert "16384" in L.last_error()
    finally:
        for v in (dx, dy, dnorm):
            v.free()
