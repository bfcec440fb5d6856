"""A second, independent restatement of MTJ's Krylov path in pure Python.

Python floats are IEEE doubles and Python never fuses a*b+c, so each
expression rounds exactly as the Java source does.  Small cases only: it is
the cross-check that pins the C oracle (oracle/mtj_oracle.c) bit for bit.
References are files of the reference project (S/ = .../matrix/sparse/,
M/ = .../matrix/).
"""
from __future__ import annotations

import bisect
import math


class NotConverged(Exception):
    def __init__(self, code, iters, resid, detail=0):
        super().__init__(code)
        self.code, self.iters, self.resid, self.detail = code, iters, resid, detail


class Unsupported(Exception):
    """UnsupportedOperationException (MatrixIterationMonitor.convergedI(double))."""


class Singular(Exception):
    pass


def jmax(a, b):
    if a != a:
        return a
    if b != b:
        return b
    return a if a >= b else b


def mult(rp, ci, v, x):
    """CompRowMatrix.mult, S/CompRowMatrix.java:295-314."""
    n = len(rp) - 1
    y = [0.0] * n
    for i in range(n):
        s = 0.0
        for k in range(rp[i], rp[i + 1]):
            s = s + v[k] * x[ci[k]]
        if s != 0:
            y[i] = s
    return y


def mult_add(rp, ci, v, alpha, x, y):
    """CompRowMatrix.multAdd, S/CompRowMatrix.java:330-347."""
    y = list(y)
    for i in range(len(rp) - 1):
        s = 0.0
        for k in range(rp[i], rp[i + 1]):
            s = s + v[k] * x[ci[k]]
        y[i] = y[i] + alpha * s
    return y


def dot(x, y):
    s = 0.0
    for a, b in zip(x, y):
        s = s + a * b
    return s


def norm2(x):
    s = 0.0
    for a in x:
        s = s + a * a
    return math.sqrt(s)


class Monitor:
    """DefaultIterationMonitor, S/DefaultIterationMonitor.java:133-156."""

    def __init__(self, max_iter, rtol, atol=1e-50, dtol=1e5):
        self.max_iter, self.rtol, self.atol, self.dtol = max_iter, rtol, atol, dtol
        self.iter = 0
        self.initR = 0.0
        self.residual = 0.0
        self.hist = []

    def converged(self, r, x=None):
        """converged(r, x) with the iterate, converged(r) without (GMRES's
        inner test)."""
        self.hist.append((r, self.iter))
        self.residual = r
        if self.iter == 0:
            self.initR = r
        if r < jmax(self._tol_base(x), self.atol):
            return True
        if r > self.dtol * self.initR:
            raise NotConverged(2, self.iter, r)
        if self.iter >= self.max_iter:
            raise NotConverged(1, self.iter, r)
        if r != r:
            raise NotConverged(2, self.iter, r)
        return False

    def _tol_base(self, x):
        return self.rtol * self.initR


class MatrixMonitor(Monitor):
    """MatrixIterationMonitor, S/MatrixIterationMonitor.java:101-129: the
    test against rtol (normA |x|_2 + normb); converged(double) unsupported."""

    def __init__(self, normA, normb, max_iter, rtol, atol=1e-50, dtol=1e5):
        super().__init__(max_iter, rtol, atol, dtol)
        self.normA, self.normb = normA, normb

    def converged(self, r, x=None):
        if x is None:
            self.hist.append((r, self.iter))
            self.residual = r
            raise Unsupported()
        return super().converged(r, x)

    def _tol_base(self, x):
        return self.rtol * (self.normA * norm2(x) + self.normb)


def jacobi(rp, ci, v):
    """DiagonalPreconditioner.setMatrix, S/DiagonalPreconditioner.java:64-76."""
    n = len(rp) - 1
    inv = [0.0] * n
    for i in range(n):
        cols = ci[rp[i]:rp[i + 1]]
        j = bisect.bisect_left(cols, i)
        d = v[rp[i] + j] if j < len(cols) and cols[j] == i else 0.0
        if d == 0:
            raise RuntimeError(f"Zero diagonal on row {i + 1}")
        inv[i] = 1 / d
    return lambda b: [b[i] * inv[i] for i in range(n)]


def diag_positions(rp, ci):
    out = []
    for k in range(len(rp) - 1):
        cols = ci[rp[k]:rp[k + 1]]
        j = bisect.bisect_left(cols, k)
        if j >= len(cols) or cols[j] != k:
            raise RuntimeError(f"Missing diagonal entry on row {k + 1}")
        out.append(rp[k] + j)
    return out


def ilu_factor(rp, ci, v):
    """ILU.factor, S/ILU.java:86-125 (with its scan past the row end)."""
    n = len(rp) - 1
    data = list(v)
    cix = list(ci) + [-1]  # an index past the last row reads nothing that matches
    dg = diag_positions(rp, ci)
    for k in range(1, n):
        for i in range(rp[k], dg[k]):
            index = cix[i]
            piv = data[dg[index]]
            if piv == 0:
                raise RuntimeError(f"Zero pivot encountered on row {i + 1} during ILU process")
            data[i] = data[i] / piv
            lki = data[i]
            l = rp[k] + 1
            for j in range(dg[index] + 1, rp[index + 1]):
                while l < rp[k + 1] and cix[l] < cix[j]:
                    l += 1
                if cix[l] == cix[j]:
                    data[l] = data[l] - lki * data[j]
    return data, dg


def ilu_apply(rp, ci, data, dg, b):
    """ILU.apply (S/ILU.java:64-70): unit-lower then upper gather solves."""
    n = len(rp) - 1
    y = [0.0] * n
    for i in range(n):
        s = 0.0
        for k in range(rp[i], dg[i]):
            s = s + data[k] * y[ci[k]]
        y[i] = b[i] - s
    x = [0.0] * n
    for i in range(n - 1, -1, -1):
        s = 0.0
        for k in range(dg[i] + 1, rp[i + 1]):
            s = s + data[k] * x[ci[k]]
        x[i] = (y[i] - s) / data[dg[i]]
    return x


def icc_factor(rp, ci, v):
    """ICC.factor, S/ICC.java:85-139, literally (O(n^2))."""
    n = len(rp) - 1
    data = list(v)
    dg = diag_positions(rp, ci)
    for k in range(n):
        Rk = [0.0] * n
        for e in range(rp[k], rp[k + 1]):
            Rk[ci[e]] = data[e]
        for i in range(k):
            Rii = data[dg[i]]
            if Rii == 0:
                raise RuntimeError("zero pivot")
            Rki = Rk[i] / Rii
            if Rki == 0:
                continue
            for j in range(dg[i] + 1, rp[i + 1]):
                Rk[ci[j]] = Rk[ci[j]] - Rki * data[j]
        if Rk[k] == 0:
            raise RuntimeError("zero diagonal")
        sq = math.sqrt(Rk[k])
        for e in range(dg[k], rp[k + 1]):
            data[e] = Rk[ci[e]] / sq
    return data, dg


def icc_apply(rp, ci, data, dg, b):
    """ICC.apply (S/ICC.java:67-73): R' scatter solve then R gather solve."""
    n = len(rp) - 1
    y = list(b)
    for i in range(n):
        y[i] = y[i] / data[dg[i]]
        for k in range(dg[i] + 1, rp[i + 1]):
            y[ci[k]] = y[ci[k]] - data[k] * y[i]
    x = [0.0] * n
    for i in range(n - 1, -1, -1):
        s = 0.0
        for k in range(dg[i] + 1, rp[i + 1]):
            s = s + data[k] * x[ci[k]]
        x[i] = (y[i] - s) / data[dg[i]]
    return x


def cg(rp, ci, v, b, x, M, mon):
    """CG.solve, S/CG.java:58-87."""
    n = len(b)
    x = list(x)
    r = mult_add(rp, ci, v, -1.0, x, b)
    p = [0.0] * n
    rho_1 = 0.0
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        z = M(r)
        rho = dot(r, z)
        if mon.iter == 0:
            p = list(z)
        else:
            beta = rho / rho_1
            p = [p[i] * beta for i in range(n)]
            p = [p[i] + z[i] for i in range(n)]
        q = mult(rp, ci, v, p)
        alpha = rho / dot(p, q)
        if alpha != 0:
            x = [x[i] + alpha * p[i] for i in range(n)]
            r = [r[i] + (-alpha) * q[i] for i in range(n)]
        rho_1 = rho
        mon.iter += 1
    return x


def bicgstab(rp, ci, v, b, x, M, mon):
    """BiCGstab.solve, S/BiCGstab.java:65-116."""
    n = len(b)
    x = list(x)
    rho_1 = rho_2 = alpha = beta = omega = 1.0
    r = mult_add(rp, ci, v, -1.0, x, b)
    rt = list(r)
    p = [0.0] * n
    vv = [0.0] * n
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        rho_1 = dot(rt, r)
        if rho_1 == 0:
            raise NotConverged(3, mon.iter, mon.residual, 1)
        if omega == 0:
            raise NotConverged(3, mon.iter, mon.residual, 2)
        if mon.iter == 0:
            p = list(r)
        else:
            beta = (rho_1 / rho_2) * (alpha / omega)
            temp = [(-omega) * vv[i] for i in range(n)]
            temp = [temp[i] + p[i] for i in range(n)]
            p = list(r) if beta == 0 else [r[i] + beta * temp[i] for i in range(n)]
        phat = M(p)
        vv = mult(rp, ci, v, phat)
        alpha = rho_1 / dot(rt, vv)
        s = list(r) if alpha == 0 else [r[i] + (-alpha) * vv[i] for i in range(n)]
        if alpha != 0:
            x = [x[i] + alpha * phat[i] for i in range(n)]
        if mon.converged(norm2(s), x):
            return x
        shat = M(s)
        t = mult(rp, ci, v, shat)
        omega = dot(t, s) / dot(t, t)
        if omega != 0:
            x = [x[i] + omega * shat[i] for i in range(n)]
        r = list(s) if omega == 0 else [s[i] + (-omega) * t[i] for i in range(n)]
        rho_2 = rho_1
        mon.iter += 1
    return x


def _givens(a, b):
    """GivensRotation(x, y), M/GivensRotation.java:42-58."""
    roe = a if abs(a) > abs(b) else b
    scale = abs(a) + abs(b)
    if scale != 0:
        xs, ys = a / scale, b / scale
        r = scale * math.sqrt(xs * xs + ys * ys)
        if roe < 0:
            r *= -1
        return a / r, b / r
    return 1.0, 0.0


def _rot(c, s, a1, a2):
    return c * a1 + s * a2, -s * a1 + c * a2


def gmres(rp, ci, v, b, x, M, mon, restart=30):
    """GMRES.solve, S/GMRES.java:127-176 with dtrtrs per the netlib reference."""
    n = len(b)
    x = list(x)
    H = [[0.0] * restart for _ in range(restart + 1)]
    rots = [None] * (restart + 1)
    u = mult_add(rp, ci, v, -1.0, x, b)
    r = M(u)
    normr = norm2(r)
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        a = 1 / normr
        V = [[0.0] * n if a == 0 else [a * r[j] for j in range(n)]]
        s = [0.0] * (restart + 1)
        s[0] = normr
        i = 0
        while i < restart and not mon.converged(abs(s[i])):
            u = mult(rp, ci, v, V[i])
            w = M(u)
            for k in range(i + 1):
                H[k][i] = dot(w, V[k])
                h = -H[k][i]
                if h != 0:
                    w = [w[j] + h * V[k][j] for j in range(n)]
            H[i + 1][i] = norm2(w)
            a = 1. / H[i + 1][i]
            V.append([0.0] * n if a == 0 else [a * w[j] for j in range(n)])
            for k in range(i):
                H[k][i], H[k + 1][i] = _rot(rots[k][0], rots[k][1], H[k][i], H[k + 1][i])
            rots[i] = _givens(H[i][i], H[i + 1][i])
            H[i][i], H[i + 1][i] = _rot(rots[i][0], rots[i][1], H[i][i], H[i + 1][i])
            s[i], s[i + 1] = _rot(rots[i][0], rots[i][1], s[i], s[i + 1])
            i += 1
            mon.iter += 1
        for k in range(i):
            if H[k][k] == 0:
                raise Singular()
        for k in range(i - 1, -1, -1):
            if s[k] != 0:
                s[k] = s[k] / H[k][k]
                for q in range(k):
                    s[q] = s[q] - s[k] * H[q][k]
        for j in range(i):
            if s[j] != 0:
                x = [x[t] + s[j] * V[j][t] for t in range(n)]
        u = mult_add(rp, ci, v, -1.0, x, b)
        r = M(u)
        normr = norm2(r)
        mon.iter += 1
    return x


# --------------------------------------------- BiCG, CGS, QMR, Chebyshev, IR
def trans_mult(rp, ci, v, x, m):
    """CompRowMatrix.transMult, S/CompRowMatrix.java:350-366 (scatter)."""
    y = [0.0] * m
    for i in range(len(rp) - 1):
        for k in range(rp[i], rp[i + 1]):
            y[ci[k]] = y[ci[k]] + v[k] * x[i]
    return y


def trans_mult_add(rp, ci, v, alpha, x, y):
    """CompRowMatrix.transMultAdd, S/CompRowMatrix.java:369-388."""
    y = [yi * (1 / alpha) for yi in y]
    for i in range(len(rp) - 1):
        for k in range(rp[i], rp[i + 1]):
            y[ci[k]] = y[ci[k]] + v[k] * x[i]
    return [yi * alpha for yi in y]


def ilu_trans_apply(rp, ci, data, dg, b):
    """ILU.transApply (S/ILU.java:72-78): U' then L' scatter solves
    (S/UpperCompRowMatrix.java:70-90, S/UnitLowerCompRowMatrix.java:70-86)."""
    n = len(rp) - 1
    y = list(b)
    for i in range(n):
        y[i] = y[i] / data[dg[i]]
        for k in range(dg[i] + 1, rp[i + 1]):
            y[ci[k]] = y[ci[k]] - data[k] * y[i]
    x = list(y)
    for i in range(n - 1, -1, -1):
        for k in range(rp[i], dg[i]):
            x[ci[k]] = x[ci[k]] - data[k] * x[i]
    return x


def _set(alpha, y):  # DenseVector.set(alpha, y), M/DenseVector.java:216-231
    return [0.0] * len(y) if alpha == 0 else [alpha * t for t in y]


def _add(d, alpha, y):  # DenseVector.add(alpha, y), M/DenseVector.java:249-264
    return list(d) if alpha == 0 else [d[i] + alpha * y[i] for i in range(len(d))]


def bicg(rp, ci, v, b, x, M, Mt, mon):
    """BiCG.solve, S/BiCG.java:63-102."""
    n = len(b)
    x = list(x)
    rho_1 = rho_2 = 1.0
    r = mult_add(rp, ci, v, -1.0, x, b)
    rt = list(r)
    p = pt = [0.0] * n
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        z = M(r)
        zt = Mt(rt)
        rho_1 = dot(z, rt)
        if rho_1 == 0:
            raise NotConverged(3, mon.iter, mon.residual, 1)
        if mon.iter == 0:
            p, pt = list(z), list(zt)
        else:
            beta = rho_1 / rho_2
            p = [p[i] * beta + z[i] for i in range(n)]
            pt = [pt[i] * beta + zt[i] for i in range(n)]
        q = mult(rp, ci, v, p)
        qt = trans_mult(rp, ci, v, pt, n)
        alpha = rho_1 / dot(pt, q)
        x = _add(x, alpha, p)
        r = _add(r, -alpha, q)
        rt = _add(rt, -alpha, qt)
        rho_2 = rho_1
        mon.iter += 1
    return x


def cgs(rp, ci, v, b, x, M, mon):
    """CGS.solve, S/CGS.java:65-105."""
    n = len(b)
    x = list(x)
    rho_2 = 0.0
    r = mult_add(rp, ci, v, -1.0, x, b)
    rt = list(r)
    p = q = [0.0] * n
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        rho_1 = dot(rt, r)
        if rho_1 == 0:
            raise NotConverged(3, mon.iter, mon.residual, 1)
        if mon.iter == 0:
            u = list(r)
            p = list(u)
        else:
            beta = rho_1 / rho_2
            u = _add(r, beta, q)
            s = _add(q, beta, p)
            p = _add(u, beta, s)
        phat = M(p)
        vhat = mult(rp, ci, v, phat)
        alpha = rho_1 / dot(rt, vhat)
        q = _set(-alpha, vhat)
        q = [q[i] + u[i] for i in range(n)]
        s = [u[i] + q[i] for i in range(n)]
        uhat = M(s)
        x = _add(x, alpha, uhat)
        qhat = mult(rp, ci, v, uhat)
        r = _add(r, -alpha, qhat)
        rho_2 = rho_1
        mon.iter += 1
    return x


def qmr(rp, ci, v, b, x, M, Mt, mon):
    """QMR.solve, S/QMR.java:117-213 with M1 = M2 = M."""
    n = len(b)
    x = list(x)
    rho_1 = xi = gamma_1 = theta = theta_1 = delta = ep = beta = 0.0
    gamma, eta = 1.0, -1.0
    r = mult_add(rp, ci, v, -1.0, x, b)
    v_tld = list(r)
    y = M(v_tld)
    rho = norm2(y)
    w_tld = list(r)
    z = Mt(w_tld)
    xi = norm2(z)
    p = q = d = s = [0.0] * n
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        if rho == 0:
            raise NotConverged(3, mon.iter, mon.residual, 1)
        if xi == 0:
            raise NotConverged(3, mon.iter, mon.residual, 3)
        vv = _set(1 / rho, v_tld)
        y = [t * (1 / rho) for t in y]
        w = _set(1 / xi, w_tld)
        z = [t * (1 / xi) for t in z]
        delta = dot(z, y)
        if delta == 0:
            raise NotConverged(3, mon.iter, mon.residual, 4)
        y_tld = M(y)
        z_tld = Mt(z)
        if mon.iter == 0:
            p, q = list(y_tld), list(z_tld)
        else:
            cp = -xi * delta / ep
            cq = -rho * delta / ep
            p = [p[i] * cp + y_tld[i] for i in range(n)]
            q = [q[i] * cq + z_tld[i] for i in range(n)]
        p_tld = mult(rp, ci, v, p)
        ep = dot(q, p_tld)
        if ep == 0:
            raise NotConverged(3, mon.iter, mon.residual, 5)
        beta = ep / delta
        if beta == 0:
            raise NotConverged(3, mon.iter, mon.residual, 6)
        v_tld = _set(-beta, vv)
        v_tld = [v_tld[i] + p_tld[i] for i in range(n)]
        y = M(v_tld)
        rho_1 = rho
        rho = norm2(y)
        w_tld = trans_mult_add(rp, ci, v, 1.0, q, _set(-beta, w))
        z = Mt(w_tld)
        xi = norm2(z)
        gamma_1 = gamma
        theta_1 = theta
        theta = rho / (gamma_1 * beta)
        gamma = 1 / math.sqrt(1 + theta * theta)
        if gamma == 0:
            raise NotConverged(3, mon.iter, mon.residual, 7)
        eta = -eta * rho_1 * gamma * gamma / (beta * gamma_1 * gamma_1)
        if mon.iter == 0:
            d = _set(eta, p)
            s = _set(eta, p_tld)
        else:
            val = theta_1 * theta_1 * gamma * gamma
            d = _add([t * val for t in d], eta, p)
            s = _add([t * val for t in s], eta, p_tld)
        x = [x[i] + d[i] for i in range(n)]
        r = _add(r, -1.0, s)
        mon.iter += 1
    return x


def chebyshev(rp, ci, v, b, x, M, mon, eigmin, eigmax):
    """Chebyshev.solve, S/Chebyshev.java:90-120."""
    n = len(b)
    x = list(x)
    alpha = 0.0
    r = mult_add(rp, ci, v, -1.0, x, b)
    c = (eigmax - eigmin) / 2.0
    d = (eigmax + eigmin) / 2.0
    p = [0.0] * n
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        z = M(r)
        if mon.iter == 0:
            p = list(z)
            alpha = 2.0 / d
        else:
            beta = (alpha * c) / 2.0
            beta *= beta
            alpha = 1.0 / (d - beta)
            p = [p[i] * beta + z[i] for i in range(n)]
        q = mult(rp, ci, v, p)
        x = _add(x, alpha, p)
        r = _add(r, -alpha, q)
        mon.iter += 1
    return x


def ir(rp, ci, v, b, x, M, mon):
    """IR.solve, S/IR.java:57-70."""
    n = len(b)
    x = list(x)
    r = mult_add(rp, ci, v, -1.0, x, b)
    mon.iter = 0
    while not mon.converged(norm2(r), x):
        z = M(r)
        x = [x[i] + z[i] for i in range(n)]
        r = mult_add(rp, ci, v, -1.0, x, b)
        mon.iter += 1
    return x


# ---------------------------------------------------------- SSOR and ILUT
def ssor_apply(rp, ci, v, dg, b, x, omega_f=1.0, omega_r=1.0, reverse=True):
    """SSOR.apply, S/SSOR.java:148-192: one symmetric SOR sweep starting
    from x's content; returns the new x."""
    n = len(rp) - 1
    xd = list(x)
    xx = list(x)
    for i in range(n):
        sigma = 0.0
        for j in range(rp[i], dg[i]):
            sigma = sigma + v[j] * xx[ci[j]]
        for j in range(dg[i] + 1, rp[i + 1]):
            sigma = sigma + v[j] * xd[ci[j]]
        sigma = (b[i] - sigma) / v[dg[i]]
        xx[i] = xd[i] + omega_f * (sigma - xd[i])
    if not reverse:
        return xx
    for i in range(n - 1, -1, -1):
        sigma = 0.0
        for j in range(rp[i], dg[i]):
            sigma = sigma + v[j] * xx[ci[j]]
        for j in range(dg[i] + 1, rp[i + 1]):
            sigma = sigma + v[j] * xd[ci[j]]
        sigma = (b[i] - sigma) / v[dg[i]]
        xd[i] = xx[i] + omega_r * (sigma - xx[i])
    return xd


class SparseRow:
    """SparseVector's storage (S/SparseVector.java): sorted index[:used];
    the slots past used keep their old contents; full storage doubles (at
    most to `size`) into fresh zeroed arrays (getIndex, :188-231)."""

    def __init__(self, size, index, data):
        self.size = size
        self.index = list(index)
        self.data = list(data)
        self.used = len(index)

    def _find_greater(self, key):  # Arrays.binarySearchGreater over [0, used)
        lo, hi = 0, self.used
        while lo < hi:
            mid = (lo + hi) // 2
            if self.index[mid] < key:
                lo = mid + 1
            else:
                hi = mid
        return lo

    def set(self, ind, value):
        i = self._find_greater(ind)
        if not (i < self.used and self.index[i] == ind):
            self.used += 1
            if self.used > len(self.data):
                cap = len(self.data) * 2 if self.data else 1
                cap = min(cap, self.size)
                ni, nd = self.index[:i] + [0] * (cap - i), self.data[:i] + [0.0] * (cap - i)
            else:
                ni, nd = self.index, self.data
            tail_i = self.index[i:self.used - 1]
            tail_d = self.data[i:self.used - 1]
            ni[i + 1:self.used] = tail_i
            nd[i + 1:self.used] = tail_d
            ni[i], nd[i] = ind, 0.0
            self.index, self.data = ni, nd
        self.data[i] = value

    def zero(self):
        self.data = [0.0] * len(self.data)
        self.used = 0


def ilut_factor(rp, ci, v, tau=1e-6, p=25):
    """ILUT.setMatrix + factor, S/ILUT.java:119-272, literally; returns
    (rows, diagind) or raises RuntimeError."""
    n = len(rp) - 1
    rows = []
    for k in range(n):
        pairs = [(ci[j], v[j]) for j in range(rp[k], rp[k + 1]) if v[j] != 0.0]
        rows.append(SparseRow(n, [c for c, _ in pairs], [x for _, x in pairs]))
    diag = []
    for k in range(n):
        r = rows[k]
        j = bisect.bisect_left(r.index[:r.used], k)
        if j >= r.used or r.index[j] != k:
            raise RuntimeError(f"Missing diagonal entry on row {k + 1}")
        diag.append(j)
    for i in range(1, n):
        rowi = rows[i]
        s = 0.0
        for t in range(rowi.used):
            s = s + rowi.data[t] * rowi.data[t]
        taui = math.sqrt(s) * tau
        z = [0.0] * n
        for t in range(rowi.used):
            z[rowi.index[t]] = rowi.data[t]
        for k in range(i):
            rk = rows[k]
            dk = rk.data[diag[k]]
            if dk == 0:
                raise RuntimeError(f"Zero diagonal entry on row {k + 1} during ILU process")
            lik = z[k] / dk
            if abs(lik) <= taui:
                continue
            for j in range(diag[k] + 1, rk.used):
                z[rk.index[j]] = z[rk.index[j]] - lik * rk.data[j]
            z[k] = lik
        nl = sum(1 for t in range(rowi.used) if rowi.index[t] < i)
        nu = sum(1 for t in range(rowi.used) if rowi.index[t] > i)
        rowi.zero()
        lower = [(c, z[c]) for c in range(i) if abs(z[c]) > taui]
        upper = [(c, z[c]) for c in range(i + 1, n) if abs(z[c]) > taui]
        lower.sort(key=lambda e: -abs(e[1]))  # stable, as Collections.sort
        upper.sort(key=lambda e: -abs(e[1]))
        rowi.set(i, z[i])
        for c, x in lower[:min(nl + p, len(lower))]:
            rowi.set(c, x)
        for c, x in upper[:min(nu + p, len(upper))]:
            rowi.set(c, x)
        d = diag[i]
        if d >= len(rowi.index) or rowi.index[d] != i:
            j = bisect.bisect_left(rowi.index[:rowi.used], i)
            diag[i] = j
    return rows, diag


def ilut_apply(rows, diag, b, y):
    """ILUT.apply (S/ILUT.java:111-113): the unit lower solve into y (whose
    previous content it may read, as MTJ does), then the upper solve."""
    n = len(rows)
    y = list(y)
    for i in range(n):
        r = rows[i]
        s = 0.0
        for j in range(diag[i]):
            s = s + r.data[j] * y[r.index[j]]
        y[i] = b[i] - s
    x = [0.0] * n
    for i in range(n - 1, -1, -1):
        r = rows[i]
        s = 0.0
        for j in range(diag[i] + 1, r.used):
            s = s + r.data[j] * x[r.index[j]]
        x[i] = (y[i] - s) / r.data[diag[i]] if r.data[diag[i]] != 0 else math.copysign(math.inf, y[i] - s)
    return x, y
