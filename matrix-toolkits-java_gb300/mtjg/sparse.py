"""Host-side mirror of MTJ's ``no.uib.cipr.matrix.sparse`` iterative API.

Same class and method names, argument meaning and error behaviour as the
reference (citations are files of the reference project, S/ =
src/main/java/no/uib/cipr/matrix/sparse/, M/ = src/main/java/no/uib/cipr/matrix/):

  CompRowMatrix               S/CompRowMatrix.java   (device CSR)
  DiagonalPreconditioner      S/DiagonalPreconditioner.java
  ILU, ICC                    S/ILU.java, S/ICC.java
  CG, BiCGstab, GMRES         S/CG.java, S/BiCGstab.java, S/GMRES.java
  BiCG, CGS, QMR, Chebyshev, IR  S/BiCG.java, S/CGS.java, S/QMR.java, S/Chebyshev.java, S/IR.java
  DefaultIterationMonitor     S/DefaultIterationMonitor.java
  IterativeSolverNotConvergedException, NotConvergedException.Reason

Vectors are float64 numpy arrays (the DenseVector analogue); ``solve``
overwrites ``x`` in place and returns it, as IterativeSolver.solve does.
Everything computes on the GPU through libmtjg.so.
"""
from __future__ import annotations

import ctypes as C
import enum
import sys

import numpy as np

from . import _lib as L


# ---------------------------------------------------------------- errors
class IllegalArgumentException(ValueError):
    pass


class IndexOutOfBoundsException(IndexError):
    pass


class MatrixSingularException(RuntimeError):
    """M/MatrixSingularException.java (GMRES's triangular solve)."""


class CudaError(RuntimeError):
    pass


class UnsupportedOperationException(RuntimeError):
    pass


class NotConvergedException(Exception):
    class Reason(enum.Enum):  # M/NotConvergedException.java:33-49
        Iterations = 1
        Divergence = 2
        Breakdown = 3


class IterativeSolverNotConvergedException(NotConvergedException):
    """S/IterativeSolverNotConvergedException.java: reason, residual, iterations."""

    def __init__(self, reason, residual, iterations, message=""):
        super().__init__(f"{reason.name}{': ' + message if message else ''} "
                         f"(residual={residual}, iterations={iterations})")
        self.reason = reason
        self._r = residual
        self._it = iterations
        self.message = message

    def getReason(self):
        return self.reason

    def getResidual(self):
        return self._r

    def getIterations(self):
        return self._it


# mtjg_result.detail of a breakdown -> the name MTJ's exception message carries
BREAKDOWN = {1: "rho", 2: "omega", 3: "xi", 4: "delta", 5: "ep", 6: "beta", 7: "gamma"}


def _raise(code: int, what: str = ""):
    if code == L.OK:
        return
    msg = L.last_error()
    if code in (L.ERR_ILLEGAL_ARGUMENT,):
        raise IllegalArgumentException(msg)
    if code == L.ERR_INDEX_OUT_OF_BOUNDS:
        raise IndexOutOfBoundsException(msg)
    if code in (L.ERR_ZERO_PIVOT, L.ERR_ZERO_DIAGONAL, L.ERR_MISSING_DIAGONAL):
        raise RuntimeError(msg)
    if code == L.ERR_IO:
        raise IOError(msg)
    if code == L.ERR_UNSUPPORTED:
        raise UnsupportedOperationException(msg)
    if code == L.ERR_SINGULAR:
        raise MatrixSingularException(msg)
    raise CudaError(f"{what}: code {code}: {msg}")


# --------------------------------------------------------------- context
class Context:
    """One CUDA device and stream (all objects made with it share them)."""

    def __init__(self, device: int = 0, numerics: int = L.NUMERICS_FAST):
        self._lib = L.load()
        h = C.c_void_p()
        _raise(self._lib.mtjg_ctx_create(device, C.byref(h)), "mtjg_ctx_create")
        self.h = h
        self.setNumerics(numerics)

    def setNumerics(self, numerics: int):
        _raise(self._lib.mtjg_ctx_set_numerics(self.h, numerics), "set_numerics")
        self.numerics = numerics

    def launchCount(self) -> int:
        return int(self._lib.mtjg_ctx_launch_count(self.h))

    def synchronize(self):
        _raise(self._lib.mtjg_ctx_synchronize(self.h), "synchronize")

    def close(self):
        if getattr(self, "h", None):
            self._lib.mtjg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        # at interpreter shutdown the process is about to release the device
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


_default = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default


# ---------------------------------------------------------- CompRowMatrix
class CompRowMatrix:
    """CSR matrix resident on the device (S/CompRowMatrix.java).

    ``CompRowMatrix(numRows, numColumns, rowptr, colind, data)`` takes MTJ's
    0-based arrays (ascending columns per row); ``CompRowMatrix.fromDense``
    builds the pattern of the nonzeros of a dense array.
    """

    def __init__(self, numRows, numColumns, rowptr, colind, data, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self._lib = self.ctx._lib
        self.rowptr = L.i32(rowptr)
        self.colind = L.i32(colind)
        self.data = L.f64(data)
        self.n, self.m = int(numRows), int(numColumns)
        if len(self.rowptr) != self.n + 1:
            raise IllegalArgumentException("rowptr.length != numRows + 1")
        nnz = int(self.rowptr[-1]) if self.n >= 0 else 0
        if len(self.colind) < nnz or len(self.data) < nnz:
            raise IllegalArgumentException("colind/data shorter than rowptr[numRows]")
        h = C.c_void_p()
        _raise(self._lib.mtjg_csr_upload(self.ctx.h, self.n, self.m, L.iptr(self.rowptr), L.iptr(self.colind),
                                         L.dptr(self.data), C.byref(h)), "csr_upload")
        self.h = h

    @classmethod
    def fromDense(cls, A, ctx=None, keep_zeros_on_diagonal=True):
        A = np.asarray(A, dtype=np.float64)
        n, m = A.shape
        rows, cols, vals = [], [], []
        rp = [0]
        for i in range(n):
            for j in range(m):
                if A[i, j] != 0 or (keep_zeros_on_diagonal and i == j):
                    cols.append(j)
                    vals.append(A[i, j])
            rp.append(len(cols))
        return cls(n, m, np.array(rp), np.array(cols, dtype=np.int32), np.array(vals), ctx)

    @classmethod
    def fromMatrixMarket(cls, source, ctx=None):
        """new CompRowMatrix(new MatrixVectorReader(...)) (S/CompRowMatrix.java:86-166).

        ``source`` is a path, or the file's text as bytes.  The library reads
        and parses it and uploads the CSR (mtjg_csr_read_matrix_market /
        mtjg_csr_parse_matrix_market); the host arrays behind the getters
        are copied back from the device."""
        self = cls.__new__(cls)
        self.ctx = ctx or default_context()
        self._lib = self.ctx._lib
        h = C.c_void_p()
        if isinstance(source, (bytes, bytearray)):
            buf = bytes(source)
            _raise(self._lib.mtjg_csr_parse_matrix_market(self.ctx.h, buf, len(buf), C.byref(h)), "matrix market")
        else:
            _raise(self._lib.mtjg_csr_read_matrix_market(self.ctx.h, str(source).encode(), C.byref(h)),
                   "matrix market")
        self.h = h
        n, m, nnz = C.c_int(), C.c_int(), C.c_int64()
        _raise(self._lib.mtjg_csr_dims(h, C.byref(n), C.byref(m), C.byref(nnz)), "dims")
        self.n, self.m = n.value, m.value
        self.rowptr = np.empty(self.n + 1, dtype=np.int32)
        self.colind = np.empty(max(nnz.value, 1), dtype=np.int32)
        self.data = np.empty(max(nnz.value, 1))
        _raise(self._lib.mtjg_csr_to_host(h, L.iptr(self.rowptr), L.iptr(self.colind), L.dptr(self.data)), "to_host")
        self.colind, self.data = self.colind[:nnz.value], self.data[:nnz.value]
        return self

    @classmethod
    def _adopt(cls, ctx, h):
        self = cls.__new__(cls)
        self.ctx = ctx
        self._lib = ctx._lib
        self.h = h
        n, m, nnz = C.c_int(), C.c_int(), C.c_int64()
        _raise(self._lib.mtjg_csr_dims(h, C.byref(n), C.byref(m), C.byref(nnz)), "dims")
        self.n, self.m = n.value, m.value
        self.rowptr = np.empty(self.n + 1, dtype=np.int32)
        self.colind = np.empty(max(nnz.value, 1), dtype=np.int32)
        self.data = np.empty(max(nnz.value, 1))
        _raise(self._lib.mtjg_csr_to_host(h, L.iptr(self.rowptr), L.iptr(self.colind), L.dptr(self.data)), "to_host")
        self.colind, self.data = self.colind[:nnz.value], self.data[:nnz.value]
        return self

    @classmethod
    def fromCompColMatrix(cls, numRows, numColumns, colptr, rowind, data, ctx=None):
        """new CompRowMatrix(CompColMatrix A) (S/CompRowMatrix.java:210-243):
        A's CSC arrays, converted on the device (mtjg_csr_upload_csc)."""
        ctx = ctx or default_context()
        cp, ri, v = L.i32(colptr), L.i32(rowind), L.f64(data)
        h = C.c_void_p()
        _raise(ctx._lib.mtjg_csr_upload_csc(ctx.h, int(numRows), int(numColumns), L.iptr(cp), L.iptr(ri), L.dptr(v),
                                            C.byref(h)), "upload_csc")
        return cls._adopt(ctx, h)

    @classmethod
    def fromFlexCompRowMatrix(cls, numColumns, rows, ctx=None, slack=0):
        """new CompRowMatrix(FlexCompRowMatrix A) (S/CompRowMatrix.java:210-243):
        ``rows`` holds each row's SparseVector as (index, data) (sorted
        indices); they are laid out in one slab, each row's storage `slack`
        entries longer than its used part as a SparseVector's may be, and
        compacted on the device (mtjg_csr_upload_rows)."""
        ctx = ctx or default_context()
        n = len(rows)
        used = np.array([len(r[0]) for r in rows], dtype=np.int32)
        start = np.zeros(n, dtype=np.int64)
        if n:
            start[1:] = np.cumsum(used.astype(np.int64) + slack)[:-1]
        total = int(start[-1] + used[-1] + slack) if n else 0
        index = np.full(max(total, 1), -7, dtype=np.int32)
        data = np.full(max(total, 1), np.nan)
        for i, (ix, dv) in enumerate(rows):
            index[start[i]:start[i] + used[i]] = ix
            data[start[i]:start[i] + used[i]] = dv
        h = C.c_void_p()
        _raise(ctx._lib.mtjg_csr_upload_rows(ctx.h, n, int(numColumns), start.ctypes.data_as(C.POINTER(C.c_int64)),
                                             L.iptr(used), L.iptr(index), L.dptr(data), total, C.byref(h)),
               "upload_rows")
        return cls._adopt(ctx, h)

    def numRows(self):
        return self.n

    def numColumns(self):
        return self.m

    def isSquare(self):
        return self.n == self.m

    def getRowPointers(self):
        return self.rowptr

    def getColumnIndices(self):
        return self.colind

    def getData(self):
        return self.data

    def setData(self, data):
        """New values with the same pattern."""
        self.data = L.f64(data)
        _raise(self._lib.mtjg_csr_update_values(self.h, L.dptr(self.data)), "update_values")

    def _vec(self, v, size, name):
        v = L.f64(v)
        if v.shape != (size,):
            raise IndexOutOfBoundsException(f"{name}.size != {size}")
        return v

    def mult(self, x, y=None):
        """y = A x (S/CompRowMatrix.java:295-314)."""
        x = self._vec(x, self.m, "x")
        out = np.empty(self.n) if y is None else y
        _raise(self._lib.mtjg_csr_mult(self.h, L.dptr(x), L.dptr(out)), "mult")
        return out

    def multAdd(self, alpha, x, y):
        """y = alpha A x + y, in place (S/CompRowMatrix.java:330-347)."""
        x = self._vec(x, self.m, "x")
        if y.dtype != np.float64 or not y.flags.c_contiguous or y.shape != (self.n,):
            raise IllegalArgumentException("y must be a contiguous float64 vector of numRows")
        _raise(self._lib.mtjg_csr_mult_add(self.h, float(alpha), L.dptr(x), L.dptr(y)), "multAdd")
        return y

    def transMult(self, x, y=None):
        """y = A' x (S/CompRowMatrix.java:350-366)."""
        x = self._vec(x, self.n, "x")
        out = np.empty(self.m) if y is None else y
        _raise(self._lib.mtjg_csr_trans_mult(self.h, L.dptr(x), L.dptr(out)), "transMult")
        return out

    def transMultAdd(self, alpha, x, y):
        """y = alpha A' x + y, in place (S/CompRowMatrix.java:369-388)."""
        x = self._vec(x, self.n, "x")
        if y.dtype != np.float64 or not y.flags.c_contiguous or y.shape != (self.m,):
            raise IllegalArgumentException("y must be a contiguous float64 vector of numColumns")
        _raise(self._lib.mtjg_csr_trans_mult_add(self.h, float(alpha), L.dptr(x), L.dptr(y)), "transMultAdd")
        return y

    def close(self):
        if getattr(self, "h", None):
            self._lib.mtjg_csr_destroy(self.h)
            self.h = None

    def __del__(self):
        # at interpreter shutdown the process is about to release the device
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def parseMatrixMarket(text: bytes):
    """The CSR that CompRowMatrix(MatrixVectorReader) builds from Matrix
    Market text, parsed by the library on the host (no device needed):
    returns (numRows, numColumns, rowptr, colind, data)."""
    lib = L.load()
    text = bytes(text)
    n, m, nnz = C.c_int(), C.c_int(), C.c_int64()
    _raise(lib.mtjg_csr_parse_matrix_market_host(text, len(text), C.byref(n), C.byref(m), C.byref(nnz), None, None,
                                                 None, 0), "matrix market")
    rp = np.empty(n.value + 1, dtype=np.int32)
    ci = np.empty(max(nnz.value, 1), dtype=np.int32)
    v = np.empty(max(nnz.value, 1))
    _raise(lib.mtjg_csr_parse_matrix_market_host(text, len(text), C.byref(n), C.byref(m), C.byref(nnz), L.iptr(rp),
                                                 L.iptr(ci), L.dptr(v), nnz.value), "matrix market")
    return n.value, m.value, rp, ci[:nnz.value], v[:nnz.value]


def readVector(source):
    """new DenseVector(new MatrixVectorReader(...)) (M/DenseVector.java:52-96):
    a path or the text as bytes; returns a float64 numpy vector."""
    lib = L.load()
    size = C.c_int64()
    if isinstance(source, (bytes, bytearray)):
        buf = bytes(source)
        _raise(lib.mtjg_vector_parse_matrix_market(buf, len(buf), None, 0, C.byref(size)), "vector")
        out = np.empty(max(size.value, 1))
        _raise(lib.mtjg_vector_parse_matrix_market(buf, len(buf), L.dptr(out), size.value, C.byref(size)), "vector")
    else:
        path = str(source).encode()
        _raise(lib.mtjg_vector_read_matrix_market(path, None, 0, C.byref(size)), "vector")
        out = np.empty(max(size.value, 1))
        _raise(lib.mtjg_vector_read_matrix_market(path, L.dptr(out), size.value, C.byref(size)), "vector")
    return out[:size.value]


def block_diagonal(systems):
    """Concatenates CSR systems [(n, rowptr, colind, data), ...] into one
    block-diagonal CSR; returns (sys_rows, rowptr, colind, data)."""
    sizes = [int(s[0]) for s in systems]
    sys_rows = np.zeros(len(systems) + 1, dtype=np.int64)
    sys_rows[1:] = np.cumsum(sizes)
    nnzs = [int(s[1][-1]) for s in systems]
    nz_off = np.zeros(len(systems) + 1, dtype=np.int64)
    nz_off[1:] = np.cumsum(nnzs)
    if sys_rows[-1] >= 2 ** 31 or nz_off[-1] >= 2 ** 31:
        raise IllegalArgumentException("batch exceeds 32-bit row or entry indices")
    rowptr = np.empty(int(sys_rows[-1]) + 1, dtype=np.int32)
    colind = np.empty(int(nz_off[-1]), dtype=np.int32)
    data = np.empty(int(nz_off[-1]), dtype=np.float64)
    for k, (n, rp, ci, v) in enumerate(systems):
        r0, z0 = int(sys_rows[k]), int(nz_off[k])
        rowptr[r0:r0 + n] = np.asarray(rp[:n], dtype=np.int64) + z0
        colind[z0:z0 + nnzs[k]] = np.asarray(ci[:nnzs[k]], dtype=np.int64) + r0
        data[z0:z0 + nnzs[k]] = v[:nnzs[k]]
    rowptr[-1] = int(nz_off[-1])
    return sys_rows.astype(np.int32), rowptr, colind, data


class BatchCompRowMatrix(CompRowMatrix):
    """A batch of independent square systems held as one block-diagonal CSR
    on the device (mtjg_batch_upload).  A CG or BiCGstab solver of the total
    size solves all systems in the same launches; ``solveBatch`` returns each
    system's outcome.  No counterpart in the reference, which solves one
    system per call."""

    def __init__(self, systems, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self._lib = self.ctx._lib
        self.sys_rows, self.rowptr, self.colind, self.data = block_diagonal(systems)
        self.n = self.m = int(self.sys_rows[-1])
        h = C.c_void_p()
        _raise(self._lib.mtjg_batch_upload(self.ctx.h, len(systems), L.iptr(self.sys_rows), L.iptr(self.rowptr),
                                           L.iptr(self.colind), L.dptr(self.data), C.byref(h)), "batch_upload")
        self.h = h

    def numSystems(self):
        return len(self.sys_rows) - 1

    def systemRows(self, s):
        return int(self.sys_rows[s]), int(self.sys_rows[s + 1])


# -------------------------------------------------------- preconditioners
class Preconditioner:
    """S/Preconditioner.java: setMatrix(A), apply(b, x), transApply(b, x)."""

    kind = L.PC_IDENTITY

    def __init__(self, n: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self._lib = self.ctx._lib
        self.n = int(n)
        h = C.c_void_p()
        _raise(self._lib.mtjg_precond_create(self.ctx.h, self.kind, self.n, C.byref(h)), "precond_create")
        self.h = h
        self.error_row = 0

    def setMatrix(self, A: CompRowMatrix):
        row = C.c_int(0)
        code = self._lib.mtjg_precond_set_matrix(self.h, A.h, C.byref(row))
        self.error_row = row.value
        _raise(code, "setMatrix")

    def apply(self, b, x=None):
        b = L.f64(b)
        out = np.empty(self.n) if x is None else x
        _raise(self._lib.mtjg_precond_apply(self.h, L.dptr(b), L.dptr(out)), "apply")
        return out

    def transApply(self, b, x=None):
        b = L.f64(b)
        out = np.empty(self.n) if x is None else x
        _raise(self._lib.mtjg_precond_trans_apply(self.h, L.dptr(b), L.dptr(out)), "transApply")
        return out

    def values(self) -> np.ndarray:
        """The factored values (ILU/ICC data array; Jacobi inverse diagonal)."""
        ln = C.c_int64(0)
        _raise(self._lib.mtjg_precond_values(self.h, None, 0, C.byref(ln)), "values")
        out = np.empty(ln.value)
        if ln.value:
            _raise(self._lib.mtjg_precond_values(self.h, L.dptr(out), ln.value, C.byref(ln)), "values")
        return out

    def pattern(self):
        """(rowptr, colind, diag) of the factor, in the layout of values();
        diag holds each row's diagonal position within the row."""
        nnz = C.c_int64(0)
        _raise(self._lib.mtjg_precond_pattern(self.h, None, None, None, 0, C.byref(nnz)), "pattern")
        rp = np.empty(self.n + 1, dtype=np.int32)
        ci = np.empty(max(nnz.value, 1), dtype=np.int32)
        dg = np.empty(max(self.n, 1), dtype=np.int32)
        _raise(self._lib.mtjg_precond_pattern(self.h, L.iptr(rp), L.iptr(ci), L.iptr(dg), nnz.value, C.byref(nnz)),
               "pattern")
        return rp, ci[:nnz.value], dg[:self.n]

    def close(self):
        if getattr(self, "h", None):
            self._lib.mtjg_precond_destroy(self.h)
            self.h = None

    def __del__(self):
        # at interpreter shutdown the process is about to release the device
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class IdentityPreconditioner(Preconditioner):
    kind = L.PC_IDENTITY


class DiagonalPreconditioner(Preconditioner):
    """new DiagonalPreconditioner(n) (S/DiagonalPreconditioner.java:43-45)."""

    kind = L.PC_JACOBI


class ILU(Preconditioner):
    """new ILU(CompRowMatrix LU) (S/ILU.java:54-62): LU gives the size."""

    kind = L.PC_ILU

    def __init__(self, LU, ctx=None):
        n = LU.numRows() if hasattr(LU, "numRows") else int(LU)
        if hasattr(LU, "isSquare") and not LU.isSquare():
            raise IllegalArgumentException("ILU only applies to square matrices")
        super().__init__(n, ctx or getattr(LU, "ctx", None))


class SSOR(Preconditioner):
    """new SSOR(CompRowMatrix F, reverse, omegaF, omegaR) (S/SSOR.java:62-77).
    apply(b, x) is one symmetric SOR sweep starting from x's content, as in
    MTJ (S/SSOR.java:148-192): pass the x to start from (zeros when None)."""

    kind = L.PC_SSOR

    def __init__(self, F, reverse=True, omegaF=1.0, omegaR=1.0, ctx=None):
        n = F.numRows() if hasattr(F, "numRows") else int(F)
        if hasattr(F, "isSquare") and not F.isSquare():
            raise IllegalArgumentException("SSOR only applies to square matrices")
        super().__init__(n, ctx or getattr(F, "ctx", None))
        self.reverse = bool(reverse)
        self.setOmega(omegaF, omegaR)

    def setOmega(self, omegaF, omegaR):
        """SSOR.setOmega, S/SSOR.java:87-96."""
        _raise(self._lib.mtjg_precond_set_ssor(self.h, 1 if self.reverse else 0, float(omegaF), float(omegaR)),
               "setOmega")
        self.omegaF, self.omegaR = float(omegaF), float(omegaR)

    def apply(self, b, x=None):
        out = np.zeros(self.n) if x is None else x
        return super().apply(b, out)

    def transApply(self, b, x=None):
        out = np.zeros(self.n) if x is None else x
        return super().transApply(b, out)


class ILUT(Preconditioner):
    """new ILUT(FlexCompRowMatrix LU, tau, p) (S/ILUT.java:68-97); LU gives the
    size (a CompRowMatrix or the row count)."""

    kind = L.PC_ILUT

    def __init__(self, LU, tau=1e-6, p=25, ctx=None):
        n = LU.numRows() if hasattr(LU, "numRows") else int(LU)
        if hasattr(LU, "isSquare") and not LU.isSquare():
            raise IllegalArgumentException("ILU only applies to square matrices")
        super().__init__(n, ctx or getattr(LU, "ctx", None))
        _raise(self._lib.mtjg_precond_set_ilut(self.h, float(tau), int(p)), "ILUT")
        self.tau, self.p = float(tau), int(p)


class ICC(Preconditioner):
    """new ICC(CompRowMatrix R) (S/ICC.java:57-65)."""

    kind = L.PC_ICC

    def __init__(self, R, ctx=None):
        n = R.numRows() if hasattr(R, "numRows") else int(R)
        if hasattr(R, "isSquare") and not R.isSquare():
            raise IllegalArgumentException("ICC only applies to square matrices")
        super().__init__(n, ctx or getattr(R, "ctx", None))


# --------------------------------------------------------------- monitor
class Norm(enum.IntEnum):  # M/Vector.java:159-182
    One = L.NORM_ONE
    Two = L.NORM_TWO
    TwoRobust = L.NORM_TWO_ROBUST
    Infinity = L.NORM_INFINITY


class IterationReporter:
    """S/IterationReporter.java: monitor(r, i) per convergence test."""

    def monitor(self, r, i):
        pass


class DefaultIterationMonitor:
    """S/DefaultIterationMonitor.java (defaults 100000, 1e-5, 1e-50, 1e+5).

    The reporter is replayed after the solve from the residual history that
    the device records at every convergence test; per-iteration x is not
    available to it.
    """

    def __init__(self, maxIter=100000, rtol=1e-5, atol=1e-50, dtol=1e+5):
        self.maxIter, self.rtol, self.atol, self.dtol = int(maxIter), float(rtol), float(atol), float(dtol)
        self.normType = Norm.Two
        self.reporter = None
        self.history_cap = 0
        self._iter = 0
        self._residual = 0.0

    def setMaxIterations(self, m):
        self.maxIter = int(m)

    def setRelativeTolerance(self, r):
        self.rtol = float(r)

    def setAbsoluteTolerance(self, a):
        self.atol = float(a)

    def setDivergenceTolerance(self, d):
        self.dtol = float(d)

    def setNormType(self, t):
        self.normType = Norm(t)

    def getNormType(self):
        return self.normType

    def setIterationReporter(self, reporter, history_cap=None):
        self.reporter = reporter
        if history_cap is None:
            history_cap = self.maxIter * 2 + 64
        self.history_cap = int(history_cap)

    def getIterationReporter(self):
        return self.reporter

    def iterations(self):
        return self._iter

    def residual(self):
        return self._residual

    def _struct(self) -> L.Monitor:
        return L.Monitor(self.maxIter, self.rtol, self.atol, self.dtol, int(self.normType), self.history_cap)

    def _matrix_norms(self):
        return None


class MatrixIterationMonitor(DefaultIterationMonitor):
    """S/MatrixIterationMonitor.java: converged iff r < max(rtol (normA |x|
    + normb), atol), |x| the current iterate's norm in the monitor's norm
    type (formed on the device before each test).  GMRES's inner test is
    converged(double), which this monitor does not support: such a solve
    raises UnsupportedOperationException, as in MTJ."""

    def __init__(self, normA, normb, maxIter=100000, rtol=1e-5, atol=1e-50, dtol=1e+5):
        super().__init__(maxIter, rtol, atol, dtol)
        self.normA, self.normb = float(normA), float(normb)

    def setMatrixNorm(self, normA):
        self.normA = float(normA)

    def setVectorNorm(self, normb):
        self.normb = float(normb)

    def _matrix_norms(self):
        return (self.normA, self.normb)


# --------------------------------------------------------------- solvers
class AbstractIterativeSolver:
    """S/AbstractIterativeSolver.java: identity preconditioner and default
    monitor until set."""

    kind = L.CG

    def __init__(self, template, restart=0, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self._lib = self.ctx._lib
        self.n = len(template) if not isinstance(template, int) else template
        h = C.c_void_p()
        _raise(self._lib.mtjg_solver_create(self.ctx.h, self.kind, self.n, restart, C.byref(h)), "solver_create")
        self.h = h
        self.M = IdentityPreconditioner(self.n, self.ctx)
        self.iter = DefaultIterationMonitor()
        self._mon_key = None
        self.history = (np.empty(0), np.empty(0, dtype=np.int32))

    def setPreconditioner(self, M: Preconditioner):
        self.M = M
        _raise(self._lib.mtjg_solver_set_precond(self.h, M.h), "set_precond")

    def getPreconditioner(self):
        return self.M

    def setIterationMonitor(self, mon: DefaultIterationMonitor):
        # the monitor runs on the device: MTJ's two monitors only
        if not isinstance(mon, DefaultIterationMonitor):
            raise UnsupportedOperationException("only DefaultIterationMonitor and MatrixIterationMonitor run on the GPU")
        self.iter = mon

    def getIterationMonitor(self):
        return self.iter

    def setMixedPrecision(self, enable=True, inner_rtol=1e-4, inner_max_iter=1000):
        """FP32 inner solves inside FP64 iterative refinement
        (mtjg_solver_set_mixed): CG (identity or Jacobi), GMRES and BiCGstab
        (identity, Jacobi, ILU or ILUT).  iterations() then counts refinement
        steps and innerIterations() the FP32 iterations."""
        _raise(self._lib.mtjg_solver_set_mixed(self.h, 1 if enable else 0, float(inner_rtol), int(inner_max_iter)),
               "set_mixed")

    def setGraphLaunch(self, enable=True):
        """Run every iteration as graph-captured phase launches
        (mtjg_solver_set_launch MTJG_LAUNCH_GRAPH), also where a small CG
        solve would otherwise run its loop in one launch; enable=False
        restores the default.  The results are the same either way."""
        _raise(self._lib.mtjg_solver_set_launch(self.h, 1 if enable else 0), "set_launch")

    def innerIterations(self):
        r = getattr(self, "last_result", None)
        return r.inner_iterations if r is not None else 0

    def _sync_monitor(self):
        s = self.iter._struct()
        mn = self.iter._matrix_norms()
        key = (s.max_iter, s.rtol, s.atol, s.dtol, s.norm, s.history_cap, mn)
        if key != self._mon_key:
            _raise(self._lib.mtjg_solver_set_monitor(self.h, C.byref(s)), "set_monitor")
            _raise(self._lib.mtjg_solver_set_matrix_monitor(self.h, 1 if mn else 0, *(mn or (0.0, 0.0))),
                   "set_matrix_monitor")
            self._mon_key = key

    def solve(self, A: CompRowMatrix, b, x):
        """IterativeSolver.solve(A, b, x) (S/IterativeSolver.java:30-44)."""
        if not A.isSquare():
            raise IllegalArgumentException("!A.isSquare()")
        b = L.f64(b)
        if b.shape != (A.numRows(),):
            raise IllegalArgumentException("b.size() != A.numRows()")
        if not isinstance(x, np.ndarray) or x.dtype != np.float64 or not x.flags.c_contiguous:
            raise IllegalArgumentException("x must be a contiguous float64 numpy vector")
        if x.shape != b.shape:
            raise IllegalArgumentException("b.size() != x.size()")
        self._sync_monitor()
        res = L.Result()
        code = self._lib.mtjg_solver_solve(self.h, A.h, L.dptr(b), L.dptr(x), C.byref(res))
        self.iter._iter = res.iterations
        self.iter._residual = res.residual
        self.last_result = res
        self._replay()
        if code in (L.NOT_CONVERGED_ITERATIONS, L.NOT_CONVERGED_DIVERGENCE, L.NOT_CONVERGED_BREAKDOWN):
            reason = NotConvergedException.Reason(code)
            msg = BREAKDOWN.get(res.detail, "") if code == L.NOT_CONVERGED_BREAKDOWN else ""
            raise IterativeSolverNotConvergedException(reason, res.residual, res.iterations, msg)
        _raise(code, "solve")
        return x

    def solveBatch(self, A: BatchCompRowMatrix, b, x):
        """Solves every system of a batch; x is overwritten in place.  Returns
        one (status, iterations, residual) per system and raises only for
        errors that are not a system's own convergence failure."""
        b = L.f64(b)
        if b.shape != (A.numRows(),) or x.shape != b.shape or x.dtype != np.float64 or not x.flags.c_contiguous:
            raise IllegalArgumentException("b and x must be float64 vectors of the batch's total size")
        self._sync_monitor()
        res = L.Result()
        code = self._lib.mtjg_solver_solve(self.h, A.h, L.dptr(b), L.dptr(x), C.byref(res))
        if code not in (L.OK, L.NOT_CONVERGED_ITERATIONS, L.NOT_CONVERGED_DIVERGENCE, L.NOT_CONVERGED_BREAKDOWN):
            _raise(code, "solveBatch")
        ns = A.numSystems()
        out = (L.Result * ns)()
        _raise(self._lib.mtjg_solver_batch_results(self.h, out, ns), "batch_results")
        return [(r.status, r.iterations, r.residual) for r in out]

    def batchHistory(self, s):
        cap = self.iter.history_cap
        r = np.empty(max(cap, 1))
        it = np.empty(max(cap, 1), dtype=np.int32)
        ln = C.c_int(0)
        _raise(self._lib.mtjg_solver_batch_history(self.h, s, L.dptr(r), L.iptr(it), cap, C.byref(ln)), "history")
        return r[: ln.value].copy(), it[: ln.value].copy()

    def _replay(self):
        cap = self.iter.history_cap
        if cap <= 0:
            self.history = (np.empty(0), np.empty(0, dtype=np.int32))
            return
        r = np.empty(cap)
        it = np.empty(cap, dtype=np.int32)
        ln = C.c_int(0)
        _raise(self._lib.mtjg_solver_history(self.h, L.dptr(r), L.iptr(it), cap, C.byref(ln)), "history")
        self.history = (r[: ln.value].copy(), it[: ln.value].copy())
        if self.iter.reporter is not None:
            for rv, iv in zip(*self.history):
                self.iter.reporter.monitor(float(rv), int(iv))

    def close(self):
        if getattr(self, "h", None):
            self._lib.mtjg_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        # at interpreter shutdown the process is about to release the device
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


class CG(AbstractIterativeSolver):
    """S/CG.java"""

    kind = L.CG


class BiCGstab(AbstractIterativeSolver):
    """S/BiCGstab.java"""

    kind = L.BICGSTAB


class BiCG(AbstractIterativeSolver):
    """S/BiCG.java (uses M.transApply and A.transMult)."""

    kind = L.BICG


class CGS(AbstractIterativeSolver):
    """S/CGS.java"""

    kind = L.CGS


class QMR(AbstractIterativeSolver):
    """S/QMR.java with M1 = M2 = the solver's preconditioner (QMR(Vector),
    :65-80; setPreconditioner, :216-220)."""

    kind = L.QMR


class IR(AbstractIterativeSolver):
    """S/IR.java (Richardson iteration with the preconditioner)."""

    kind = L.IR


class Chebyshev(AbstractIterativeSolver):
    """S/Chebyshev.java: new Chebyshev(template, eigmin, eigmax)."""

    kind = L.CHEBYSHEV

    def __init__(self, template, eigmin, eigmax, ctx=None):
        super().__init__(template, 0, ctx)
        self.setEigenvalues(eigmin, eigmax)

    def setEigenvalues(self, eigmin, eigmax):
        """Chebyshev.setEigenvalues, S/Chebyshev.java:78-88."""
        _raise(self._lib.mtjg_solver_set_eigenvalues(self.h, float(eigmin), float(eigmax)), "setEigenvalues")
        self.eigmin, self.eigmax = float(eigmin), float(eigmax)


class GMRES(AbstractIterativeSolver):
    """S/GMRES.java; restart defaults to 30 (:84-86)."""

    kind = L.GMRES

    def __init__(self, template, restart=30, ctx=None):
        if restart <= 0:
            raise IllegalArgumentException("restart must be a positive integer")
        super().__init__(template, restart, ctx)
        self.restart = restart
