/*
 * mtjg.h -- C ABI of the GB300 preconditioned Krylov library.
 *
 * Drop-in for the sparse iterative path of MTJ (no.uib.cipr.matrix.sparse):
 * CompRowMatrix's products, the CG / BiCGstab / GMRES(m) solvers, the
 * Jacobi / ILU(0) / ICC preconditioners and DefaultIterationMonitor.  Each
 * declaration names the reference method it replaces (file:line inside the
 * reference project; S/ = src/main/java/no/uib/cipr/matrix/sparse/,
 * M/ = src/main/java/no/uib/cipr/matrix/).
 *
 * Conventions
 *  - Every function returns an int status: MTJG_OK (0) or a code below.
 *    Nothing throws.  mtjg_last_error() gives the message of the calling
 *    thread's last failure.  The codes map one to one onto the exceptions
 *    the reference throws.
 *  - CSR is MTJ's: 0-based int32 row pointers and column indices, column
 *    indices ascending inside each row, float64 values.
 *  - Host pointers are borrowed for the duration of the call only.  "_dev"
 *    variants take device pointers that stay valid until the call returns.
 *  - Handles are not thread-safe (as the Java objects are not): one thread
 *    per context, or an external lock.  All work of a context runs in order
 *    on that context's CUDA stream.
 */
#ifndef MTJG_H
#define MTJG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MTJG_API __attribute__((visibility("default")))
#else
#define MTJG_API
#endif

/* ---- status codes ---------------------------------------------------- */
enum {
    MTJG_OK = 0,
    /* IterativeSolverNotConvergedException(Reason.*), S/IterativeSolverNotConvergedException.java:29-91,
     * reasons M/NotConvergedException.java:33-49 */
    MTJG_NOT_CONVERGED_ITERATIONS = 1,
    MTJG_NOT_CONVERGED_DIVERGENCE = 2,
    MTJG_NOT_CONVERGED_BREAKDOWN = 3,
    /* IllegalArgumentException (sizes, S/AbstractIterativeSolver.java:70-77) */
    MTJG_ERR_ILLEGAL_ARGUMENT = 10,
    /* IndexOutOfBoundsException (M/AbstractMatrix.java:170-177) */
    MTJG_ERR_INDEX_OUT_OF_BOUNDS = 11,
    /* java.io.IOException / EOFException / NumberFormatException while reading
     * Matrix Market text (M/io/MatrixVectorReader.java) */
    MTJG_ERR_IO = 12,
    /* RuntimeException("Zero pivot encountered on row ..."), S/ILU.java:105-107, S/ICC.java:112-114 */
    MTJG_ERR_ZERO_PIVOT = 20,
    /* "Zero diagonal entry encountered on row ..." S/ICC.java:128-131,
     * "Zero diagonal on row ..." S/DiagonalPreconditioner.java:71-72 */
    MTJG_ERR_ZERO_DIAGONAL = 21,
    /* "Missing diagonal entry on row ..." S/ILU.java:134-136, S/ICC.java:148-150 */
    MTJG_ERR_MISSING_DIAGONAL = 22,
    /* MatrixSingularException from GMRES's triangular solve, M/AbstractTriangDenseMatrix.java:251-252 */
    MTJG_ERR_SINGULAR = 23,
    MTJG_ERR_UNSUPPORTED = 30,
    MTJG_ERR_CUDA = 40,
    MTJG_ERR_OUT_OF_MEMORY = 41,
    /* a bounded wait on the device gave up; the context stays usable */
    MTJG_ERR_DEVICE_TIMEOUT = 42
};

/* Vector.Norm, M/Vector.java:159-182 */
enum { MTJG_NORM_ONE = 0, MTJG_NORM_TWO = 1, MTJG_NORM_TWO_ROBUST = 2, MTJG_NORM_INFINITY = 3 };

/* Preconditioner kinds: identity (S/AbstractIterativeSolver.java:82-96),
 * DiagonalPreconditioner, ILU, ICC, SSOR, ILUT */
enum { MTJG_PC_IDENTITY = 0, MTJG_PC_JACOBI = 1, MTJG_PC_ILU = 2, MTJG_PC_ICC = 3, MTJG_PC_SSOR = 4, MTJG_PC_ILUT = 5 };

/* IterativeSolver implementations: S/CG.java, S/BiCGstab.java, S/GMRES.java,
 * S/BiCG.java, S/CGS.java, S/QMR.java, S/Chebyshev.java, S/IR.java */
enum {
    MTJG_CG = 0, MTJG_BICGSTAB = 1, MTJG_GMRES = 2, MTJG_BICG = 3, MTJG_CGS = 4, MTJG_QMR = 5,
    MTJG_CHEBYSHEV = 6, MTJG_IR = 7
};

/* Arithmetic of the products and vector updates.  FAST uses fused
 * multiply-add.  STRICT rounds every product and sum separately, as Java
 * does, which makes CSR products bit-identical to CompRowMatrix.mult; only
 * the order of the dot-product and norm reductions then differs from MTJ. */
enum { MTJG_NUMERICS_FAST = 0, MTJG_NUMERICS_STRICT = 1 };

/* DefaultIterationMonitor(maxIter, rtol, atol, dtol), S/DefaultIterationMonitor.java:72-90,
 * with the norm of AbstractIterationMonitor.setNormType (S/AbstractIterationMonitor.java:110-112).
 * history_cap > 0 records the residual and the iteration number passed to
 * IterationReporter.monitor at every convergence test (S/AbstractIterationMonitor.java:81-93). */
typedef struct mtjg_monitor {
    int max_iter;      /* default 100000 */
    double rtol;       /* default 1e-5   */
    double atol;       /* default 1e-50  */
    double dtol;       /* default 1e+5   */
    int norm;          /* default MTJG_NORM_TWO */
    int history_cap;   /* 0: no history */
} mtjg_monitor;

/* Outcome of a solve: IterationMonitor.iterations()/residual() at exit and
 * the exception reason, if any.  detail names the quantity of a breakdown:
 * 1 "rho", 2 "omega" (S/BiCGstab.java:77-83), 3 "xi", 4 "delta", 5 "ep",
 * 6 "beta", 7 "gamma" (S/QMR.java:134-195). */
typedef struct mtjg_result {
    int status;
    int iterations;
    double residual;
    int detail;
    int history_len;   /* convergence tests made (may exceed history_cap) */
    int inner_iterations;  /* mixed precision: FP32 inner iterations of all refinement steps */
} mtjg_result;

typedef struct mtjg_ctx mtjg_ctx;
typedef struct mtjg_csr mtjg_csr;
typedef struct mtjg_precond mtjg_precond;
typedef struct mtjg_solver mtjg_solver;

/* ---- library and context --------------------------------------------- */
MTJG_API const char *mtjg_last_error(void);
MTJG_API const char *mtjg_version(void);
/* Default DefaultIterationMonitor settings (S/DefaultIterationMonitor.java:85-90). */
MTJG_API void mtjg_monitor_defaults(mtjg_monitor *mon);

/* A context owns one CUDA device and one stream. */
MTJG_API int mtjg_ctx_create(int device, mtjg_ctx **out);
MTJG_API int mtjg_ctx_destroy(mtjg_ctx *ctx);
MTJG_API int mtjg_ctx_set_numerics(mtjg_ctx *ctx, int numerics);
MTJG_API int mtjg_ctx_synchronize(mtjg_ctx *ctx);
/* Number of this library's kernel launches on the context so far. */
MTJG_API int64_t mtjg_ctx_launch_count(mtjg_ctx *ctx);
/* CUDA events on the context's stream, for timing: record into slot 0..15,
 * elapsed milliseconds between two recorded slots (synchronizes on b). */
MTJG_API int mtjg_ctx_event_record(mtjg_ctx *ctx, int slot);
MTJG_API int mtjg_ctx_event_elapsed(mtjg_ctx *ctx, int a, int b, float *ms);
/* Device memory of `bytes` bytes on ctx's device (cudaMalloc), for callers
 * that keep vectors on the GPU; copies below are ordered on ctx's stream and
 * return when done. */
MTJG_API int mtjg_dev_alloc(mtjg_ctx *ctx, int64_t bytes, void **dptr);
MTJG_API int mtjg_dev_free(mtjg_ctx *ctx, void *dptr);
MTJG_API int mtjg_memcpy_h2d(mtjg_ctx *ctx, void *dst, const void *src, int64_t bytes);
MTJG_API int mtjg_memcpy_d2h(mtjg_ctx *ctx, void *dst, const void *src, int64_t bytes);

/* ---- CompRowMatrix ----------------------------------------------------- */
/* CompRowMatrix(numRows, numColumns, nz) + data, S/CompRowMatrix.java:178-208:
 * copies the CSR to the device.  Rejects unsorted or out-of-range column
 * indices (S/CompRowMatrix.java:200-203) with MTJG_ERR_ILLEGAL_ARGUMENT. */
MTJG_API int mtjg_csr_upload(mtjg_ctx *ctx, int num_rows, int num_cols,
                             const int *rowptr, const int *colind, const double *val,
                             mtjg_csr **out);
/* A batch of independent square systems as one block-diagonal CSR: system s
 * owns rows [sys_rows[s], sys_rows[s+1]) and references only columns in that
 * range (checked).  Solving it with a CG or BiCGstab solver of size
 * sys_rows[num_systems] runs every system in the same launches, each with
 * its own scalars and DefaultIterationMonitor; a system's results do not
 * depend on the other systems of the batch (they equal a batch of that one
 * system; a batch groups its dot products in larger blocks than a lone
 * mtjg_csr_upload, so results differ from that by rounding).  No reference counterpart: MTJ
 * solves one system per call (IterativeSolver.solve, S/IterativeSolver.java:30-44). */
MTJG_API int mtjg_batch_upload(mtjg_ctx *ctx, int num_systems, const int *sys_rows, const int *rowptr,
                               const int *colind, const double *val, mtjg_csr **out);
/* new CompRowMatrix(new MatrixVectorReader(reader)), S/CompRowMatrix.java:86-166:
 * reads a Matrix Market file (or text of `len` bytes) and uploads it as a
 * device CSR.  Coordinate real or integer, general / symmetric /
 * skew-symmetric (mirrored entries added after the file's own; the last
 * value assigned to a position wins, as CompRowMatrix.set overwrites).
 * Pattern, array (dense) and complex files are MTJG_ERR_UNSUPPORTED, as in
 * MTJ; malformed text MTJG_ERR_IO; an entry on a row outside the matrix
 * MTJG_ERR_INDEX_OUT_OF_BOUNDS, on a column outside it
 * MTJG_ERR_ILLEGAL_ARGUMENT.  Without a "%%MatrixMarket" first line the text
 * is coordinate real general (M/io/MatrixVectorReader.java:122-240). */
MTJG_API int mtjg_csr_read_matrix_market(mtjg_ctx *ctx, const char *path, mtjg_csr **out);
MTJG_API int mtjg_csr_parse_matrix_market(mtjg_ctx *ctx, const char *text, int64_t len, mtjg_csr **out);
/* The same parse into host arrays, without a device: call with NULL arrays
 * to learn the sizes, then with rowptr[num_rows + 1] and colind / val of
 * `cap` >= nnz entries. */
MTJG_API int mtjg_csr_parse_matrix_market_host(const char *text, int64_t len, int *num_rows, int *num_cols,
                                               int64_t *nnz, int *rowptr, int *colind, double *val, int64_t cap);
/* new DenseVector(new MatrixVectorReader(reader)), M/DenseVector.java:52-96:
 * coordinate or array, real or integer; *size receives the vector's size and
 * the first min(cap, size) entries go to out. */
MTJG_API int mtjg_vector_read_matrix_market(const char *path, double *out, int64_t cap, int64_t *size);
MTJG_API int mtjg_vector_parse_matrix_market(const char *text, int64_t len, double *out, int64_t cap,
                                             int64_t *size);
/* CompRowMatrix.getRowPointers / getColumnIndices / getData
 * (S/CompRowMatrix.java:255-271): the device CSR copied to host arrays of
 * num_rows + 1 and nnz entries (any of them may be NULL). */
MTJG_API int mtjg_csr_to_host(const mtjg_csr *A, int *rowptr, int *colind, double *val);
/* new CompRowMatrix(A) for a CompColMatrix A (S/CompRowMatrix.java:210-243,
 * S/CompColMatrix.java:190-215): 0-based column pointers and row indices
 * (strictly ascending within a column), converted to the device CSR on the
 * device.  The result is a CompRowMatrix: its products round as
 * CompRowMatrix's do. */
MTJG_API int mtjg_csr_upload_csc(mtjg_ctx *ctx, int num_rows, int num_cols, const int *colptr, const int *rowind,
                                 const double *val, mtjg_csr **out);
/* new CompRowMatrix(A) for a FlexCompRowMatrix A (S/CompRowMatrix.java:210-243,
 * S/FlexCompRowMatrix.java): its rows' SparseVector storage in one slab of
 * `slab` entries -- row i's indices (strictly ascending, in [0, num_cols))
 * and values at [row_start[i], row_start[i] + row_used[i]) -- compacted into
 * the device CSR on the device. */
MTJG_API int mtjg_csr_upload_rows(mtjg_ctx *ctx, int num_rows, int num_cols, const int64_t *row_start,
                                  const int *row_used, const int *index, const double *data, int64_t slab,
                                  mtjg_csr **out);
/* The lanes per row the batch autotuner chose for systems of `rows` rows and
 * `nnz` entries (its class: bands of rows and of entries per row); 0 while
 * no batch of that class has been solved.  A batch from mtjg_batch_upload
 * solved by CG with the identity or Jacobi preconditioner (FP64 or mixed)
 * runs as one persistent launch: each CTA takes whole systems, largest
 * first, and runs their CG to the end.  On the first batch holding a class,
 * short probe solves time each lanes-per-row candidate; the fastest is kept
 * for the process (MTJG_TUNE=0 in the environment: the entries-per-row rule
 * instead).  No counterpart in the reference. */
MTJG_API int mtjg_batch_tuning(int64_t rows, int64_t nnz, int *lanes_per_row);
/* New values, same pattern (CompRowMatrix.set on the data array). */
MTJG_API int mtjg_csr_update_values(mtjg_csr *A, const double *val);
MTJG_API int mtjg_csr_destroy(mtjg_csr *A);
MTJG_API int mtjg_csr_dims(const mtjg_csr *A, int *num_rows, int *num_cols, int64_t *nnz);

/* CompRowMatrix.mult(Vector x, Vector y): y = A x, S/CompRowMatrix.java:295-314 */
MTJG_API int mtjg_csr_mult(mtjg_csr *A, const double *x, double *y);
/* CompRowMatrix.multAdd(alpha, x, y): y += alpha A x, S/CompRowMatrix.java:330-347 */
MTJG_API int mtjg_csr_mult_add(mtjg_csr *A, double alpha, const double *x, double *y);
/* CompRowMatrix.transMult(x, y): y = A' x, S/CompRowMatrix.java:350-366 */
MTJG_API int mtjg_csr_trans_mult(mtjg_csr *A, const double *x, double *y);
/* CompRowMatrix.transMultAdd(alpha, x, y): y = alpha A' x + y, S/CompRowMatrix.java:369-388 */
MTJG_API int mtjg_csr_trans_mult_add(mtjg_csr *A, double alpha, const double *x, double *y);
/* Device-pointer forms of mult / multAdd / transMult (no host copies). */
MTJG_API int mtjg_csr_mult_dev(mtjg_csr *A, const double *dx, double *dy);
MTJG_API int mtjg_csr_mult_add_dev(mtjg_csr *A, double alpha, const double *dx, double *dy);
MTJG_API int mtjg_csr_trans_mult_dev(mtjg_csr *A, const double *dx, double *dy);

/* y = alpha A x + y (as mtjg_csr_mult_add_dev) and the two-norm of the new y,
 * written to dnorm[0] -- one norm per system, dnorm[s], for a batch from
 * mtjg_batch_upload.  All pointers are device pointers; the call is
 * asynchronous on A's context stream.  With alpha = -1 and y = b it is the
 * residual step r = b - A x, |r| of an iterative refinement loop.  No
 * counterpart in the reference.
 *
 * This call allocates nothing: its reduction scratch is a fixed 512 KB array
 * in the library's device image.  It is for callers that may not allocate
 * device memory once set up: hosts whose device memory is a fixed arena
 * handed out at start-up (a JVM off-heap pool, a serving process with a
 * memory budget), and loops that cannot afford cudaMalloc/cudaFree, which may
 * synchronise the device.
 *   - Limit: A's product tiling may have at most 16384 reduction groups.  A
 *     group is at most 8 product tiles of at most 1152 entries, so one system
 *     fits up to about 16384 * 8 * 1152 = 151 million entries (about 21
 *     million rows at 7 entries per row); a batch fits at most 16384
 *     systems.  Larger A gives MTJG_ERR_ILLEGAL_ARGUMENT.
 *   - Nothing has to start at zero: partials are written before they are read
 *     within the call, and each norm is stored, not accumulated.
 *   - In FAST numerics, rows longer than a product stage (1152 entries) are
 *     summed ahead into scratch that belongs to A (allocated when A was
 *     uploaded, not by this call); overlapping calls on one A race there too.
 *   - The scratch is one array per device, shared by all contexts and threads:
 *     calls that overlap on one device (two streams, contexts or threads)
 *     race and return wrong norms.  Calls in order on one stream are safe.
 *   - The first call on each device looks the scratch's address up once
 *     (with that device current).  A caller that captures streams makes one
 *     call before capture begins, so this set-up is not inside a capture.
 *   - cudaDeviceReset by the host ends every handle of this library on that
 *     device, this entry's saved scratch address included: make new handles
 *     (and so a new first call) after a reset. */
MTJG_API int mtjg_csr_mult_add_norm_noalloc(mtjg_csr *A, double alpha, const double *dx, double *dy,
                                            double *dnorm);

/* ---- Preconditioner ---------------------------------------------------- */
/* new DiagonalPreconditioner(n) / new ILU(CompRowMatrix) / new ICC(CompRowMatrix) /
 * new SSOR(CompRowMatrix) / new ILUT(FlexCompRowMatrix),
 * S/DiagonalPreconditioner.java:43-45, S/ILU.java:54-62, S/ICC.java:57-65,
 * S/SSOR.java:75-77, S/ILUT.java:95-97 (SSOR: reverse, omegaF = omegaR = 1;
 * ILUT: tau = 1e-6, p = 25) */
MTJG_API int mtjg_precond_create(mtjg_ctx *ctx, int kind, int n, mtjg_precond **out);
/* SSOR(F, reverse, omegaF, omegaR) / SSOR.setOmega, S/SSOR.java:62-96: omegas
 * outside [0, 2] are MTJG_ERR_ILLEGAL_ARGUMENT.  SSOR's apply(b, x) is one
 * symmetric SOR sweep starting from x's content (S/SSOR.java:148-192), so x
 * is read as well as written. */
MTJG_API int mtjg_precond_set_ssor(mtjg_precond *M, int reverse, double omega_f, double omega_r);
/* ILUT(LU, tau, p), S/ILUT.java:68-85: drop tolerance and fill per row; takes
 * effect at the next setMatrix.  The factor runs on the host (it is a chain
 * over the rows), its solves on the device. */
MTJG_API int mtjg_precond_set_ilut(mtjg_precond *M, double tau, int p);
/* Preconditioner.setMatrix(A), S/Preconditioner.java:56-63: Jacobi extracts
 * the inverse diagonal, ILU and ICC copy A and factor it.  On a setup error
 * *err_row receives the number MTJ's message prints. */
MTJG_API int mtjg_precond_set_matrix(mtjg_precond *M, mtjg_csr *A, int *err_row);
/* Preconditioner.apply(b, x) / transApply(b, x), S/Preconditioner.java:30-54 */
MTJG_API int mtjg_precond_apply(mtjg_precond *M, const double *b, double *x);
MTJG_API int mtjg_precond_trans_apply(mtjg_precond *M, const double *b, double *x);
MTJG_API int mtjg_precond_apply_dev(mtjg_precond *M, const double *db, double *dx);
/* The factored values (ILU/ICC: the in-place CSR data array of MTJ's copy,
 * Jacobi: the inverse diagonal), copied to host; returns the count in *len. */
MTJG_API int mtjg_precond_values(mtjg_precond *M, double *out, int64_t cap, int64_t *len);
/* The factor's pattern (ILU, ICC, SSOR: A's; ILUT: its rows after the factor,
 * positions [0, max(stored, diagonal + 1)) of each), with each row's
 * diagonal position within the row, in the layout of mtjg_precond_values. */
MTJG_API int mtjg_precond_pattern(mtjg_precond *M, int *rowptr, int *colind, int *diag, int64_t cap,
                                  int64_t *nnz);
MTJG_API int mtjg_precond_destroy(mtjg_precond *M);

/* ---- IterativeSolver ---------------------------------------------------- */
/* new CG(template) / new BiCGstab(template) / new GMRES(template, restart) /
 * new BiCG / CGS / QMR / IR(template) / new Chebyshev(template, eigmin,
 * eigmax): scratch vectors of size n live on the device with the solver
 * (S/CG.java:51-56, S/BiCGstab.java:53-63, S/GMRES.java:99-125,
 * S/BiCG.java:52-61, S/CGS.java:52-63, S/QMR.java:65-80, S/IR.java:52-55,
 * S/Chebyshev.java:62-68).  restart <= 0 for GMRES is
 * MTJG_ERR_ILLEGAL_ARGUMENT (S/GMRES.java:114-116).  A Chebyshev solver
 * needs mtjg_solver_set_eigenvalues before it solves. */
MTJG_API int mtjg_solver_create(mtjg_ctx *ctx, int kind, int n, int restart,
                                mtjg_solver **out);
/* Chebyshev.setEigenvalues(eigmin, eigmax), S/Chebyshev.java:78-88: bounds of
 * the spectrum of M^-1 A; eigmin <= 0, eigmax <= 0 or eigmin > eigmax is
 * MTJG_ERR_ILLEGAL_ARGUMENT. */
MTJG_API int mtjg_solver_set_eigenvalues(mtjg_solver *S, double eigmin, double eigmax);
/* setPreconditioner(M) (NULL = identity), S/AbstractIterativeSolver.java:50-52 */
MTJG_API int mtjg_solver_set_precond(mtjg_solver *S, mtjg_precond *M);
/* setIterationMonitor(new DefaultIterationMonitor(...)), S/AbstractIterativeSolver.java:62-64 */
MTJG_API int mtjg_solver_set_monitor(mtjg_solver *S, const mtjg_monitor *mon);
/* IterativeSolver.solve(A, b, x), S/IterativeSolver.java:30-44: x is the
 * initial guess and receives the solution (also on a not-converged status,
 * where it holds the iterate MTJ would leave). */
MTJG_API int mtjg_solver_solve(mtjg_solver *S, mtjg_csr *A, const double *b, double *x,
                               mtjg_result *res);
MTJG_API int mtjg_solver_solve_dev(mtjg_solver *S, mtjg_csr *A, const double *db,
                                   double *dx, mtjg_result *res);
/* Mixed precision for CG with the identity or Jacobi preconditioner (also
 * batched), and for GMRES(m <= 63) and BiCGstab with the identity, Jacobi,
 * ILU or ILUT preconditioner (one system).  The solve becomes iterative
 * refinement in the shape of MTJ's IR (S/IR.java:57-70): the outer loop keeps
 * x, the true residual r = b - A x and the monitor's test in FP64, exactly as
 * DefaultIterationMonitor sees them, and each correction comes from an inner
 * solve of the same kind (CG; right-preconditioned GMRES(m) or BiCGstab)
 * whose matrix values, vectors, products and preconditioner (an FP32 copy of
 * the factor or diagonal) are FP32, run until its residual falls by
 * inner_rtol or for inner_max_iter iterations (GMRES: in all, per solve).
 * iterations() then counts refinement steps; mtjg_result.inner_iterations
 * the inner ones.  Other solvers are MTJG_ERR_UNSUPPORTED here, other
 * preconditioners at solve time.  enable = 0 restores the FP64 solver.  No
 * counterpart in the reference. */
MTJG_API int mtjg_solver_set_mixed(mtjg_solver *S, int enable, double inner_rtol, int inner_max_iter);
/* setIterationMonitor(new MatrixIterationMonitor(normA, normb, ...))
 * (S/MatrixIterationMonitor.java): with enable != 0 every convergence test
 * converges iff r < max(rtol (normA |x| + normb), atol), |x| the current
 * iterate's norm in the monitor's norm type, formed on the device before the
 * test; divergence, iteration and NaN tests as DefaultIterationMonitor.  The
 * other settings (maxIter, tolerances, norm) come from mtjg_solver_set_monitor.
 * GMRES's inner test calls converged(double), which MatrixIterationMonitor
 * does not support: a GMRES solve that does not converge at its first test
 * ends MTJG_ERR_UNSUPPORTED (UnsupportedOperationException), as in MTJ.
 * Single-system FP64 solves only (batched or mixed: MTJG_ERR_UNSUPPORTED at
 * solve time).  enable = 0 restores DefaultIterationMonitor. */
MTJG_API int mtjg_solver_set_matrix_monitor(mtjg_solver *S, int enable, double normA, double normb);
/* How the iterations of a solve are launched.  MTJG_LAUNCH_AUTO (the
 * default): CG with the identity or Jacobi preconditioner on one system of at
 * most 512 product tiles (about 80k rows at 7 entries per row, no row longer
 * than 1152 entries) runs its whole loop in one cooperative launch, the
 * matrix held in shared memory, with the results of the graph path bit for
 * bit; every other solve runs a captured graph of its phase launches.
 * MTJG_LAUNCH_GRAPH: always the graph.  No counterpart in the reference. */
enum { MTJG_LAUNCH_AUTO = 0, MTJG_LAUNCH_GRAPH = 1 };
MTJG_API int mtjg_solver_set_launch(mtjg_solver *S, int mode);
/* Residual history of the last solve: the (residual, iteration) pairs passed
 * to IterationReporter.monitor, oldest first (up to history_cap); for a
 * batch, that of the system the result describes (the first that did not
 * converge, else system 0). */
MTJG_API int mtjg_solver_history(mtjg_solver *S, double *resid, int *iters, int cap, int *len);
/* Per-system outcome and residual history of the last batched solve (the
 * aggregate mtjg_result reports the first system that did not converge). */
MTJG_API int mtjg_solver_batch_results(mtjg_solver *S, mtjg_result *out, int count);
MTJG_API int mtjg_solver_batch_history(mtjg_solver *S, int sys, double *resid, int *iters, int cap, int *len);
MTJG_API int mtjg_solver_destroy(mtjg_solver *S);

/* ---- Serving ------------------------------------------------------------
 * A continuous-batching solve server.  No counterpart in the reference,
 * which solves one system per IterativeSolver.solve call.  Matrices are
 * registered once; a resident matrix holds its CSR with FP64 and FP32 values
 * and its Jacobi diagonal (about 16 bytes per entry + 8 per row).  Requests
 * (matrix, b, x0) queue on the host; a scheduler thread admits each into a
 * free slot as soon as a slot, a segment of the pooled vector workspace (40
 * bytes per row) and room for its matrix are free (admission by device-memory
 * footprint), runs a chunk of mixed-precision CG + Jacobi iterations over
 * every admitted system at once, and retires finished systems between chunks,
 * so requests that arrive while others are on the GPU join the running batch.
 * With matrix_budget > 0 the resident matrices stay within that many bytes:
 * each keeps a host copy, is uploaded when first needed, and idle ones (no
 * system in flight) are evicted least recently used and uploaded again on
 * their next request; a request whose matrix cannot get room waits at the
 * head of the queue.  A system's result does not depend on the other systems
 * in flight nor on evictions.  The server runs on a context and stream of its
 * own, on ctx's device; ctx stays free for other work.  mtjg_server_destroy
 * abandons unfinished requests.                                              */
typedef struct mtjg_server mtjg_server;

typedef struct mtjg_server_config {
    int max_systems;       /* concurrent systems on the device */
    int64_t pool_rows;     /* rows of pooled vector workspace (< 2^31) */
    int max_iter;          /* refinement steps (DefaultIterationMonitor maxIter) */
    double rtol, atol, dtol;
    double inner_rtol;     /* FP32 inner CG: residual decrease per refinement step */
    int inner_max_iter;
    int64_t matrix_budget; /* device bytes for resident matrices; 0: no limit, no eviction */
} mtjg_server_config;

typedef struct mtjg_server_result {
    int64_t ticket;
    int matrix;
    mtjg_result result;
    double latency_s;      /* submission to result on the host */
    double queue_s;        /* submission to admission */
} mtjg_server_result;

MTJG_API void mtjg_server_config_defaults(mtjg_server_config *cfg);
MTJG_API int mtjg_server_create(mtjg_ctx *ctx, const mtjg_server_config *cfg, mtjg_server **out);
/* Registers an SPD matrix (0-based CSR, sorted columns, with a nonzero
 * diagonal); *matrix_id identifies it in submissions.  It is uploaded now if
 * it fits the matrix budget without evicting, else on its first request; a
 * matrix larger than the whole budget is refused (MTJG_ERR_ILLEGAL_ARGUMENT). */
MTJG_API int mtjg_server_add_matrix(mtjg_server *S, int n, const int *rowptr, const int *colind,
                                    const double *val, int *matrix_id);
/* Releases a registered matrix: new submissions naming it fail at once;
 * requests already submitted still finish, and its device memory is freed
 * when the last of them has completed (its x written to x_out), at once when
 * none is outstanding. */
MTJG_API int mtjg_server_remove_matrix(mtjg_server *S, int matrix_id);
/* Queues a solve of A x = b (x0 may be NULL for zeros).  b and x0 are copied;
 * x_out receives the solution and must stay valid until the request is
 * reported by mtjg_server_poll. */
MTJG_API int mtjg_server_submit(mtjg_server *S, int matrix_id, const double *b, const double *x0,
                                double *x_out, int64_t *ticket);
/* mtjg_server_submit with a choice of solver: MTJG_CG (the batched lane
 * above), or MTJG_GMRES / MTJG_BICGSTAB, which a second lane solves one at a
 * time on its own stream -- mixed-precision GMRES(30) or BiCGstab with the
 * Jacobi preconditioner and the server's monitor and inner settings, as
 * mtjg_solver_solve would -- on the resident matrix, pinned for the solve
 * under the same matrix budget, concurrently with the CG batch.  Other
 * solvers are MTJG_ERR_UNSUPPORTED. */
MTJG_API int mtjg_server_submit_solver(mtjg_server *S, int matrix_id, int solver, const double *b,
                                       const double *x0, double *x_out, int64_t *ticket);
/* Finished requests since the last poll (non-blocking). */
MTJG_API int mtjg_server_poll(mtjg_server *S, mtjg_server_result *out, int cap, int *count);
/* Waits until every submitted request has finished (or the timeout). */
MTJG_API int mtjg_server_drain(mtjg_server *S, double timeout_s);
/* Chunks run, requests admitted, largest number of systems in flight, and
 * the server's clock (seconds since creation). */
MTJG_API int mtjg_server_stats(mtjg_server *S, int64_t *chunks, int64_t *admitted, int64_t *max_active,
                               double *clock_s);
/* Bytes and number of the matrices resident (or being uploaded), uploads so
 * far (registrations included) and evictions. */
MTJG_API int mtjg_server_residency(mtjg_server *S, int64_t *resident_bytes, int64_t *resident_matrices,
                                   int64_t *uploads, int64_t *evictions);
/* Where the scheduler's time went: GPU time of the chunks (CUDA events),
 * host time spent retiring, admitting and queueing, host time waiting for a
 * chunk, and the mean number of admitted rows per chunk. */
MTJG_API int mtjg_server_timing(mtjg_server *S, double *gpu_s, double *host_s, double *wait_s,
                                double *mean_rows);
/* The server's own context: its stream carries every kernel the server runs,
 * so mtjg_ctx_event_record/_elapsed and mtjg_ctx_launch_count on it time and
 * count the server's device work.  Owned by the server (do not destroy). */
MTJG_API int mtjg_server_context(mtjg_server *S, mtjg_ctx **ctx);
MTJG_API int mtjg_server_destroy(mtjg_server *S);

#ifdef __cplusplus
}
#endif
#endif
