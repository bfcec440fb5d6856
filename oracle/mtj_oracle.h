/*
 * mtj_oracle.h -- CPU restatement of MTJ's preconditioned Krylov path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the GPU library is
 * compared against; nothing in the product links or calls it.  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark use it.
 *
 * Every function restates one Java method of MTJ (no.uib.cipr.matrix),
 * keeping its loop order, its operation order and its short-circuits, and is
 * compiled with -ffp-contract=off so that a*b+c is rounded twice as in Java.
 * Citations are file:line inside the reference project, with
 *   S/ = src/main/java/no/uib/cipr/matrix/sparse/
 *   M/ = src/main/java/no/uib/cipr/matrix/
 *
 * Parity pinning: the reference ships no golden vectors (all its test inputs
 * come from unseeded Math.random).  The oracle is pinned against the
 * properties the reference's own tests check (tests/test_oracle_*.py) and
 * against an independent pure-Python restatement on small cases.  GMRES's
 * dtrtrs step follows the netlib reference BLAS/LAPACK algorithm (the F2J
 * build of netlib-java 1.1.2); a native LAPACK may round differently, so that
 * one step is unpinned beyond the reference test's 1e-4.
 */
#ifndef MTJ_ORACLE_H
#define MTJ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes: identical numbering to include/mtjg.h */
enum {
    OR_OK = 0,
    OR_NC_ITERATIONS = 1,
    OR_NC_DIVERGENCE = 2,
    OR_NC_BREAKDOWN = 3,
    OR_ERR_ILLEGAL_ARGUMENT = 10,
    OR_ERR_ZERO_PIVOT = 20,
    OR_ERR_ZERO_DIAGONAL = 21,
    OR_ERR_MISSING_DIAGONAL = 22,
    OR_ERR_SINGULAR = 23,
    OR_ERR_UNSUPPORTED = 30
};

enum { OR_NORM_ONE = 0, OR_NORM_TWO = 1, OR_NORM_TWO_ROBUST = 2, OR_NORM_INFINITY = 3 };
enum { OR_PC_IDENTITY = 0, OR_PC_JACOBI = 1, OR_PC_ILU = 2, OR_PC_ICC = 3, OR_PC_ICC_LITERAL = 4, OR_PC_SSOR = 5,
       OR_PC_ILUT = 6 };
enum { OR_CG = 0, OR_BICGSTAB = 1, OR_GMRES = 2, OR_BICG = 3, OR_CGS = 4, OR_QMR = 5, OR_CHEBYSHEV = 6, OR_IR = 7 };
/* or_result.detail of a breakdown: which quantity became zero */
enum { OR_BD_RHO = 1, OR_BD_OMEGA = 2, OR_BD_XI = 3, OR_BD_DELTA = 4, OR_BD_EP = 5, OR_BD_BETA = 6, OR_BD_GAMMA = 7 };

/* DefaultIterationMonitor, or MatrixIterationMonitor when matrix != 0
 * (S/MatrixIterationMonitor.java: convergence against rtol (normA |x| +
 * normb) instead of rtol initR) */
typedef struct or_monitor {
    int max_iter;
    double rtol, atol, dtol;
    int norm;
    int matrix;
    double normA, normb;
} or_monitor;

typedef struct or_result {
    int status;
    int iterations;
    double residual;
    int detail;        /* breakdown: OR_BD_* ("rho", "omega", "xi", "delta", "ep", "beta", "gamma") */
    int history_len;   /* monitor calls made (may exceed the history capacity) */
} or_result;

/* CompRowMatrix (S/CompRowMatrix.java) */
void or_mult(int n, const int *rowptr, const int *colind, const double *val,
             const double *x, double *y);
void or_mult_add(int n, const int *rowptr, const int *colind, const double *val,
                 double alpha, const double *x, double *y);
void or_trans_mult(int n, int m, const int *rowptr, const int *colind,
                   const double *val, const double *x, double *y);
void or_trans_mult_add(int n, int m, const int *rowptr, const int *colind,
                       const double *val, double alpha, const double *x, double *y);

/* DenseVector (M/DenseVector.java) */
double or_dot(int n, const double *x, const double *y);
double or_norm(int n, const double *x, int type);
/* 0 (default): MTJ's sequential sums.  B > 0: sums of B-entry blocks combined
 * pairwise, used only to measure a solver's sensitivity to the order of its
 * reductions. */
void or_set_sum_order(int mode);

/* Preconditioners (S/DiagonalPreconditioner.java, S/ILU.java, S/ICC.java) */
typedef struct or_pc or_pc;
or_pc *or_pc_new(int kind, int n);
void or_pc_free(or_pc *pc);
/* returns a status; *detail gets the number MTJ prints in its message */
int or_pc_set_matrix(or_pc *pc, int n, const int *rowptr, const int *colind,
                     const double *val, int *detail);
void or_pc_apply(or_pc *pc, const double *b, double *x);
void or_pc_trans_apply(or_pc *pc, const double *b, double *x);
/* factor values (ILU/ICC: the in-place data array; Jacobi: invdiag; ILUT:
 * its rows' stored values, positions [0, max(used, diagind + 1)) per row) */
int or_pc_values(const or_pc *pc, double *out, int cap);
/* the factor's pattern in the layout of or_pc_values (returns the entry count) */
int or_pc_pattern(const or_pc *pc, int *rowptr, int *colind, int cap);
int or_pc_diag(const or_pc *pc, int *diag);
/* SSOR: (omegaF, omegaR, reverse) (S/SSOR.java:62-96); ILUT: (tau, -, p)
 * (S/ILUT.java:68-85).  Call before or_pc_set_matrix. */
int or_pc_set_params(or_pc *pc, double a, double b, int c);

/* IterativeSolver.solve (S/CG.java, S/BiCGstab.java, S/GMRES.java, S/BiCG.java,
 * S/CGS.java, S/QMR.java, S/Chebyshev.java, S/IR.java); pc NULL = identity */
int or_solve(int kind, int restart, int n, const int *rowptr, const int *colind,
             const double *val, or_pc *pc, const double *b, double *x,
             const or_monitor *mon, or_result *res,
             double *hist_r, int *hist_it, int hist_cap);
/* the same with Chebyshev's eigenvalue bounds (ignored by the other kinds) */
int or_solve_ex(int kind, int restart, double eigmin, double eigmax, int n, const int *rowptr,
                const int *colind, const double *val, or_pc *pc, const double *b, double *x,
                const or_monitor *mon, or_result *res, double *hist_r, int *hist_it, int hist_cap);

#ifdef __cplusplus
}
#endif
#endif
