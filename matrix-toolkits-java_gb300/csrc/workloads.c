/*
 * workloads.c -- seeded synthetic sparse systems of the benchmark shapes.
 *
 * Host-only C (no CUDA): the CSR matrices and vectors every measured
 * configuration is built from, shared by the GPU library's tests, the
 * benchmark and the CPU baseline so that all of them read identical inputs.
 *
 * Random numbers: splitmix64 (Steele, Lea and Flood, "Fast splittable
 * pseudorandom number generators", OOPSLA 2014); a double in [0,1) is the top
 * 53 bits times 2^-53.
 *
 * All matrices are 0-based CSR with ascending column indices inside each row
 * and an explicit diagonal, the storage MTJ's CompRowMatrix keeps
 * (S/CompRowMatrix.java:44-54, :183-208 in the reference).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#if defined(_WIN32)
#define MTJW_API __declspec(dllexport)
#else
#define MTJW_API __attribute__((visibility("default")))
#endif

static uint64_t sm64_next(uint64_t *s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static double sm64_u01(uint64_t *s)
{
    return (double)(sm64_next(s) >> 11) * (1.0 / 9007199254740992.0);
}

/* n values uniform in [lo, hi) from splitmix64 seeded with `seed`. */
MTJW_API void mtjw_uniform(int64_t n, uint64_t seed, double lo, double hi, double *out)
{
    uint64_t s = seed;
    for (int64_t i = 0; i < n; ++i) out[i] = lo + (hi - lo) * sm64_u01(&s);
}

/* Number of nonzeros of the d-dimensional (2*d+1)-point stencil on an N^d
 * grid with Dirichlet boundaries: n + 2*d*(N-1)*N^(d-1). */
MTJW_API int64_t mtjw_stencil_nnz(int dim, int N)
{
    int64_t n = 1, face = 1;
    for (int d = 0; d < dim; ++d) n *= N;
    for (int d = 0; d < dim - 1; ++d) face *= N;
    return n + 2LL * dim * (int64_t)(N - 1) * face;
}

/* Fills one stencil matrix on an N^dim grid (dim 2 or 3), natural ordering
 * i = x + N*y (+ N^2*z).  Off-diagonal weight per axis and side:
 * lower[d] for the neighbour at -1 along axis d, upper[d] for +1. */
static void stencil_fill(int dim, int N, double diag, const double *lower,
                         const double *upper, int *rowptr, int *colind, double *val)
{
    int64_t n = (dim == 2) ? (int64_t)N * N : (int64_t)N * N * N;
    int64_t stride[3] = {1, N, (int64_t)N * N};
    int64_t k = 0;
    rowptr[0] = 0;
    for (int64_t i = 0; i < n; ++i) {
        int64_t c[3] = {i % N, (i / N) % N, dim == 3 ? i / ((int64_t)N * N) : 0};
        for (int d = dim - 1; d >= 0; --d)
            if (c[d] > 0) { colind[k] = (int)(i - stride[d]); val[k++] = lower[d]; }
        colind[k] = (int)i; val[k++] = diag;
        for (int d = 0; d < dim; ++d)
            if (c[d] < N - 1) { colind[k] = (int)(i + stride[d]); val[k++] = upper[d]; }
        rowptr[i + 1] = (int)k;
    }
}

/* 2D 5-point Poisson, 4 on the diagonal and -1 off it. */
MTJW_API void mtjw_poisson2d(int N, int *rowptr, int *colind, double *val)
{
    double m1[3] = {-1, -1, -1};
    stencil_fill(2, N, 4.0, m1, m1, rowptr, colind, val);
}

/* 3D 7-point Poisson, 6 on the diagonal and -1 off it. */
MTJW_API void mtjw_poisson3d(int N, int *rowptr, int *colind, double *val)
{
    double m1[3] = {-1, -1, -1};
    stencil_fill(3, N, 6.0, m1, m1, rowptr, colind, val);
}

/* 3D upwind convection-diffusion, 7-point, scaled by h^2 with D = 1 and a
 * constant velocity along (1, 0.5, 0.25) whose largest cell Peclet number
 * |v|_inf*h/(2D) is 0.5, so the per-axis Peclet numbers are (0.5, 0.25,
 * 0.125).  Diagonal 6 + 2*sum(Pe); the upwind neighbour (the -1 side, as the
 * velocity is positive) carries -1 - 2*Pe_d; the downwind neighbour -1. */
MTJW_API void mtjw_convdiff3d(int N, int *rowptr, int *colind, double *val)
{
    double pe[3] = {0.5, 0.25, 0.125};
    double lower[3], upper[3], diag = 6.0;
    for (int d = 0; d < 3; ++d) {
        lower[d] = -1.0 - 2.0 * pe[d];
        upper[d] = -1.0;
        diag += 2.0 * pe[d];
    }
    stencil_fill(3, N, diag, lower, upper, rowptr, colind, val);
}

/* Sizes of a batch of random graph Laplacians: n_s = floor(exp(U[ln lo,
 * ln hi])) drawn in order from splitmix64 seeded with seed ^ 0x5EED5EED. */
MTJW_API void mtjw_batch_sizes(int count, uint64_t seed, int lo, int hi, int *sizes)
{
    uint64_t s = seed ^ 0x5EED5EEDULL;
    double a = log((double)lo), b = log((double)hi);
    for (int i = 0; i < count; ++i) {
        int v = (int)floor(exp(a + (b - a) * sm64_u01(&s)));
        if (v < lo) v = lo;
        if (v > hi) v = hi;
        sizes[i] = v;
    }
}

#define LAP_MAXDEG 29

/* Random SPD graph Laplacian with a diagonal shift.  Rows are visited in
 * order; row i draws k ~ U{4..14} new neighbours j != i (redrawing repeats
 * and endpoints that already have LAP_MAXDEG neighbours, at most 64k draws)
 * and joins them by undirected edges of weight w ~ U[0.1, 1).  A_ij = -w and
 * A_ii = sum of the row's weights + shift, so rows hold 5..30 entries.
 * Writes nnz; fills the arrays when they are non-NULL (call twice: once to
 * size, once to fill; both calls draw the same numbers). */
MTJW_API int64_t mtjw_laplacian(int n, uint64_t seed, double shift,
                                int *rowptr, int *colind, double *val)
{
    int *nb = (int *)malloc(sizeof(int) * (size_t)n * LAP_MAXDEG);
    double *wt = (double *)malloc(sizeof(double) * (size_t)n * LAP_MAXDEG);
    int *deg = (int *)calloc((size_t)n, sizeof(int));
    uint64_t s = seed;
    for (int i = 0; i < n; ++i) {
        int k = 4 + (int)(sm64_u01(&s) * 11.0);
        int added = 0;
        for (int att = 0; added < k && att < 64 * k; ++att) {
            if (deg[i] >= LAP_MAXDEG) break;
            int j = (int)(sm64_u01(&s) * (double)n);
            if (j == i || j >= n) continue;
            if (deg[j] >= LAP_MAXDEG) continue;
            int dup = 0;
            for (int q = 0; q < deg[i]; ++q)
                if (nb[(size_t)i * LAP_MAXDEG + q] == j) { dup = 1; break; }
            if (dup) continue;
            double w = 0.1 + 0.9 * sm64_u01(&s);
            nb[(size_t)i * LAP_MAXDEG + deg[i]] = j;
            wt[(size_t)i * LAP_MAXDEG + deg[i]++] = w;
            nb[(size_t)j * LAP_MAXDEG + deg[j]] = i;
            wt[(size_t)j * LAP_MAXDEG + deg[j]++] = w;
            added++;
        }
    }
    int64_t nnz = 0;
    for (int i = 0; i < n; ++i) nnz += deg[i] + 1;
    if (rowptr && colind && val) {
        int64_t k = 0;
        rowptr[0] = 0;
        for (int i = 0; i < n; ++i) {
            int *a = nb + (size_t)i * LAP_MAXDEG;
            double *w = wt + (size_t)i * LAP_MAXDEG;
            int d = deg[i];
            /* insertion sort of the neighbour list by column */
            for (int p = 1; p < d; ++p) {
                int cj = a[p];
                double cw = w[p];
                int q = p - 1;
                while (q >= 0 && a[q] > cj) { a[q + 1] = a[q]; w[q + 1] = w[q]; --q; }
                a[q + 1] = cj;
                w[q + 1] = cw;
            }
            double sum = 0.0;
            for (int p = 0; p < d; ++p) sum += w[p];
            int p = 0;
            for (; p < d && a[p] < i; ++p) { colind[k] = a[p]; val[k++] = -w[p]; }
            colind[k] = i;
            val[k++] = sum + shift;
            for (; p < d; ++p) { colind[k] = a[p]; val[k++] = -w[p]; }
            rowptr[i + 1] = (int)k;
        }
    }
    free(nb);
    free(wt);
    free(deg);
    return nnz;
}
