/*
 * mtj_oracle.c -- CPU restatement of MTJ's preconditioned Krylov path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): see
 * mtj_oracle.h.  Build with -ffp-contract=off; Java never fuses a*b+c.
 */
#include "mtj_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- helpers */

/* java.lang.Math.max for doubles: NaN wins, otherwise the larger value. */
static double jmax(double a, double b)
{
    if (a != a) return a;
    if (b != b) return b;
    return a >= b ? a : b;
}

/* java.util.Arrays.binarySearch(int[], from, to, key) as used through
 * S/Arrays.java:119-121: index if found, negative otherwise. */
static int jbinsearch(const int *a, int from, int to, int key)
{
    int lo = from, hi = to - 1;
    while (lo <= hi) {
        int mid = (int)(((unsigned)lo + (unsigned)hi) >> 1);
        int v = a[mid];
        if (v < key) lo = mid + 1;
        else if (v > key) hi = mid - 1;
        else return mid;
    }
    return -(lo + 1);
}

/* ------------------------------------------------------- CompRowMatrix */

/* CompRowMatrix.mult(Vector,Vector), S/CompRowMatrix.java:295-314:
 * y.zero(); row sums in ascending entry order; stored only if != 0. */
void or_mult(int n, const int *rowptr, const int *colind, const double *val,
             const double *x, double *y)
{
    for (int i = 0; i < n; ++i) y[i] = 0.0;
    for (int i = 0; i < n; ++i) {
        double dot = 0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; j++)
            dot += val[j] * x[colind[j]];
        if (dot != 0) y[i] = dot;
    }
}

/* CompRowMatrix.multAdd, S/CompRowMatrix.java:330-347: y_i += alpha*dot. */
void or_mult_add(int n, const int *rowptr, const int *colind, const double *val,
                 double alpha, const double *x, double *y)
{
    for (int i = 0; i < n; ++i) {
        double dot = 0;
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j)
            dot += val[j] * x[colind[j]];
        y[i] += alpha * dot;
    }
}

/* CompRowMatrix.transMult, S/CompRowMatrix.java:350-366: scatter form. */
void or_trans_mult(int n, int m, const int *rowptr, const int *colind,
                   const double *val, const double *x, double *y)
{
    for (int i = 0; i < m; ++i) y[i] = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j)
            y[colind[j]] += val[j] * x[i];
}

/* CompRowMatrix.transMultAdd, S/CompRowMatrix.java:369-388: y scaled by
 * 1/alpha, scatter-added, then scaled by alpha (alpha == 0 gives Inf/NaN,
 * as in the reference). */
void or_trans_mult_add(int n, int m, const int *rowptr, const int *colind,
                       const double *val, double alpha, const double *x, double *y)
{
    double inv = 1. / alpha;
    for (int i = 0; i < m; ++i) y[i] *= inv;
    for (int i = 0; i < n; ++i)
        for (int j = rowptr[i]; j < rowptr[i + 1]; ++j)
            y[colind[j]] += val[j] * x[i];
    for (int i = 0; i < m; ++i) y[i] *= alpha;
}

/* ---------------------------------------------------------- DenseVector */

/* Summation order of dot products and two-norms: 0 = MTJ's sequential loop
 * (the restatement); B > 0 = blocks of B entries summed sequentially, then
 * the block sums combined pairwise.  B > 0 exists only to measure how far a
 * solver's residual history moves when nothing but the order of these sums
 * changes. */
static int g_sum_order = 0;

void or_set_sum_order(int mode) { g_sum_order = mode; }

static double blocked_sum_sq(int n, const double *x, const double *y)
{
    const int B = g_sum_order;
    int nb = (n + B - 1) / B;
    double *part = (double *)malloc(sizeof(double) * (size_t)(nb > 0 ? nb : 1));
    for (int b = 0; b < nb; ++b) {
        double s = 0.;
        int e = (b + 1) * B < n ? (b + 1) * B : n;
        for (int i = b * B; i < e; ++i) s += x[i] * y[i];
        part[b] = s;
    }
    for (int w = 1; w < nb; w *= 2)
        for (int b = 0; b + w < nb; b += 2 * w) part[b] += part[b + w];
    double r = nb ? part[0] : 0.;
    free(part);
    return r;
}

/* DenseVector.dot, M/DenseVector.java:267-279 */
double or_dot(int n, const double *x, const double *y)
{
    if (g_sum_order > 0) return blocked_sum_sq(n, x, y);
    double dot = 0.;
    for (int i = 0; i < n; ++i) dot += x[i] * y[i];
    return dot;
}

/* AbstractVector.norm dispatch M/AbstractVector.java:180-190 onto
 * DenseVector.norm1/norm2/norm2_robust/normInf, M/DenseVector.java:282-318 */
double or_norm(int n, const double *x, int type)
{
    if (type == OR_NORM_ONE) {
        double sum = 0;
        for (int i = 0; i < n; ++i) sum += fabs(x[i]);
        return sum;
    } else if (type == OR_NORM_TWO) {
        if (g_sum_order > 0) return sqrt(blocked_sum_sq(n, x, x));
        double norm = 0;
        for (int i = 0; i < n; ++i) norm += x[i] * x[i];
        return sqrt(norm);
    } else if (type == OR_NORM_TWO_ROBUST) {
        double scale = 0, ssq = 1;
        for (int i = 0; i < n; ++i)
            if (x[i] != 0) {
                double absxi = fabs(x[i]);
                if (scale < absxi) {
                    ssq = 1 + ssq * (scale / absxi) * (scale / absxi);
                    scale = absxi;
                } else
                    ssq += (absxi / scale) * (absxi / scale);
            }
        return scale * sqrt(ssq);
    } else {
        double max = 0;
        for (int i = 0; i < n; ++i) max = jmax(fabs(x[i]), max);
        return max;
    }
}

/* DenseVector.set(alpha, y), M/DenseVector.java:216-231 (alpha==0 zeroes) */
static void vset_a(int n, double *d, double alpha, const double *y)
{
    if (alpha == 0) { for (int i = 0; i < n; ++i) d[i] = 0.0; return; }
    for (int i = 0; i < n; ++i) d[i] = alpha * y[i];
}

/* DenseVector.add(alpha, y), M/DenseVector.java:249-264 (alpha==0 no-op) */
static void vadd_a(int n, double *d, double alpha, const double *y)
{
    if (alpha == 0) return;
    for (int i = 0; i < n; i++) d[i] += alpha * y[i];
}

/* DenseVector.add(y), M/DenseVector.java:234-246 */
static void vadd(int n, double *d, const double *y)
{
    for (int i = 0; i < n; i++) d[i] += y[i];
}

/* DenseVector.scale, M/DenseVector.java:196-200 */
static void vscale(int n, double *d, double alpha)
{
    for (int i = 0; i < n; ++i) d[i] *= alpha;
}

/* ------------------------------------------------------ iteration monitor */

typedef struct mon_state {
    const or_monitor *cfg;
    int n;
    const double *x;  /* the solver's iterate (MatrixIterationMonitor reads its norm) */
    int iter;
    double initR;
    double residual;
    double *hist_r;
    int *hist_it;
    int hist_cap;
    int hist_len;
} mon_state;

/* AbstractIterationMonitor.converged(double), S/AbstractIterationMonitor.java
 * :81-93 (reporter hook, then residual, then convergedI) and
 * DefaultIterationMonitor.convergedI, S/DefaultIterationMonitor.java:133-156.
 * Returns -1 while running, OR_OK when converged, or a not-converged code. */
static int mon_check(mon_state *m, double r)
{
    if (m->hist_len < m->hist_cap) {
        m->hist_r[m->hist_len] = r;
        m->hist_it[m->hist_len] = m->iter;
    }
    m->hist_len++;
    m->residual = r;
    if (m->iter == 0) m->initR = r;
    if (r < jmax(m->cfg->rtol * m->initR, m->cfg->atol)) return OR_OK;
    if (r > m->cfg->dtol * m->initR) return OR_NC_DIVERGENCE;
    if (m->iter >= m->cfg->max_iter) return OR_NC_ITERATIONS;
    if (r != r) return OR_NC_DIVERGENCE;
    return -1;
}

/* AbstractIterationMonitor.converged(Vector r, Vector x) (:76-86).  With a
 * MatrixIterationMonitor, its convergedI(r, x)
 * (S/MatrixIterationMonitor.java:101-124): initR on the first test; converged
 * iff r < max(rtol (normA |x| + normb), atol), |x| in the monitor's norm;
 * then DefaultIterationMonitor's divergence, iteration and NaN tests. */
static int mon_check_vec(mon_state *m, int n, const double *r)
{
    const double rn = or_norm(n, r, m->cfg->norm);
    if (!m->cfg->matrix) return mon_check(m, rn);
    if (m->hist_len < m->hist_cap) {
        m->hist_r[m->hist_len] = rn;
        m->hist_it[m->hist_len] = m->iter;
    }
    m->hist_len++;
    m->residual = rn;
    if (m->iter == 0) m->initR = rn;
    const double xn = or_norm(m->n, m->x, m->cfg->norm);
    if (rn < jmax(m->cfg->rtol * (m->cfg->normA * xn + m->cfg->normb), m->cfg->atol)) return OR_OK;
    if (rn > m->cfg->dtol * m->initR) return OR_NC_DIVERGENCE;
    if (m->iter >= m->cfg->max_iter) return OR_NC_ITERATIONS;
    if (rn != rn) return OR_NC_DIVERGENCE;
    return -1;
}

/* AbstractIterationMonitor.converged(double r) (:88-93): the reporter and the
 * residual, then convergedI(r), which a MatrixIterationMonitor does not
 * support (S/MatrixIterationMonitor.java:127-129). */
static int mon_check_scalar(mon_state *m, double r)
{
    if (!m->cfg->matrix) return mon_check(m, r);
    if (m->hist_len < m->hist_cap) {
        m->hist_r[m->hist_len] = r;
        m->hist_it[m->hist_len] = m->iter;
    }
    m->hist_len++;
    m->residual = r;
    return OR_ERR_UNSUPPORTED;
}

/* ------------------------------------------------------- preconditioners */

/* SparseVector storage (S/SparseVector.java): sorted indices in
 * index[0, used), capacity cap; slots past used keep whatever they held. */
typedef struct svec {
    int *index;
    double *data;
    int cap, used;
} svec;

struct or_pc {
    int kind;
    int n;
    /* SSOR (S/SSOR.java:37-52) and ILUT (S/ILUT.java:68-85) parameters */
    int reverse, p;
    double omega_f, omega_r, tau;
    svec *rows;          /* ILUT factor rows */
    double *xx;          /* SSOR half iterate */
    /* Jacobi */
    double *invdiag;
    /* ILU / ICC: private CSR copy factored in place + diagonal positions */
    int *rowptr, *colind, *diagind;
    double *data;
    int nnz;
    double *y; /* the temporary vector of ILU/ICC apply */
};

or_pc *or_pc_new(int kind, int n)
{
    or_pc *pc = (or_pc *)calloc(1, sizeof(or_pc));
    pc->kind = kind;
    pc->n = n;
    pc->y = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    pc->xx = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    /* new SSOR(F) = SSOR(F, true, 1, 1) (S/SSOR.java:75-77); new ILUT(LU) =
     * ILUT(LU, 1e-6, 25) (S/ILUT.java:95-97) */
    pc->reverse = 1;
    pc->omega_f = pc->omega_r = 1;
    pc->tau = 1e-6;
    pc->p = 25;
    if (kind == OR_PC_JACOBI)
        pc->invdiag = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    return pc;
}

static void free_rows(or_pc *pc)
{
    if (!pc->rows) return;
    for (int i = 0; i < pc->n; ++i) {
        free(pc->rows[i].index);
        free(pc->rows[i].data);
    }
    free(pc->rows);
    pc->rows = NULL;
}

void or_pc_free(or_pc *pc)
{
    if (!pc) return;
    free_rows(pc);
    free(pc->xx);
    free(pc->invdiag);
    free(pc->rowptr);
    free(pc->colind);
    free(pc->diagind);
    free(pc->data);
    free(pc->y);
    free(pc);
}

/* ILU.findDiagonalIndices S/ILU.java:127-140 / ICC S/ICC.java:141-154 */
static int find_diag(or_pc *pc, int *detail)
{
    int n = pc->n;
    pc->diagind = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int k = 0; k < n; ++k) {
        pc->diagind[k] = jbinsearch(pc->colind, pc->rowptr[k], pc->rowptr[k + 1], k);
        if (pc->diagind[k] < 0) { *detail = k + 1; return OR_ERR_MISSING_DIAGONAL; }
    }
    return OR_OK;
}

/* ILU.factor, S/ILU.java:86-125, including the read of colind[l] after the
 * scan has left row k (l == rowptr[k+1]), which may update the first entry
 * of row k+1 when the pattern is structurally nonsymmetric. */
static int ilu_factor(or_pc *pc, int *detail)
{
    int n = pc->n;
    const int *colind = pc->colind, *rowptr = pc->rowptr, *diagind = pc->diagind;
    double *data = pc->data;
    for (int k = 1; k < n; ++k)
        for (int i = rowptr[k]; i < diagind[k]; ++i) {
            int index = colind[i];
            double LUii = data[diagind[index]];
            if (LUii == 0) { *detail = i + 1; return OR_ERR_ZERO_PIVOT; }
            double LUki = (data[i] /= LUii);
            for (int j = diagind[index] + 1, l = rowptr[k] + 1; j < rowptr[index + 1]; ++j) {
                while (l < rowptr[k + 1] && colind[l] < colind[j]) l++;
                if (colind[l] == colind[j]) data[l] -= LUki * data[j];
            }
        }
    return OR_OK;
}

/* ICC.factor, S/ICC.java:85-139, literally: dense row workspace and a scan
 * over every earlier row.  O(n^2); used on small cases to pin the fast one. */
static int icc_factor_literal(or_pc *pc, int *detail)
{
    int n = pc->n;
    const int *colind = pc->colind, *rowptr = pc->rowptr, *diagind = pc->diagind;
    double *data = pc->data;
    double *Rk = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    for (int k = 0; k < n; ++k) {
        for (int c = 0; c < n; ++c) Rk[c] = 0;
        for (int i = rowptr[k]; i < rowptr[k + 1]; ++i) Rk[colind[i]] = data[i];
        for (int i = 0; i < k; ++i) {
            double Rii = data[diagind[i]];
            if (Rii == 0) { free(Rk); *detail = i + 1; return OR_ERR_ZERO_PIVOT; }
            double Rki = Rk[i] / Rii;
            if (Rki == 0) continue;
            for (int j = diagind[i] + 1; j < rowptr[i + 1]; ++j)
                Rk[colind[j]] -= Rki * data[j];
        }
        if (Rk[k] == 0) { free(Rk); *detail = k + 1; return OR_ERR_ZERO_DIAGONAL; }
        double sqRkk = sqrt(Rk[k]);
        for (int i = diagind[k]; i < rowptr[k + 1]; ++i) data[i] = Rk[colind[i]] / sqRkk;
    }
    free(Rk);
    return OR_OK;
}

/* min-heap of column indices for the reach-based ICC */
typedef struct { int *a; int len, cap; } iheap;
static void hpush(iheap *h, int v)
{
    if (h->len == h->cap) {
        h->cap = h->cap ? 2 * h->cap : 64;
        h->a = (int *)realloc(h->a, sizeof(int) * (size_t)h->cap);
    }
    int i = h->len++;
    while (i > 0) {
        int p = (i - 1) / 2;
        if (h->a[p] <= v) break;
        h->a[i] = h->a[p];
        i = p;
    }
    h->a[i] = v;
}
static int hpop(iheap *h)
{
    int top = h->a[0], v = h->a[--h->len], i = 0;
    for (;;) {
        int c = 2 * i + 1;
        if (c >= h->len) break;
        if (c + 1 < h->len && h->a[c + 1] < h->a[c]) c++;
        if (h->a[c] >= v) break;
        h->a[i] = h->a[c];
        i = c;
    }
    if (h->len) h->a[i] = v;
    return top;
}

/* ICC.factor restated over the reach of each row: the literal loop visits
 * every i < k but only changes Rk through rows i whose Rk[i] is nonzero, and
 * Rk[i] can only become nonzero by being in row k's pattern or by an update
 * from a visited row.  Visiting exactly those columns in ascending order
 * performs the same floating-point operations in the same order.  Rows whose
 * diagonal became NaN (a negative pivot) make 0/NaN != 0, so the literal loop
 * applies them to every later row; they are added to every reach. */
static int icc_factor_reach(or_pc *pc, int *detail)
{
    int n = pc->n;
    const int *colind = pc->colind, *rowptr = pc->rowptr, *diagind = pc->diagind;
    double *data = pc->data;
    double *Rk = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    unsigned char *mark = (unsigned char *)calloc((size_t)(n > 0 ? n : 1), 1);
    int *touched = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int *nanrows = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    int nnan = 0;
    iheap h = {0, 0, 0};
    int st = OR_OK;
    for (int k = 0; k < n && st == OR_OK; ++k) {
        int nt = 0;
        for (int i = rowptr[k]; i < rowptr[k + 1]; ++i) {
            int c = colind[i];
            Rk[c] = data[i];
            if (!mark[c]) { mark[c] = 1; touched[nt++] = c; if (c < k) hpush(&h, c); }
        }
        for (int q = 0; q < nnan; ++q) {
            int c = nanrows[q];
            if (!mark[c]) { mark[c] = 1; touched[nt++] = c; hpush(&h, c); }
        }
        while (h.len) {
            int i = hpop(&h);
            double Rii = data[diagind[i]];
            if (Rii == 0) { *detail = i + 1; st = OR_ERR_ZERO_PIVOT; break; }
            double Rki = Rk[i] / Rii;
            if (Rki == 0) continue;
            for (int j = diagind[i] + 1; j < rowptr[i + 1]; ++j) {
                int c = colind[j];
                Rk[c] -= Rki * data[j];
                if (!mark[c]) { mark[c] = 1; touched[nt++] = c; if (c < k) hpush(&h, c); }
            }
        }
        if (st == OR_OK) {
            if (Rk[k] == 0) { *detail = k + 1; st = OR_ERR_ZERO_DIAGONAL; }
            else {
                double sqRkk = sqrt(Rk[k]);
                for (int i = diagind[k]; i < rowptr[k + 1]; ++i) data[i] = Rk[colind[i]] / sqRkk;
                if (data[diagind[k]] != data[diagind[k]]) nanrows[nnan++] = k;
            }
        }
        for (int t = 0; t < nt; ++t) { Rk[touched[t]] = 0; mark[touched[t]] = 0; }
        h.len = 0;
    }
    free(h.a);
    free(Rk);
    free(mark);
    free(touched);
    free(nanrows);
    return st;
}

/* ------------------------------------------------------------------ ILUT */

/* Arrays.binarySearchGreater(index, key, 0, used) (S/Arrays.java:51-54,
 * :123-156): the first position whose index is >= key, else used. */
static int sv_greater(const svec *v, int key)
{
    int begin = 0, end = v->used;
    if (begin == end) return end;
    end--;
    int mid = (end + begin) >> 1;
    while (begin <= end) {
        mid = (end + begin) >> 1;
        if (v->index[mid] < key) begin = mid + 1;
        else if (v->index[mid] > key) end = mid - 1;
        else return mid;
    }
    return v->index[mid] >= key ? mid : mid + 1;
}

/* SparseVector.getIndex (S/SparseVector.java:188-231): position of ind,
 * inserted (value 0) when absent; the storage doubles (at most `size`) when
 * full, into fresh zero-filled arrays. */
static int sv_get_index(svec *v, int ind, int size)
{
    int i = sv_greater(v, ind);
    if (i < v->used && v->index[i] == ind) return i;
    int *ni = v->index;
    double *nd = v->data;
    int grew = 0;
    if (++v->used > v->cap) {
        int len = v->cap != 0 ? v->cap << 1 : 1;
        if (len > size) len = size;
        ni = (int *)calloc((size_t)(len > 0 ? len : 1), sizeof(int));
        nd = (double *)calloc((size_t)(len > 0 ? len : 1), sizeof(double));
        if (i) {
            memcpy(ni, v->index, sizeof(int) * (size_t)i);
            memcpy(nd, v->data, sizeof(double) * (size_t)i);
        }
        v->cap = len;
        grew = 1;
    }
    int tail = v->used - i - 1;
    if (tail > 0) {
        memmove(ni + i + 1, v->index + i, sizeof(int) * (size_t)tail);
        memmove(nd + i + 1, v->data + i, sizeof(double) * (size_t)tail);
    }
    ni[i] = ind;
    nd[i] = 0.;
    if (grew) {
        free(v->index);
        free(v->data);
    }
    v->index = ni;
    v->data = nd;
    return i;
}

/* SparseVector.set (S/SparseVector.java:157-164): the position first (it may
 * reallocate the storage), then the value */
static void sv_set(svec *v, int ind, double value, int size)
{
    int i = sv_get_index(v, ind, size);
    v->data[i] = value;
}

/* SparseVector.zero (S/SparseVector.java:238-242): values cleared, used = 0,
 * the index array keeps its contents */
static void sv_zero(svec *v)
{
    for (int i = 0; i < v->cap; ++i) v->data[i] = 0;
    v->used = 0;
}

/* SparseVector.norm2 (S/SparseVector.java:282-287) */
static double sv_norm2(const svec *v)
{
    double norm = 0;
    for (int i = 0; i < v->used; ++i) norm += v->data[i] * v->data[i];
    return sqrt(norm);
}

typedef struct {
    int index;
    double value;
} ide;

/* Collections.sort of ILUT.IntDoubleEntry (S/ILUT.java:282-302): by
 * decreasing magnitude, stable (a merge sort keeps equal magnitudes in the
 * order they were added, i.e. by increasing index) */
static void ide_sort(ide *a, ide *tmp, int n)
{
    if (n < 2) return;
    int h = n / 2;
    ide_sort(a, tmp, h);
    ide_sort(a + h, tmp, n - h);
    int i = 0, j = h, k = 0;
    while (i < h && j < n) {
        if (fabs(a[j].value) > fabs(a[i].value)) tmp[k++] = a[j++];
        else tmp[k++] = a[i++];
    }
    while (i < h) tmp[k++] = a[i++];
    while (j < n) tmp[k++] = a[j++];
    memcpy(a, tmp, sizeof(ide) * (size_t)n);
}

/* ILUT.gather (S/ILUT.java:225-272) of the dense row z into row v (row d) */
static void ilut_gather(or_pc *pc, const double *z, svec *v, double taui, int d, ide *lo, ide *up, ide *tmp)
{
    int n = pc->n, nl = 0, nu = 0, nlo = 0, nup = 0;
    for (int i = 0; i < v->used; ++i) {
        if (v->index[i] < d) nl++;
        else if (v->index[i] > d) nu++;
    }
    sv_zero(v);
    for (int i = 0; i < d; ++i)
        if (fabs(z[i]) > taui) { lo[nlo].index = i; lo[nlo].value = z[i]; nlo++; }
    for (int i = d + 1; i < n; ++i)
        if (fabs(z[i]) > taui) { up[nup].index = i; up[nup].value = z[i]; nup++; }
    ide_sort(lo, tmp, nlo);
    ide_sort(up, tmp, nup);
    sv_set(v, d, z[d], n);
    int ml = nl + pc->p < nlo ? nl + pc->p : nlo, mu = nu + pc->p < nup ? nu + pc->p : nup;
    for (int i = 0; i < ml; ++i) sv_set(v, lo[i].index, lo[i].value, n);
    for (int i = 0; i < mu; ++i) sv_set(v, up[i].index, up[i].value, n);
}

/* ILUT.setMatrix + factor (S/ILUT.java:119-208), literally: the dense work
 * row LUi, every earlier row k visited (O(n^2)).  LU.set(A); LU.compact()
 * leaves each row holding A's nonzero entries, storage exactly full. */
static int ilut_factor(or_pc *pc, const int *rowptr, const int *colind, const double *val, int *detail)
{
    int n = pc->n, st = OR_OK;
    free_rows(pc);
    pc->rows = (svec *)calloc((size_t)(n > 0 ? n : 1), sizeof(svec));
    pc->diagind = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    for (int k = 0; k < n; ++k) {
        int nz = 0;
        for (int j = rowptr[k]; j < rowptr[k + 1]; ++j) nz += val[j] != 0.;
        svec *v = &pc->rows[k];
        v->cap = v->used = nz;
        v->index = (int *)calloc((size_t)(nz > 0 ? nz : 1), sizeof(int));
        v->data = (double *)calloc((size_t)(nz > 0 ? nz : 1), sizeof(double));
        for (int j = rowptr[k], q = 0; j < rowptr[k + 1]; ++j)
            if (val[j] != 0.) { v->index[q] = colind[j]; v->data[q] = val[j]; q++; }
    }
    for (int k = 0; k < n; ++k) {
        pc->diagind[k] = jbinsearch(pc->rows[k].index, 0, pc->rows[k].used, k);
        if (pc->diagind[k] < 0) { *detail = k + 1; return OR_ERR_MISSING_DIAGONAL; }
    }
    double *LUi = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    ide *lo = (ide *)malloc(sizeof(ide) * (size_t)(n > 0 ? n : 1));
    ide *up = (ide *)malloc(sizeof(ide) * (size_t)(n > 0 ? n : 1));
    ide *tmp = (ide *)malloc(sizeof(ide) * (size_t)(n > 0 ? n : 1));
    for (int i = 1; i < n && st == OR_OK; ++i) {
        svec *rowi = &pc->rows[i];
        double taui = sv_norm2(rowi) * pc->tau;
        for (int c = 0; c < n; ++c) LUi[c] = 0;
        for (int j = 0; j < rowi->used; ++j) LUi[rowi->index[j]] = rowi->data[j];
        for (int k = 0; k < i; ++k) {
            const svec *rk = &pc->rows[k];
            double dk = rk->data[pc->diagind[k]];
            if (dk == 0) { *detail = k + 1; st = OR_ERR_ZERO_DIAGONAL; break; }
            double LUik = LUi[k] / dk;
            if (fabs(LUik) <= taui) continue;
            for (int j = pc->diagind[k] + 1; j < rk->used; ++j) LUi[rk->index[j]] -= LUik * rk->data[j];
            LUi[k] = LUik;
        }
        if (st != OR_OK) break;
        ilut_gather(pc, LUi, rowi, taui, i, lo, up, tmp);
        int di = pc->diagind[i];
        if (di >= rowi->cap || rowi->index[di] != i) {
            pc->diagind[i] = jbinsearch(rowi->index, 0, rowi->used, i);
            if (pc->diagind[i] < 0) { *detail = i + 1; st = OR_ERR_MISSING_DIAGONAL; }
        }
    }
    free(LUi); free(lo); free(up); free(tmp);
    return st;
}

/* positions of row i the factor's triangular solves read: [0, diagind] and
 * the stored entries */
static int ilut_row_len(const or_pc *pc, int i)
{
    int u = pc->rows[i].used, d = pc->diagind[i] + 1;
    return u > d ? u : d;
}

/* ILUT.apply (S/ILUT.java:111-113): UnitLowerFlexCompRowMatrix.solve (:321-336)
 * into y, then UpperFlexCompRowMatrix.solve (:375-391) */
static void ilut_apply(or_pc *pc, const double *b, double *x)
{
    int n = pc->n;
    double *y = pc->y;
    for (int i = 0; i < n; ++i) {
        const svec *r = &pc->rows[i];
        double sum = 0;
        for (int j = 0; j < pc->diagind[i]; ++j) sum += r->data[j] * y[r->index[j]];
        y[i] = b[i] - sum;
    }
    for (int i = n - 1; i >= 0; --i) {
        const svec *r = &pc->rows[i];
        double sum = 0;
        for (int j = pc->diagind[i] + 1; j < r->used; ++j) sum += r->data[j] * x[r->index[j]];
        x[i] = (y[i] - sum) / r->data[pc->diagind[i]];
    }
}

/* ILUT.transApply (S/ILUT.java:115-117): UpperFlexCompRowMatrix.transSolve
 * (:393-410) into y, then UnitLowerFlexCompRowMatrix.transSolve (:338-353) */
static void ilut_trans_apply(or_pc *pc, const double *b, double *x)
{
    int n = pc->n;
    double *y = pc->y;
    if (y != b) memcpy(y, b, sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const svec *r = &pc->rows[i];
        y[i] /= r->data[pc->diagind[i]];
        for (int j = pc->diagind[i] + 1; j < r->used; ++j) y[r->index[j]] -= r->data[j] * y[i];
    }
    if (x != y) memcpy(x, y, sizeof(double) * (size_t)n);
    for (int i = n - 1; i >= 0; --i) {
        const svec *r = &pc->rows[i];
        for (int j = 0; j < pc->diagind[i]; ++j) x[r->index[j]] -= r->data[j] * x[i];
    }
}

/* ------------------------------------------------------------------ SSOR */

/* SSOR.apply (S/SSOR.java:148-192): one symmetric SOR sweep from the current
 * content of x (forward into xx, then backward into x when reverse) */
static void ssor_apply(or_pc *pc, const double *b, double *x)
{
    int n = pc->n;
    const int *rp = pc->rowptr, *ci = pc->colind, *dg = pc->diagind;
    const double *d = pc->data;
    double *xx = pc->xx;
    memcpy(xx, x, sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        double sigma = 0;
        for (int j = rp[i]; j < dg[i]; ++j) sigma += d[j] * xx[ci[j]];
        for (int j = dg[i] + 1; j < rp[i + 1]; ++j) sigma += d[j] * x[ci[j]];
        sigma = (b[i] - sigma) / d[dg[i]];
        xx[i] = x[i] + pc->omega_f * (sigma - x[i]);
    }
    if (!pc->reverse) {
        memcpy(x, xx, sizeof(double) * (size_t)n);
        return;
    }
    for (int i = n - 1; i >= 0; --i) {
        double sigma = 0;
        for (int j = rp[i]; j < dg[i]; ++j) sigma += d[j] * xx[ci[j]];
        for (int j = dg[i] + 1; j < rp[i + 1]; ++j) sigma += d[j] * x[ci[j]];
        sigma = (b[i] - sigma) / d[dg[i]];
        x[i] = xx[i] + pc->omega_r * (sigma - xx[i]);
    }
}

int or_pc_set_params(or_pc *pc, double a, double b, int c)
{
    if (pc->kind == OR_PC_SSOR) {
        /* SSOR.setOmega, S/SSOR.java:87-96 */
        if (a < 0 || a > 2 || b < 0 || b > 2) return OR_ERR_ILLEGAL_ARGUMENT;
        pc->omega_f = a;
        pc->omega_r = b;
        pc->reverse = c;
    } else if (pc->kind == OR_PC_ILUT) {
        pc->tau = a;
        pc->p = c;
    }
    return OR_OK;
}

int or_pc_pattern(const or_pc *pc, int *rowptr, int *colind, int cap)
{
    if (pc->kind == OR_PC_ILUT) {
        int tot = 0;
        if (rowptr) rowptr[0] = 0;
        for (int i = 0; i < pc->n; ++i) {
            int len = ilut_row_len(pc, i);
            for (int j = 0; j < len; ++j)
                if (colind && tot + j < cap) colind[tot + j] = pc->rows[i].index[j];
            tot += len;
            if (rowptr) rowptr[i + 1] = tot;
        }
        return tot;
    }
    if (!pc->rowptr) return 0;
    if (rowptr) memcpy(rowptr, pc->rowptr, sizeof(int) * (size_t)(pc->n + 1));
    int m = pc->nnz < cap ? pc->nnz : cap;
    if (colind) memcpy(colind, pc->colind, sizeof(int) * (size_t)m);
    return pc->nnz;
}

/* position of each row's diagonal in or_pc_pattern's rows */
int or_pc_diag(const or_pc *pc, int *diag)
{
    if (!pc->diagind) return 0;
    memcpy(diag, pc->diagind, sizeof(int) * (size_t)pc->n);
    return pc->n;
}

int or_pc_set_matrix(or_pc *pc, int n, const int *rowptr, const int *colind,
                     const double *val, int *detail)
{
    int dummy;
    if (!detail) detail = &dummy;
    *detail = 0;
    if (n != pc->n) return OR_ERR_ILLEGAL_ARGUMENT;
    if (pc->kind == OR_PC_IDENTITY) return OR_OK;
    if (pc->kind == OR_PC_JACOBI) {
        /* DiagonalPreconditioner.setMatrix, S/DiagonalPreconditioner.java:64-76,
         * with CompRowMatrix.get (binary search) S/CompRowMatrix.java:407-417 */
        for (int i = 0; i < n; ++i) {
            int idx = jbinsearch(colind, rowptr[i], rowptr[i + 1], i);
            double d = idx >= 0 ? val[idx] : 0.0;
            if (d == 0) { *detail = i + 1; return OR_ERR_ZERO_DIAGONAL; }
            pc->invdiag[i] = 1 / d;
        }
        return OR_OK;
    }
    /* ILU/ICC: LU.set(A) / R.set(A) copies A into the private CSR
     * (S/ILU.java:80-84, S/ICC.java:79-83) */
    int nnz = rowptr[n];
    free(pc->rowptr); free(pc->colind); free(pc->data); free(pc->diagind);
    pc->diagind = NULL;
    pc->nnz = nnz;
    pc->rowptr = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    pc->colind = (int *)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    pc->data = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
    memcpy(pc->rowptr, rowptr, sizeof(int) * (size_t)(n + 1));
    if (nnz) {
        memcpy(pc->colind, colind, sizeof(int) * (size_t)nnz);
        memcpy(pc->data, val, sizeof(double) * (size_t)nnz);
    }
    if (pc->kind == OR_PC_ILUT) return ilut_factor(pc, rowptr, colind, val, detail);
    int st = find_diag(pc, detail);
    if (st != OR_OK) return st;
    if (pc->kind == OR_PC_SSOR) return OR_OK;  /* SSOR.setMatrix, S/SSOR.java:98-113 */
    if (pc->kind == OR_PC_ILU) return ilu_factor(pc, detail);
    if (pc->kind == OR_PC_ICC_LITERAL) return icc_factor_literal(pc, detail);
    return icc_factor_reach(pc, detail);
}

int or_pc_values(const or_pc *pc, double *out, int cap)
{
    if (pc->kind == OR_PC_ILUT) {
        int tot = 0;
        for (int i = 0; pc->rows && i < pc->n; ++i) {
            int len = ilut_row_len(pc, i);
            for (int j = 0; j < len; ++j)
                if (out && tot + j < cap) out[tot + j] = pc->rows[i].data[j];
            tot += len;
        }
        return tot;
    }
    if (pc->kind == OR_PC_JACOBI) {
        int m = pc->n < cap ? pc->n : cap;
        memcpy(out, pc->invdiag, sizeof(double) * (size_t)m);
        return pc->n;
    }
    if (!pc->data) return 0;
    int m = pc->nnz < cap ? pc->nnz : cap;
    memcpy(out, pc->data, sizeof(double) * (size_t)m);
    return pc->nnz;
}

/* UnitLowerCompRowMatrix.solve, S/UnitLowerCompRowMatrix.java:49-67 */
static void lower_solve(const or_pc *pc, const double *b, double *x)
{
    for (int i = 0; i < pc->n; ++i) {
        double sum = 0;
        for (int j = pc->rowptr[i]; j < pc->diagind[i]; ++j)
            sum += pc->data[j] * x[pc->colind[j]];
        x[i] = b[i] - sum;
    }
}

/* UnitLowerCompRowMatrix.transSolve, S/UnitLowerCompRowMatrix.java:70-86 */
static void lower_trans_solve(const or_pc *pc, const double *b, double *x)
{
    if (x != b) memcpy(x, b, sizeof(double) * (size_t)pc->n);
    for (int i = pc->n - 1; i >= 0; --i)
        for (int j = pc->rowptr[i]; j < pc->diagind[i]; ++j)
            x[pc->colind[j]] -= pc->data[j] * x[i];
}

/* UpperCompRowMatrix.solve, S/UpperCompRowMatrix.java:49-67 */
static void upper_solve(const or_pc *pc, const double *b, double *x)
{
    for (int i = pc->n - 1; i >= 0; --i) {
        double sum = 0;
        for (int j = pc->diagind[i] + 1; j < pc->rowptr[i + 1]; ++j)
            sum += pc->data[j] * x[pc->colind[j]];
        x[i] = (b[i] - sum) / pc->data[pc->diagind[i]];
    }
}

/* UpperCompRowMatrix.transSolve, S/UpperCompRowMatrix.java:70-90 */
static void upper_trans_solve(const or_pc *pc, const double *b, double *x)
{
    if (x != b) memcpy(x, b, sizeof(double) * (size_t)pc->n);
    for (int i = 0; i < pc->n; ++i) {
        x[i] /= pc->data[pc->diagind[i]];
        for (int j = pc->diagind[i] + 1; j < pc->rowptr[i + 1]; ++j)
            x[pc->colind[j]] -= pc->data[j] * x[i];
    }
}

void or_pc_apply(or_pc *pc, const double *b, double *x)
{
    int n = pc->n;
    switch (pc->kind) {
    case OR_PC_IDENTITY: /* S/AbstractIterativeSolver.java:82-96 */
        if (x != b) memcpy(x, b, sizeof(double) * (size_t)n);
        break;
    case OR_PC_JACOBI: /* S/DiagonalPreconditioner.java:47-58 */
        for (int i = 0; i < n; ++i) x[i] = b[i] * pc->invdiag[i];
        break;
    case OR_PC_ILU: /* S/ILU.java:64-70 */
        lower_solve(pc, b, pc->y);
        upper_solve(pc, pc->y, x);
        break;
    case OR_PC_SSOR:
        ssor_apply(pc, b, x);
        break;
    case OR_PC_ILUT:
        ilut_apply(pc, b, x);
        break;
    default: /* ICC.apply S/ICC.java:67-73 */
        upper_trans_solve(pc, b, pc->y);
        upper_solve(pc, pc->y, x);
        break;
    }
}

void or_pc_trans_apply(or_pc *pc, const double *b, double *x)
{
    if (pc->kind == OR_PC_ILU) { /* S/ILU.java:72-78 */
        upper_trans_solve(pc, b, pc->y);
        lower_trans_solve(pc, pc->y, x);
    } else if (pc->kind == OR_PC_ILUT) {
        ilut_trans_apply(pc, b, x);
    } else { /* SSOR.transApply assumes a symmetric matrix (S/SSOR.java:194-197) */
        or_pc_apply(pc, b, x);
    }
}

/* ---------------------------------------------------------------- solvers */

static void pc_apply_or_identity(or_pc *pc, int n, const double *b, double *x)
{
    if (pc) or_pc_apply(pc, b, x);
    else if (x != b) memcpy(x, b, sizeof(double) * (size_t)n);
}

/* CG.solve, S/CG.java:58-87 */
static int cg_solve(int n, const int *rp, const int *ci, const double *v, or_pc *pc,
                    const double *b, double *x, mon_state *m, int *detail)
{
    (void)detail;
    double alpha = 0, beta = 0, rho = 0, rho_1 = 0;
    double *p = calloc((size_t)n + 1, 8), *z = calloc((size_t)n + 1, 8);
    double *q = calloc((size_t)n + 1, 8), *r = calloc((size_t)n + 1, 8);
    memcpy(r, b, sizeof(double) * (size_t)n);
    or_mult_add(n, rp, ci, v, -1, x, r);
    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        pc_apply_or_identity(pc, n, r, z);
        rho = or_dot(n, r, z);
        if (m->iter == 0)
            memcpy(p, z, sizeof(double) * (size_t)n);
        else {
            beta = rho / rho_1;
            vscale(n, p, beta);
            vadd(n, p, z);
        }
        or_mult(n, rp, ci, v, p, q);
        alpha = rho / or_dot(n, p, q);
        vadd_a(n, x, alpha, p);
        vadd_a(n, r, -alpha, q);
        rho_1 = rho;
    }
    free(p); free(z); free(q); free(r);
    return st;
}

/* BiCGstab.solve, S/BiCGstab.java:65-116 */
static int bicgstab_solve(int n, const int *rp, const int *ci, const double *v, or_pc *pc,
                          const double *b, double *x, mon_state *m, int *detail)
{
    double rho_1 = 1, rho_2 = 1, alpha = 1, beta = 1, omega = 1;
    size_t sz = (size_t)n + 1;
    double *p = calloc(sz, 8), *s = calloc(sz, 8), *phat = calloc(sz, 8), *shat = calloc(sz, 8);
    double *t = calloc(sz, 8), *vv = calloc(sz, 8), *temp = calloc(sz, 8), *r = calloc(sz, 8);
    double *rtilde = calloc(sz, 8);
    memcpy(r, b, sizeof(double) * (size_t)n);
    or_mult_add(n, rp, ci, v, -1, x, r);
    memcpy(rtilde, r, sizeof(double) * (size_t)n);
    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        rho_1 = or_dot(n, rtilde, r);
        if (rho_1 == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_RHO; break; }
        if (omega == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_OMEGA; break; }
        if (m->iter == 0)
            memcpy(p, r, sizeof(double) * (size_t)n);
        else {
            beta = (rho_1 / rho_2) * (alpha / omega);
            vset_a(n, temp, -omega, vv);
            vadd(n, temp, p);
            memcpy(p, r, sizeof(double) * (size_t)n);
            vadd_a(n, p, beta, temp);
        }
        pc_apply_or_identity(pc, n, p, phat);
        or_mult(n, rp, ci, v, phat, vv);
        alpha = rho_1 / or_dot(n, rtilde, vv);
        memcpy(s, r, sizeof(double) * (size_t)n);
        vadd_a(n, s, -alpha, vv);
        vadd_a(n, x, alpha, phat);
        st = mon_check_vec(m, n, s);
        if (st >= 0) break;
        pc_apply_or_identity(pc, n, s, shat);
        or_mult(n, rp, ci, v, shat, t);
        omega = or_dot(n, t, s) / or_dot(n, t, t);
        vadd_a(n, x, omega, shat);
        memcpy(r, s, sizeof(double) * (size_t)n);
        vadd_a(n, r, -omega, t);
        rho_2 = rho_1;
    }
    free(p); free(s); free(phat); free(shat); free(t); free(vv); free(temp); free(r); free(rtilde);
    return st;
}

/* GivensRotation(x, y), M/GivensRotation.java:42-58 */
static void givens(double x, double y, double *c, double *s)
{
    double roe = fabs(x) > fabs(y) ? x : y;
    double scale = fabs(x) + fabs(y);
    if (scale != 0) {
        double xs = x / scale;
        double ys = y / scale;
        double r = scale * sqrt(xs * xs + ys * ys);
        if (roe < 0) r *= -1;
        *c = x / r;
        *s = y / r;
    } else {
        *c = 1;
        *s = 0;
    }
}

/* GivensRotation.apply on two entries, M/GivensRotation.java:72-92 */
static void givens_apply(double c, double s, double *a1, double *a2)
{
    double temp = c * *a1 + s * *a2;
    *a2 = -s * *a1 + c * *a2;
    *a1 = temp;
}

/* UpperTriangDenseMatrix(H, i, false).solve(s, s), S/GMRES.java:166 ->
 * M/AbstractTriangDenseMatrix.java:228-257 -> LAPACK dtrtrs('U','N','N').
 * dtrtrs reports info = k when A(k,k) == 0 (checked first, k ascending),
 * otherwise solves with dtrsm; the netlib reference dtrsm for one right-hand
 * side, Left/Upper/NoTrans/NonUnit, walks k = n..1: when b(k) != 0,
 * b(k) /= A(k,k) and b(i) -= b(k)*A(i,k) for i < k. */
static int dtrtrs_upper(int nn, const double *H, int ld, double *b)
{
    for (int k = 0; k < nn; ++k)
        if (H[k + (size_t)k * ld] == 0) return k + 1;
    for (int k = nn - 1; k >= 0; --k) {
        if (b[k] != 0) {
            b[k] = b[k] / H[k + (size_t)k * ld];
            for (int i = 0; i < k; ++i) b[i] = b[i] - b[k] * H[i + (size_t)k * ld];
        }
    }
    return 0;
}

/* GMRES.solve, S/GMRES.java:127-176 (restart from GMRES(template, restart),
 * :99-125).  The reference also computes M.apply(b, u) at :134; u is
 * overwritten before any read, so that dead call is not repeated here. */
static int gmres_solve(int restart, int n, const int *rp, const int *ci, const double *v,
                       or_pc *pc, const double *b, double *x, mon_state *m, int *detail)
{
    (void)detail;
    size_t sz = (size_t)n + 1;
    int ld = restart + 1;
    double *w = calloc(sz, 8), *u = calloc(sz, 8), *r = calloc(sz, 8);
    double *s = calloc((size_t)restart + 1, 8);
    double *H = calloc((size_t)(restart + 1) * (size_t)restart, 8);
    double *rc = calloc((size_t)restart + 1, 8), *rs = calloc((size_t)restart + 1, 8);
    double **V = malloc(sizeof(double *) * (size_t)(restart + 1));
    for (int i = 0; i <= restart; ++i) V[i] = calloc(sz, 8);

    memcpy(u, b, sizeof(double) * (size_t)n);
    or_mult_add(n, rp, ci, v, -1, x, u);
    pc_apply_or_identity(pc, n, u, r);
    double normr = or_norm(n, r, OR_NORM_TWO);

    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        vset_a(n, V[0], 1 / normr, r);
        for (int k = 0; k <= restart; ++k) s[k] = 0;
        s[0] = normr;
        int i = 0;
        for (; i < restart; i++, m->iter++) {
            st = mon_check_scalar(m, fabs(s[i]));
            if (st > 0) goto done;     /* exception out of the inner loop */
            if (st == OR_OK) break;
            or_mult(n, rp, ci, v, V[i], u);
            pc_apply_or_identity(pc, n, u, w);
            for (int k = 0; k <= i; k++) {
                H[k + (size_t)i * ld] = or_dot(n, w, V[k]);
                vadd_a(n, w, -H[k + (size_t)i * ld], V[k]);
            }
            H[i + 1 + (size_t)i * ld] = or_norm(n, w, OR_NORM_TWO);
            vset_a(n, V[i + 1], 1. / H[i + 1 + (size_t)i * ld], w);
            for (int k = 0; k < i; ++k)
                givens_apply(rc[k], rs[k], &H[k + (size_t)i * ld], &H[k + 1 + (size_t)i * ld]);
            givens(H[i + (size_t)i * ld], H[i + 1 + (size_t)i * ld], &rc[i], &rs[i]);
            givens_apply(rc[i], rs[i], &H[i + (size_t)i * ld], &H[i + 1 + (size_t)i * ld]);
            givens_apply(rc[i], rs[i], &s[i], &s[i + 1]);
        }
        if (dtrtrs_upper(i, H, ld, s) != 0) { st = OR_ERR_SINGULAR; goto done; }
        for (int j = 0; j < i; j++) vadd_a(n, x, s[j], V[j]);
        memcpy(u, b, sizeof(double) * (size_t)n);
        or_mult_add(n, rp, ci, v, -1, x, u);
        pc_apply_or_identity(pc, n, u, r);
        normr = or_norm(n, r, OR_NORM_TWO);
    }
done:
    for (int i = 0; i <= restart; ++i) free(V[i]);
    free(V); free(w); free(u); free(r); free(s); free(H); free(rc); free(rs);
    return st;
}

static void pc_trans_apply_or_identity(or_pc *pc, int n, const double *b, double *x)
{
    if (pc) or_pc_trans_apply(pc, b, x);
    else if (x != b) memcpy(x, b, sizeof(double) * (size_t)n);
}

static void vcopy(int n, double *d, const double *s) { memcpy(d, s, sizeof(double) * (size_t)n); }

/* BiCG.solve, S/BiCG.java:63-102 */
static int bicg_solve(int n, const int *rp, const int *ci, const double *v, or_pc *pc,
                      const double *b, double *x, mon_state *m, int *detail)
{
    double rho_1 = 1, rho_2 = 1, alpha = 1, beta = 1;
    size_t sz = (size_t)n + 1;
    double *z = calloc(sz, 8), *p = calloc(sz, 8), *q = calloc(sz, 8), *r = calloc(sz, 8);
    double *zt = calloc(sz, 8), *pt = calloc(sz, 8), *qt = calloc(sz, 8), *rt = calloc(sz, 8);
    vcopy(n, r, b);
    or_mult_add(n, rp, ci, v, -1, x, r);
    vcopy(n, rt, r);
    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        pc_apply_or_identity(pc, n, r, z);
        pc_trans_apply_or_identity(pc, n, rt, zt);
        rho_1 = or_dot(n, z, rt);
        if (rho_1 == 0.) { st = OR_NC_BREAKDOWN; *detail = OR_BD_RHO; break; }
        if (m->iter == 0) {
            vcopy(n, p, z);
            vcopy(n, pt, zt);
        } else {
            beta = rho_1 / rho_2;
            vscale(n, p, beta);
            vadd(n, p, z);
            vscale(n, pt, beta);
            vadd(n, pt, zt);
        }
        or_mult(n, rp, ci, v, p, q);
        or_trans_mult(n, n, rp, ci, v, pt, qt);
        alpha = rho_1 / or_dot(n, pt, q);
        vadd_a(n, x, alpha, p);
        vadd_a(n, r, -alpha, q);
        vadd_a(n, rt, -alpha, qt);
        rho_2 = rho_1;
    }
    free(z); free(p); free(q); free(r); free(zt); free(pt); free(qt); free(rt);
    return st;
}

/* CGS.solve, S/CGS.java:65-105 */
static int cgs_solve(int n, const int *rp, const int *ci, const double *v, or_pc *pc,
                     const double *b, double *x, mon_state *m, int *detail)
{
    double rho_1 = 0, rho_2 = 0, alpha = 0, beta = 0;
    size_t sz = (size_t)n + 1;
    double *p = calloc(sz, 8), *q = calloc(sz, 8), *u = calloc(sz, 8), *phat = calloc(sz, 8);
    double *qhat = calloc(sz, 8), *vhat = calloc(sz, 8), *uhat = calloc(sz, 8), *sum = calloc(sz, 8);
    double *r = calloc(sz, 8), *rt = calloc(sz, 8);
    vcopy(n, r, b);
    or_mult_add(n, rp, ci, v, -1, x, r);
    vcopy(n, rt, r);
    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        rho_1 = or_dot(n, rt, r);
        if (rho_1 == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_RHO; break; }
        if (m->iter == 0) {
            vcopy(n, u, r);
            vcopy(n, p, u);
        } else {
            beta = rho_1 / rho_2;
            vcopy(n, u, r);
            vadd_a(n, u, beta, q);
            vcopy(n, sum, q);
            vadd_a(n, sum, beta, p);
            vcopy(n, p, u);
            vadd_a(n, p, beta, sum);
        }
        pc_apply_or_identity(pc, n, p, phat);
        or_mult(n, rp, ci, v, phat, vhat);
        alpha = rho_1 / or_dot(n, rt, vhat);
        vset_a(n, q, -alpha, vhat);
        vadd(n, q, u);
        vcopy(n, sum, u);
        vadd(n, sum, q);
        pc_apply_or_identity(pc, n, sum, uhat);
        vadd_a(n, x, alpha, uhat);
        or_mult(n, rp, ci, v, uhat, qhat);
        vadd_a(n, r, -alpha, qhat);
        rho_2 = rho_1;
    }
    free(p); free(q); free(u); free(phat); free(qhat); free(vhat); free(uhat); free(sum); free(r); free(rt);
    return st;
}

/* QMR.solve, S/QMR.java:117-213, with M1 = M2 = the solver's preconditioner
 * (QMR(Vector), :65-80, and setPreconditioner, :216-220) */
static int qmr_solve(int n, const int *rp, const int *ci, const double *vals, or_pc *pc,
                     const double *b, double *x, mon_state *m, int *detail)
{
    double rho = 0, rho_1 = 0, xi = 0, gamma = 1., gamma_1 = 0, theta = 0, theta_1 = 0,
           eta = -1., delta = 0, ep = 0, beta = 0;
    size_t sz = (size_t)n + 1;
    double *r = calloc(sz, 8), *y = calloc(sz, 8), *z = calloc(sz, 8), *v = calloc(sz, 8);
    double *w = calloc(sz, 8), *p = calloc(sz, 8), *q = calloc(sz, 8), *d = calloc(sz, 8);
    double *s = calloc(sz, 8), *v_tld = calloc(sz, 8), *w_tld = calloc(sz, 8), *y_tld = calloc(sz, 8);
    double *z_tld = calloc(sz, 8), *p_tld = calloc(sz, 8);
    vcopy(n, r, b);
    or_mult_add(n, rp, ci, vals, -1, x, r);
    vcopy(n, v_tld, r);
    pc_apply_or_identity(pc, n, v_tld, y);
    rho = or_norm(n, y, OR_NORM_TWO);
    vcopy(n, w_tld, r);
    pc_trans_apply_or_identity(pc, n, w_tld, z);
    xi = or_norm(n, z, OR_NORM_TWO);
    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        if (rho == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_RHO; break; }
        if (xi == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_XI; break; }
        vset_a(n, v, 1 / rho, v_tld);
        vscale(n, y, 1 / rho);
        vset_a(n, w, 1 / xi, w_tld);
        vscale(n, z, 1 / xi);
        delta = or_dot(n, z, y);
        if (delta == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_DELTA; break; }
        pc_apply_or_identity(pc, n, y, y_tld);
        pc_trans_apply_or_identity(pc, n, z, z_tld);
        if (m->iter == 0) {
            vcopy(n, p, y_tld);
            vcopy(n, q, z_tld);
        } else {
            vscale(n, p, -xi * delta / ep);
            vadd(n, p, y_tld);
            vscale(n, q, -rho * delta / ep);
            vadd(n, q, z_tld);
        }
        or_mult(n, rp, ci, vals, p, p_tld);
        ep = or_dot(n, q, p_tld);
        if (ep == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_EP; break; }
        beta = ep / delta;
        if (beta == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_BETA; break; }
        vset_a(n, v_tld, -beta, v);
        vadd(n, v_tld, p_tld);
        pc_apply_or_identity(pc, n, v_tld, y);
        rho_1 = rho;
        rho = or_norm(n, y, OR_NORM_TWO);
        /* A.transMultAdd(q, w_tld.set(-beta, w)): transMultAdd(1, q, w_tld) */
        vset_a(n, w_tld, -beta, w);
        or_trans_mult_add(n, n, rp, ci, vals, 1, q, w_tld);
        pc_trans_apply_or_identity(pc, n, w_tld, z);
        xi = or_norm(n, z, OR_NORM_TWO);
        gamma_1 = gamma;
        theta_1 = theta;
        theta = rho / (gamma_1 * beta);
        gamma = 1 / sqrt(1 + theta * theta);
        if (gamma == 0) { st = OR_NC_BREAKDOWN; *detail = OR_BD_GAMMA; break; }
        eta = -eta * rho_1 * gamma * gamma / (beta * gamma_1 * gamma_1);
        if (m->iter == 0) {
            vset_a(n, d, eta, p);
            vset_a(n, s, eta, p_tld);
        } else {
            double val = theta_1 * theta_1 * gamma * gamma;
            vscale(n, d, val);
            vadd_a(n, d, eta, p);
            vscale(n, s, val);
            vadd_a(n, s, eta, p_tld);
        }
        vadd(n, x, d);
        vadd_a(n, r, -1, s);
    }
    free(r); free(y); free(z); free(v); free(w); free(p); free(q); free(d); free(s);
    free(v_tld); free(w_tld); free(y_tld); free(z_tld); free(p_tld);
    return st;
}

/* Chebyshev.solve, S/Chebyshev.java:90-120 */
static int chebyshev_solve(double eigmin, double eigmax, int n, const int *rp, const int *ci, const double *v,
                           or_pc *pc, const double *b, double *x, mon_state *m)
{
    double alpha = 0, beta = 0, c = 0, d = 0;
    size_t sz = (size_t)n + 1;
    double *p = calloc(sz, 8), *z = calloc(sz, 8), *r = calloc(sz, 8), *q = calloc(sz, 8);
    vcopy(n, r, b);
    or_mult_add(n, rp, ci, v, -1, x, r);
    c = (eigmax - eigmin) / 2.0;
    d = (eigmax + eigmin) / 2.0;
    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        pc_apply_or_identity(pc, n, r, z);
        if (m->iter == 0) {
            vcopy(n, p, z);
            alpha = 2.0 / d;
        } else {
            beta = (alpha * c) / 2.0;
            beta *= beta;
            alpha = 1.0 / (d - beta);
            vscale(n, p, beta);
            vadd(n, p, z);
        }
        or_mult(n, rp, ci, v, p, q);
        vadd_a(n, x, alpha, p);
        vadd_a(n, r, -alpha, q);
    }
    free(p); free(z); free(r); free(q);
    return st;
}

/* IR.solve, S/IR.java:57-70 */
static int ir_solve(int n, const int *rp, const int *ci, const double *v, or_pc *pc, const double *b,
                    double *x, mon_state *m)
{
    size_t sz = (size_t)n + 1;
    double *z = calloc(sz, 8), *r = calloc(sz, 8);
    vcopy(n, r, b);
    or_mult_add(n, rp, ci, v, -1, x, r);
    int st;
    for (m->iter = 0; (st = mon_check_vec(m, n, r)) < 0; m->iter++) {
        pc_apply_or_identity(pc, n, r, z);
        vadd(n, x, z);
        vcopy(n, r, b);
        or_mult_add(n, rp, ci, v, -1, x, r);
    }
    free(z); free(r);
    return st;
}

int or_solve(int kind, int restart, int n, const int *rowptr, const int *colind,
             const double *val, or_pc *pc, const double *b, double *x,
             const or_monitor *mon, or_result *res,
             double *hist_r, int *hist_it, int hist_cap)
{
    return or_solve_ex(kind, restart, 0.0, 0.0, n, rowptr, colind, val, pc, b, x, mon, res, hist_r, hist_it,
                       hist_cap);
}

int or_solve_ex(int kind, int restart, double eigmin, double eigmax, int n, const int *rowptr,
                const int *colind, const double *val, or_pc *pc, const double *b, double *x,
                const or_monitor *mon, or_result *res, double *hist_r, int *hist_it, int hist_cap)
{
    mon_state m;
    memset(&m, 0, sizeof(m));
    m.cfg = mon;
    m.n = n;
    m.x = x;
    m.hist_r = hist_r;
    m.hist_it = hist_it;
    m.hist_cap = hist_r && hist_it ? hist_cap : 0;
    int detail = 0, st;
    if (pc && pc->n != n) return OR_ERR_ILLEGAL_ARGUMENT;
    if (kind == OR_CG) st = cg_solve(n, rowptr, colind, val, pc, b, x, &m, &detail);
    else if (kind == OR_BICGSTAB) st = bicgstab_solve(n, rowptr, colind, val, pc, b, x, &m, &detail);
    else if (kind == OR_BICG) st = bicg_solve(n, rowptr, colind, val, pc, b, x, &m, &detail);
    else if (kind == OR_CGS) st = cgs_solve(n, rowptr, colind, val, pc, b, x, &m, &detail);
    else if (kind == OR_QMR) st = qmr_solve(n, rowptr, colind, val, pc, b, x, &m, &detail);
    else if (kind == OR_CHEBYSHEV) {
        /* Chebyshev.setEigenvalues, S/Chebyshev.java:78-88 */
        if (eigmin <= 0 || eigmax <= 0 || eigmin > eigmax) return OR_ERR_ILLEGAL_ARGUMENT;
        st = chebyshev_solve(eigmin, eigmax, n, rowptr, colind, val, pc, b, x, &m);
    } else if (kind == OR_IR) st = ir_solve(n, rowptr, colind, val, pc, b, x, &m);
    else {
        if (restart <= 0) return OR_ERR_ILLEGAL_ARGUMENT;
        st = gmres_solve(restart, n, rowptr, colind, val, pc, b, x, &m, &detail);
    }
    if (res) {
        res->status = st;
        res->iterations = m.iter;
        res->residual = m.residual;
        res->detail = detail;
        res->history_len = m.hist_len;
    }
    return st;
}
