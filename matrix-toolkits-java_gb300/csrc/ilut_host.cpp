// ilut_host.cpp -- MTJ's ILUT factor (S/ILUT.java:119-272) on the host.
//
// MTJ's ILUT is a row-by-row elimination with a dense work row: row i is
// scattered into LUi, every earlier row k (in ascending order) whose
// multiplier LUi[k] / u_kk is larger in magnitude than taui = tau |row i|_2
// is eliminated, and the row is gathered back keeping the diagonal, the
// (nl + p) largest lower and (nu + p) largest upper entries above taui (nl,
// nu: the row's entry counts before).  Row i reads every finished earlier
// row, so the factor is a chain over the rows: set-up work, run once per
// matrix on the host; its two triangular solves run on the GPU.
//
// Restated over row reaches: an earlier row k changes the work row only when
// LUi[k] is nonzero (a zero multiplier is at most taui when taui >= 0), and
// LUi[k] becomes nonzero only by being in row i or by an update from a row
// already visited; visiting exactly those k in ascending order performs the
// same floating-point operations in the same order.  A row whose taui is
// negative or NaN visits every k, as the Java loop does.  The zero-diagonal
// check of the Java loop (every k < i, at every row i) reduces to row i - 1
// at row i: the earlier rows were checked at the rows before.
//
// The gathered rows keep SparseVector's storage rules (S/SparseVector.java:
// 157-242): zero() clears values and the used count but not the index
// array, inserts shift within the storage or move to doubled, zero-filled
// storage.  MTJ then keeps a row's old diagonal position whenever the index
// array still holds i there (S/ILUT.java:200-207) -- true of a stale slot
// too.  That can only leave the last row without its stored diagonal (any
// earlier row would fail the next row's zero-diagonal check); MTJ's solves
// would then divide by that empty slot and read the previous apply's work
// vector.  That one case is reported as unsupported.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <queue>
#include <string>
#include <vector>

#include "internal.h"

namespace mtjg {
namespace {

struct SvRow {
    std::vector<int> index;   // capacity = size()
    std::vector<double> data;
    int used = 0;
};

// Arrays.binarySearchGreater(index, key, 0, used) (S/Arrays.java:123-156)
int sv_greater(const SvRow &v, int key)
{
    int begin = 0, end = v.used;
    if (begin == end) return end;
    end--;
    int mid = (end + begin) >> 1;
    while (begin <= end) {
        mid = (end + begin) >> 1;
        if (v.index[mid] < key) begin = mid + 1;
        else if (v.index[mid] > key) end = mid - 1;
        else return mid;
    }
    return v.index[mid] >= key ? mid : mid + 1;
}

// SparseVector.set via getIndex (S/SparseVector.java:157-164, :188-231)
void sv_set(SvRow &v, int ind, double value, int size)
{
    int i = sv_greater(v, ind);
    if (!(i < v.used && v.index[i] == ind)) {
        const int tail = v.used - i;  // entries that move one slot up
        v.used++;
        if (v.used > (int)v.data.size()) {
            int len = v.data.empty() ? 1 : (int)v.data.size() << 1;
            len = std::min(len, size);
            std::vector<int> ni(len, 0);
            std::vector<double> nd(len, 0.0);
            std::copy(v.index.begin(), v.index.begin() + i, ni.begin());
            std::copy(v.data.begin(), v.data.begin() + i, nd.begin());
            std::copy(v.index.begin() + i, v.index.begin() + i + tail, ni.begin() + i + 1);
            std::copy(v.data.begin() + i, v.data.begin() + i + tail, nd.begin() + i + 1);
            v.index.swap(ni);
            v.data.swap(nd);
        } else if (tail > 0) {
            std::copy_backward(v.index.begin() + i, v.index.begin() + i + tail, v.index.begin() + i + tail + 1);
            std::copy_backward(v.data.begin() + i, v.data.begin() + i + tail, v.data.begin() + i + tail + 1);
        }
        v.index[i] = ind;
        v.data[i] = 0.;
    }
    v.data[i] = value;
}

// java.util.Arrays.binarySearch over [0, used)
int sv_find(const SvRow &v, int key)
{
    int lo = 0, hi = v.used - 1;
    while (lo <= hi) {
        const int mid = (int)(((unsigned)lo + (unsigned)hi) >> 1);
        if (v.index[mid] < key) lo = mid + 1;
        else if (v.index[mid] > key) hi = mid - 1;
        else return mid;
    }
    return -(lo + 1);
}

struct Cand {
    int index;
    double value;
};

}  // namespace

// Factors A (0-based CSR) as ILUT(tau, p).  Out: the factor's rows in CSR
// form (positions [0, max(used, diag + 1)) of each row's storage), the
// diagonal's absolute position per row.  *err_row gets the number MTJ's
// message prints.
int ilut_factor_host(int n, const int *rowptr, const int *colind, const double *val, double tau, int p,
                     std::vector<int> &out_rp, std::vector<int> &out_ci, std::vector<double> &out_v,
                     std::vector<int> &out_diag, int *err_row)
{
    std::vector<SvRow> rows((size_t)n);
    // LU.set(A); LU.compact(): each row holds A's nonzero entries, storage full
    for (int k = 0; k < n; ++k) {
        SvRow &r = rows[(size_t)k];
        for (int j = rowptr[k]; j < rowptr[k + 1]; ++j)
            if (val[j] != 0.) {
                r.index.push_back(colind[j]);
                r.data.push_back(val[j]);
            }
        r.used = (int)r.index.size();
    }
    std::vector<int> diag((size_t)n);
    for (int k = 0; k < n; ++k) {
        diag[(size_t)k] = sv_find(rows[(size_t)k], k);
        if (diag[(size_t)k] < 0) {
            *err_row = k + 1;
            return fail(MTJG_ERR_MISSING_DIAGONAL, "Missing diagonal entry on row " + std::to_string(k + 1));
        }
    }
    std::vector<double> LUi((size_t)std::max(1, n), 0.0);
    std::vector<unsigned char> mark((size_t)std::max(1, n), 0);
    std::vector<int> touched;
    std::vector<Cand> lower, upper;
    std::priority_queue<int, std::vector<int>, std::greater<int>> heap;
    for (int i = 1; i < n; ++i) {
        SvRow &rowi = rows[(size_t)i];
        // the zero-diagonal check of row i - 1 (S/ILUT.java:163-166)
        {
            const SvRow &rk = rows[(size_t)(i - 1)];
            if (rk.data[(size_t)diag[(size_t)(i - 1)]] == 0) {
                *err_row = i;
                return fail(MTJG_ERR_ZERO_DIAGONAL,
                            "Zero diagonal entry on row " + std::to_string(i) + " during ILU process");
            }
        }
        double norm = 0;
        for (int j = 0; j < rowi.used; ++j) norm += rowi.data[(size_t)j] * rowi.data[(size_t)j];
        const double taui = std::sqrt(norm) * tau;
        touched.clear();
        for (int j = 0; j < rowi.used; ++j) {
            const int c = rowi.index[(size_t)j];
            LUi[(size_t)c] = rowi.data[(size_t)j];
            mark[(size_t)c] = 1;
            touched.push_back(c);
            if (c < i) heap.push(c);
        }
        auto eliminate = [&](int k) {
            const SvRow &rk = rows[(size_t)k];
            const int dk = diag[(size_t)k];
            const double LUik = LUi[(size_t)k] / rk.data[(size_t)dk];
            if (std::fabs(LUik) <= taui) return;
            for (int j = dk + 1; j < rk.used; ++j) {
                const int c = rk.index[(size_t)j];
                LUi[(size_t)c] -= LUik * rk.data[(size_t)j];
                if (!mark[(size_t)c]) {
                    mark[(size_t)c] = 1;
                    touched.push_back(c);
                    if (c < i) heap.push(c);
                }
            }
            LUi[(size_t)k] = LUik;
        };
        if (taui >= 0) {
            while (!heap.empty()) {
                const int k = heap.top();
                heap.pop();
                eliminate(k);
            }
        } else {
            while (!heap.empty()) heap.pop();
            for (int k = 0; k < i; ++k) {
                if (!mark[(size_t)k]) {
                    mark[(size_t)k] = 1;
                    touched.push_back(k);
                }
                eliminate(k);
            }
        }
        // ILUT.gather (S/ILUT.java:225-272)
        int nl = 0, nu = 0;
        for (int j = 0; j < rowi.used; ++j) {
            if (rowi.index[(size_t)j] < i) nl++;
            else if (rowi.index[(size_t)j] > i) nu++;
        }
        std::fill(rowi.data.begin(), rowi.data.end(), 0.0);
        rowi.used = 0;
        std::sort(touched.begin(), touched.end());
        lower.clear();
        upper.clear();
        if (taui >= 0) {
            // an entry never touched is 0, which is not above taui
            for (int c : touched) {
                const double z = LUi[(size_t)c];
                if (c < i && std::fabs(z) > taui) lower.push_back(Cand{c, z});
                else if (c > i && std::fabs(z) > taui) upper.push_back(Cand{c, z});
            }
        } else {
            for (int c = 0; c < n; ++c) {
                const double z = LUi[(size_t)c];
                if (c < i && std::fabs(z) > taui) lower.push_back(Cand{c, z});
                else if (c > i && std::fabs(z) > taui) upper.push_back(Cand{c, z});
            }
        }
        auto by_mag = [](const Cand &a, const Cand &b) { return std::fabs(a.value) > std::fabs(b.value); };
        std::stable_sort(lower.begin(), lower.end(), by_mag);
        std::stable_sort(upper.begin(), upper.end(), by_mag);
        sv_set(rowi, i, LUi[(size_t)i], n);
        const int ml = std::min(nl + p, (int)lower.size()), mu = std::min(nu + p, (int)upper.size());
        for (int t = 0; t < ml; ++t) sv_set(rowi, lower[(size_t)t].index, lower[(size_t)t].value, n);
        for (int t = 0; t < mu; ++t) sv_set(rowi, upper[(size_t)t].index, upper[(size_t)t].value, n);
        const int di = diag[(size_t)i];
        if (di >= (int)rowi.index.size() || rowi.index[(size_t)di] != i) diag[(size_t)i] = sv_find(rowi, i);
        for (int c : touched) {
            LUi[(size_t)c] = 0.0;
            mark[(size_t)c] = 0;
        }
    }
    if (n > 0 && diag[(size_t)(n - 1)] >= rows[(size_t)(n - 1)].used) {
        *err_row = n;
        return fail(MTJG_ERR_UNSUPPORTED, "ILUT left row " + std::to_string(n) +
                                              " without its stored diagonal (MTJ's solves would divide by an "
                                              "empty slot and read the previous apply's work vector)");
    }
    out_rp.assign((size_t)n + 1, 0);
    out_ci.clear();
    out_v.clear();
    out_diag.assign((size_t)n, 0);
    for (int i = 0; i < n; ++i) {
        const SvRow &r = rows[(size_t)i];
        const int len = std::max(r.used, diag[(size_t)i] + 1);
        out_diag[(size_t)i] = (int)out_ci.size() + diag[(size_t)i];
        out_ci.insert(out_ci.end(), r.index.begin(), r.index.begin() + len);
        out_v.insert(out_v.end(), r.data.begin(), r.data.begin() + len);
        out_rp[(size_t)i + 1] = (int)out_ci.size();
    }
    return MTJG_OK;
}

}  // namespace mtjg
