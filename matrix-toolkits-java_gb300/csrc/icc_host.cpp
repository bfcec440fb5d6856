// icc_host.cpp -- MTJ's ICC factorization (S/ICC.java:85-139) on the host.
//
// MTJ's ICC is not textbook IC(0): row k is expanded into a dense work row,
// every earlier row i with a nonzero multiplier Rk[i]/R_ii updates it over
// row i's stored upper pattern, and fill created left of the diagonal keeps
// acting as a multiplier.  Only row k's own pattern (diagonal and right) is
// stored, divided by sqrt(Rk[k]).  The literal loop visits every i < k
// (O(n^2)); only rows whose work entry can be nonzero change anything, so
// this version visits exactly the columns reached from row k's pattern, in
// ascending order, through a three-level bitmap, and performs the same
// floating-point operations in the same order.  Must be compiled with
// -ffp-contract=off.
//
// Rows form a dependency chain (row k reads the finished rows of its reach),
// so the factor is pipelined over host threads: row k goes to thread
// k mod T, and before it reads row i it waits for row i's completion flag.
// The order of every row's own operations does not change.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace mtjg {

namespace {

class OrderedSet {
public:
    explicit OrderedSet(int n) : n_(n)
    {
        w0_.assign((size_t)((n + 63) / 64) + 1, 0);
        w1_.assign(w0_.size() / 64 + 2, 0);
        w2_.assign(w1_.size() / 64 + 2, 0);
    }
    void set(int c)
    {
        const size_t a = (size_t)c >> 6, b = a >> 6, d = b >> 6;
        w0_[a] |= 1ULL << (c & 63);
        w1_[b] |= 1ULL << (a & 63);
        w2_[d] |= 1ULL << (b & 63);
    }
    void clear(int c)
    {
        const size_t a = (size_t)c >> 6, b = a >> 6, d = b >> 6;
        w0_[a] &= ~(1ULL << (c & 63));
        if (w0_[a] == 0) {
            w1_[b] &= ~(1ULL << (a & 63));
            if (w1_[b] == 0) w2_[d] &= ~(1ULL << (b & 63));
        }
    }
    // smallest member >= p, or -1
    int next(int p) const
    {
        if (p >= n_) return -1;
        size_t a = (size_t)p >> 6;
        uint64_t bits = w0_[a] & (~0ULL << (p & 63));
        if (bits) return (int)(a * 64 + __builtin_ctzll(bits));
        size_t a1 = a + 1;
        size_t b = a1 >> 6;
        if (b < w1_.size()) {
            uint64_t bb = w1_[b] & (a1 & 63 ? (~0ULL << (a1 & 63)) : ~0ULL);
            if (bb) {
                size_t aa = b * 64 + __builtin_ctzll(bb);
                return (int)(aa * 64 + __builtin_ctzll(w0_[aa]));
            }
        }
        size_t b1 = b + 1;
        size_t d = b1 >> 6;
        for (size_t dd = d; dd < w2_.size(); ++dd) {
            uint64_t db = w2_[dd];
            if (dd == d) db &= (b1 & 63 ? (~0ULL << (b1 & 63)) : ~0ULL);
            if (db) {
                size_t bb = dd * 64 + __builtin_ctzll(db);
                size_t aa = bb * 64 + __builtin_ctzll(w1_[bb]);
                return (int)(aa * 64 + __builtin_ctzll(w0_[aa]));
            }
        }
        return -1;
    }

private:
    int n_;
    std::vector<uint64_t> w0_, w1_, w2_;
};

struct Shared {
    int n;
    const int *rowptr, *colind, *diag;
    const double *orig;  // A's values (row k's expansion reads them)
    double *data;        // factor, written row by row
    std::atomic<uint8_t> *done;  // 0 pending, 1 finished, 2 failed
    std::atomic<int> err_row;    // smallest failing row message number
    std::atomic<int> err_code;
    std::atomic<int> nan_row;    // smallest row whose stored diagonal is NaN (n if none)
};

// Waits for row i; returns false if it failed.
inline bool wait_row(Shared &sh, int i)
{
    uint8_t v = sh.done[i].load(std::memory_order_acquire);
    int spins = 0;
    while (v == 0) {
        if (++spins > 64) std::this_thread::yield();
        v = sh.done[i].load(std::memory_order_acquire);
    }
    return v == 1;
}

inline void record_error(Shared &sh, int code, int row)
{
    int cur = sh.err_row.load();
    while (row < cur && !sh.err_row.compare_exchange_weak(cur, row)) {
    }
    if (sh.err_row.load() == row) sh.err_code.store(code);
}

// Factors row k.  nan_rows: rows < k whose diagonal is NaN (only used by
// the sequential pass after a NaN appeared).  Returns 1 ok, 2 failed.
int factor_row(Shared &sh, int k, std::vector<double> &Rk, std::vector<unsigned char> &mark,
               std::vector<int> &touched, OrderedSet &pending, const std::vector<int> *nan_rows, bool wait)
{
    const int *rp = sh.rowptr, *ci = sh.colind, *dg = sh.diag;
    double *data = sh.data;
    touched.clear();
    for (int e = rp[k]; e < rp[k + 1]; ++e) {
        const int c = ci[e];
        Rk[c] = sh.orig[e];
        if (!mark[c]) {
            mark[c] = 1;
            touched.push_back(c);
        }
        if (c < k) pending.set(c);
    }
    if (nan_rows)
        for (int c : *nan_rows) {
            if (c >= k) break;
            if (!mark[c]) {
                mark[c] = 1;
                touched.push_back(c);
            }
            pending.set(c);
        }
    int status = 1;
    for (int i = pending.next(0); i >= 0 && i < k; i = pending.next(i + 1)) {
        pending.clear(i);
        if (wait && !wait_row(sh, i)) {
            status = 2;
            break;
        }
        const double Rii = data[dg[i]];
        if (Rii == 0) {
            record_error(sh, MTJG_ERR_ZERO_PIVOT, i + 1);
            status = 2;
            break;
        }
        const double Rki = Rk[i] / Rii;
        if (Rki == 0) continue;
        for (int j = dg[i] + 1; j < rp[i + 1]; ++j) {
            const int c = ci[j];
            Rk[c] -= Rki * data[j];
            if (!mark[c]) {
                mark[c] = 1;
                touched.push_back(c);
                if (c < k) pending.set(c);
            }
        }
    }
    if (status == 1) {
        if (Rk[k] == 0) {
            record_error(sh, MTJG_ERR_ZERO_DIAGONAL, k + 1);
            status = 2;
        } else {
            const double sq = std::sqrt(Rk[k]);
            for (int e = dg[k]; e < rp[k + 1]; ++e) data[e] = Rk[ci[e]] / sq;
            if (std::isnan(data[dg[k]])) {
                int cur = sh.nan_row.load();
                while (k < cur && !sh.nan_row.compare_exchange_weak(cur, k)) {
                }
            }
        }
    }
    // drain pending entries left by an early exit
    for (int i = pending.next(0); i >= 0; i = pending.next(i + 1)) pending.clear(i);
    for (int c : touched) {
        Rk[c] = 0.0;
        mark[c] = 0;
    }
    return status;
}

}  // namespace

int icc_factor_host(int n, const int *rowptr, const int *colind, const int *diag, double *data, int *err_row)
{
    if (n == 0) return MTJG_OK;
    const int64_t nnz = rowptr[n];
    std::vector<double> orig(data, data + nnz);
    std::vector<std::atomic<uint8_t>> done(n);
    for (auto &d : done) d.store(0, std::memory_order_relaxed);
    Shared sh;
    sh.n = n;
    sh.rowptr = rowptr;
    sh.colind = colind;
    sh.diag = diag;
    sh.orig = orig.data();
    sh.data = data;
    sh.done = done.data();
    sh.err_row.store(0x7fffffff);
    sh.err_code.store(MTJG_OK);
    sh.nan_row.store(n);

    unsigned hw = std::thread::hardware_concurrency();
    int T = (int)std::min<unsigned>(hw ? hw : 1, 16);
    if (n < 4096) T = 1;
    auto worker = [&](int tid) {
        std::vector<double> Rk((size_t)n, 0.0);
        std::vector<unsigned char> mark((size_t)n, 0);
        std::vector<int> touched;
        OrderedSet pending(n);
        for (int k = tid; k < n; k += T) {
            int st = factor_row(sh, k, Rk, mark, touched, pending, nullptr, T > 1);
            sh.done[k].store((uint8_t)st, std::memory_order_release);
        }
    };
    if (T == 1) {
        worker(0);
    } else {
        std::vector<std::thread> th;
        for (int t = 0; t < T; ++t) th.emplace_back(worker, t);
        for (auto &t : th) t.join();
    }
    // A NaN diagonal (negative pivot) makes MTJ's 0/NaN multiplier nonzero,
    // so that row then updates every later row: redo the rows after the
    // first NaN row sequentially with those rows added to every reach.
    const int first_nan = sh.nan_row.load();
    const int first_err = sh.err_row.load();
    if (first_nan < n && (first_err == 0x7fffffff || first_err - 1 > first_nan)) {
        if (first_err != 0x7fffffff) {
            sh.err_row.store(0x7fffffff);
            sh.err_code.store(MTJG_OK);
        }
        std::vector<double> Rk((size_t)n, 0.0);
        std::vector<unsigned char> mark((size_t)n, 0);
        std::vector<int> touched, nan_rows = {first_nan};
        OrderedSet pending(n);
        for (int k = first_nan + 1; k < n; ++k) {
            for (int e = diag[k]; e < rowptr[k + 1]; ++e) data[e] = orig[e];
            if (factor_row(sh, k, Rk, mark, touched, pending, &nan_rows, false) != 1) break;
            if (std::isnan(data[diag[k]])) nan_rows.push_back(k);
        }
    }
    if (sh.err_row.load() != 0x7fffffff) {
        *err_row = sh.err_row.load();
        const int code = sh.err_code.load();
        if (code == MTJG_ERR_ZERO_DIAGONAL)
            return fail(code, "Zero diagonal entry encountered on row " + std::to_string(*err_row) +
                                  " during ICC process");
        return fail(code, "Zero pivot encountered on row " + std::to_string(*err_row) + " during ICC process");
    }
    return MTJG_OK;
}

}  // namespace mtjg
