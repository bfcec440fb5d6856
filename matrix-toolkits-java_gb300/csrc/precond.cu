// precond.cu -- Jacobi, ILU(0) and ICC preconditioners (S/DiagonalPreconditioner.java,
// S/ILU.java, S/ICC.java) with level-scheduled triangular solves.
//
// Levels of a triangular operator are found on the device by k_levels: warps
// take rows in dependency order from a ticket counter and each row waits
// (bounded) for the levels of the rows it reads, so one launch finds all
// levels in O(nnz).  The rows are then grouped by level on the host (a
// counting sort, stable in row index) and cut into chunks of at most 32 rows
// of one level.
//
// A triangular solve is one launch (k_trsv_sweep).  Its output vector is
// first filled with kPending, a signalling NaN that no arithmetic produces
// (an operation on a signalling NaN returns a quiet one).  Warps take chunks
// in level order from a ticket counter, one row per lane; a row reads the
// entries x_c it depends on with relaxed loads, polling (bounded) while one
// still holds kPending, and stores its own x_i with a single 64-bit store.
// The value is its own ready flag: no fence, no counter, no level barrier,
// and a row starts as soon as the rows it reads are done, so the sweep runs
// at the depth of the dependency graph times one L2 round trip.  A row waits
// only on rows of lower levels, whose tickets were all handed to running
// warps before its own, so the sweep cannot deadlock.  Each row sums in
// MTJ's entry order, so results are those of the row-by-row Java loop.
#include <algorithm>
#include <cstdlib>
#include <cstring>

#include "spmv.cuh"

namespace mtjg {

int icc_factor_host(int n, const int *rowptr, const int *colind, const int *diag, double *data, int *err_row);
int ilut_factor_host(int n, const int *rowptr, const int *colind, const double *val, double tau, int p,
                     std::vector<int> &out_rp, std::vector<int> &out_ci, std::vector<double> &out_v,
                     std::vector<int> &out_diag, int *err_row);

constexpr long long kSpinLimit = 1LL << 24;

// ------------------------------------------------------------- kernels
__global__ void k_find_diag(int n, const int *rp, const int *ci, int *diag, int *err_min)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int lo = rp[k], hi = rp[k + 1] - 1, pos = -1;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            int v = ci[mid];
            if (v < k) lo = mid + 1;
            else if (v > k) hi = mid - 1;
            else { pos = mid; break; }
        }
        diag[k] = pos;
        if (pos < 0) atomicMin(err_min, k + 1);
    }
}

// DiagonalPreconditioner.setMatrix, S/DiagonalPreconditioner.java:64-76:
// invdiag = 1 / A.get(i,i) (binary search, CompRowMatrix.get S/CompRowMatrix.java:407-417).
__global__ void k_jacobi_set(int n, const int *rp, const int *ci, const double *val, double *invdiag, int *err_min)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        int lo = rp[k], hi = rp[k + 1] - 1;
        double d = 0.0;
        while (lo <= hi) {
            int mid = (lo + hi) >> 1;
            int v = ci[mid];
            if (v < k) lo = mid + 1;
            else if (v > k) hi = mid - 1;
            else { d = val[mid]; break; }
        }
        if (d == 0) atomicMin(err_min, k + 1);
        invdiag[k] = 1 / d;
    }
}

// DiagonalPreconditioner.apply, S/DiagonalPreconditioner.java:54-55
__global__ void k_jacobi_apply(int n, const double *invdiag, const double *b, double *x, const int *status)
{
    if (status && *status != ST_RUNNING) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = b[i] * invdiag[i];
}

__global__ void k_copy(int n, const double *b, double *x, const int *status)
{
    if (status && *status != ST_RUNNING) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = b[i];
}

__device__ __forceinline__ int wait_level(const int *level, int d, bool &bad)
{
    const volatile int *L = level;
    int v = L[d];
    long long polls = 0;
    while (v < 0) {
        if (++polls > kSpinLimit) {
            bad = true;
            return 0;
        }
        __nanosleep(32);
        v = L[d];
    }
    return v;
}

// Dependency levels.  Row i reads rows ci[k] for k in its range:
//   range 0: [rp[i], rp[i+1]), range 1: [rp[i], diag[i]), range 2: (diag[i], rp[i+1]).
// desc: rows are taken from n-1 down (dependencies have larger indices).
// quirk (ILU factor only): row i also reads row i-1 when quirk[i-1] is set.
__global__ void k_levels(int n, int desc, int range, const int *rp, const int *ci, const int *diag,
                         const unsigned char *quirk, int *level, unsigned *ticket, int *err)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned base = 0;
        if (lane == 0) base = atomicAdd(ticket, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= (unsigned)n) return;
        const unsigned t = base + lane;
        if (t < (unsigned)n) {
            const int i = desc ? n - 1 - (int)t : (int)t;
            int b, e;
            if (range == 0) { b = rp[i]; e = rp[i + 1]; }
            else if (range == 1) { b = rp[i]; e = diag[i]; }
            else { b = diag[i] + 1; e = rp[i + 1]; }
            bool bad = false;
            int lvl = 0;
            for (int k = b; k < e; ++k) lvl = max(lvl, wait_level(level, ci[k], bad) + 1);
            if (quirk && i > 0 && quirk[i - 1]) lvl = max(lvl, wait_level(level, i - 1, bad) + 1);
            if (bad) atomicExch(err, 1);
            __threadfence();
            ((volatile int *)level)[i] = lvl;
        }
    }
}

// Marks rows k whose ILU elimination (S/ILU.java:113-120) ends a scan at
// l == rowptr[k+1] on a matching column, i.e. updates the first entry of row
// k+1.  Row k+1 must then be factored after row k.
__global__ void k_ilu_quirk(int n, const int *rp, const int *ci, const int *diag, unsigned char *quirk)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        unsigned char q = 0;
        if (k >= 1 && k + 1 < n) {
            for (int i = rp[k]; i < diag[k]; ++i) {
                const int index = ci[i];
                for (int j = diag[index] + 1, l = rp[k] + 1; j < rp[index + 1]; ++j) {
                    while (l < rp[k + 1] && ci[l] < ci[j]) l++;
                    if (l == rp[k + 1] && ci[l] == ci[j]) q = 1;
                }
            }
        }
        quirk[k] = q;
    }
}

// ILU.factor for the rows of one level (S/ILU.java:98-121), rounding each
// product and difference separately as Java does, so the factor is
// bit-identical to MTJ's.  err_min collects MTJ's message number (entry i+1)
// of the first zero pivot.
__global__ void k_ilu_level(const int *perm, int beg, int cnt, const int *rp, const int *ci, const int *diag,
                            double *data, int *err_min)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt) return;
    const int k = perm[beg + t];
    if (k == 0) return;
    for (int i = rp[k]; i < diag[k]; ++i) {
        const int index = ci[i];
        const double LUii = data[diag[index]];
        if (LUii == 0) {
            atomicMin(err_min, i + 1);
            return;
        }
        const double LUki = data[i] / LUii;
        data[i] = LUki;
        for (int j = diag[index] + 1, l = rp[k] + 1; j < rp[index + 1]; ++j) {
            while (l < rp[k + 1] && ci[l] < ci[j]) l++;
            if (ci[l] == ci[j]) data[l] = __dsub_rn(data[l], __dmul_rn(LUki, data[j]));
        }
    }
}

// ---------------------------------------------------- triangular sweeps
// x entries not yet solved hold this signalling NaN (FP64; kPending32 in the
// FP32 sweeps of the mixed-precision inner solves).
constexpr unsigned long long kPending = 0x7FF40000DEADBEEFull;
constexpr unsigned long long kQuietNaN = 0x7FF8000000000000ull;
constexpr unsigned kPending32 = 0x7FA0BEEFu;
constexpr unsigned kQuietNaN32 = 0x7FC00000u;
constexpr long long kSweepSpinLimit = 1LL << 21;
constexpr int kSweepBlock = 128;
// warps per SM a sweep launches, and polls of a pending entry before the
// poller starts to sleep between polls; both can be set in the environment
// (MTJG_SWEEP_WARPS, MTJG_SWEEP_SPIN) to tune them
// (measured on GB300, 3D Poisson 128^3 ICC and 96^3 convection-diffusion
// ILU applies: sleeping between polls costs more than the polls -- 2.6 vs
// 1.7 ms per ICC apply at 4 warps per SM -- and fewer pollers win: 32 warps
// per SM 2.2 ms against 1.7 ms at 4 or 8)
constexpr int kSweepWarpsPerSm = 8;
constexpr int kSweepSpin = 4096;

static int env_int(const char *name, int dflt, int lo, int hi)
{
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    const int x = atoi(v);
    return x < lo ? lo : (x > hi ? hi : x);
}

// the sweep modes (bit m: MODE m, m <= 2) that look ahead; the environment
// (MTJG_SWEEP_LOOKAHEAD, a bit mask) can change the set
static bool sweep_lookahead(int mode, int dflt)
{
    return (env_int("MTJG_SWEEP_LOOKAHEAD", dflt, 0, 7) >> mode) & 1;
}

__device__ __forceinline__ double ld_relaxed(const double *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return __longlong_as_double((long long)v);
}

__device__ __forceinline__ void st_relaxed(double *p, double v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"((unsigned long long)__double_as_longlong(v))
                 : "memory");
}

__device__ __forceinline__ float ld_relaxed(const float *p)
{
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return __uint_as_float(v);
}

__device__ __forceinline__ void st_relaxed(float *p, float v)
{
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(__float_as_uint(v)) : "memory");
}

__device__ __forceinline__ bool pending(double v) { return (unsigned long long)__double_as_longlong(v) == kPending; }
__device__ __forceinline__ bool pending(float v) { return __float_as_uint(v) == kPending32; }
template <class T>
__device__ __forceinline__ T pending_value();
template <>
__device__ __forceinline__ double pending_value<double>() { return __longlong_as_double((long long)kPending); }
template <>
__device__ __forceinline__ float pending_value<float>() { return __uint_as_float(kPending32); }
// a result that happens to carry the pending pattern is stored as a quiet NaN
__device__ __forceinline__ double unpend(double v) { return pending(v) ? __longlong_as_double((long long)kQuietNaN) : v; }
__device__ __forceinline__ float unpend(float v) { return pending(v) ? __uint_as_float(kQuietNaN32) : v; }

// Fills the outputs of the coming sweeps with the pending pattern and resets
// their ticket counters.  x2 may be null.
template <class T>
__global__ void k_sweep_prep(int n, T *x1, T *x2, unsigned *t1, unsigned *t2, const int *status)
{
    if (status && *status != ST_RUNNING) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (t1) *t1 = 0u;
        if (t2) *t2 = 0u;
    }
    const T p = pending_value<T>();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x1[i] = p;
        if (x2) x2[i] = p;
    }
}

// x_c for a row of the sweep: a relaxed load, polled while it is pending.
// Gives up (bad) after kSweepSpinLimit polls or when another wait has given
// up (the context's error flag is set).
template <class T>
__device__ __forceinline__ T wait_x(const T *x, int c, const int *err, int spin, bool &bad)
{
    T v = ld_relaxed(x + c);
    if (!pending(v)) return v;
    unsigned ns = 32;
    for (long long polls = 1;; ++polls) {
        if (polls > spin) {
            __nanosleep(ns);
            ns = ns < 256 ? 2 * ns : ns;
        }
        v = ld_relaxed(x + c);
        if (!pending(v)) return v;
        if (polls > kSweepSpinLimit || ((polls & 31) == 0 && *(volatile const int *)err)) {
            bad = true;
            return T(0);
        }
    }
}

// Lookahead (MODE 0-2): a row whose dependency x_c is still pending computes
// x_c itself -- the operations of row c's own lane, in the same order, so
// the same bits (the stored, unpended form) -- from the values of row c's
// dependencies, two levels back.  Row c's entries (at most kDepMax) and its
// finishing operands are loaded when the chunk starts, before any wait, so
// a published value travels two levels per L2 round trip instead of one.
constexpr int kDepMax = 4;
// Modes that look ahead by default (bit m: MODE m), measured on GB300 with
// the results unchanged.  FP32 L and U sweeps (the mixed C3 solves' ILU):
// 8-10 % faster solves.  FP64: the L sweep gains (C3 BiCGstab + ILU 111.2 ->
// 107.3 ms); the U sweep and ICC's transposed gather lose 3-4 % each, as
// their recomputed rows repeat a division on the narrow FP64 pipe.
constexpr int kLookaheadModes32 = 3;
#ifndef MTJG_LOOKAHEAD64
#define MTJG_LOOKAHEAD64 1
#endif
constexpr int kLookaheadModes64 = MTJG_LOOKAHEAD64;

template <class T>
struct DepRow {
    int n;  // entries of row c in the sweep's range; -1: not held (wait for x_c instead)
    int col[kDepMax];
    T val[kDepMax];
    T b, dfin;
};

template <int MODE>
__device__ __forceinline__ void sweep_range(int i, const int *rp, const int *diag, int &kb, int &ke)
{
    if constexpr (MODE == 0) {
        kb = rp[i];
        ke = diag[i];
    } else if constexpr (MODE == 1) {
        kb = diag[i] + 1;
        ke = rp[i + 1];
    } else {
        kb = rp[i];
        ke = rp[i + 1];
    }
}

template <int MODE, class T>
__device__ __forceinline__ void dep_load(DepRow<T> &d, int c, const int *rp, const int *ci, const T *v,
                                         const int *diag, const T *diagv, const T *b)
{
    d.n = -1;
    if (c < 0) return;
    int kb, ke;
    sweep_range<MODE>(c, rp, diag, kb, ke);
    if (ke - kb > kDepMax) return;
    d.n = ke - kb;
#pragma unroll
    for (int w = 0; w < kDepMax; ++w) {
        d.col[w] = w < d.n ? ci[kb + w] : -1;
        d.val[w] = w < d.n ? v[kb + w] : T(0);
    }
    d.b = b[c];
    if constexpr (MODE == 1) d.dfin = v[diag[c]];
    else if constexpr (MODE == 2) d.dfin = diagv[c];
    else d.dfin = T(1);
}

// x_c as row c's lane computes and stores it (MODE 0: b - sum; 1: (b - sum)
// / diagonal; 2: (b - sum) / diagonal with the sum folded into b)
template <bool S, int MODE, class T>
__device__ __forceinline__ T dep_value(const DepRow<T> &d, const T *x, const int *err, int spin, bool &bad)
{
    T xv[kDepMax];
#pragma unroll
    for (int w = 0; w < kDepMax; ++w) xv[w] = d.col[w] < 0 ? T(0) : ld_relaxed(x + d.col[w]);
    T acc = MODE == 2 ? d.b : T(0);
#pragma unroll
    for (int w = 0; w < kDepMax; ++w) {
        if (d.col[w] < 0 || bad) continue;
        if (pending(xv[w])) xv[w] = wait_x(x, d.col[w], err, spin, bad);
        if constexpr (MODE <= 1) acc = fmac<S>(d.val[w], xv[w], acc);
        else acc = fmac<S>(-d.val[w], xv[w], acc);
    }
    T r;
    if constexpr (MODE == 0) r = d.b - acc;
    else if constexpr (MODE == 1) r = (d.b - acc) / d.dfin;
    else r = acc / d.dfin;
    return unpend(r);
}

// One triangular solve, one launch.  Rows (one per lane) and their entries,
// in MTJ's order:
//  MODE 0: UnitLowerCompRowMatrix.solve   x_i = b_i - sum_{k<diag} v_k x_ck  (S/UnitLowerCompRowMatrix.java:56-64)
//  MODE 1: UpperCompRowMatrix.solve       x_i = (b_i - sum_{k>diag} v_k x_ck) / v_diag (S/UpperCompRowMatrix.java:56-64)
//  MODE 2: UpperCompRowMatrix.transSolve in gather form on the transpose of
//          the strict upper part: x_c = b_c, minus R_ic x_i for ascending
//          source rows i, then divided by R_cc (S/UpperCompRowMatrix.java:78-87)
//  MODE 3: UnitLowerCompRowMatrix.transSolve in gather form on the
//          transpose of the strict lower part, source rows descending
//          (S/UnitLowerCompRowMatrix.java:78-83)
//  MODE 4: SSOR's forward sweep (S/SSOR.java:163-172): sigma over the row in
//          entry order, lower entries from the new iterate x (waited for),
//          upper entries from aux (the old x); x_i = aux_i + omega (sigma' - aux_i)
//  MODE 5: SSOR's backward sweep (S/SSOR.java:180-189): lower entries from
//          aux (the forward iterate), upper entries from the new x (waited
//          for); x_i = aux_i + omega (sigma' - aux_i)
// A row's entries are read in groups of kGrp, whose x loads are all in
// flight before the first wait, and the operands that finish the row (the
// diagonal, SSOR's old iterate) are loaded before the waits too: once the
// last dependency arrives a row is arithmetic and one store, not further
// dependent loads.  T = float: the FP32 sweeps (MODE 0 and 1) of the
// mixed-precision inner solves, on an FP32 copy of the factor.
template <bool S, int MODE, class T = double, bool LA = false>
__global__ void __launch_bounds__(kSweepBlock) k_trsv_sweep(const int *__restrict__ perm,
                                                          const int *__restrict__ chunk, int num_chunks,
                                                          const int *__restrict__ rp, const int *__restrict__ ci,
                                                          const T *__restrict__ v,
                                                          const int *__restrict__ diag,
                                                          const T *__restrict__ diagv, const T *b,
                                                          T *x, unsigned *ticket, const int *status, int *err,
                                                          int spin, const T *__restrict__ aux, T omega)
{
    constexpr int kGrp = 4;
    if (status && *status != ST_RUNNING) return;
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned c = 0;
        if (lane == 0) c = atomicAdd(ticket, 1u);
        c = __shfl_sync(0xffffffffu, c, 0);
        if (c >= (unsigned)num_chunks) return;
        const int beg = chunk[c], cnt = chunk[c + 1] - beg;
        bool bad = false;
        if (lane < cnt) {
            const int i = perm[beg + lane];
            const T bi = b[i];
            // entry range, walked upwards from kb (MODE 3: downwards from ke - 1)
            int kb, ke, dk = -1;
            if constexpr (MODE == 0) {
                kb = rp[i];
                ke = diag[i];
            } else if constexpr (MODE == 1) {
                kb = diag[i] + 1;
                ke = rp[i + 1];
            } else {
                kb = rp[i];
                ke = rp[i + 1];
            }
            if constexpr (MODE >= 4) dk = diag[i];
            // the row's finishing operands, ahead of the waits
            T dfin = T(1), old = T(0);
            if constexpr (MODE == 1) dfin = v[diag[i]];
            else if constexpr (MODE == 2) dfin = diagv[i];
            else if constexpr (MODE >= 4) {
                dfin = v[dk];
                old = aux[i];
            }
            T acc = (MODE == 2 || MODE == 3) ? bi : T(0);
            for (int k0 = 0; k0 < ke - kb && !bad; k0 += kGrp) {
                int cc[kGrp];
                T vv[kGrp], xv[kGrp];
                bool wt[kGrp];  // the entry is read from the sweep's own output
#pragma unroll
                for (int u = 0; u < kGrp; ++u) {
                    const int k = MODE == 3 ? ke - 1 - (k0 + u) : kb + k0 + u;
                    const bool in = k0 + u < ke - kb && k != dk;
                    cc[u] = in ? ci[k] : -1;
                    vv[u] = in ? v[k] : T(0);
                    wt[u] = MODE == 4 ? k < dk : (MODE == 5 ? k > dk : true);
                }
                // lookahead: the first group's dependency rows, before any wait
                constexpr bool kLA = LA && MODE <= 2 && kGrp == kDepMax;
                DepRow<T> dr[kLA ? kGrp : 1];
                if constexpr (kLA) {
                    if (k0 == 0) {
#pragma unroll
                        for (int u = 0; u < kGrp; ++u) dep_load<MODE>(dr[u], cc[u], rp, ci, v, diag, diagv, b);
                    }
                }
#pragma unroll
                for (int u = 0; u < kGrp; ++u)
                    xv[u] = cc[u] < 0 ? T(0) : (wt[u] ? ld_relaxed(x + cc[u]) : aux[cc[u]]);
#pragma unroll
                for (int u = 0; u < kGrp; ++u) {
                    if (cc[u] < 0 || bad) continue;
                    if constexpr (kLA) {
                        if (k0 == 0 && pending(xv[u]) && dr[u].n >= 0) {
                            // x_c may have been published meanwhile
                            xv[u] = ld_relaxed(x + cc[u]);
                            if (pending(xv[u])) xv[u] = dep_value<S, MODE>(dr[u], x, err, spin, bad);
                        }
                    }
                    if (wt[u] && pending(xv[u])) xv[u] = wait_x(x, cc[u], err, spin, bad);
                    if constexpr (MODE <= 1 || MODE >= 4) acc = fmac<S>(vv[u], xv[u], acc);
                    else acc = fmac<S>(-vv[u], xv[u], acc);
                }
            }
            T xi;
            if constexpr (MODE == 0) xi = bi - acc;
            else if constexpr (MODE == 1) xi = (bi - acc) / dfin;
            else if constexpr (MODE == 2) xi = acc / dfin;
            else if constexpr (MODE == 3) xi = acc;
            else {
                // sigma = (b_i - sigma) / a_ii; x_i = old_i + omega (sigma - old_i)
                const T sig = (bi - acc) / dfin;
                if constexpr (S) xi = __dadd_rn(old, __dmul_rn(omega, __dsub_rn(sig, old)));
                else xi = fma(omega, sig - old, old);
            }
            // a stored pending pattern would read as "not solved": store a quiet NaN
            if (!bad) st_relaxed(x + i, unpend(xi));
        }
        if (__any_sync(0xffffffffu, bad)) {
            if (lane == 0) atomicExch(err, 1);
            return;
        }
    }
}

__global__ void k_gather_diag(int n, const int *diag, const double *data, double *diagv)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) diagv[i] = data[diag[i]];
}

// ------------------------------------------------------------- host side
static int grid_for(mtjg_ctx *ctx, int n)
{
    return std::max(1, std::min((n + kBlock - 1) / kBlock, ctx->num_sms * 8));
}

static void free_sched(LevelSchedule &s)
{
    cudaFree(s.perm);
    cudaFree(s.chunk);
    cudaFree(s.ticket);
    s.perm = s.chunk = nullptr;
    s.ticket = nullptr;
    s.level_ptr.clear();
    s.num_levels = 0;
    s.num_chunks = 0;
}

// Finds the levels on the device, then groups rows by level.
static int build_levels(mtjg_ctx *ctx, int n, int desc, int range, const int *rp, const int *ci, const int *diag,
                        const unsigned char *quirk, LevelSchedule &out)
{
    free_sched(out);
    out.n = n;
    if (n == 0) {
        out.level_ptr = {0};
        return MTJG_OK;
    }
    int *level = nullptr;
    unsigned *ticket = nullptr;
    MTJG_CUDA(cudaMalloc(&level, sizeof(int) * (size_t)n));
    MTJG_CUDA(cudaMalloc(&ticket, sizeof(unsigned)));
    MTJG_CUDA(cudaMemsetAsync(level, 0xff, sizeof(int) * (size_t)n, ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned), ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    k_levels<<<ctx->num_sms * 4, kBlock, 0, ctx->stream>>>(n, desc, range, rp, ci, diag, quirk, level, ticket,
                                                            ctx->d_flag);
    ctx->launches++;
    MTJG_CUDA(cudaGetLastError());
    std::vector<int> h(n);
    MTJG_CUDA(cudaMemcpyAsync(h.data(), level, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    int flag = 0;
    MTJG_CUDA(cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(level);
    cudaFree(ticket);
    if (flag) {
        cudaMemset(ctx->d_flag, 0, sizeof(int));
        return fail(MTJG_ERR_DEVICE_TIMEOUT, "level analysis: a bounded wait gave up");
    }
    int nl = 0;
    for (int i = 0; i < n; ++i) nl = std::max(nl, h[i] + 1);
    out.num_levels = nl;
    out.level_ptr.assign(nl + 1, 0);
    for (int i = 0; i < n; ++i) out.level_ptr[h[i] + 1]++;
    for (int l = 0; l < nl; ++l) out.level_ptr[l + 1] += out.level_ptr[l];
    std::vector<int> pos(out.level_ptr.begin(), out.level_ptr.end() - 1), perm(n);
    for (int i = 0; i < n; ++i) perm[pos[h[i]]++] = i;
    // chunks of at most 32 rows, never straddling two levels
    std::vector<int> chunk;
    for (int l = 0; l < nl; ++l)
        for (int p = out.level_ptr[l]; p < out.level_ptr[l + 1]; p += 32) chunk.push_back(p);
    out.num_chunks = (int)chunk.size();
    chunk.push_back(n);
    MTJG_CUDA(cudaMalloc(&out.perm, sizeof(int) * (size_t)n));
    MTJG_CUDA(cudaMemcpy(out.perm, perm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
    MTJG_CUDA(cudaMalloc(&out.chunk, sizeof(int) * chunk.size()));
    MTJG_CUDA(cudaMemcpy(out.chunk, chunk.data(), sizeof(int) * chunk.size(), cudaMemcpyHostToDevice));
    MTJG_CUDA(cudaMalloc(&out.ticket, sizeof(unsigned)));
    MTJG_CUDA(cudaMemset(out.ticket, 0, sizeof(unsigned)));
    return MTJG_OK;
}

// Fills the outputs of the next sweeps (x2 may be null) with kPending and
// resets their tickets.
static cudaError_t sweep_prep(mtjg_ctx *ctx, int n, double *x1, double *x2, LevelSchedule *s1, LevelSchedule *s2,
                              const int *status)
{
    k_sweep_prep<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, x1, x2, s1 ? s1->ticket : nullptr,
                                                               s2 ? s2->ticket : nullptr, status);
    ctx->launches++;
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t sweep_t(mtjg_ctx *ctx, bool strict, const LevelSchedule &s, const int *rp, const int *ci,
                           const double *v, const int *diag, const double *diagv, const double *b, double *x,
                           const int *status, const double *aux = nullptr, double omega = 0.0)
{
    if (s.num_chunks == 0) return cudaSuccess;
    const int warps = ctx->num_sms * env_int("MTJG_SWEEP_WARPS", kSweepWarpsPerSm, 1, 40);
    const int spin = env_int("MTJG_SWEEP_SPIN", kSweepSpin, 0, 1 << 20);
    const int grid = (std::min(warps, s.num_chunks) + kSweepBlock / 32 - 1) / (kSweepBlock / 32);
    auto go = [&](auto kernel) {
        kernel<<<grid, kSweepBlock, 0, ctx->stream>>>(s.perm, s.chunk, s.num_chunks, rp, ci, v, diag, diagv, b, x,
                                                      s.ticket, status, ctx->d_flag, spin, aux, omega);
    };
    if constexpr (MODE <= 2) {
        if (sweep_lookahead(MODE, kLookaheadModes64)) {
            if (strict) go(k_trsv_sweep<true, MODE, double, true>);
            else go(k_trsv_sweep<false, MODE, double, true>);
            ctx->launches++;
            return cudaGetLastError();
        }
    }
    if (strict) go(k_trsv_sweep<true, MODE>);
    else go(k_trsv_sweep<false, MODE>);
    ctx->launches++;
    return cudaGetLastError();
}

// One triangular solve x = T \ b.  x must have been filled with kPending and
// s's ticket reset (sweep_prep) since its last sweep, and x must not alias b.
static cudaError_t sweep(mtjg_ctx *ctx, int mode, const LevelSchedule &s, const int *rp, const int *ci,
                         const double *v, const int *diag, const double *diagv, const double *b, double *x,
                         const int *status)
{
    const bool strict = ctx->numerics == MTJG_NUMERICS_STRICT;
    switch (mode) {
    case 0: return sweep_t<0>(ctx, strict, s, rp, ci, v, diag, diagv, b, x, status);
    case 1: return sweep_t<1>(ctx, strict, s, rp, ci, v, diag, diagv, b, x, status);
    case 2: return sweep_t<2>(ctx, strict, s, rp, ci, v, diag, diagv, b, x, status);
    default: return sweep_t<3>(ctx, strict, s, rp, ci, v, diag, diagv, b, x, status);
    }
}

// Two sweeps, b -> y (first operator) -> x (second): y and (when it does not
// alias b) x are filled in one pass before the first; an x that aliases b is
// filled between the two.
static cudaError_t sweep_pair(mtjg_ctx *ctx, int n, int mode1, LevelSchedule &s1, const int *rp1, const int *ci1,
                              const double *v1, const int *diag1, const double *diagv1, int mode2, LevelSchedule &s2,
                              const int *rp2, const int *ci2, const double *v2, const int *diag2,
                              const double *diagv2, const double *b, double *y, double *x, const int *status)
{
    const bool alias = x == b;
    cudaError_t e = sweep_prep(ctx, n, y, alias ? nullptr : x, &s1, &s2, status);
    if (e == cudaSuccess) e = sweep(ctx, mode1, s1, rp1, ci1, v1, diag1, diagv1, b, y, status);
    if (e == cudaSuccess && alias) e = sweep_prep(ctx, n, x, nullptr, nullptr, nullptr, status);
    if (e == cudaSuccess) e = sweep(ctx, mode2, s2, rp2, ci2, v2, diag2, diagv2, y, x, status);
    return e;
}

static int read_err_min(mtjg_ctx *ctx, int *err_min_dev, int *out)
{
    MTJG_CUDA(cudaMemcpyAsync(out, err_min_dev, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    return MTJG_OK;
}

// Applies M to device vectors: x = M \ b.  `status` (nullable) makes every
// kernel a no-op unless the solve it belongs to is running.
int precond_apply_dev(mtjg_precond *M, const double *b, double *x, const int *status)
{
    mtjg_ctx *ctx = M->ctx;
    const int n = M->n;
    if (n == 0) return MTJG_OK;
    cudaError_t e = cudaSuccess;
    switch (M->kind) {
    case MTJG_PC_IDENTITY:
        if (x != b) {
            k_copy<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, b, x, status);
            ctx->launches++;
        }
        e = cudaGetLastError();
        break;
    case MTJG_PC_JACOBI:
        k_jacobi_apply<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, M->invdiag, b, x, status);
        ctx->launches++;
        e = cudaGetLastError();
        break;
    case MTJG_PC_SSOR: {  // S/SSOR.java:148-192: forward sweep into y, then backward into x
        if (x == b) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "SSOR apply needs distinct b and x");
        const bool strict = ctx->numerics == MTJG_NUMERICS_STRICT;
        e = sweep_prep(ctx, n, M->y, nullptr, &M->lo, &M->up, status);
        if (e == cudaSuccess)
            e = sweep_t<4>(ctx, strict, M->lo, M->rowptr, M->colind, M->data, M->diag, nullptr, b, M->y, status, x,
                           M->omega_f);
        if (e == cudaSuccess && M->reverse) {
            e = sweep_prep(ctx, n, x, nullptr, nullptr, nullptr, status);
            if (e == cudaSuccess)
                e = sweep_t<5>(ctx, strict, M->up, M->rowptr, M->colind, M->data, M->diag, nullptr, b, x, status,
                               M->y, M->omega_r);
        } else if (e == cudaSuccess) {
            k_copy<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, M->y, x, status);
            ctx->launches++;
            e = cudaGetLastError();
        }
        break;
    }
    case MTJG_PC_ILU:   // L y = b, then U x = y (S/ILU.java:64-70)
    case MTJG_PC_ILUT:  // the same solves on the ILUT factor (S/ILUT.java:111-113)
        e = sweep_pair(ctx, n, 0, M->lo, M->rowptr, M->colind, M->data, M->diag, nullptr, 1, M->up, M->rowptr,
                       M->colind, M->data, M->diag, nullptr, b, M->y, x, status);
        break;
    default:  // ICC: R' y = b, then R x = y (S/ICC.java:67-73)
        e = sweep_pair(ctx, n, 2, M->lo, M->rt_rowptr, M->rt_colind, M->rt_val, nullptr, M->diagv, 1, M->up,
                       M->rowptr, M->colind, M->data, M->diag, nullptr, b, M->y, x, status);
        break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "preconditioner apply");
    return MTJG_OK;
}

// ------------------------------------------------ FP32 copies and applies
// The mixed-precision inner solves apply M in FP32: an FP32 copy of the
// ILU / ILUT factor values (sweeps with the FP64 factor's levels) or of the
// Jacobi inverse diagonal.  precond_prepare32 builds the copy (it allocates,
// so it runs before a solve's loop) and rebuilds it after setMatrix.
int precond_prepare32(mtjg_precond *M);
int precond_apply32(mtjg_precond *M, const float *b, float *x, const int *status);

__global__ void k_copy32(int n, const float *b, float *x, const int *status)
{
    if (status && *status != ST_RUNNING) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = b[i];
}

__global__ void k_jacobi_apply32(int n, const float *invdiag, const float *b, float *x, const int *status)
{
    if (status && *status != ST_RUNNING) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = b[i] * invdiag[i];
}

__global__ void k_narrow(int64_t n, const double *a, float *b)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

template <int MODE>
static cudaError_t sweep32(mtjg_ctx *ctx, const LevelSchedule &s, const int *rp, const int *ci, const float *v,
                           const int *diag, const float *b, float *x, const int *status)
{
    if (s.num_chunks == 0) return cudaSuccess;
    const int warps = ctx->num_sms * env_int("MTJG_SWEEP_WARPS", kSweepWarpsPerSm, 1, 40);
    const int spin = env_int("MTJG_SWEEP_SPIN", kSweepSpin, 0, 1 << 20);
    const int grid = (std::min(warps, s.num_chunks) + kSweepBlock / 32 - 1) / (kSweepBlock / 32);
    if (sweep_lookahead(MODE, kLookaheadModes32))
        k_trsv_sweep<false, MODE, float, true><<<grid, kSweepBlock, 0, ctx->stream>>>(
            s.perm, s.chunk, s.num_chunks, rp, ci, v, diag, nullptr, b, x, s.ticket, status, ctx->d_flag, spin,
            nullptr, 0.0f);
    else
        k_trsv_sweep<false, MODE, float><<<grid, kSweepBlock, 0, ctx->stream>>>(
            s.perm, s.chunk, s.num_chunks, rp, ci, v, diag, nullptr, b, x, s.ticket, status, ctx->d_flag, spin,
            nullptr, 0.0f);
    ctx->launches++;
    return cudaGetLastError();
}

int precond_prepare32(mtjg_precond *M)
{
    if (!M->ready) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "preconditioner has no matrix (call setMatrix first)");
    if (M->kind != MTJG_PC_IDENTITY && M->kind != MTJG_PC_JACOBI && M->kind != MTJG_PC_ILU &&
        M->kind != MTJG_PC_ILUT)
        return fail(MTJG_ERR_UNSUPPORTED, "mixed precision applies the identity, Jacobi, ILU or ILUT preconditioner");
    if (M->v32 == M->version) return MTJG_OK;
    mtjg_ctx *ctx = M->ctx;
    cudaFree(M->data32);
    cudaFree(M->invdiag32);
    cudaFree(M->y32);
    M->data32 = M->invdiag32 = M->y32 = nullptr;
    const int n = M->n;
    if (M->kind == MTJG_PC_JACOBI) {
        MTJG_CUDA(cudaMalloc(&M->invdiag32, sizeof(float) * (size_t)std::max(1, n)));
        if (n) k_narrow<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, M->invdiag, M->invdiag32);
        ctx->launches++;
    } else if (M->kind != MTJG_PC_IDENTITY) {
        MTJG_CUDA(cudaMalloc(&M->data32, sizeof(float) * (size_t)std::max<int64_t>(1, M->nnz)));
        MTJG_CUDA(cudaMalloc(&M->y32, sizeof(float) * (size_t)std::max(1, n)));
        if (M->nnz) k_narrow<<<ctx->num_sms * 8, kBlock, 0, ctx->stream>>>(M->nnz, M->data, M->data32);
        ctx->launches++;
    }
    MTJG_CUDA(cudaGetLastError());
    M->v32 = M->version;
    return MTJG_OK;
}

// x = M \ b in FP32, gated like precond_apply_dev; needs precond_prepare32.
int precond_apply32(mtjg_precond *M, const float *b, float *x, const int *status)
{
    mtjg_ctx *ctx = M->ctx;
    const int n = M->n;
    if (n == 0) return MTJG_OK;
    if (M->v32 != M->version) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "FP32 preconditioner copy is stale");
    cudaError_t e = cudaSuccess;
    switch (M->kind) {
    case MTJG_PC_IDENTITY:
        if (x != b) {
            k_copy32<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, b, x, status);
            ctx->launches++;
        }
        e = cudaGetLastError();
        break;
    case MTJG_PC_JACOBI:
        k_jacobi_apply32<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, M->invdiag32, b, x, status);
        ctx->launches++;
        e = cudaGetLastError();
        break;
    default: {  // ILU / ILUT: L y = b, then U x = y, on the FP32 factor
        const bool alias = x == b;
        k_sweep_prep<float><<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, M->y32, alias ? nullptr : x,
                                                                          M->lo.ticket, M->up.ticket, status);
        ctx->launches++;
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = sweep32<0>(ctx, M->lo, M->rowptr, M->colind, M->data32, M->diag, b, M->y32, status);
        if (e == cudaSuccess && alias) {
            k_sweep_prep<float><<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, x, nullptr, nullptr, nullptr,
                                                                              status);
            ctx->launches++;
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = sweep32<1>(ctx, M->up, M->rowptr, M->colind, M->data32, M->diag, M->y32, x, status);
        break;
    }
    }
    if (e != cudaSuccess) return cuda_fail(e, "FP32 preconditioner apply");
    return MTJG_OK;
}

// Preconditioner.transApply on device vectors, gated like
// precond_apply_dev; and the set-up it needs (ILU's transposed factors),
// which allocates and so must run before any stream capture.
int precond_trans_apply_dev(mtjg_precond *M, const double *b, double *x, const int *status);
int precond_prepare_trans(mtjg_precond *M);

// ILU.transApply (S/ILU.java:72-78): U'y = b, then L'x = y.  Built on first use.
struct IluTrans {
    int *ut_rp = nullptr, *ut_ci = nullptr;
    double *ut_v = nullptr;
    int *lt_rp = nullptr, *lt_ci = nullptr;
    double *lt_v = nullptr;
    LevelSchedule ut, lt;
};

}  // namespace mtjg

using namespace mtjg;

static void precond_release(mtjg_precond *M)
{
    cudaFree(M->invdiag);
    cudaFree(M->rowptr);
    cudaFree(M->colind);
    cudaFree(M->diag);
    cudaFree(M->data);
    cudaFree(M->rt_rowptr);
    cudaFree(M->rt_colind);
    cudaFree(M->rt_val);
    cudaFree(M->diagv);
    cudaFree(M->data32);
    cudaFree(M->invdiag32);
    cudaFree(M->y32);
    M->data32 = M->invdiag32 = M->y32 = nullptr;
    M->v32 = -1;
    free_sched(M->lo);
    free_sched(M->up);
    M->invdiag = M->data = M->rt_val = M->diagv = nullptr;
    M->rowptr = M->colind = M->diag = M->rt_rowptr = M->rt_colind = nullptr;
    if (M->trans) {
        IluTrans *t = static_cast<IluTrans *>(M->trans);
        cudaFree(t->ut_rp);
        cudaFree(t->ut_ci);
        cudaFree(t->ut_v);
        cudaFree(t->lt_rp);
        cudaFree(t->lt_ci);
        cudaFree(t->lt_v);
        free_sched(t->ut);
        free_sched(t->lt);
        delete t;
        M->trans = nullptr;
    }
    M->ready = false;
}

extern "C" int mtjg_precond_create(mtjg_ctx *ctx, int kind, int n, mtjg_precond **out)
{
    if (!ctx || !out) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (kind < MTJG_PC_IDENTITY || kind > MTJG_PC_ILUT) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "unknown preconditioner");
    if (n < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "negative size");
    MTJG_CUDA(cudaSetDevice(ctx->device));
    mtjg_precond *M = new mtjg_precond();
    M->ctx = ctx;
    ctx_retain(ctx);
    M->kind = kind;
    M->n = n;
    const size_t nb = sizeof(double) * (size_t)std::max(1, n);
    if (cudaMalloc(&M->y, nb) != cudaSuccess || cudaMalloc(&M->d_b, nb) != cudaSuccess ||
        cudaMalloc(&M->d_x, nb) != cudaSuccess) {
        mtjg_precond_destroy(M);
        return fail(MTJG_ERR_OUT_OF_MEMORY, "cudaMalloc failed for the preconditioner");
    }
    if (kind == MTJG_PC_IDENTITY) M->ready = true;
    *out = M;
    return MTJG_OK;
}

extern "C" int mtjg_precond_destroy(mtjg_precond *M)
{
    if (!M) return MTJG_OK;
    cudaSetDevice(M->ctx->device);
    cudaStreamSynchronize(M->ctx->stream);
    precond_release(M);
    cudaFree(M->y);
    cudaFree(M->d_b);
    cudaFree(M->d_x);
    mtjg_ctx *ctx = M->ctx;
    delete M;
    ctx_release(ctx);
    return MTJG_OK;
}

static int copy_pattern(mtjg_precond *M, mtjg_csr *A)
{
    const int n = A->n;
    M->nnz = A->nnz;
    MTJG_CUDA(cudaMalloc(&M->rowptr, sizeof(int) * (size_t)(n + 1)));
    MTJG_CUDA(cudaMalloc(&M->colind, sizeof(int) * (size_t)(A->nnz + 4)));
    MTJG_CUDA(cudaMalloc(&M->data, sizeof(double) * (size_t)(A->nnz + 2)));
    MTJG_CUDA(cudaMalloc(&M->diag, sizeof(int) * (size_t)std::max(1, n)));
    MTJG_CUDA(cudaMemcpyAsync(M->rowptr, A->rowptr, sizeof(int) * (size_t)(n + 1), cudaMemcpyDeviceToDevice,
                              M->ctx->stream));
    MTJG_CUDA(cudaMemcpyAsync(M->colind, A->colind, sizeof(int) * (size_t)(A->nnz + 4), cudaMemcpyDeviceToDevice,
                              M->ctx->stream));
    MTJG_CUDA(cudaMemcpyAsync(M->data, A->val, sizeof(double) * (size_t)(A->nnz + 2), cudaMemcpyDeviceToDevice,
                              M->ctx->stream));
    return MTJG_OK;
}

static int find_diagonal(mtjg_precond *M, int *err_row)
{
    mtjg_ctx *ctx = M->ctx;
    int *err = ctx->d_flag + 1;
    const int big = 0x7fffffff;
    MTJG_CUDA(cudaMemcpyAsync(err, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if (M->n) {
        k_find_diag<<<grid_for(ctx, M->n), kBlock, 0, ctx->stream>>>(M->n, M->rowptr, M->colind, M->diag, err);
        ctx->launches++;
    }
    int e = big;
    int st = read_err_min(ctx, err, &e);
    if (st != MTJG_OK) return st;
    if (e != big) {
        *err_row = e;
        return fail(MTJG_ERR_MISSING_DIAGONAL, "Missing diagonal entry on row " + std::to_string(e));
    }
    return MTJG_OK;
}

static int ilu_setup(mtjg_precond *M, int *err_row)
{
    mtjg_ctx *ctx = M->ctx;
    const int n = M->n;
    int st = find_diagonal(M, err_row);
    if (st != MTJG_OK) return st;
    unsigned char *quirk = nullptr;
    MTJG_CUDA(cudaMalloc(&quirk, (size_t)std::max(1, n)));
    if (n) {
        k_ilu_quirk<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, M->rowptr, M->colind, M->diag, quirk);
        ctx->launches++;
    }
    LevelSchedule fac;
    st = build_levels(ctx, n, 0, 1, M->rowptr, M->colind, M->diag, quirk, fac);
    cudaFree(quirk);
    if (st != MTJG_OK) return st;
    int *err = ctx->d_flag + 1;
    const int big = 0x7fffffff;
    MTJG_CUDA(cudaMemcpyAsync(err, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    for (int l = 0; l < fac.num_levels; ++l) {
        const int beg = fac.level_ptr[l], cnt = fac.level_ptr[l + 1] - beg;
        k_ilu_level<<<(cnt + kBlock - 1) / kBlock, kBlock, 0, ctx->stream>>>(fac.perm, beg, cnt, M->rowptr,
                                                                            M->colind, M->diag, M->data, err);
        ctx->launches++;
    }
    MTJG_CUDA(cudaGetLastError());
    int e = big;
    st = read_err_min(ctx, err, &e);
    free_sched(fac);
    if (st != MTJG_OK) return st;
    if (e != big) {
        *err_row = e;
        return fail(MTJG_ERR_ZERO_PIVOT, "Zero pivot encountered on row " + std::to_string(e) + " during ILU process");
    }
    // solve schedules: L (rows ascending, lower range), U (descending, upper range)
    st = build_levels(ctx, n, 0, 1, M->rowptr, M->colind, M->diag, nullptr, M->lo);
    if (st != MTJG_OK) return st;
    return build_levels(ctx, n, 1, 2, M->rowptr, M->colind, M->diag, nullptr, M->up);
}

static int icc_setup(mtjg_precond *M, mtjg_csr *A, int *err_row)
{
    mtjg_ctx *ctx = M->ctx;
    const int n = M->n;
    int st = find_diagonal(M, err_row);
    if (st != MTJG_OK) return st;
    // ICC.factor (S/ICC.java:85-139) runs on the host over the row reaches,
    // then the factor returns to the device.
    std::vector<int> ci((size_t)A->nnz), diag((size_t)n);
    std::vector<double> data((size_t)A->nnz);
    if (A->nnz) {
        MTJG_CUDA(cudaMemcpy(ci.data(), A->colind, sizeof(int) * (size_t)A->nnz, cudaMemcpyDeviceToHost));
        MTJG_CUDA(cudaMemcpy(data.data(), A->val, sizeof(double) * (size_t)A->nnz, cudaMemcpyDeviceToHost));
    }
    if (n) MTJG_CUDA(cudaMemcpy(diag.data(), M->diag, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
    st = icc_factor_host(n, A->h_rowptr.data(), ci.data(), diag.data(), data.data(), err_row);
    if (st != MTJG_OK) return st;
    if (A->nnz)
        MTJG_CUDA(cudaMemcpy(M->data, data.data(), sizeof(double) * (size_t)A->nnz, cudaMemcpyHostToDevice));
    int64_t tn = 0;
    st = csr_transpose(ctx, n, n, M->rowptr, M->colind, M->data, 1, &M->rt_rowptr, &M->rt_colind, &M->rt_val, &tn);
    if (st != MTJG_OK) return st;
    MTJG_CUDA(cudaMalloc(&M->diagv, sizeof(double) * (size_t)std::max(1, n)));
    if (n) {
        k_gather_diag<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, M->diag, M->data, M->diagv);
        ctx->launches++;
    }
    st = build_levels(ctx, n, 0, 0, M->rt_rowptr, M->rt_colind, nullptr, nullptr, M->lo);
    if (st != MTJG_OK) return st;
    return build_levels(ctx, n, 1, 2, M->rowptr, M->colind, M->diag, nullptr, M->up);
}

// SSOR.setMatrix (S/SSOR.java:98-113): F.set(A), the diagonal positions;
// the sweeps' dependency levels (forward: the lower part, backward: the upper)
static int ssor_setup(mtjg_precond *M, int *err_row)
{
    int st = find_diagonal(M, err_row);
    if (st == MTJG_ERR_MISSING_DIAGONAL) return fail(st, "Missing diagonal on row " + std::to_string(*err_row));
    if (st != MTJG_OK) return st;
    st = build_levels(M->ctx, M->n, 0, 1, M->rowptr, M->colind, M->diag, nullptr, M->lo);
    if (st != MTJG_OK) return st;
    return build_levels(M->ctx, M->n, 1, 2, M->rowptr, M->colind, M->diag, nullptr, M->up);
}

// ILUT.setMatrix (S/ILUT.java:119-123): the factor on the host
// (ilut_host.cpp), its rows uploaded as a CSR, then ILU's solve levels.
static int ilut_setup(mtjg_precond *M, mtjg_csr *A, int *err_row)
{
    mtjg_ctx *ctx = M->ctx;
    const int n = M->n;
    std::vector<int> ci((size_t)A->nnz);
    std::vector<double> val((size_t)A->nnz);
    if (A->nnz) {
        MTJG_CUDA(cudaMemcpy(ci.data(), A->colind, sizeof(int) * (size_t)A->nnz, cudaMemcpyDeviceToHost));
        MTJG_CUDA(cudaMemcpy(val.data(), A->val, sizeof(double) * (size_t)A->nnz, cudaMemcpyDeviceToHost));
    }
    std::vector<int> frp, fci, fdiag;
    std::vector<double> fv;
    int st = ilut_factor_host(n, A->h_rowptr.data(), ci.data(), val.data(), M->tau, M->p, frp, fci, fv, fdiag,
                              err_row);
    if (st != MTJG_OK) return st;
    const int64_t nnz = frp[(size_t)n];
    M->nnz = nnz;
    MTJG_CUDA(cudaMalloc(&M->rowptr, sizeof(int) * (size_t)(n + 1 + kRowptrPad)));
    MTJG_CUDA(cudaMalloc(&M->colind, sizeof(int) * (size_t)(nnz + 4)));
    MTJG_CUDA(cudaMalloc(&M->data, sizeof(double) * (size_t)(nnz + 2)));
    MTJG_CUDA(cudaMalloc(&M->diag, sizeof(int) * (size_t)std::max(1, n)));
    MTJG_CUDA(cudaMemcpy(M->rowptr, frp.data(), sizeof(int) * (size_t)(n + 1), cudaMemcpyHostToDevice));
    if (nnz) {
        MTJG_CUDA(cudaMemcpy(M->colind, fci.data(), sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice));
        MTJG_CUDA(cudaMemcpy(M->data, fv.data(), sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice));
    }
    if (n) MTJG_CUDA(cudaMemcpy(M->diag, fdiag.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice));
    st = build_levels(ctx, n, 0, 1, M->rowptr, M->colind, M->diag, nullptr, M->lo);
    if (st != MTJG_OK) return st;
    return build_levels(ctx, n, 1, 2, M->rowptr, M->colind, M->diag, nullptr, M->up);
}

extern "C" int mtjg_precond_set_ssor(mtjg_precond *M, int reverse, double omega_f, double omega_r)
{
    if (!M) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL preconditioner");
    if (M->kind != MTJG_PC_SSOR) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "not an SSOR preconditioner");
    // SSOR.setOmega, S/SSOR.java:87-96
    if (omega_f < 0 || omega_f > 2) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "omegaF must be between 0 and 2");
    if (omega_r < 0 || omega_r > 2) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "omegaR must be between 0 and 2");
    M->reverse = reverse != 0;
    M->omega_f = omega_f;
    M->omega_r = omega_r;
    M->version++;
    return MTJG_OK;
}

extern "C" int mtjg_precond_set_ilut(mtjg_precond *M, double tau, int p)
{
    if (!M) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL preconditioner");
    if (M->kind != MTJG_PC_ILUT) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "not an ILUT preconditioner");
    M->tau = tau;
    M->p = p;
    return MTJG_OK;
}

extern "C" int mtjg_precond_pattern(mtjg_precond *M, int *rowptr, int *colind, int *diag, int64_t cap,
                                    int64_t *nnz)
{
    if (!M) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL preconditioner");
    MTJG_CUDA(cudaSetDevice(M->ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(M->ctx->stream));
    const bool has = M->rowptr && M->kind != MTJG_PC_JACOBI;
    if (nnz) *nnz = has ? M->nnz : 0;
    if (!has) return MTJG_OK;
    if (rowptr) MTJG_CUDA(cudaMemcpy(rowptr, M->rowptr, sizeof(int) * (size_t)(M->n + 1), cudaMemcpyDeviceToHost));
    const int64_t m = std::min(cap, M->nnz);
    if (colind && m > 0) MTJG_CUDA(cudaMemcpy(colind, M->colind, sizeof(int) * (size_t)m, cudaMemcpyDeviceToHost));
    if (diag && M->n) {
        std::vector<int> d((size_t)M->n), rp((size_t)M->n + 1);
        MTJG_CUDA(cudaMemcpy(d.data(), M->diag, sizeof(int) * (size_t)M->n, cudaMemcpyDeviceToHost));
        MTJG_CUDA(cudaMemcpy(rp.data(), M->rowptr, sizeof(int) * (size_t)(M->n + 1), cudaMemcpyDeviceToHost));
        for (int i = 0; i < M->n; ++i) diag[i] = d[(size_t)i] - rp[(size_t)i];  // position within the row
    }
    return MTJG_OK;
}

extern "C" int mtjg_precond_set_matrix(mtjg_precond *M, mtjg_csr *A, int *err_row)
{
    int dummy = 0;
    if (!err_row) err_row = &dummy;
    *err_row = 0;
    if (!M || !A) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (A->ctx != M->ctx) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "matrix and preconditioner use different contexts");
    if (M->kind == MTJG_PC_IDENTITY) return MTJG_OK;
    if (A->n != M->n)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "Matrix size differs from preconditioner size");
    if (M->kind != MTJG_PC_JACOBI && A->n != A->m)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, M->kind == MTJG_PC_ICC    ? "ICC only applies to square matrices"
                                               : M->kind == MTJG_PC_SSOR ? "SSOR only applies to square matrices"
                                                                         : "ILU only applies to square matrices");
    mtjg_ctx *ctx = M->ctx;
    MTJG_CUDA(cudaSetDevice(ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    precond_release(M);
    static int64_t s_version = 0;
    M->version = ++s_version;
    const int n = M->n;
    if (M->kind == MTJG_PC_JACOBI) {
        MTJG_CUDA(cudaMalloc(&M->invdiag, sizeof(double) * (size_t)std::max(1, n)));
        int *err = ctx->d_flag + 1;
        const int big = 0x7fffffff;
        MTJG_CUDA(cudaMemcpyAsync(err, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        if (n) {
            k_jacobi_set<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, A->rowptr, A->colind, A->val, M->invdiag,
                                                                       err);
            ctx->launches++;
        }
        int e = big;
        int st = read_err_min(ctx, err, &e);
        if (st != MTJG_OK) return st;
        if (e != big) {
            *err_row = e;
            return fail(MTJG_ERR_ZERO_DIAGONAL, "Zero diagonal on row " + std::to_string(e));
        }
        M->ready = true;
        return MTJG_OK;
    }
    int st = M->kind == MTJG_PC_ILUT ? ilut_setup(M, A, err_row) : copy_pattern(M, A);
    if (st != MTJG_OK) return st;
    if (M->kind == MTJG_PC_ILU) st = ilu_setup(M, err_row);
    else if (M->kind == MTJG_PC_ICC) st = icc_setup(M, A, err_row);
    else if (M->kind == MTJG_PC_SSOR) st = ssor_setup(M, err_row);
    if (st != MTJG_OK) return st;
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    M->ready = true;
    return MTJG_OK;
}

static int ilu_trans_setup(mtjg_precond *M)
{
    if (M->trans) return MTJG_OK;
    mtjg_ctx *ctx = M->ctx;
    IluTrans *t = new IluTrans();
    M->trans = t;
    int64_t tn = 0;
    int st = csr_transpose(ctx, M->n, M->n, M->rowptr, M->colind, M->data, 1, &t->ut_rp, &t->ut_ci, &t->ut_v, &tn);
    if (st != MTJG_OK) return st;
    st = csr_transpose(ctx, M->n, M->n, M->rowptr, M->colind, M->data, 2, &t->lt_rp, &t->lt_ci, &t->lt_v, &tn);
    if (st != MTJG_OK) return st;
    if (!M->diagv) {
        MTJG_CUDA(cudaMalloc(&M->diagv, sizeof(double) * (size_t)std::max(1, M->n)));
        if (M->n) {
            k_gather_diag<<<grid_for(ctx, M->n), kBlock, 0, ctx->stream>>>(M->n, M->diag, M->data, M->diagv);
            ctx->launches++;
        }
    }
    st = build_levels(ctx, M->n, 0, 0, t->ut_rp, t->ut_ci, nullptr, nullptr, t->ut);
    if (st != MTJG_OK) return st;
    return build_levels(ctx, M->n, 1, 0, t->lt_rp, t->lt_ci, nullptr, nullptr, t->lt);
}

static bool lu_kind(const mtjg_precond *M) { return M->kind == MTJG_PC_ILU || M->kind == MTJG_PC_ILUT; }

int mtjg::precond_prepare_trans(mtjg_precond *M)
{
    return lu_kind(M) ? ilu_trans_setup(M) : MTJG_OK;
}

// DiagonalPreconditioner, ICC and SSOR are their own transposes here
// (S/DiagonalPreconditioner.java:60-62, S/ICC.java:75-77, S/SSOR.java:194-197);
// ILU and ILUT sweep U' then L' (S/ILU.java:72-78, S/ILUT.java:115-117).
int mtjg::precond_trans_apply_dev(mtjg_precond *M, const double *b, double *x, const int *status)
{
    if (!lu_kind(M)) return precond_apply_dev(M, b, x, status);
    int st = ilu_trans_setup(M);
    if (st != MTJG_OK) return st;
    IluTrans *t = static_cast<IluTrans *>(M->trans);
    cudaError_t e = sweep_pair(M->ctx, M->n, 2, t->ut, t->ut_rp, t->ut_ci, t->ut_v, nullptr, M->diagv, 3, t->lt,
                               t->lt_rp, t->lt_ci, t->lt_v, nullptr, nullptr, b, M->y, x, status);
    if (e != cudaSuccess) return cuda_fail(e, "ILU transApply");
    return MTJG_OK;
}

static int precond_host_call(mtjg_precond *M, const double *b, double *x, bool trans)
{
    if (!M || (!b && M->n) || (!x && M->n)) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (!M->ready) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "setMatrix has not been called");
    mtjg_ctx *ctx = M->ctx;
    MTJG_CUDA(cudaSetDevice(ctx->device));
    const size_t nb = sizeof(double) * (size_t)M->n;
    if (M->n == 0) return MTJG_OK;
    MTJG_CUDA(cudaMemcpyAsync(M->d_b, b, nb, cudaMemcpyHostToDevice, ctx->stream));
    // SSOR's sweep starts from x's content (S/SSOR.java:160)
    if (M->kind == MTJG_PC_SSOR) MTJG_CUDA(cudaMemcpyAsync(M->d_x, x, nb, cudaMemcpyHostToDevice, ctx->stream));
    int st = trans ? precond_trans_apply_dev(M, M->d_b, M->d_x, nullptr) : precond_apply_dev(M, M->d_b, M->d_x, nullptr);
    if (st != MTJG_OK) return st;
    MTJG_CUDA(cudaMemcpyAsync(x, M->d_x, nb, cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    return MTJG_OK;
}

extern "C" int mtjg_precond_apply(mtjg_precond *M, const double *b, double *x)
{
    return precond_host_call(M, b, x, false);
}

extern "C" int mtjg_precond_trans_apply(mtjg_precond *M, const double *b, double *x)
{
    return precond_host_call(M, b, x, true);
}

extern "C" int mtjg_precond_apply_dev(mtjg_precond *M, const double *db, double *dx)
{
    if (!M || !db || !dx) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (!M->ready) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "setMatrix has not been called");
    MTJG_CUDA(cudaSetDevice(M->ctx->device));
    return precond_apply_dev(M, db, dx, nullptr);
}

extern "C" int mtjg_precond_values(mtjg_precond *M, double *out, int64_t cap, int64_t *len)
{
    if (!M) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL preconditioner");
    MTJG_CUDA(cudaSetDevice(M->ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(M->ctx->stream));
    int64_t total = 0;
    const double *src = nullptr;
    if (M->kind == MTJG_PC_JACOBI) {
        total = M->invdiag ? M->n : 0;
        src = M->invdiag;
    } else if (M->kind != MTJG_PC_IDENTITY) {
        total = M->data ? M->nnz : 0;
        src = M->data;
    }
    if (len) *len = total;
    const int64_t m = std::min(total, cap);
    if (m > 0 && out) MTJG_CUDA(cudaMemcpy(out, src, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost));
    return MTJG_OK;
}
