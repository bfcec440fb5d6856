// batch.cu -- a batch of independent systems solved by CG in one persistent
// launch (the batching form): every CTA takes whole systems, largest first,
// from a ticket counter and runs each one's complete CG loop on the chip --
// products, vector updates, fixed-order block reductions, MTJ's monitor --
// with block barriers only, so thousands of uneven systems need no
// grid-wide phase, no launch per iteration and no host round trip.  A
// system's convergence ends its loop (per-system masks), its CTA takes the
// next system.
//
// Arithmetic per system is that of the CG phases (S/CG.java:58-87 with
// DiagonalPreconditioner, or the FP32-inner / FP64-refinement form of
// phases.cuh): same operation order per row and per vector update; dot
// products and norms are fixed-order block trees.  A system's results
// depend only on the system and its lanes per row (chosen per system class
// by the autotuner below), never on the batch around it or on which CTA
// takes it: alone and in any batch they are bit-identical.
//
// Autotuner: a system class is (rows band, entries-per-row band).  On the
// first batch that holds a class, short probe solves (kProbeIters
// iterations on up to kProbeSystems of its systems) are timed with CUDA
// events for each lanes-per-row candidate; the fastest is kept for the rest
// of the process.  MTJG_TUNE=0 in the environment skips the probes and
// takes the entries-per-row rule of the tiled products instead.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <numeric>

#include "batch.cuh"

namespace mtjg {

constexpr int kBatchBlock = 256;
// resident CTAs per SM the batched CG is compiled for (its register cap).
// Measured on GB300 (C4, FP64 / mixed): 3 (80 registers) 168.5 / 115.7 ms;
// 4 (64 registers) 200.9 / 128.0 ms; 5: 238.6 / 152.8 ms -- the rows a
// thread keeps in flight matter more than resident warps.
#ifndef MTJG_BATCH_MINB
#define MTJG_BATCH_MINB 3
#endif
constexpr int kBatchMinBlocks = MTJG_BATCH_MINB;
constexpr int kProbeIters = 12;
constexpr int kProbeSystems = 24;
constexpr int kVecCandidates[] = {1, 2, 4, 8, 32};
constexpr unsigned char kPairFlag = 0x80;  // in a system's lanes byte: pair its FP32 product rows

namespace {

// Fixed-order block reduction: a fixed butterfly inside each warp, then
// warps in order by thread 0; the result is broadcast through `out`.
template <int SLOTS>
__device__ __forceinline__ void cta_reduce(Acc &a, int type, Acc *warp_acc, Acc &out)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if constexpr ((SLOTS & kSlotD2) != 0) a.v[2] += (double)a.f[0];
    if constexpr ((SLOTS & kSlotD3) != 0) a.v[3] += (double)a.f[1];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc_shfl_down<SLOTS>(a, off, type);
    if (lane == 0) warp_acc[w] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        Acc s = warp_acc[0];
        for (int k = 1; k < kBatchBlock / 32; ++k) acc_merge_m<SLOTS>(s, warp_acc[k], type);
        out = s;
    }
    __syncthreads();
}

// row i of A (x gathered), summed by VEC lanes in entry order per lane and a
// fixed butterfly; every lane of the group returns the sum.  The matrix is
// read-only for the launch (read-only path); x was written by this CTA
// earlier in the launch, so it is read with coherent loads.
template <int VEC, bool S, class T>
__device__ __forceinline__ T row_dot(const int *__restrict__ rp, const int *__restrict__ ci,
                                     const T *__restrict__ v, const T *x, int i, bool in, int l)
{
    T sum = T(0);
    if (in) {
        const int b = __ldg(rp + i), e = __ldg(rp + i + 1);
#pragma unroll 4
        for (int k = b + l; k < e; k += VEC) sum = fmac<S>(__ldg(v + k), x[__ldg(ci + k)], sum);
    }
#pragma unroll
    for (int off = VEC / 2; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off, VEC);
    return sum;
}

// Build-time knob: MTJG_BATCH_U is the rows per thread and step of the
// element-wise loops (1: one row at a time); it changes no result.
#ifndef MTJG_BATCH_U
#define MTJG_BATCH_U 4
#endif

// Rows ia and ib of a product step.  Paired (`pair`), their gathers are in
// flight at once, so a thread waits one latency round for both; else one
// after the other.  Each row keeps its entry order and its butterfly, so
// the sums are the same either way.  Measured on GB300 (C4 and a batch of
// 2D Poisson grids): pairing made the FP32 inner products of 5-entry rows
// 10 % faster and those of ~19-entry rows, and every FP64 product, slower;
// a system pairs its FP32 products when its rows average under 12 entries
// (kPairFlag in its lanes byte).
template <int VEC, bool S, class T>
__device__ __forceinline__ void row_dot2(const int *__restrict__ rp, const int *__restrict__ ci,
                                         const T *__restrict__ v, const T *x, int ia, bool ina, int ib, bool inb,
                                         int l, T &sa, T &sb, bool pair)
{
    if (!pair) {
        sa = row_dot<VEC, S>(rp, ci, v, x, ia, ina, l);
        sb = row_dot<VEC, S>(rp, ci, v, x, ib, inb, l);
        return;
    }
    T a = T(0), b = T(0);
    const int ba = ina ? __ldg(rp + ia) : 0, la = ina ? __ldg(rp + ia + 1) - ba : 0;
    const int bb = inb ? __ldg(rp + ib) : 0, lb = inb ? __ldg(rp + ib + 1) - bb : 0;
    const int lm = la > lb ? la : lb;
#pragma unroll 4
    for (int k = l; k < lm; k += VEC) {
        if (k < la) a = fmac<S>(__ldg(v + ba + k), x[__ldg(ci + ba + k)], a);
        if (k < lb) b = fmac<S>(__ldg(v + bb + k), x[__ldg(ci + bb + k)], b);
    }
#pragma unroll
    for (int off = VEC / 2; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off, VEC);
        b += __shfl_xor_sync(0xffffffffu, b, off, VEC);
    }
    sa = a;
    sb = b;
}

// Element-wise loops over a system's rows take kU rows per thread and step:
// every load of the step is issued before its first store (the vectors may
// alias, so the compiler cannot hoist them itself); rows are still visited,
// and accumulated, in the order i = r0 + tid, r0 + tid + kBatchBlock, ...
constexpr int kU = MTJG_BATCH_U;
constexpr int kU2 = kU > 2 ? 2 : kU;  // the FP64 update loop, whose rows carry five doubles

__device__ __forceinline__ int batch_check(const BatchCg &a, SysState &t, int sys, double r)
{
    const size_t h = (size_t)sys * a.mon.hist_cap;
    return monitor_check(t, a.mon, r, a.hist_r + h, a.hist_it + h);
}

struct Shared {
    Acc warp_acc[kBatchBlock / 32];
    Acc out;
    double sc[4];
    int status, iter, flag, k;
};

// CG + identity / Jacobi on rows [r0, r1): CgInit, then CgP, CgQ, CgUpd per
// iteration (solver.cu), in one CTA
template <int VEC, bool S>
__device__ void cg_system(const BatchCg &a, int sys, Shared &sh)
{
    const int r0 = a.sys_rows[sys], r1 = a.sys_rows[sys + 1];
    const int tid = threadIdx.x, g = tid / VEC, l = tid % VEC;
    constexpr int RPS = kBatchBlock / VEC;
    const int nt = a.mon.norm;
    const bool jac = a.pc == kPcJacobi;
    // z is r itself without a preconditioner: no restrict on the vectors
    double *r = a.r, *z = jac ? a.z : a.r, *p = a.p, *q = a.q, *x = a.x;
    const double *inv = a.invdiag;
    Acc acc;
    acc_zero(acc);
    for (int base = r0; base < r1; base += 2 * RPS) {  // r = b - A x; z = M r; |r|; r.z
        double dv[2];
        row_dot2<VEC, S>(a.rowptr, a.colind, a.val, (const double *)x, base + g, base + g < r1, base + RPS + g,
                         base + RPS + g < r1, l, dv[0], dv[1], false);
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int i = base + u * RPS + g;
            if (i < r1 && l == 0) {
                const double rr = a.b[i] - dv[u];
                r[i] = rr;
                norm_add<S>(acc, rr, nt);
                if (jac) {
                    const double zz = rr * inv[i];
                    z[i] = zz;
                    acc.v[2] = fmac<S>(rr, zz, acc.v[2]);
                } else {
                    acc.v[2] = fmac<S>(rr, rr, acc.v[2]);
                }
            }
        }
    }
    cta_reduce<kSlotNorm | kSlotD2>(acc, nt, sh.warp_acc, sh.out);
    if (tid == 0) {
        SysState &t = a.st[sys];
        t.iter = 0;
        const int c = batch_check(a, t, sys, norm_finish(sh.out.v, nt));
        if (c == ST_RUNNING) t.rho = sh.out.v[2];
        t.status = c;
        sh.status = c;
        sh.iter = 0;
        sh.sc[1] = t.beta;
    }
    __syncthreads();
    while (sh.status == ST_RUNNING) {
        const bool first = sh.iter == 0;
        const double beta = sh.sc[1];
        for (int base = r0 + tid; base < r1; base += kU * kBatchBlock) {  // p = z or p = beta p + z
            double zv[kU], pv[kU];
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int i = base + u * kBatchBlock;
                zv[u] = i < r1 ? z[i] : 0.0;
                pv[u] = i < r1 && !first ? p[i] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kU; ++u) {
                const int i = base + u * kBatchBlock;
                if (i < r1) p[i] = first ? zv[u] : fmac<S>(pv[u], beta, zv[u]);
            }
        }
        __syncthreads();
        acc_zero(acc);
        for (int base = r0; base < r1; base += 2 * RPS) {  // q = A p; p.q
            double dv[2];
            row_dot2<VEC, S>(a.rowptr, a.colind, a.val, (const double *)p, base + g, base + g < r1, base + RPS + g,
                             base + RPS + g < r1, l, dv[0], dv[1], false);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int i = base + u * RPS + g;
                if (i < r1 && l == 0) {
                    const double qq = mtj_assign(dv[u]);
                    q[i] = qq;
                    acc.v[2] = fmac<S>(p[i], qq, acc.v[2]);
                }
            }
        }
        cta_reduce<kSlotD2>(acc, nt, sh.warp_acc, sh.out);
        if (tid == 0) {
            SysState &t = a.st[sys];
            t.alpha = t.rho / sh.out.v[2];
            sh.sc[0] = t.alpha;
        }
        __syncthreads();
        const double al = sh.sc[0];
        acc_zero(acc);
        for (int base = r0 + tid; base < r1; base += kU2 * kBatchBlock) {  // x += alpha p; r -= alpha q; z = M r
            double rv[kU2], xv[kU2], pv[kU2], qv[kU2], iv[kU2];
#pragma unroll
            for (int u = 0; u < kU2; ++u) {
                const int i = base + u * kBatchBlock;
                const bool in = i < r1;
                rv[u] = in ? r[i] : 0.0;
                xv[u] = in && al != 0 ? x[i] : 0.0;
                pv[u] = in && al != 0 ? p[i] : 0.0;
                qv[u] = in && al != 0 ? q[i] : 0.0;
                iv[u] = in && jac ? inv[i] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < kU2; ++u) {
                const int i = base + u * kBatchBlock;
                if (i >= r1) break;
                double rr = rv[u];
                if (al != 0) {
                    x[i] = fmac<S>(al, pv[u], xv[u]);
                    rr = fmac<S>(-al, qv[u], rr);
                    r[i] = rr;
                }
                norm_add<S>(acc, rr, nt);
                if (jac) {
                    const double zz = rr * iv[u];
                    z[i] = zz;
                    acc.v[2] = fmac<S>(rr, zz, acc.v[2]);
                } else {
                    acc.v[2] = fmac<S>(rr, rr, acc.v[2]);
                }
            }
        }
        cta_reduce<kSlotNorm | kSlotD2>(acc, nt, sh.warp_acc, sh.out);
        if (tid == 0) {
            SysState &t = a.st[sys];
            t.rho_1 = t.rho;
            t.iter++;
            const int c = batch_check(a, t, sys, norm_finish(sh.out.v, nt));
            if (c == ST_RUNNING) {
                t.rho = sh.out.v[2];
                t.beta = t.rho / t.rho_1;
            }
            t.status = c;
            sh.status = c;
            sh.iter = t.iter;
            sh.sc[1] = t.beta;
        }
        __syncthreads();
    }
}

// Mixed precision on rows [r0, r1): the outer step and inner FP32 CG of
// phases.cuh (MxX, MxOuter, MxP, MxQ, MxUpd), in one CTA
template <int VEC, bool S>
__device__ void mixed_system(const BatchCg &a, int sys, Shared &sh)
{
    const bool pair = (a.vec[sys] & kPairFlag) != 0;
    const int r0 = a.sys_rows[sys], r1 = a.sys_rows[sys + 1];
    const int tid = threadIdx.x, g = tid / VEC, l = tid % VEC;
    constexpr int RPS = kBatchBlock / VEC;
    const int nt = a.mon.norm;
    const bool jac = a.pc == kPcJacobi;
    // z is rin itself without a preconditioner: no restrict on the vectors
    float *rin = a.r32, *z = jac ? a.z32 : a.r32, *p = a.p32, *q = a.q32, *d = a.d32;
    const float *inv = a.invdiag32;
    double *x = a.x;
    for (;;) {
        // the outer step: x += d when a correction is pending (MxX) ...
        if (tid == 0) sh.flag = a.st[sys].pending;
        __syncthreads();
        const bool pend = sh.flag != 0;
        __syncthreads();  // every thread has read the flag before it is rewritten
        if (pend) {
            for (int base = r0 + tid; base < r1; base += kU * kBatchBlock) {
                double xv[kU];
                float dv[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int i = base + u * kBatchBlock;
                    xv[u] = i < r1 ? x[i] : 0.0;
                    dv[u] = i < r1 ? d[i] : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int i = base + u * kBatchBlock;
                    if (i < r1) x[i] = xv[u] + (double)dv[u];
                }
            }
            __syncthreads();
            if (tid == 0) {
                SysState &t = a.st[sys];
                t.pending = 0;
                t.iter++;
            }
        }
        // ... then r = b - A x in FP64, the monitor's test, the inner start (MxOuter)
        Acc acc;
        acc_zero(acc);
        for (int base = r0; base < r1; base += 2 * RPS) {
            double dv[2];
            row_dot2<VEC, S>(a.rowptr, a.colind, a.val, (const double *)x, base + g, base + g < r1, base + RPS + g,
                             base + RPS + g < r1, l, dv[0], dv[1], false);
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int i = base + u * RPS + g;
                if (i < r1 && l == 0) {
                    const double rr = a.b[i] - dv[u];
                    norm_add<false>(acc, rr, nt);
                    const float rf = (float)rr;
                    rin[i] = rf;
                    d[i] = 0.0f;
                    float zf = rf;
                    if (jac) {
                        zf = rf * inv[i];
                        z[i] = zf;
                    }
                    acc.f[0] = fmaf(rf, zf, acc.f[0]);
                    acc.f[1] = fmaf(rf, rf, acc.f[1]);
                }
            }
        }
        cta_reduce<kSlotNorm | kSlotD2 | kSlotD3>(acc, nt, sh.warp_acc, sh.out);
        if (tid == 0) {
            SysState &t = a.st[sys];
            const int c = batch_check(a, t, sys, norm_finish(sh.out.v, nt));
            if (c == ST_RUNNING) {
                t.phase = 1;
                t.pending = 1;
                t.in_iter = 0;
                t.in_fresh = 1;
                t.in_rho = sh.out.v[2];
                t.in_r0 = sqrt(sh.out.v[3]);
            }
            t.status = c;
            sh.status = c;
        }
        __syncthreads();
        if (sh.status != ST_RUNNING) return;
        // inner FP32 CG until its stopping test ends the refinement step
        for (;;) {
            if (tid == 0) {
                const SysState &t = a.st[sys];
                sh.flag = t.in_fresh;
                sh.sc[1] = t.in_beta;
            }
            __syncthreads();
            const bool fresh = sh.flag != 0;
            const float beta = (float)sh.sc[1];
            __syncthreads();  // read before thread 0 rewrites them
            for (int base = r0 + tid; base < r1; base += kU * kBatchBlock) {
                float zv[kU], pv[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int i = base + u * kBatchBlock;
                    zv[u] = i < r1 ? z[i] : 0.0f;
                    pv[u] = i < r1 && !fresh ? p[i] : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int i = base + u * kBatchBlock;
                    if (i < r1) p[i] = fresh ? zv[u] : fmaf(pv[u], beta, zv[u]);
                }
            }
            __syncthreads();
            acc_zero(acc);
            for (int base = r0; base < r1; base += 2 * RPS) {  // q = A32 p; p.q
                float dv[2];
                row_dot2<VEC, false>(a.rowptr, a.colind, a.val32, (const float *)p, base + g, base + g < r1,
                                     base + RPS + g, base + RPS + g < r1, l, dv[0], dv[1], pair);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int i = base + u * RPS + g;
                    if (i < r1 && l == 0) {
                        q[i] = dv[u];
                        acc.f[0] = fmaf(p[i], dv[u], acc.f[0]);
                    }
                }
            }
            cta_reduce<kSlotD2>(acc, nt, sh.warp_acc, sh.out);
            if (tid == 0) {
                SysState &t = a.st[sys];
                t.in_alpha = t.in_rho / sh.out.v[2];
                sh.sc[0] = t.in_alpha;
            }
            __syncthreads();
            const float al = (float)sh.sc[0];
            acc_zero(acc);
            for (int base = r0 + tid; base < r1; base += kU * kBatchBlock) {  // d += alpha p; rin -= alpha q; z = M rin
                float dv[kU], pv[kU], qv[kU], rv[kU], iv[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int i = base + u * kBatchBlock;
                    const bool in = i < r1;
                    dv[u] = in ? d[i] : 0.0f;
                    pv[u] = in ? p[i] : 0.0f;
                    qv[u] = in ? q[i] : 0.0f;
                    rv[u] = in ? rin[i] : 0.0f;
                    iv[u] = in && jac ? inv[i] : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int i = base + u * kBatchBlock;
                    if (i >= r1) break;
                    d[i] = fmaf(al, pv[u], dv[u]);
                    const float rf = fmaf(-al, qv[u], rv[u]);
                    rin[i] = rf;
                    float zf = rf;
                    if (jac) {
                        zf = rf * iv[u];
                        z[i] = zf;
                    }
                    acc.f[0] = fmaf(rf, zf, acc.f[0]);
                    acc.f[1] = fmaf(rf, rf, acc.f[1]);
                }
            }
            cta_reduce<kSlotD2 | kSlotD3>(acc, nt, sh.warp_acc, sh.out);
            if (tid == 0) {
                SysState &t = a.st[sys];
                t.in_iter++;
                t.in_total++;
                t.in_fresh = 0;
                const double rn = sqrt(sh.out.v[3]);
                const double target = jmax(a.mix.rtol * t.initR, a.mix.atol);
                if (!(rn > a.mix.in_rtol * t.in_r0) || !(rn > target) || t.in_iter >= a.mix.in_max) {
                    t.phase = 0;
                } else {
                    t.in_rho_1 = t.in_rho;
                    t.in_rho = sh.out.v[2];
                    t.in_beta = t.in_rho / t.in_rho_1;
                }
                sh.flag = t.phase;
            }
            __syncthreads();
            const bool stop = sh.flag == 0;
            __syncthreads();  // every thread has read the flag before it is rewritten
            if (stop) break;
        }
    }
}

template <bool S, bool MIXED>
__global__ void __launch_bounds__(kBatchBlock, kBatchMinBlocks) k_batch_cg(BatchCg a)
{
    __shared__ Shared sh;
    for (;;) {
        if (threadIdx.x == 0) sh.k = (int)atomicAdd(a.ticket, 1u);
        __syncthreads();
        const int k = sh.k;
        __syncthreads();
        if (k >= a.count) return;
        const int sys = a.order[k];
        const int vec = S ? 1 : (a.vec[sys] & ~kPairFlag);
        if constexpr (MIXED) {
            switch (vec) {
            case 2: mixed_system<2, S>(a, sys, sh); break;
            case 4: mixed_system<4, S>(a, sys, sh); break;
            case 8: mixed_system<8, S>(a, sys, sh); break;
            case 32: mixed_system<32, S>(a, sys, sh); break;
            default: mixed_system<1, S>(a, sys, sh); break;
            }
        } else {
            switch (vec) {
            case 2: cg_system<2, S>(a, sys, sh); break;
            case 4: cg_system<4, S>(a, sys, sh); break;
            case 8: cg_system<8, S>(a, sys, sh); break;
            case 32: cg_system<32, S>(a, sys, sh); break;
            default: cg_system<1, S>(a, sys, sh); break;
            }
        }
        __syncthreads();
    }
}

template <bool S, bool MIXED>
cudaError_t launch_one(mtjg_ctx *ctx, const BatchCg &a)
{
    auto k = k_batch_cg<S, MIXED>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBatchBlock, 0);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min(a.count, ctx->num_sms * std::max(1, per_sm)));
    k<<<grid, kBatchBlock, 0, ctx->stream>>>(a);
    ctx->launches++;
    return cudaGetLastError();
}

// ----------------------------------------------------------- autotuner
std::mutex g_tune_mu;
std::map<int, int> g_tuned;  // class -> lanes per row

int band(double v, const double *edges, int count)
{
    int k = 0;
    while (k < count && v >= edges[k]) ++k;
    return k;
}

}  // namespace

cudaError_t batch_launch(mtjg_ctx *ctx, const BatchCg &a, bool mixed)
{
    const bool strict = ctx->numerics == MTJG_NUMERICS_STRICT;
    if (strict) return mixed ? launch_one<true, true>(ctx, a) : launch_one<true, false>(ctx, a);
    return mixed ? launch_one<false, true>(ctx, a) : launch_one<false, false>(ctx, a);
}

// The class of a system: bands of its rows and of its entries per row.
int batch_class(int64_t rows, int64_t nnz)
{
    static const double kRows[] = {2048, 8192, 32768, 131072};
    static const double kPerRow[] = {6, 12, 24, 48};
    const double per = rows > 0 ? (double)nnz / (double)rows : 0.0;
    return band((double)rows, kRows, 4) * 8 + band(per, kPerRow, 4);
}

int batch_tuned(int cls)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(cls);
    return it == g_tuned.end() ? 0 : it->second;
}

// Lanes per row of each system of the batch; classes not tuned yet are
// probed first (solve() restores x and the system states afterwards).
// `probe(order, vec, iters)` runs the persistent solve on the systems in
// `order` with every system's lanes set from `vec`, capped at `iters`
// iterations, and returns its milliseconds (negative on an error).
int batch_vec(int num_sys, const int *sys_rows, const int *h_rowptr, std::vector<unsigned char> &vec,
              const std::function<double(const std::vector<int> &, int, int)> &probe)
{
    vec.assign((size_t)num_sys, 1);
    const char *env = getenv("MTJG_TUNE");
    const bool tune = !(env && env[0] == '0');
    std::map<int, std::vector<int>> by_class;
    for (int s = 0; s < num_sys; ++s) {
        const int64_t rows = sys_rows[s + 1] - sys_rows[s];
        const int64_t nnz = (int64_t)h_rowptr[sys_rows[s + 1]] - h_rowptr[sys_rows[s]];
        by_class[batch_class(rows, nnz)].push_back(s);
    }
    for (auto &kv : by_class) {
        int v = batch_tuned(kv.first);
        if (v == 0) {
            const std::vector<int> &ss = kv.second;
            int64_t rows = 0, nnz = 0;
            for (int s : ss) {
                rows += sys_rows[s + 1] - sys_rows[s];
                nnz += (int64_t)h_rowptr[sys_rows[s + 1]] - h_rowptr[sys_rows[s]];
            }
            v = choose_vec(nnz, rows);
            if (tune) {
                // the largest systems of the class: they carry most of its time
                std::vector<int> pick(ss);
                std::sort(pick.begin(), pick.end(), [&](int x, int y) {
                    return sys_rows[x + 1] - sys_rows[x] > sys_rows[y + 1] - sys_rows[y];
                });
                if ((int)pick.size() > kProbeSystems) pick.resize(kProbeSystems);
                double best = -1;
                for (int cand : kVecCandidates) {
                    probe(pick, cand, kProbeIters);  // warm-up
                    const double ms = probe(pick, cand, kProbeIters);
                    if (ms < 0) return MTJG_ERR_CUDA;
                    if (best < 0 || ms < best) {
                        best = ms;
                        v = cand;
                    }
                }
            }
            std::lock_guard<std::mutex> lk(g_tune_mu);
            if (tune) g_tuned.emplace(kv.first, v);
        }
        for (int s : kv.second) {
            const int64_t rows = sys_rows[s + 1] - sys_rows[s];
            const int64_t nnz = (int64_t)h_rowptr[sys_rows[s + 1]] - h_rowptr[sys_rows[s]];
            vec[(size_t)s] = (unsigned char)(v | (nnz < 12 * rows ? kPairFlag : 0));
        }
    }
    return MTJG_OK;
}

}  // namespace mtjg

using namespace mtjg;

extern "C" int mtjg_batch_tuning(int64_t rows, int64_t nnz, int *lanes_per_row)
{
    if (!lanes_per_row) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *lanes_per_row = batch_tuned(batch_class(rows, nnz));
    return MTJG_OK;
}
