// phases.cuh -- solver phases shared by the solver (solver.cu) and the
// serving engine (server.cu): the monitor plumbing and the mixed-precision
// refinement phases.
#pragma once

#include "spmv.cuh"

// resident blocks per SM the FP32 update of the inner solve is compiled for
#ifndef MTJG_MXUPD_MINB
#define MTJG_MXUPD_MINB 0
#endif
// resident CTAs per SM of the FP32 product of the inner solve: 4, as many
// as the 2560-entry FP32 stages fit (with 1728-entry stages 5 had measured
// 8 % faster than 6 on the served mix, leaving L1 room for the gathers)
#ifndef MTJG_MXQ_CTAS
#define MTJG_MXQ_CTAS 4
#endif

namespace mtjg {

constexpr int kPcIdentity = 0, kPcJacobi = 1, kPcExternal = 2;

// Mixed precision: inner iterations per outer step slot of a loop body.
constexpr int kInnerPerBody = 8;

struct MonPtrs {
    SysState *st;
    MonCfgDev mon;
    double *hr;
    int *hi;
    int *num_running;
    __device__ __forceinline__ void finish(SysState &t, int code) const
    {
        t.status = code;
        t.gate = code == ST_RUNNING ? ST_RUNNING : 1;
        if (code != ST_RUNNING) atomicSub(num_running, 1);
    }
    __device__ __forceinline__ int check(SysState &t, int sys, double r) const
    {
        return monitor_check(t, mon, r, hr + (size_t)sys * mon.hist_cap, hi + (size_t)sys * mon.hist_cap);
    }
    // converged(double): GMRES's inner test
    __device__ __forceinline__ int check_scalar(SysState &t, int sys, double r) const
    {
        return monitor_check_scalar(t, mon, r, hr + (size_t)sys * mon.hist_cap, hi + (size_t)sys * mon.hist_cap);
    }
};

// ===================================================== mixed precision
// Iterative refinement around an FP32 CG (the loop of S/IR.java:57-70 with
// the inner solve in the role of the preconditioner).  The inner CG runs in
// FP32 (values, vectors, preconditioner) until its residual has fallen by
// in_rtol, or below the monitor's target; then the outer step adds the FP32
// correction d to the FP64 x, forms the true residual r = b - A x in FP64,
// lets the monitor test it and restarts the inner CG on it.  (Keeping the
// search direction across the replacement -- reliable updates -- was
// measured slower on the served 2D Poisson mix: 1297 FP32 iterations per
// request against 889 restarted, as FP32 CG loses its superlinear phase.)
// Per system, `phase` says whether the outer step is due (0) or inner FP32
// iterations run (1); every kernel is gated on it, so the systems of a batch
// move through their own refinement steps independently.
struct MixCfg {
    double in_rtol;  // residual reduction of one inner solve
    int in_max;      // inner iterations per outer step, at most
    int pad;
    double rtol, atol;  // the monitor's target (an inner solve also ends below it)
};

// x += d (the FP32 correction, widened exactly); iter.next() of the outer loop
struct MxX {
    double *x;
    const float *d;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = 0;
    __device__ bool active(int sys) const
    {
        const SysState &t = st[sys];
        return t.status == ST_RUNNING && t.phase == 0 && t.pending;
    }
    static constexpr bool kBatched = true;
    __device__ void row(int i, int, Acc &) const { x[i] = x[i] + (double)d[i]; }
    __device__ void rows(int base, int end, int, Acc &) const
    {
        double xv[kRowsPerThread];
        float dv[kRowsPerThread];
#pragma unroll
        for (int u = 0; u < kRowsPerThread; ++u) {
            const int i = base + u * kBlock;
            xv[u] = i < end ? x[i] : 0.0;
            dv[u] = i < end ? __ldg(d + i) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < kRowsPerThread; ++u) {
            const int i = base + u * kBlock;
            if (i < end) x[i] = xv[u] + (double)dv[u];
        }
    }
    __device__ void scalar(int sys, const Acc &)
    {
        SysState &t = st[sys];
        t.pending = 0;
        t.iter++;
    }
};

// r = b - A x in FP64, the monitor's test on it, then the inner system's
// right-hand side rin = (float) r, d = 0 and z = M rin in FP32
struct MxOuter {
    const double *b;
    float *rin, *z, *d;
    const float *invdiag;
    int pc;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const
    {
        const SysState &t = m.st[sys];
        return t.status == ST_RUNNING && t.phase == 0 && !t.pending;
    }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double dd, double, Acc &a) const
    {
        const double rr = b[i] - dd;
        norm_add<false>(a, rr, m.mon.norm);
        const float rf = (float)rr;
        rin[i] = rf;
        d[i] = 0.0f;
        float zf = rf;
        if (pc == kPcJacobi) {
            zf = rf * invdiag[i];
            z[i] = zf;
        }
        a.f[0] = fmaf(rf, zf, a.f[0]);
        a.f[1] = fmaf(rf, rf, a.f[1]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        const int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING) {
            t.phase = 1;
            t.pending = 1;
            t.in_iter = 0;
            t.in_fresh = 1;  // the inner CG restarts: p = z
            t.in_rho = s.v[2];
            t.in_r0 = sqrt(s.v[3]);
        }
        m.finish(t, c);
    }
};

struct MxP {  // p = z (first) or p = beta p + z, FP32
    float *p;
    const float *z;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING && st[sys].phase == 1; }
    static constexpr bool kBatched = true;
    __device__ void row(int i, int sys, Acc &) const
    {
        const SysState &t = st[sys];
        p[i] = t.in_fresh ? z[i] : fmaf(p[i], (float)t.in_beta, z[i]);
    }
    __device__ void rows(int base, int end, int sys, Acc &) const
    {
        const bool first = st[sys].in_fresh != 0;
        const float beta = (float)st[sys].in_beta;
        float zv[kRowsPerThread], pv[kRowsPerThread];
#pragma unroll
        for (int u = 0; u < kRowsPerThread; ++u) {
            const int i = base + u * kBlock;
            zv[u] = i < end ? __ldg(z + i) : 0.0f;
            pv[u] = i < end && !first ? p[i] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < kRowsPerThread; ++u) {
            const int i = base + u * kBlock;
            if (i < end) p[i] = first ? zv[u] : fmaf(pv[u], beta, zv[u]);
        }
    }
    __device__ void scalar(int, const Acc &) {}
};

struct MxQ {  // q = A32 p (FP32 row sums); alpha = rho / p.q
    float *q;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = true;
    static constexpr int kSlots = kSlotD2;
    static constexpr int kCtas = MTJG_MXQ_CTAS;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING && st[sys].phase == 1; }
    __device__ float init(int, int) const { return 0.0f; }
    __device__ void row(int i, int, float dd, float pi, Acc &a) const
    {
        q[i] = dd;
        a.f[0] = fmaf(pi, dd, a.f[0]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.in_alpha = t.in_rho / s.v[2];
    }
};

struct MxUpd {  // d += alpha p; rin -= alpha q; z = M rin; inner stopping test
    float *d, *rin, *z;
    const float *p, *q, *invdiag;
    int pc;
    SysState *st;
    MixCfg cfg;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2 | kSlotD3;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING && st[sys].phase == 1; }
    static constexpr bool kBatched = true;
    static constexpr int kMinBlocks = MTJG_MXUPD_MINB;
    __device__ void row(int i, int sys, Acc &a) const
    {
        const float al = (float)st[sys].in_alpha;
        d[i] = fmaf(al, p[i], d[i]);
        const float rf = fmaf(-al, q[i], rin[i]);
        rin[i] = rf;
        float zf = rf;
        if (pc == kPcJacobi) {
            zf = rf * invdiag[i];
            z[i] = zf;
        }
        a.f[0] = fmaf(rf, zf, a.f[0]);
        a.f[1] = fmaf(rf, rf, a.f[1]);
    }
    __device__ void rows(int base, int end, int sys, Acc &a) const
    {
        constexpr int U = kRowsPerThread;
        const float al = (float)st[sys].in_alpha;
        float dv[U], pv[U], qv[U], rv[U], iv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = base + u * kBlock;
            const bool in = i < end;
            dv[u] = in ? d[i] : 0.0f;
            pv[u] = in ? __ldg(p + i) : 0.0f;
            qv[u] = in ? __ldg(q + i) : 0.0f;
            rv[u] = in ? rin[i] : 0.0f;
            iv[u] = in && pc == kPcJacobi ? __ldg(invdiag + i) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = base + u * kBlock;
            if (i >= end) break;
            d[i] = fmaf(al, pv[u], dv[u]);
            const float rf = fmaf(-al, qv[u], rv[u]);
            rin[i] = rf;
            float zf = rf;
            if (pc == kPcJacobi) {
                zf = rf * iv[u];
                z[i] = zf;
            }
            a.f[0] = fmaf(rf, zf, a.f[0]);
            a.f[1] = fmaf(rf, rf, a.f[1]);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.in_iter++;
        t.in_total++;
        t.in_fresh = 0;
        const double rn = sqrt(s.v[3]);
        const double target = jmax(cfg.rtol * t.initR, cfg.atol);
        if (!(rn > cfg.in_rtol * t.in_r0) || !(rn > target) || t.in_iter >= cfg.in_max) {
            t.phase = 0;  // the correction in d goes to x in the next outer step
        } else {
            t.in_rho_1 = t.in_rho;
            t.in_rho = s.v[2];
            t.in_beta = t.in_rho / t.in_rho_1;
        }
    }
};

static __global__ void k_to_f32(int64_t n, const double *a, float *b)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

}  // namespace mtjg
