// solver.cu -- CG, BiCGstab and GMRES(m) (S/CG.java, S/BiCGstab.java,
// S/GMRES.java) as fused device phases.
//
// Every phase is one kernel over the matrix's tiles: a CSR product with a
// fused epilogue or a row kernel, whose per-tile partial sums a small
// finalize launch reduces in tile order before running the phase's scalar
// step (alpha, beta, omega, Givens rotations, the iteration monitor) on the
// device.  The host never reads a scalar during a solve: the loop
// body is captured once into a CUDA graph, replayed in chunks, and every
// kernel of a finished solve returns at once.  The host only polls the
// status word between chunks.
#include <algorithm>
#include <cstring>
#include <numeric>

#include "batch.cuh"
#include "krylov_ext.cuh"
#include "mixed_ir_phases.cuh"

// resident blocks per SM the CG update is compiled for (it keeps four rows of
// five FP64 vectors in flight per thread)
#ifndef MTJG_CGUPD_MINB
#define MTJG_CGUPD_MINB 4
#endif
// resident CTAs per SM of the CG product (40 registers without spills in
// FAST numerics; its one-slot reduction leaves room in shared memory)
#ifndef MTJG_CGQ_CTAS
#define MTJG_CGQ_CTAS 6
#endif

namespace mtjg {

int precond_apply_dev(mtjg_precond *M, const double *b, double *x, const int *status);
int precond_trans_apply_dev(mtjg_precond *M, const double *b, double *x, const int *status);
int precond_prepare_trans(mtjg_precond *M);
int precond_prepare32(mtjg_precond *M);
int precond_apply32(mtjg_precond *M, const float *b, float *x, const int *status);
int csr_ensure_transpose(mtjg_csr *A);


// ================================================================== CG
// S/CG.java:58-87.  pc == kPcExternal (ILU/ICC): z = M r runs as its own
// kernels between the monitor test and CgDot.
template <bool S>
struct CgInit {  // r = b - A x (A.multAdd(-1, x, r.set(b)), :64); fused z = M r and r.z
    const double *b;
    double *r, *z;
    const double *invdiag;
    int pc;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm | kSlotD2;
    __device__ bool active(int) const { return true; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double rr = b[i] - d;
        r[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
        if (pc == kPcJacobi) {
            const double zz = rr * invdiag[i];
            z[i] = zz;
            a.v[2] = fmac<S>(rr, zz, a.v[2]);
        } else if (pc == kPcIdentity) {
            a.v[2] = fmac<S>(rr, rr, a.v[2]);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.iter = 0;
        const int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING && pc != kPcExternal) t.rho = s.v[2];
        m.finish(t, c);
    }
};

template <bool S>
struct CgP {  // p = z (first) or p = beta*p + z (p.scale(beta).add(z), :70-75)
    double *p;
    const double *z;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    static constexpr bool kBatched = true;
    __device__ void row(int i, int sys, Acc &) const
    {
        const SysState &t = st[sys];
        p[i] = t.iter == 0 ? z[i] : fmac<S>(p[i], t.beta, z[i]);
    }
    __device__ void rows(int base, int end, int sys, Acc &) const
    {
        const bool first = st[sys].iter == 0;
        const double beta = st[sys].beta;
        double zv[kRowsPerThread], pv[kRowsPerThread];
#pragma unroll
        for (int u = 0; u < kRowsPerThread; ++u) {
            const int i = base + u * kBlock;
            zv[u] = i < end ? __ldg(z + i) : 0.0;
            pv[u] = i < end && !first ? p[i] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < kRowsPerThread; ++u) {
            const int i = base + u * kBlock;
            if (i < end) p[i] = first ? zv[u] : fmac<S>(pv[u], beta, zv[u]);
        }
    }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct CgQ {  // q = A p; alpha = rho / p.q (:77-78)
    const double *p;
    double *q;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = true;  // p_i arrives with the row's diagonal gather
    static constexpr int kSlots = kSlotD2;
    static constexpr int kCtas = MTJG_CGQ_CTAS;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double pi, Acc &a) const
    {
        const double qq = mtj_assign(d);
        q[i] = qq;
        a.v[2] = fmac<S>(pi, qq, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.alpha = t.rho / s.v[2];
    }
};

template <bool S>
struct CgUpd {  // x += alpha p; r -= alpha q; next monitor test; fused z = M r, r.z (:80-83, :66-68)
    double *x, *r, *z;
    const double *p, *q, *invdiag;
    int pc;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm | kSlotD2;
    static constexpr bool kBatched = true;
    static constexpr int kMinBlocks = MTJG_CGUPD_MINB;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &a) const
    {
        const double al = m.st[sys].alpha;
        double rr = r[i];
        if (al != 0) {
            x[i] = fmac<S>(al, p[i], x[i]);
            rr = fmac<S>(-al, q[i], rr);
            r[i] = rr;
        }
        norm_add<S>(a, rr, m.mon.norm);
        if (pc == kPcJacobi) {
            const double zz = rr * invdiag[i];
            z[i] = zz;
            a.v[2] = fmac<S>(rr, zz, a.v[2]);
        } else if (pc == kPcIdentity) {
            a.v[2] = fmac<S>(rr, rr, a.v[2]);
        }
    }
    __device__ void rows(int base, int end, int sys, Acc &a) const
    {
        constexpr int U = kRowsPerThread;
        const double al = m.st[sys].alpha;
        const int nt = m.mon.norm;
        double rv[U], xv[U], pv[U], qv[U], dv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = base + u * kBlock;
            const bool in = i < end;
            rv[u] = in ? r[i] : 0.0;
            xv[u] = in && al != 0 ? x[i] : 0.0;
            pv[u] = in && al != 0 ? __ldg(p + i) : 0.0;
            qv[u] = in && al != 0 ? __ldg(q + i) : 0.0;
            dv[u] = in && pc == kPcJacobi ? __ldg(invdiag + i) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = base + u * kBlock;
            if (i >= end) break;
            double rr = rv[u];
            if (al != 0) {
                x[i] = fmac<S>(al, pv[u], xv[u]);
                rr = fmac<S>(-al, qv[u], rr);
                r[i] = rr;
            }
            norm_add<S>(a, rr, nt);
            if (pc == kPcJacobi) {
                const double zz = rr * dv[u];
                z[i] = zz;
                a.v[2] = fmac<S>(rr, zz, a.v[2]);
            } else if (pc == kPcIdentity) {
                a.v[2] = fmac<S>(rr, rr, a.v[2]);
            }
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.rho_1 = t.rho;
        t.iter++;
        const int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING && pc != kPcExternal) {
            t.rho = s.v[2];
            t.beta = t.rho / t.rho_1;
        }
        m.finish(t, c);
    }
};

template <bool S>
struct CgDot {  // rho = r.z after an external preconditioner (:68, :73)
    const double *r, *z;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int, Acc &a) const { a.v[2] = fmac<S>(r[i], z[i], a.v[2]); }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.rho = s.v[2];
        if (t.iter > 0) t.beta = t.rho / t.rho_1;
    }
};

// ============================================================ BiCGstab
// S/BiCGstab.java:65-116
__device__ __forceinline__ void bicg_breakdown(SysState &t, int &c)
{
    if (t.rho_1 == 0) {
        c = MTJG_NOT_CONVERGED_BREAKDOWN;
        t.detail = 1;
    } else if (t.omega == 0) {
        c = MTJG_NOT_CONVERGED_BREAKDOWN;
        t.detail = 2;
    }
}

template <bool S>
struct BiInit {  // r = b - A x; rtilde = r (:71-72); first test; rho_1 = rtilde.r (:75)
    const double *b;
    double *r, *rt;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int) const { return true; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double rr = b[i] - d;
        r[i] = rr;
        rt[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
        a.v[2] = fmac<S>(rr, rr, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.iter = 0;
        int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING) {
            t.rho_1 = s.v[2];
            bicg_breakdown(t, c);
        }
        m.finish(t, c);
    }
};

template <bool S>
struct BiP {  // p = r (first) or p = r + beta (p - omega v) (:85-95); fused phat = M p
    double *p, *phat;
    const double *r, *v, *invdiag;
    int pc;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &) const
    {
        const SysState &t = st[sys];
        double pp;
        if (t.iter == 0) {
            pp = r[i];
        } else {
            const double tmp = fmac<S>(-t.omega, v[i], p[i]);
            pp = t.beta != 0 ? fmac<S>(t.beta, tmp, r[i]) : r[i];
        }
        p[i] = pp;
        if (pc == kPcJacobi) phat[i] = pp * invdiag[i];
    }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct BiV {  // v = A phat; alpha = rho_1 / rtilde.v (:98-99)
    double *v;
    const double *rt;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double vv = mtj_assign(d);
        v[i] = vv;
        a.v[2] = fmac<S>(rt[i], vv, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.alpha = t.rho_1 / s.v[2];
    }
};

template <bool S>
struct BiS {  // s = r - alpha v; x += alpha phat; test on s (:100-104); fused shat = M s
    double *s, *x, *shat;
    const double *r, *v, *phat, *invdiag;
    int pc;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &a) const
    {
        const double al = m.st[sys].alpha;
        double ss = r[i];
        if (al != 0) {
            ss = fmac<S>(-al, v[i], ss);
            x[i] = fmac<S>(al, phat[i], x[i]);
        }
        s[i] = ss;
        norm_add<S>(a, ss, m.mon.norm);
        if (pc == kPcJacobi) shat[i] = ss * invdiag[i];
    }
    __device__ void scalar(int sys, const Acc &sm)
    {
        SysState &t = m.st[sys];
        m.finish(t, m.check(t, sys, norm_finish(sm.v, m.mon.norm)));
    }
};

template <bool S>
struct BiT {  // t = A shat; omega = t.s / t.t (:107-108)
    double *t;
    const double *s;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double tt = mtj_assign(d);
        t[i] = tt;
        a.v[2] = fmac<S>(tt, s[i], a.v[2]);
        a.v[3] = fmac<S>(tt, tt, a.v[3]);
    }
    __device__ void scalar(int sys, const Acc &sm)
    {
        SysState &q = st[sys];
        q.omega = sm.v[2] / sm.v[3];
    }
};

template <bool S>
struct BiR {  // x += omega shat; r = s - omega t (:109-110); next test; rho_1, breakdown, beta
    double *x, *r;
    const double *s, *shat, *t, *rt;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &a) const
    {
        const double w = m.st[sys].omega;
        double rr = s[i];
        if (w != 0) {
            x[i] = fmac<S>(w, shat[i], x[i]);
            rr = fmac<S>(-w, t[i], rr);
        }
        r[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
        a.v[2] = fmac<S>(rt[i], rr, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &sm)
    {
        SysState &q = m.st[sys];
        q.rho_2 = q.rho_1;
        q.iter++;
        int c = m.check(q, sys, norm_finish(sm.v, m.mon.norm));
        if (c == ST_RUNNING) {
            q.rho_1 = sm.v[2];
            bicg_breakdown(q, c);
            if (c == ST_RUNNING) q.beta = (q.rho_1 / q.rho_2) * (q.alpha / q.omega);
        }
        m.finish(q, c);
    }
};

// =============================================================== GMRES
// S/GMRES.java:127-176, GivensRotation M/GivensRotation.java:42-92.  The
// scalar work (Hessenberg column, rotations, triangular solve) runs on one
// thread with every product and sum rounded separately, as in Java.
struct GmData {
    double *H;   // (restart+1) x restart, column-major, ld = restart+1
    double *s;   // restart+1
    double *gc, *gs;  // rotations
    int restart;
};

__device__ __forceinline__ double jmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double jadd(double a, double b) { return __dadd_rn(a, b); }

__device__ void givens_make(double x, double y, double &c, double &s)
{
    const double roe = fabs(x) > fabs(y) ? x : y;
    const double scale = jadd(fabs(x), fabs(y));
    if (scale != 0) {
        const double xs = x / scale, ys = y / scale;
        double r = jmul(scale, sqrt(jadd(jmul(xs, xs), jmul(ys, ys))));
        if (roe < 0) r = -r;
        c = x / r;
        s = y / r;
    } else {
        c = 1;
        s = 0;
    }
}

__device__ __forceinline__ void givens_apply(double c, double s, double &a1, double &a2)
{
    const double temp = jadd(jmul(c, a1), jmul(s, a2));
    a2 = jadd(jmul(-s, a1), jmul(c, a2));
    a1 = temp;
}

// residual phase: u = b - A x
struct GmU {
    const double *b;
    double *u;
    SysState *st;
    bool always;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return always || st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &) const { u[i] = b[i] - d; }
    __device__ void scalar(int, const Acc &) {}
};

// inner step product u = A v_i (A.mult, :146), while the inner loop runs
struct GmAv {
    double *u;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].gate == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &) const { u[i] = mtj_assign(d); }
    __device__ void scalar(int, const Acc &) {}
};

// norms of r = M u: the monitor's norm and ||r||2; outer test (:133, :137,
// :172); on running, a new cycle: s = [normr, 0...], inner test on |s_0| (:144)
template <bool S>
struct GmNorm {
    const double *r;
    MonPtrs m;
    GmData g;
    bool first;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return first || m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int, Acc &a) const
    {
        const double rr = r[i];
        norm_add<S>(a, rr, m.mon.norm);
        a.v[2] = fmac<S>(rr, rr, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &sm)
    {
        SysState &t = m.st[sys];
        if (first) t.iter = 0;
        else t.iter++;
        t.normr = sqrt(sm.v[2]);
        int c = m.check(t, sys, norm_finish(sm.v, m.mon.norm));
        if (c == ST_RUNNING) {
            for (int k = 0; k <= g.restart; ++k) g.s[k] = 0.0;
            g.s[0] = t.normr;
            t.inner = 0;
            t.inner_done = 0;
            t.scratch[0] = 1 / t.normr;  // v[0].set(1 / normr, r)
            if (g.restart > 0) {
                c = m.check_scalar(t, sys, fabs(g.s[0]));
                if (c == ST_DONE) {
                    t.inner_done = 1;
                    c = ST_RUNNING;
                }
            } else {
                t.inner_done = 1;
            }
        }
        m.finish(t, c);
        if (c == ST_RUNNING && t.inner_done) t.gate = 1;
    }
};

// v_{k} = alpha * w (DenseVector.set(alpha, y): alpha == 0 zeroes, M/DenseVector.java:216-231)
template <bool S>
struct GmScale {
    double *v;
    const double *w;
    SysState *st;
    bool gated;  // use the inner gate (v_{i+1}) or the status (v_0)
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return gated ? st[sys].gate == ST_RUNNING : st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &) const
    {
        const double al = st[sys].scratch[0];
        v[i] = al == 0 ? 0.0 : al * w[i];
    }
    __device__ void scalar(int, const Acc &) {}
};

// Modified Gram-Schmidt pass k of inner step i (:149-153): w -= H[k-1,i] v_{k-1}
// (k > 0), then H[k,i] = w.v_k (k <= i) or H[i+1,i] = ||w||2 (k == i+1);
// the last pass also rotates column i and s and runs the next inner test.
template <bool S>
struct GmMgs {
    double *w;
    const double *vprev, *vk;
    int i, k;
    MonPtrs m;
    GmData g;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return m.st[sys].gate == ST_RUNNING; }
    __device__ void row(int r, int, Acc &a) const
    {
        double wr = w[r];
        if (k > 0) {
            const double h = g.H[(k - 1) + (size_t)i * (g.restart + 1)];
            if (-h != 0) {
                wr = fmac<S>(-h, vprev[r], wr);
                w[r] = wr;
            }
        }
        if (k <= i) a.v[2] = fmac<S>(wr, vk[r], a.v[2]);
        else a.v[2] = fmac<S>(wr, wr, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &sm)
    {
        SysState &t = m.st[sys];
        const int ld = g.restart + 1;
        double *Hc = g.H + (size_t)i * ld;
        if (k <= i) {
            Hc[k] = sm.v[2];
            return;
        }
        Hc[i + 1] = sqrt(sm.v[2]);
        t.scratch[0] = 1. / Hc[i + 1];
        for (int q = 0; q < i; ++q) givens_apply(g.gc[q], g.gs[q], Hc[q], Hc[q + 1]);
        givens_make(Hc[i], Hc[i + 1], g.gc[i], g.gs[i]);
        givens_apply(g.gc[i], g.gs[i], Hc[i], Hc[i + 1]);
        givens_apply(g.gc[i], g.gs[i], g.s[i], g.s[i + 1]);
        t.iter++;
        t.inner = i + 1;
        int c = ST_RUNNING;
        if (i + 1 < g.restart) {
            c = m.check_scalar(t, sys, fabs(g.s[i + 1]));
            if (c == ST_DONE) {
                t.inner_done = 1;
                c = ST_RUNNING;
            }
        } else {
            t.inner_done = 1;
        }
        m.finish(t, c);
        if (c == ST_RUNNING && t.inner_done) t.gate = 1;
    }
};

// new UpperTriangDenseMatrix(H, i, false).solve(s, s) (:166): LAPACK dtrtrs
// semantics -- info = first zero diagonal (MatrixSingularException), else the
// reference dtrsm column sweep k = i-1..0 skipping zero entries of s.
__global__ void k_gmres_trsv(SysState *st, GmData g, int *num_running)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    SysState &t = st[0];
    if (t.status != ST_RUNNING) return;
    const int n = t.inner, ld = g.restart + 1;
    for (int k = 0; k < n; ++k)
        if (g.H[k + (size_t)k * ld] == 0) {
            t.status = MTJG_ERR_SINGULAR;
            t.gate = 1;
            atomicSub(num_running, 1);
            return;
        }
    for (int k = n - 1; k >= 0; --k) {
        if (g.s[k] != 0) {
            g.s[k] = g.s[k] / g.H[k + (size_t)k * ld];
            for (int q = 0; q < k; ++q) g.s[q] = jadd(g.s[q], -jmul(g.s[k], g.H[q + (size_t)k * ld]));
        }
    }
}

// x += s_j v_j for j < i, in order (:167-168)
template <bool S>
struct GmX {
    double *x;
    const double *V;
    size_t ldv;
    GmData g;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int r, int sys, Acc &) const
    {
        const int n = st[sys].inner;
        double xr = x[r];
        for (int j = 0; j < n; ++j) {
            const double sj = g.s[j];
            if (sj != 0) xr = fmac<S>(sj, V[(size_t)j * ldv + r], xr);
        }
        x[r] = xr;
    }
    __device__ void scalar(int, const Acc &) {}
};


}  // namespace mtjg

#include "persist.cuh"

using namespace mtjg;

// ================================================================ handle
struct mtjg_solver {
    mtjg_ctx *ctx = nullptr;
    int kind = MTJG_CG;
    int n = 0;
    int restart = 30;
    mtjg_precond *M = nullptr;
    mtjg_monitor mon{};
    SysState *st = nullptr;     // one per system of the matrix being solved
    int st_alloc = 0;
    double *hist_r = nullptr;   // history_cap entries per system
    int *hist_it = nullptr;
    int64_t hist_alloc = 0;
    int num_sys = 1;            // systems of the last solve
    std::vector<SysState> last_all;
    // mixed precision
    bool mixed = false;
    MixCfg mix{1e-4, 1000, 0, 1e-10, 1e-50};
    std::vector<float *> v32;   // d, rin, z, p, q
    float *invdiag32 = nullptr;
    int64_t inv32_version = -1;
    std::vector<double *> vecs;
    double *V = nullptr;
    GmData gm{};
    // graph of one chunk of the loop body
    cudaGraphExec_t gexec = nullptr;
    const mtjg_csr *g_A = nullptr;
    const mtjg_precond *g_M = nullptr;
    int g_numerics = -1;
    int g_norm = -1;
    int64_t g_version = 0;
    int64_t g_aversion = -1;
    // Chebyshev's eigenvalue bounds (Chebyshev.setEigenvalues)
    double eigmin = 0, eigmax = 0;
    bool eig_set = false;
    int g_kernels = 0;
    int chunk = 16;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    SysState last{};
    int last_valid = 0;
    // persistent batched CG (batch.cu): work order, lanes per row, ticket,
    // and a copy of x kept while the autotuner probes
    int *b_order = nullptr;
    unsigned char *b_vec = nullptr;
    unsigned *b_ticket = nullptr;
    double *b_xsave = nullptr;
    int b_cap = 0;
    int64_t b_xcap = 0;
    int last_sys = 0;          // the system of the last solve that S->last describes
    // mixed GMRES / BiCGstab (mixed_ir.cuh): FP32 vectors, FP64 partials and
    // scalars, pinned copies of the scalars
    float *ir_f = nullptr;
    double *ir_d = nullptr, *ir_h = nullptr;
    int64_t ir_fcap = 0, ir_dcap = 0, ir_hcap = 0;
    bool last_empty = false;   // the last solve had n == 0: its history is empty_it (residuals 0)
    std::vector<int> empty_it;
    // one-launch CG (persist.cuh): MTJG_LAUNCH_*, the product's partials,
    // the barrier's arrival count and abort word
    int launch_mode = MTJG_LAUNCH_AUTO;
    double *pc_part = nullptr;
    int64_t pc_part_cap = 0;
    double *pc_p2 = nullptr;  // the second p buffer
    unsigned long long *pc_bar = nullptr;
    bool last_persistent = false;
    // MatrixIterationMonitor (mtjg_solver_set_matrix_monitor)
    int xmon = 0;
    double normA = 0, normb = 0;
};

namespace {

enum {
    V_B = 0, V_X, V_R, V_Z, V_P, V_Q, V_RT, V_PH, V_S, V_SH, V_T, V_V, V_U, V_W,
    // BiCG, CGS, QMR
    V_ZT, V_PT, V_QT, V_VH, V_UH, V_SUM, V_Y, V_D, V_VT, V_WT, V_YT, V_ZTL, V_PTL,
    V_COUNT
};

// transposed products (A.transMult / transMultAdd) and M.transApply
bool needs_transpose(int kind) { return kind == MTJG_BICG || kind == MTJG_QMR; }

MonCfgDev mon_dev(const mtjg_solver *S)
{
    MonCfgDev c;
    c.max_iter = S->mon.max_iter;
    c.norm = S->mon.norm;
    c.hist_cap = S->mon.history_cap;
    c.xmon = S->xmon;
    c.rtol = S->mon.rtol;
    c.atol = S->mon.atol;
    c.dtol = S->mon.dtol;
    return c;
}

int pc_mode(const mtjg_solver *S)
{
    if (!S->M || S->M->kind == MTJG_PC_IDENTITY) return kPcIdentity;
    if (S->M->kind == MTJG_PC_JACOBI) return kPcJacobi;
    return kPcExternal;
}

template <bool STRICT>
struct Phases {
    mtjg_solver *S;
    mtjg_csr *A;
    MonPtrs mp() const
    {
        return MonPtrs{S->st, mon_dev(S), S->hist_r, S->hist_it, A->num_running};
    }
    CsrArgs csr() const { return CsrArgs{A->rowptr, A->colind, A->val}; }
    RedCtx rc() const { return red_ctx(A, A->tiles); }
    double *v(int k) const { return S->vecs[k]; }
    const double *invdiag() const { return S->M && S->M->kind == MTJG_PC_JACOBI ? S->M->invdiag : nullptr; }
    int norm() const { return S->mon.norm; }

    // apply M (b -> x) with a gate word; identity with x == b does nothing
    int pc(const double *b, double *x, const int *gate)
    {
        if (!S->M || S->M->kind == MTJG_PC_IDENTITY) {
            if (x == b) return MTJG_OK;
            mtjg_precond tmp;
            tmp.ctx = S->ctx;
            tmp.kind = MTJG_PC_IDENTITY;
            tmp.n = S->n;
            return precond_apply_dev(&tmp, b, x, gate);
        }
        return precond_apply_dev(S->M, b, x, gate);
    }

#define PH_CHECK(e)                                                \
    do {                                                           \
        cudaError_t e__ = (e);                                     \
        if (e__ != cudaSuccess) return cuda_fail(e__, "solver phase"); \
    } while (0)

    // ---- CG
    int cg_init()
    {
        const int pcm = pc_mode(S);
        double *z = pcm == kPcIdentity ? v(V_R) : v(V_Z);
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X),
                             CgInit<STRICT>{v(V_B), v(V_R), z, invdiag(), pcm, mp()}, rc(), norm()));
        return MTJG_OK;
    }
    int cg_body()
    {
        const int pcm = pc_mode(S);
        double *z = pcm == kPcIdentity ? v(V_R) : v(V_Z);
        if (pcm == kPcExternal) {
            int st = pc(v(V_R), z, &S->st->status);
            if (st != MTJG_OK) return st;
            PH_CHECK(launch_rows(S->ctx, A->rtiles, CgDot<STRICT>{v(V_R), z, S->st}, rc(), norm()));
        }
        PH_CHECK(launch_rows(S->ctx, A->rtiles, CgP<STRICT>{v(V_P), z, S->st}, rc(), norm()));
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_P), CgQ<STRICT>{v(V_P), v(V_Q), S->st}, rc(), norm()));
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             CgUpd<STRICT>{v(V_X), v(V_R), z, v(V_P), v(V_Q), invdiag(), pcm, mp()}, rc(), norm()));
        return MTJG_OK;
    }

    // ---- BiCGstab
    int bi_init()
    {
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X), BiInit<STRICT>{v(V_B), v(V_R), v(V_RT), mp()}, rc(),
                             norm()));
        return MTJG_OK;
    }
    int bi_body()
    {
        const int pcm = pc_mode(S);
        double *phat = pcm == kPcIdentity ? v(V_P) : v(V_PH);
        double *shat = pcm == kPcIdentity ? v(V_S) : v(V_SH);
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             BiP<STRICT>{v(V_P), phat, v(V_R), v(V_V), invdiag(), pcm, S->st}, rc(), norm()));
        if (pcm == kPcExternal) {
            int st = pc(v(V_P), phat, &S->st->status);
            if (st != MTJG_OK) return st;
        }
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, phat, BiV<STRICT>{v(V_V), v(V_RT), S->st}, rc(), norm()));
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             BiS<STRICT>{v(V_S), v(V_X), shat, v(V_R), v(V_V), phat, invdiag(), pcm, mp()}, rc(),
                             norm()));
        if (pcm == kPcExternal) {
            int st = pc(v(V_S), shat, &S->st->status);
            if (st != MTJG_OK) return st;
        }
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, shat, BiT<STRICT>{v(V_T), v(V_S), S->st}, rc(), norm()));
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             BiR<STRICT>{v(V_X), v(V_R), v(V_S), shat, v(V_T), v(V_RT), mp()}, rc(), norm()));
        return MTJG_OK;
    }

    // M.transApply (b -> x) with a gate word
    int pct(const double *b, double *x, const int *gate)
    {
        if (!S->M || S->M->kind == MTJG_PC_IDENTITY) return pc(b, x, gate);
        return precond_trans_apply_dev(S->M, b, x, gate);
    }
    CsrArgs tcsr() const { return CsrArgs{A->t_rowptr, A->t_colind, A->t_val}; }
    RedCtx trc() const { return RedCtx{A->t_part, A->cnt, A->t_tiles.sys_group, A->num_running}; }
    const int *gate() const { return &S->st->status; }

    // ---- IR (S/IR.java:57-70)
    int ir_init()
    {
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X), IrRes<STRICT>{v(V_B), v(V_R), mp(), true}, rc(),
                             norm()));
        return MTJG_OK;
    }
    int ir_body()
    {
        const int pcm = pc_mode(S);
        if (pcm == kPcExternal) {
            int st = pc(v(V_R), v(V_Z), gate());
            if (st != MTJG_OK) return st;
        }
        PH_CHECK(launch_rows(S->ctx, A->rtiles, IrX<STRICT>{v(V_X), v(V_R), v(V_Z), invdiag(), pcm, S->st}, rc(),
                             norm()));
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X), IrRes<STRICT>{v(V_B), v(V_R), mp(), false}, rc(),
                             norm()));
        return MTJG_OK;
    }

    // ---- Chebyshev (S/Chebyshev.java:90-120)
    ChCfg cheb() const { return ChCfg{(S->eigmax - S->eigmin) / 2.0, (S->eigmax + S->eigmin) / 2.0}; }
    int cheb_init()
    {
        const int pcm = pc_mode(S);
        double *z = pcm == kPcIdentity ? v(V_R) : v(V_Z);
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X),
                             ChInit<STRICT>{v(V_B), v(V_R), z, invdiag(), pcm, mp(), cheb()}, rc(), norm()));
        return MTJG_OK;
    }
    int cheb_body()
    {
        const int pcm = pc_mode(S);
        double *z = pcm == kPcIdentity ? v(V_R) : v(V_Z);
        if (pcm == kPcExternal) {
            int st = pc(v(V_R), z, gate());
            if (st != MTJG_OK) return st;
        }
        PH_CHECK(launch_rows(S->ctx, A->rtiles, CgP<STRICT>{v(V_P), z, S->st}, rc(), norm()));
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_P), ChQ{v(V_Q), S->st}, rc(), norm()));
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             ChUpd<STRICT>{v(V_X), v(V_R), z, v(V_P), v(V_Q), invdiag(), pcm, mp(), cheb()}, rc(),
                             norm()));
        return MTJG_OK;
    }

    // ---- BiCG (S/BiCG.java:63-102)
    int bicg_init()
    {
        const int pcm = pc_mode(S);
        double *z = pcm == kPcIdentity ? v(V_R) : v(V_Z), *zt = pcm == kPcIdentity ? v(V_RT) : v(V_ZT);
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X),
                             BgInit<STRICT>{v(V_B), v(V_R), v(V_RT), z, zt, invdiag(), pcm, mp()}, rc(), norm()));
        return MTJG_OK;
    }
    int bicg_body()
    {
        const int pcm = pc_mode(S);
        double *z = pcm == kPcIdentity ? v(V_R) : v(V_Z), *zt = pcm == kPcIdentity ? v(V_RT) : v(V_ZT);
        if (pcm == kPcExternal) {
            int st = pc(v(V_R), z, gate());
            if (st == MTJG_OK) st = pct(v(V_RT), zt, gate());
            if (st != MTJG_OK) return st;
            PH_CHECK(launch_rows(S->ctx, A->rtiles, BgRho<STRICT>{z, v(V_RT), mp()}, rc(), norm()));
        }
        PH_CHECK(launch_rows(S->ctx, A->rtiles, BgP<STRICT>{v(V_P), v(V_PT), z, zt, S->st}, rc(), norm()));
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_P), ChQ{v(V_Q), S->st}, rc(), norm()));
        PH_CHECK(launch_spmv(S->ctx, tcsr(), A->t_tiles, v(V_PT), BgQt<STRICT>{v(V_QT), v(V_Q), S->st}, trc(),
                             norm()));
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             BgUpd<STRICT>{v(V_X), v(V_R), v(V_RT), z, zt, v(V_P), v(V_Q), v(V_QT), invdiag(), pcm,
                                           mp()},
                             rc(), norm()));
        return MTJG_OK;
    }

    // ---- CGS (S/CGS.java:65-105)
    int cgs_init()
    {
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X), CsInit<STRICT>{v(V_B), v(V_R), v(V_RT), mp()}, rc(),
                             norm()));
        return MTJG_OK;
    }
    int cgs_body()
    {
        const int pcm = pc_mode(S);
        double *phat = pcm == kPcIdentity ? v(V_P) : v(V_PH);
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             CsP<STRICT>{v(V_U), v(V_P), phat, v(V_R), v(V_Q), invdiag(), pcm, S->st}, rc(), norm()));
        if (pcm == kPcExternal) {
            int st = pc(v(V_P), phat, gate());
            if (st != MTJG_OK) return st;
        }
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, phat, CsV<STRICT>{v(V_VH), v(V_RT), S->st}, rc(), norm()));
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             CsQ<STRICT>{v(V_Q), v(V_SUM), v(V_UH), v(V_X), v(V_VH), v(V_U), invdiag(), pcm, S->st},
                             rc(), norm()));
        if (pcm == kPcExternal) {
            int st = pc(v(V_SUM), v(V_UH), gate());
            if (st != MTJG_OK) return st;
            PH_CHECK(launch_rows(S->ctx, A->rtiles, CsX<STRICT>{v(V_X), v(V_UH), S->st}, rc(), norm()));
        }
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_UH), CsQh<STRICT>{v(V_R), v(V_RT), mp()}, rc(), norm()));
        return MTJG_OK;
    }

    // ---- QMR (S/QMR.java:117-213)
    int qmr_init()
    {
        const int pcm = pc_mode(S);
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X),
                             QmInit<STRICT>{v(V_B), v(V_R), v(V_VT), v(V_WT), v(V_Y), v(V_Z), invdiag(), pcm, mp()},
                             rc(), norm()));
        if (pcm == kPcExternal) {
            int st = pc(v(V_VT), v(V_Y), gate());
            if (st == MTJG_OK) st = pct(v(V_WT), v(V_Z), gate());
            if (st != MTJG_OK) return st;
            PH_CHECK(launch_rows(S->ctx, A->rtiles, QmNorms<STRICT>{v(V_Y), v(V_Z), mp()}, rc(), norm()));
        }
        return MTJG_OK;
    }
    int qmr_body()
    {
        const int pcm = pc_mode(S);
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             QmA<STRICT>{v(V_V), v(V_Y), v(V_W), v(V_Z), v(V_YT), v(V_ZTL), v(V_VT), v(V_WT),
                                         invdiag(), pcm, mp()},
                             rc(), norm()));
        if (pcm == kPcExternal) {
            int st = pc(v(V_Y), v(V_YT), gate());
            if (st == MTJG_OK) st = pct(v(V_Z), v(V_ZTL), gate());
            if (st != MTJG_OK) return st;
        }
        PH_CHECK(launch_rows(S->ctx, A->rtiles, QmP<STRICT>{v(V_P), v(V_Q), v(V_YT), v(V_ZTL), S->st}, rc(), norm()));
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_P), QmPt<STRICT>{v(V_PTL), v(V_Q), mp()}, rc(), norm()));
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             QmV<STRICT>{v(V_VT), v(V_Y), v(V_V), v(V_PTL), invdiag(), pcm, S->st}, rc(), norm()));
        if (pcm == kPcExternal) {
            int st = pc(v(V_VT), v(V_Y), gate());
            if (st != MTJG_OK) return st;
            PH_CHECK(launch_rows(S->ctx, A->rtiles, QmRho<STRICT>{v(V_Y), S->st}, rc(), norm()));
        }
        PH_CHECK(launch_spmv(S->ctx, tcsr(), A->t_tiles, v(V_Q),
                             QmW<STRICT>{v(V_WT), v(V_Z), v(V_W), invdiag(), pcm, mp()}, trc(), norm()));
        if (pcm == kPcExternal) {
            int st = pct(v(V_WT), v(V_Z), gate());
            if (st != MTJG_OK) return st;
            PH_CHECK(launch_rows(S->ctx, A->rtiles, QmXi<STRICT>{v(V_Z), mp()}, rc(), norm()));
        }
        PH_CHECK(launch_rows(S->ctx, A->rtiles,
                             QmUpd<STRICT>{v(V_D), v(V_S), v(V_X), v(V_R), v(V_P), v(V_PTL), mp()}, rc(), norm()));
        return MTJG_OK;
    }

    // ---- GMRES
    double *basis(int k) const { return S->V + (size_t)k * (size_t)S->n; }
    int gm_residual(bool first)
    {
        const int pcm = pc_mode(S);
        double *u = v(V_U);
        double *r = pcm == kPcIdentity ? u : v(V_R);
        PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, v(V_X), GmU{v(V_B), u, S->st, first}, rc(), norm()));
        if (pcm != kPcIdentity) {
            int st = pc(u, r, first ? nullptr : &S->st->status);
            if (st != MTJG_OK) return st;
        }
        PH_CHECK(launch_rows(S->ctx, A->rtiles, GmNorm<STRICT>{r, mp(), S->gm, first}, rc(), norm()));
        return MTJG_OK;
    }
    int gm_init() { return gm_residual(true); }
    int gm_body()
    {
        const int pcm = pc_mode(S);
        double *u = v(V_U);
        double *r = pcm == kPcIdentity ? u : v(V_R);
        double *w = pcm == kPcIdentity ? u : v(V_W);
        // v_0 = r / normr
        PH_CHECK(launch_rows(S->ctx, A->rtiles, GmScale<STRICT>{basis(0), r, S->st, false}, rc(), norm()));
        for (int i = 0; i < S->restart; ++i) {
            PH_CHECK(launch_spmv(S->ctx, csr(), A->tiles, basis(i), GmAv{u, S->st}, rc(), norm()));
            if (pcm != kPcIdentity) {
                int st = pc(u, w, &S->st->gate);
                if (st != MTJG_OK) return st;
            }
            for (int k = 0; k <= i + 1; ++k) {
                const double *vprev = k > 0 ? basis(k - 1) : nullptr;
                const double *vk = k <= i ? basis(k) : nullptr;
                PH_CHECK(launch_rows(S->ctx, A->rtiles, GmMgs<STRICT>{w, vprev, vk, i, k, mp(), S->gm}, rc(),
                                     norm()));
            }
            PH_CHECK(launch_rows(S->ctx, A->rtiles, GmScale<STRICT>{basis(i + 1), w, S->st, true}, rc(), norm()));
        }
        k_gmres_trsv<<<1, 32, 0, S->ctx->stream>>>(S->st, S->gm, A->num_running);
        S->ctx->launches++;
        PH_CHECK(cudaGetLastError());
        PH_CHECK(launch_rows(S->ctx, A->rtiles, GmX<STRICT>{v(V_X), S->V, (size_t)S->n, S->gm, S->st}, rc(), norm()));
        return gm_residual(false);
    }
};

}  // namespace

// ======================================================== orchestration
namespace {

void drop_graph(mtjg_solver *S)
{
    if (S->gexec) cudaGraphExecDestroy(S->gexec);
    S->gexec = nullptr;
    S->g_A = nullptr;
    S->g_M = nullptr;
}

// Mixed precision: the body is one outer step then kInnerPerBody inner
// iterations; systems whose inner solve ends early idle until the next body.

int mixed_body(mtjg_solver *S, mtjg_csr *A)
{
    mtjg_ctx *ctx = S->ctx;
    const int pcm = pc_mode(S);
    float *d = S->v32[0], *rin = S->v32[1], *z = pcm == kPcIdentity ? S->v32[1] : S->v32[2];
    float *p = S->v32[3], *q = S->v32[4];
    const RedCtx rc = red_ctx(A, A->tiles);
    const MonPtrs mp{S->st, mon_dev(S), S->hist_r, S->hist_it, A->num_running};
    const int norm = S->mon.norm;
    MixCfg mix = S->mix;
    mix.rtol = S->mon.rtol;
    mix.atol = S->mon.atol;
    cudaError_t e = launch_rows(ctx, A->rtiles, MxX{S->vecs[V_X], d, S->st}, rc, norm);
    if (e == cudaSuccess)
        e = launch_spmv(ctx, CsrArgs{A->rowptr, A->colind, A->val}, A->tiles, (const double *)S->vecs[V_X],
                        MxOuter{S->vecs[V_B], rin, z, d, S->invdiag32, pcm, mp}, rc, norm);
    for (int k = 0; k < kInnerPerBody && e == cudaSuccess; ++k) {
        e = launch_rows(ctx, A->rtiles, MxP{p, z, S->st}, rc, norm);
        if (e == cudaSuccess)
            e = launch_spmv(ctx, CsrArgsT<float>{A->rowptr, A->colind, A->val32}, A->tiles, (const float *)p,
                            MxQ{q, S->st}, rc, norm);
        if (e == cudaSuccess)
            e = launch_rows(ctx, A->rtiles, MxUpd{d, rin, z, p, q, S->invdiag32, pcm, S->st, mix}, rc, norm);
    }
    if (e != cudaSuccess) return cuda_fail(e, "mixed-precision phase");
    return MTJG_OK;
}

// FP32 copies the mixed solver reads: the matrix values and the inverse diagonal
int mixed_prepare(mtjg_solver *S, mtjg_csr *A)
{
    mtjg_ctx *ctx = S->ctx;
    const int grid = ctx->num_sms * 8;
    if (!A->val32) {
        MTJG_CUDA(cudaMalloc(&A->val32, sizeof(float) * (size_t)(A->nnz + 4)));
        MTJG_CUDA(cudaMemsetAsync(A->val32, 0, sizeof(float) * (size_t)(A->nnz + 4), ctx->stream));
        if (A->nnz) k_to_f32<<<grid, kBlock, 0, ctx->stream>>>(A->nnz, A->val, A->val32);
        ctx->launches++;
        drop_graph(S);
    }
    if (S->M && S->M->kind == MTJG_PC_JACOBI && S->inv32_version != S->M->version) {
        if (!S->invdiag32) MTJG_CUDA(cudaMalloc(&S->invdiag32, sizeof(float) * (size_t)std::max(1, S->n)));
        if (S->n) k_to_f32<<<grid, kBlock, 0, ctx->stream>>>(S->n, S->M->invdiag, S->invdiag32);
        ctx->launches++;
        S->inv32_version = S->M->version;
    }
    MTJG_CUDA(cudaGetLastError());
    return MTJG_OK;
}

template <bool STRICT>
int run_phase(mtjg_solver *S, mtjg_csr *A, bool init)
{
    if (S->mixed) return init ? MTJG_OK : mixed_body(S, A);
    Phases<STRICT> ph{S, A};
    switch (S->kind) {
    case MTJG_CG: return init ? ph.cg_init() : ph.cg_body();
    case MTJG_BICGSTAB: return init ? ph.bi_init() : ph.bi_body();
    case MTJG_BICG: return init ? ph.bicg_init() : ph.bicg_body();
    case MTJG_CGS: return init ? ph.cgs_init() : ph.cgs_body();
    case MTJG_QMR: return init ? ph.qmr_init() : ph.qmr_body();
    case MTJG_CHEBYSHEV: return init ? ph.cheb_init() : ph.cheb_body();
    case MTJG_IR: return init ? ph.ir_init() : ph.ir_body();
    default: return init ? ph.gm_init() : ph.gm_body();
    }
}

int phase(mtjg_solver *S, mtjg_csr *A, bool init)
{
    return S->ctx->numerics == MTJG_NUMERICS_STRICT ? run_phase<true>(S, A, init) : run_phase<false>(S, A, init);
}

int capture(mtjg_solver *S, mtjg_csr *A)
{
    mtjg_ctx *ctx = S->ctx;
    drop_graph(S);
    const int64_t before = ctx->launches;
    cudaGraph_t g = nullptr;
    MTJG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int st = MTJG_OK;
    const int reps = S->kind == MTJG_GMRES ? 1 : S->mixed ? 2 : S->chunk;
    for (int c = 0; c < reps && st == MTJG_OK; ++c) st = phase(S, A, false);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (st != MTJG_OK) {
        if (g) cudaGraphDestroy(g);
        ctx->launches = before;
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&S->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    S->g_kernels = (int)(ctx->launches - before);
    ctx->launches = before;
    S->g_A = A;
    S->g_M = S->M;
    S->g_numerics = ctx->numerics;
    S->g_norm = S->mon.norm;
    S->g_version = S->M ? S->M->version : 0;
    S->g_aversion = A->version;
    return MTJG_OK;
}

int map_status(int st) { return st == ST_DONE ? MTJG_OK : st; }

// Copies the first m entries of the residual history of system `sys` of the
// last solve.
int copy_history(mtjg_solver *S, int sys, double *resid, int *iters, int m)
{
    if (m <= 0) return MTJG_OK;
    if (S->last_empty) {
        for (int k = 0; k < m; ++k) {
            if (resid) resid[k] = 0.0;
            if (iters) iters[k] = S->empty_it[(size_t)k];
        }
        return MTJG_OK;
    }
    const size_t off = (size_t)sys * (size_t)S->mon.history_cap;
    MTJG_CUDA(cudaSetDevice(S->ctx->device));
    if (resid) MTJG_CUDA(cudaMemcpy(resid, S->hist_r + off, sizeof(double) * (size_t)m, cudaMemcpyDeviceToHost));
    if (iters) MTJG_CUDA(cudaMemcpy(iters, S->hist_it + off, sizeof(int) * (size_t)m, cudaMemcpyDeviceToHost));
    return MTJG_OK;
}

// The caller's view of S->last: its result and, for a solve that did not
// converge, the message of the exception MTJ would throw.
int report(mtjg_solver *S, mtjg_result *res)
{
    const int code = map_status(S->last.status);
    if (res) {
        res->status = code;
        res->iterations = S->last.iter;
        res->residual = S->last.residual;
        res->detail = S->last.detail;
        res->history_len = S->last.hist_len;
        res->inner_iterations = S->last.in_total;
    }
    if (code == MTJG_NOT_CONVERGED_BREAKDOWN) {
        static const char *what[] = {"", "rho", "omega", "xi", "delta", "ep", "beta", "gamma"};
        const int d = S->last.detail;
        set_error(std::string("Breakdown: ") + (d >= 1 && d <= 7 ? what[d] : "?"));
    }
    else if (code == MTJG_NOT_CONVERGED_ITERATIONS)
        set_error("Iterations");
    else if (code == MTJG_NOT_CONVERGED_DIVERGENCE)
        set_error("Divergence");
    else if (code == MTJG_ERR_UNSUPPORTED)
        set_error("MatrixIterationMonitor.convergedI(double) is not supported (GMRES's inner test)");
    else if (code == MTJG_ERR_SINGULAR)
        set_error("MatrixSingularException in the GMRES triangular solve");
    return code;
}

// Device state for `ns` systems: scalars and monitor histories.
int ensure_state(mtjg_solver *S, int ns)
{
    if (ns > S->st_alloc) {
        cudaFree(S->st);
        S->st = nullptr;
        S->st_alloc = 0;
        MTJG_CUDA(cudaMalloc(&S->st, sizeof(SysState) * (size_t)ns));
        S->st_alloc = ns;
        drop_graph(S);
    }
    const int64_t need = (int64_t)ns * S->mon.history_cap;
    if (need > S->hist_alloc) {
        cudaFree(S->hist_r);
        cudaFree(S->hist_it);
        S->hist_r = nullptr;
        S->hist_it = nullptr;
        S->hist_alloc = 0;
        MTJG_CUDA(cudaMalloc(&S->hist_r, sizeof(double) * (size_t)need));
        MTJG_CUDA(cudaMalloc(&S->hist_it, sizeof(int) * (size_t)need));
        S->hist_alloc = need;
        drop_graph(S);
    }
    return MTJG_OK;
}

// CG with the identity or Jacobi preconditioner on one system of at most
// kPersistMaxTiles product tiles (no row longer than a tile) runs its loop in
// one cooperative launch (persist.cuh) unless the graph path was asked for.
bool persistent_cg(const mtjg_solver *S, const mtjg_csr *A)
{
    return S->launch_mode == MTJG_LAUNCH_AUTO && S->kind == MTJG_CG && !S->mixed && !S->xmon &&
           pc_mode(S) != kPcExternal &&
           A->sys_rows.empty() && A->tiles.num_sys == 1 && A->rtiles.num_sys == 1 && A->tiles.num_long == 0 &&
           A->tiles.num_tiles > 0 && A->tiles.num_tiles <= kPersistMaxTiles &&
           A->tiles.num_groups == A->tiles.num_tiles && A->rtiles.num_groups == A->rtiles.num_tiles;
}

struct PersistPlan {
    int grid = 0;
    int slots = 0;  // cached product tiles per CTA
    size_t smem = 0;
};

// The grid of the one-launch CG: as many co-resident CTAs as there are
// tiles, up to 4 per SM, each caching ceil(tiles / grid) product tiles in
// shared memory; fewer CTAs per SM (more slots each) when that does not fit.
// False when no grid fits: the solve takes the graph path.
template <bool STRICT>
bool persist_plan(mtjg_ctx *ctx, const mtjg_csr *A, PersistPlan &pl)
{
    auto k = k_cg_persist<STRICT>;
    int optin = 0;
    cudaFuncAttributes fa{};
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, k) != cudaSuccess)
        return false;
    const int maxdyn = optin - (int)fa.sharedSizeBytes;
    if (maxdyn < kSlotBytes || cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, maxdyn) != cudaSuccess)
        return false;
    const int NT = A->tiles.num_tiles, NR = A->rtiles.num_tiles;
    for (int per_sm = 4; per_sm >= 1; --per_sm) {
        const int G = std::min(std::max(NT, NR), per_sm * ctx->num_sms);
        const int slots = (NT + G - 1) / G;
        const size_t smem = (size_t)slots * kSlotBytes;
        if (smem > (size_t)maxdyn) continue;
        int blocks = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k, kBlock, smem) != cudaSuccess) return false;
        if ((int64_t)blocks * ctx->num_sms >= G) {
            pl.grid = G;
            pl.slots = slots;
            pl.smem = smem;
            return true;
        }
    }
    return false;
}

// The loop body of CG after cg_init, in one launch; the state and the
// running count end as the graph path leaves them.  Returns kCoopRefused,
// with nothing launched, when the device refuses the cooperative launch
// (fewer co-resident CTAs than planned, e.g. under a partitioned device):
// the solve then continues on the graph path.
constexpr int kCoopRefused = -1;

template <bool STRICT>
int run_persistent_cg(mtjg_solver *S, mtjg_csr *A, const PersistPlan &pl)
{
    mtjg_ctx *ctx = S->ctx;
    const int64_t need = (int64_t)(A->tiles.num_groups + 1) * kParts;
    if (need > S->pc_part_cap) {
        cudaFree(S->pc_part);
        S->pc_part = nullptr;
        S->pc_part_cap = 0;
        MTJG_CUDA(cudaMalloc(&S->pc_part, sizeof(double) * (size_t)need));
        S->pc_part_cap = need;
    }
    if (!S->pc_p2) MTJG_CUDA(cudaMalloc(&S->pc_p2, sizeof(double) * (size_t)std::max(1, S->n)));
    if (!S->pc_bar) MTJG_CUDA(cudaMalloc(&S->pc_bar, 2 * sizeof(unsigned long long)));
    MTJG_CUDA(cudaMemsetAsync(S->pc_bar, 0, 2 * sizeof(unsigned long long), ctx->stream));
    const int pcm = pc_mode(S);
    PersistCg c;
    c.A = CsrArgs{A->rowptr, A->colind, A->val};
    c.pt = tile_args(A->tiles);
    c.rt = tile_args(A->rtiles);
    c.invdiag = S->M && S->M->kind == MTJG_PC_JACOBI ? S->M->invdiag : nullptr;
    c.x = S->vecs[V_X];
    c.r = S->vecs[V_R];
    c.z = pcm == kPcIdentity ? S->vecs[V_R] : S->vecs[V_Z];
    c.q = S->vecs[V_Q];
    c.p[0] = S->vecs[V_P];
    c.p[1] = S->pc_p2;
    c.pc = pcm;
    c.slots = pl.slots;
    c.rcq = RedCtx{S->pc_part, A->cnt, A->tiles.sys_group, A->num_running};
    c.rcu = red_ctx(A, A->rtiles);
    c.m = MonPtrs{S->st, mon_dev(S), S->hist_r, S->hist_it, A->num_running};
    c.gb = GridBar{S->pc_bar, reinterpret_cast<int *>(S->pc_bar + 1)};
    c.err = ctx->d_flag;
    int normtype = S->mon.norm;
    void *args[] = {&c, &normtype};
    const cudaError_t e = cudaLaunchCooperativeKernel(reinterpret_cast<void *>(k_cg_persist<STRICT>), dim3(pl.grid),
                                                      dim3(kBlock), args, pl.smem, ctx->stream);
    if (e == cudaErrorCooperativeLaunchTooLarge || e == cudaErrorNotSupported) {
        (void)cudaGetLastError();  // a launch-configuration error: nothing ran, nothing is sticky
        return kCoopRefused;
    }
    MTJG_CUDA(e);
    ctx->launches++;
    return MTJG_OK;
}

int finish_run(mtjg_solver *S, mtjg_result *res);

// vectors b and x are in the solver's buffers
int run(mtjg_solver *S, mtjg_csr *A, mtjg_result *res)
{
    mtjg_ctx *ctx = S->ctx;
    const int ns = A->tiles.num_sys;
    int st = ensure_state(S, ns);
    if (st != MTJG_OK) return st;
    S->num_sys = ns;
    SysState init;
    std::memset(&init, 0, sizeof(init));
    init.status = ST_RUNNING;
    init.gate = ST_RUNNING;
    init.rho_1 = init.rho_2 = init.alpha = init.beta = init.omega = 1.0;
    if (S->xmon) {  // MatrixIterationMonitor (one system): its norms and the iterate
        init.xm_x = S->vecs[V_X];
        init.xm_n = S->n;
        init.xm_strict = ctx->numerics == MTJG_NUMERICS_STRICT ? 1 : 0;
        init.xm_normA = S->normA;
        init.xm_normb = S->normb;
    }
    S->last_all.assign(ns, init);
    if (S->mixed) {
        st = mixed_prepare(S, A);
        if (st != MTJG_OK) return st;
    }
    MTJG_CUDA(cudaMemcpyAsync(S->st, S->last_all.data(), sizeof(SysState) * (size_t)ns, cudaMemcpyHostToDevice,
                              ctx->stream));
    MTJG_CUDA(cudaMemcpyAsync(A->num_running, &S->num_sys, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(A->cnt, 0, sizeof(unsigned) * (size_t)ns, ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    // what the loop body needs that allocates: before any capture
    if (needs_transpose(S->kind)) {
        st = csr_ensure_transpose(A);
        if (st == MTJG_OK && S->M) st = precond_prepare_trans(S->M);
        if (st != MTJG_OK) return st;
    }
    st = phase(S, A, true);
    if (st != MTJG_OK) return st;
    PersistPlan pl;
    const bool strict = ctx->numerics == MTJG_NUMERICS_STRICT;
    S->last_persistent =
        persistent_cg(S, A) && (strict ? persist_plan<true>(ctx, A, pl) : persist_plan<false>(ctx, A, pl));
    if (S->last_persistent) {
        // one launch runs the loop to the monitor's verdict (a solve that
        // cg_init finished already leaves it nothing to do)
        st = strict ? run_persistent_cg<true>(S, A, pl) : run_persistent_cg<false>(S, A, pl);
        if (st == kCoopRefused) {
            S->last_persistent = false;  // the graph path below runs the loop instead
        } else {
            if (st != MTJG_OK) return st;
            return finish_run(S, res);
        }
    }
    const bool stale = !S->gexec || S->g_A != A || S->g_M != S->M || S->g_numerics != ctx->numerics ||
                       S->g_norm != S->mon.norm || S->g_version != (S->M ? S->M->version : 0) ||
                       S->g_aversion != A->version;
    if (stale) {
        st = capture(S, A);
        if (st != MTJG_OK) return st;
    }
    int *pin = ctx->h_pinned;
    MTJG_CUDA(cudaMemcpyAsync(pin, A->num_running, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (pin[0] != 0) {
        // two chunks in flight: launch k+1, then wait for the status copied after k
        int k = 0;
        MTJG_CUDA(cudaGraphLaunch(S->gexec, ctx->stream));
        ctx->launches += S->g_kernels;
        MTJG_CUDA(cudaMemcpyAsync(pin + 0, A->num_running, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        MTJG_CUDA(cudaMemcpyAsync(pin + 2, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        MTJG_CUDA(cudaEventRecord(S->ev[0], ctx->stream));
        for (;;) {
            const int nx = (k + 1) & 1;
            MTJG_CUDA(cudaGraphLaunch(S->gexec, ctx->stream));
            ctx->launches += S->g_kernels;
            MTJG_CUDA(cudaMemcpyAsync(pin + nx, A->num_running, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            MTJG_CUDA(cudaMemcpyAsync(pin + 2 + nx, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            MTJG_CUDA(cudaEventRecord(S->ev[nx], ctx->stream));
            MTJG_CUDA(cudaEventSynchronize(S->ev[k & 1]));
            if (pin[k & 1] == 0 || pin[2 + (k & 1)] != 0) break;
            // every chunk advances the iteration count by at least one, so a
            // solve that is still running after maxIter + 16 chunks is stuck
            if (++k > (int64_t)std::max(0, S->mon.max_iter) + 16) {
                MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
                return fail(MTJG_ERR_DEVICE_TIMEOUT, "solve did not finish within maxIter iterations");
            }
        }
    }
    return finish_run(S, res);
}

// After the loop: the systems' states and the error flag back to the host,
// and the caller's view of them.
int finish_run(mtjg_solver *S, mtjg_result *res)
{
    mtjg_ctx *ctx = S->ctx;
    const int ns = S->num_sys;
    MTJG_CUDA(cudaMemcpyAsync(S->last_all.data(), S->st, sizeof(SysState) * (size_t)ns, cudaMemcpyDeviceToHost,
                              ctx->stream));
    int flag = 0;
    MTJG_CUDA(cudaMemcpyAsync(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    S->last = S->last_all[0];
    S->last_valid = 1;
    S->last_empty = false;
    if (flag) {
        cudaMemset(ctx->d_flag, 0, sizeof(int));
        return fail(MTJG_ERR_DEVICE_TIMEOUT, "a bounded wait in a device kernel gave up during the solve");
    }
    // a batch reports its first system that did not converge (else system 0)
    S->last_sys = 0;
    for (size_t i = 0; i < S->last_all.size(); ++i)
        if (S->last_all[i].status != ST_DONE) {
            S->last = S->last_all[i];
            S->last_sys = (int)i;
            break;
        }
    return report(S, res);
}

#include "mixed_ir.cuh"

// A batch from mtjg_batch_upload solved by CG with the identity or Jacobi
// preconditioner runs as one persistent launch (batch.cu); other batches
// run the tiled phases.
bool batch_persistent(const mtjg_solver *S, const mtjg_csr *A)
{
    return !A->sys_rows.empty() && S->kind == MTJG_CG &&
           (!S->M || S->M->kind == MTJG_PC_IDENTITY || S->M->kind == MTJG_PC_JACOBI);
}

int run_batch(mtjg_solver *S, mtjg_csr *A, mtjg_result *res)
{
    mtjg_ctx *ctx = S->ctx;
    const int ns = (int)A->sys_rows.size() - 1;
    int st = ensure_state(S, ns);
    if (st != MTJG_OK) return st;
    S->num_sys = ns;
    SysState init;
    std::memset(&init, 0, sizeof(init));
    init.status = ST_RUNNING;
    init.gate = ST_RUNNING;
    init.rho_1 = init.rho_2 = init.alpha = init.beta = init.omega = 1.0;
    S->last_all.assign(ns, init);
    if (S->mixed) {
        st = mixed_prepare(S, A);
        if (st != MTJG_OK) return st;
    }
    if (ns > S->b_cap) {
        cudaFree(S->b_order);
        cudaFree(S->b_vec);
        S->b_order = nullptr;
        S->b_vec = nullptr;
        S->b_cap = 0;
        MTJG_CUDA(cudaMalloc(&S->b_order, sizeof(int) * (size_t)ns));
        MTJG_CUDA(cudaMalloc(&S->b_vec, (size_t)ns));
        S->b_cap = ns;
    }
    if (!S->b_ticket) MTJG_CUDA(cudaMalloc(&S->b_ticket, sizeof(unsigned)));
    const int *srow = A->sys_rows.data();
    const int *hrp = A->h_rowptr.data();
    // the systems' row offsets on the device, uploaded once per matrix
    if (!A->d_sys_rows) {
        MTJG_CUDA(cudaMalloc(&A->d_sys_rows, sizeof(int) * (size_t)(ns + 1)));
        MTJG_CUDA(cudaMemcpy(A->d_sys_rows, srow, sizeof(int) * (size_t)(ns + 1), cudaMemcpyHostToDevice));
    }
    BatchCg a{};
    a.rowptr = A->rowptr;
    a.colind = A->colind;
    a.val = A->val;
    a.val32 = A->val32;
    a.sys_rows = A->d_sys_rows;
    a.order = S->b_order;
    a.vec = S->b_vec;
    a.ticket = S->b_ticket;
    a.pc = pc_mode(S);
    a.invdiag = S->M && S->M->kind == MTJG_PC_JACOBI ? S->M->invdiag : nullptr;
    a.invdiag32 = S->invdiag32;
    a.b = S->vecs[V_B];
    a.x = S->vecs[V_X];
    a.r = S->vecs[V_R];
    a.z = S->vecs[V_Z];
    a.p = S->vecs[V_P];
    a.q = S->vecs[V_Q];
    if (S->mixed) {
        a.d32 = S->v32[0];
        a.r32 = S->v32[1];
        a.z32 = S->v32[2];
        a.p32 = S->v32[3];
        a.q32 = S->v32[4];
    }
    a.st = S->st;
    a.mon = mon_dev(S);
    a.hist_r = S->hist_r;
    a.hist_it = S->hist_it;
    a.mix = S->mix;
    a.mix.rtol = S->mon.rtol;
    a.mix.atol = S->mon.atol;
    auto upload_states = [&]() {
        return cudaMemcpyAsync(S->st, S->last_all.data(), sizeof(SysState) * (size_t)ns, cudaMemcpyHostToDevice,
                               ctx->stream);
    };
    auto go = [&](const BatchCg &args, const std::vector<int> &order) -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(S->b_order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice,
                                        ctx->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(S->b_ticket, 0, sizeof(unsigned), ctx->stream);
        if (e == cudaSuccess) e = batch_launch(ctx, args, S->mixed);
        return e;
    };
    // lanes per row: STRICT sums every row in entry order (one lane)
    std::vector<unsigned char> vec;
    if (ctx->numerics == MTJG_NUMERICS_STRICT) {
        vec.assign((size_t)ns, 1);
    } else {
        const int64_t n = A->n;
        bool saved = false;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        auto probe = [&](const std::vector<int> &pick, int lanes, int iters) -> double {
            if (!saved) {
                if (n > S->b_xcap) {
                    cudaFree(S->b_xsave);
                    S->b_xsave = nullptr;
                    S->b_xcap = 0;
                    if (cudaMalloc(&S->b_xsave, sizeof(double) * (size_t)std::max<int64_t>(1, n)) != cudaSuccess)
                        return -1;
                    S->b_xcap = n;
                }
                if (cudaMemcpyAsync(S->b_xsave, S->vecs[V_X], sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice,
                                    ctx->stream) != cudaSuccess ||
                    cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
                    return -1;
                saved = true;
            }
            std::vector<unsigned char> all((size_t)ns, (unsigned char)lanes);
            BatchCg pa = a;
            pa.count = (int)pick.size();
            pa.mon.hist_cap = 0;
            if (S->mixed) {
                pa.mon.max_iter = 1;
                pa.mix.in_max = iters;
            } else {
                pa.mon.max_iter = iters;
            }
            if (upload_states() != cudaSuccess ||
                cudaMemcpyAsync(S->b_vec, all.data(), all.size(), cudaMemcpyHostToDevice, ctx->stream) !=
                    cudaSuccess ||
                cudaEventRecord(e0, ctx->stream) != cudaSuccess || go(pa, pick) != cudaSuccess ||
                cudaEventRecord(e1, ctx->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
                return -1;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            return ms;
        };
        st = batch_vec(ns, srow, hrp, vec, probe);
        if (saved) {
            cudaMemcpyAsync(S->vecs[V_X], S->b_xsave, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice,
                            ctx->stream);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        }
        if (st != MTJG_OK) return fail(st, "batch autotuner probe failed");
    }
    // work order: largest systems first (longest-processing-time first)
    std::vector<int> order((size_t)ns);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return (int64_t)hrp[srow[x + 1]] - hrp[srow[x]] > (int64_t)hrp[srow[y + 1]] - hrp[srow[y]];
    });
    a.count = ns;
    MTJG_CUDA(cudaMemcpyAsync(S->b_vec, vec.data(), vec.size(), cudaMemcpyHostToDevice, ctx->stream));
    MTJG_CUDA(upload_states());
    MTJG_CUDA(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    MTJG_CUDA(go(a, order));
    MTJG_CUDA(cudaMemcpyAsync(S->last_all.data(), S->st, sizeof(SysState) * (size_t)ns, cudaMemcpyDeviceToHost,
                              ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    S->last = S->last_all[0];
    S->last_valid = 1;
    S->last_empty = false;
    S->last_sys = 0;
    for (size_t i = 0; i < S->last_all.size(); ++i)
        if (S->last_all[i].status != ST_DONE) {
            S->last = S->last_all[i];
            S->last_sys = (int)i;
            break;
        }
    return report(S, res);
}

// n == 0: every vector is empty and every norm 0, so the monitor sees r = 0
// at every test (DefaultIterationMonitor.convergedI,
// S/DefaultIterationMonitor.java:133-155): it converges at the first test iff
// 0 < max(rtol * 0, atol), i.e. atol > 0, and otherwise stops at maxIter.
// Short of that the solvers run on zero vectors as MTJ's do: CG tests every
// iteration up to maxIter (S/CG.java:66-86); BiCGstab breaks down on rho = 0
// at once (S/BiCGstab.java:75-79); GMRES tests the cycle's first residual
// once more inside the cycle, then every step, and a full cycle ends in a
// singular (all-zero) Hessenberg matrix (S/GMRES.java:137-166).  The
// history (all residuals 0) stays on the host.
int run_empty(mtjg_solver *S, mtjg_result *res)
{
    std::memset(&S->last, 0, sizeof(S->last));
    std::vector<int> &it = S->empty_it;
    it.assign(1, 0);
    const int mi = std::max(0, S->mon.max_iter);
    // MatrixIterationMonitor: rtol (normA |x| + normb) with |x| = 0
    const double base = S->xmon ? S->normA * 0.0 + S->normb : 0.0;
    const bool conv = 0.0 < std::max(S->mon.rtol * base, S->mon.atol);
    if (conv) {
        S->last.status = ST_DONE;
    } else if (mi == 0) {
        S->last.status = MTJG_NOT_CONVERGED_ITERATIONS;
    } else if (S->kind == MTJG_BICGSTAB || S->kind == MTJG_BICG || S->kind == MTJG_CGS || S->kind == MTJG_QMR) {
        // rho = 0: BiCGstab, BiCG and CGS form it as a dot product of zero
        // vectors, QMR as a norm (S/BiCG.java:75-79, S/CGS.java:75-79, S/QMR.java:134-137)
        S->last.status = MTJG_NOT_CONVERGED_BREAKDOWN;
        S->last.detail = 1;  // rho
    } else if (S->kind == MTJG_CG || S->kind == MTJG_CHEBYSHEV || S->kind == MTJG_IR) {
        S->last.status = MTJG_NOT_CONVERGED_ITERATIONS;
        S->last.iter = mi;
        for (int k = 1; k <= mi; ++k) it.push_back(k);
    } else if (S->xmon) {
        // GMRES: the cycle's first inner test is converged(double)
        S->last.status = MTJG_ERR_UNSUPPORTED;
        it.push_back(0);
    } else if (mi < S->restart) {
        S->last.status = MTJG_NOT_CONVERGED_ITERATIONS;
        S->last.iter = mi;
        for (int k = 0; k <= mi; ++k) it.push_back(k);
    } else {
        S->last.status = MTJG_ERR_SINGULAR;
        S->last.iter = S->restart;
        for (int k = 0; k < S->restart; ++k) it.push_back(k);
    }
    S->last.hist_len = (int)it.size();
    S->last_all.assign(1, S->last);
    S->last_sys = 0;
    S->last_valid = 1;
    S->last_empty = true;
    return report(S, res);
}

int check_sizes(mtjg_solver *S, mtjg_csr *A)
{
    // AbstractIterativeSolver.checkSizes, S/AbstractIterativeSolver.java:70-77
    if (!A) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL matrix");
    if (A->ctx != S->ctx) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "matrix and solver use different contexts");
    if (A->n != A->m) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "!A.isSquare()");
    if (S->n != A->n) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "b.size() != A.numRows()");
    if (S->M && S->M->n != A->n) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "preconditioner size differs from A");
    if (S->M && !S->M->ready) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "preconditioner setMatrix has not been called");
    if (S->kind == MTJG_CHEBYSHEV && !S->eig_set)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "Chebyshev needs its eigenvalue bounds (mtjg_solver_set_eigenvalues)");
    if (S->mixed && S->kind == MTJG_CG && S->M && S->M->kind != MTJG_PC_IDENTITY && S->M->kind != MTJG_PC_JACOBI)
        return fail(MTJG_ERR_UNSUPPORTED, "mixed-precision CG supports the identity or Jacobi preconditioner");
    if (S->mixed && S->kind != MTJG_CG) {
        if (S->M && S->M->kind != MTJG_PC_IDENTITY && S->M->kind != MTJG_PC_JACOBI && S->M->kind != MTJG_PC_ILU &&
            S->M->kind != MTJG_PC_ILUT)
            return fail(MTJG_ERR_UNSUPPORTED,
                        "mixed-precision GMRES and BiCGstab support the identity, Jacobi, ILU and ILUT preconditioners");
        if (A->tiles.num_sys > 1)
            return fail(MTJG_ERR_UNSUPPORTED, "mixed-precision GMRES and BiCGstab solve one system at a time");
        if (S->kind == MTJG_GMRES && S->restart > 63)
            return fail(MTJG_ERR_UNSUPPORTED, "mixed-precision GMRES supports restart <= 63");
    }
    if (S->xmon && (S->mixed || A->tiles.num_sys > 1 || !A->sys_rows.empty()))
        return fail(MTJG_ERR_UNSUPPORTED, "MatrixIterationMonitor runs with single-system FP64 solves");
    if (A->tiles.num_sys > 1) {
        if (S->kind == MTJG_GMRES)
            return fail(MTJG_ERR_UNSUPPORTED, "batched solves support CG and BiCGstab");
        if (S->M && S->M->kind != MTJG_PC_IDENTITY && S->M->kind != MTJG_PC_JACOBI)
            return fail(MTJG_ERR_UNSUPPORTED, "batched solves support the identity and Jacobi preconditioners");
    }
    return MTJG_OK;
}

}  // namespace

extern "C" int mtjg_solver_create(mtjg_ctx *ctx, int kind, int n, int restart, mtjg_solver **out)
{
    if (!ctx || !out) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (kind < MTJG_CG || kind > MTJG_IR) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "unknown solver kind");
    if (n < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "negative size");
    if (kind == MTJG_GMRES && restart <= 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "restart must be a positive integer");
    MTJG_CUDA(cudaSetDevice(ctx->device));
    mtjg_solver *S = new mtjg_solver();
    S->ctx = ctx;
    ctx_retain(ctx);
    S->kind = kind;
    S->n = n;
    S->restart = kind == MTJG_GMRES ? restart : 0;
    mtjg_monitor_defaults(&S->mon);
    S->vecs.assign(V_COUNT, nullptr);
    std::vector<int> need;
    if (kind == MTJG_CG || kind == MTJG_CHEBYSHEV) need = {V_B, V_X, V_R, V_Z, V_P, V_Q};
    else if (kind == MTJG_BICGSTAB) need = {V_B, V_X, V_R, V_RT, V_P, V_PH, V_S, V_SH, V_T, V_V};
    else if (kind == MTJG_BICG) need = {V_B, V_X, V_R, V_Z, V_P, V_Q, V_RT, V_ZT, V_PT, V_QT};
    else if (kind == MTJG_CGS) need = {V_B, V_X, V_R, V_RT, V_P, V_Q, V_U, V_PH, V_VH, V_UH, V_SUM};
    else if (kind == MTJG_QMR)
        need = {V_B, V_X, V_R, V_Y, V_Z, V_V, V_W, V_P, V_Q, V_D, V_S, V_VT, V_WT, V_YT, V_ZTL, V_PTL};
    else if (kind == MTJG_IR) need = {V_B, V_X, V_R, V_Z};
    else need = {V_B, V_X, V_R, V_U, V_W};
    const size_t nb = sizeof(double) * (size_t)std::max(1, n);
    bool ok = ensure_state(S, 1) == MTJG_OK;
    // scratch vectors start at zero: SSOR's apply reads its output vector
    // (MTJ's start as copies of the solver's template vector)
    for (int k : need) ok = ok && cudaMalloc(&S->vecs[k], nb) == cudaSuccess && cudaMemset(S->vecs[k], 0, nb) == cudaSuccess;
    if (kind == MTJG_GMRES) {
        const size_t ld = (size_t)restart + 1;
        ok = ok && cudaMalloc(&S->V, nb * ld) == cudaSuccess;
        ok = ok && cudaMalloc(&S->gm.H, sizeof(double) * ld * (size_t)restart) == cudaSuccess;
        ok = ok && cudaMalloc(&S->gm.s, sizeof(double) * ld) == cudaSuccess;
        ok = ok && cudaMalloc(&S->gm.gc, sizeof(double) * ld) == cudaSuccess;
        ok = ok && cudaMalloc(&S->gm.gs, sizeof(double) * ld) == cudaSuccess;
        if (ok) {
            cudaMemset(S->V, 0, nb * ld);
            cudaMemset(S->gm.H, 0, sizeof(double) * ld * (size_t)restart);
        }
        S->gm.restart = restart;
    }
    ok = ok && cudaEventCreateWithFlags(&S->ev[0], cudaEventDisableTiming) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&S->ev[1], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        mtjg_solver_destroy(S);
        return fail(MTJG_ERR_OUT_OF_MEMORY, "cudaMalloc failed for the solver's work vectors");
    }
    *out = S;
    return MTJG_OK;
}

extern "C" int mtjg_solver_destroy(mtjg_solver *S)
{
    if (!S) return MTJG_OK;
    cudaSetDevice(S->ctx->device);
    cudaStreamSynchronize(S->ctx->stream);
    drop_graph(S);
    for (double *p : S->vecs) cudaFree(p);
    for (float *p : S->v32) cudaFree(p);
    cudaFree(S->pc_part);
    cudaFree(S->pc_p2);
    cudaFree(S->pc_bar);
    cudaFree(S->invdiag32);
    cudaFree(S->V);
    cudaFree(S->gm.H);
    cudaFree(S->gm.s);
    cudaFree(S->gm.gc);
    cudaFree(S->gm.gs);
    cudaFree(S->st);
    cudaFree(S->hist_r);
    cudaFree(S->hist_it);
    cudaFree(S->b_order);
    cudaFree(S->b_vec);
    cudaFree(S->b_ticket);
    cudaFree(S->b_xsave);
    cudaFree(S->ir_f);
    cudaFree(S->ir_d);
    if (S->ir_h) cudaFreeHost(S->ir_h);
    if (S->ev[0]) cudaEventDestroy(S->ev[0]);
    if (S->ev[1]) cudaEventDestroy(S->ev[1]);
    mtjg_ctx *ctx = S->ctx;
    delete S;
    ctx_release(ctx);
    return MTJG_OK;
}

extern "C" int mtjg_solver_set_precond(mtjg_solver *S, mtjg_precond *M)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    if (M && M->ctx != S->ctx) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "preconditioner uses another context");
    if (M && M->n != S->n) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "preconditioner size differs from the solver's");
    S->M = M;
    drop_graph(S);
    return MTJG_OK;
}

extern "C" int mtjg_solver_set_monitor(mtjg_solver *S, const mtjg_monitor *mon)
{
    if (!S || !mon) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (mon->norm < MTJG_NORM_ONE || mon->norm > MTJG_NORM_INFINITY || mon->history_cap < 0)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "bad monitor settings");
    MTJG_CUDA(cudaSetDevice(S->ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(S->ctx->stream));
    S->mon = *mon;
    drop_graph(S);
    return ensure_state(S, std::max(1, S->num_sys));
}

extern "C" int mtjg_solver_set_eigenvalues(mtjg_solver *S, double eigmin, double eigmax)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    if (S->kind != MTJG_CHEBYSHEV) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "eigenvalue bounds are Chebyshev's");
    // Chebyshev.setEigenvalues, S/Chebyshev.java:78-88
    if (eigmin <= 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "eigmin <= 0");
    if (eigmax <= 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "eigmax <= 0");
    if (eigmin > eigmax) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "eigmin > eigmax");
    MTJG_CUDA(cudaSetDevice(S->ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(S->ctx->stream));
    S->eigmin = eigmin;
    S->eigmax = eigmax;
    S->eig_set = true;
    drop_graph(S);
    return MTJG_OK;
}

extern "C" int mtjg_solver_set_mixed(mtjg_solver *S, int enable, double inner_rtol, int inner_max_iter)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    if (enable && S->kind != MTJG_CG && S->kind != MTJG_GMRES && S->kind != MTJG_BICGSTAB)
        return fail(MTJG_ERR_UNSUPPORTED, "mixed precision supports CG, GMRES and BiCGstab");
    if (enable && (!(inner_rtol > 0.0 && inner_rtol < 1.0) || inner_max_iter <= 0))
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "inner_rtol must lie in (0, 1) and inner_max_iter be positive");
    MTJG_CUDA(cudaSetDevice(S->ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(S->ctx->stream));
    if (enable && S->v32.empty()) {
        S->v32.assign(5, nullptr);
        for (auto &p : S->v32)
            if (cudaMalloc(&p, sizeof(float) * (size_t)std::max(1, S->n)) != cudaSuccess)
                return fail(MTJG_ERR_OUT_OF_MEMORY, "cudaMalloc failed for the FP32 work vectors");
    }
    S->mixed = enable != 0;
    if (enable) S->mix = MixCfg{inner_rtol, inner_max_iter, 0, 0.0, 0.0};
    drop_graph(S);
    return MTJG_OK;
}

extern "C" int mtjg_solver_set_matrix_monitor(mtjg_solver *S, int enable, double normA, double normb)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    S->xmon = enable ? 1 : 0;
    S->normA = enable ? normA : 0.0;
    S->normb = enable ? normb : 0.0;
    drop_graph(S);
    return MTJG_OK;
}

extern "C" int mtjg_solver_set_launch(mtjg_solver *S, int mode)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    if (mode != MTJG_LAUNCH_AUTO && mode != MTJG_LAUNCH_GRAPH)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "launch mode must be MTJG_LAUNCH_AUTO or MTJG_LAUNCH_GRAPH");
    S->launch_mode = mode;
    return MTJG_OK;
}

extern "C" int mtjg_solver_batch_results(mtjg_solver *S, mtjg_result *out, int count)
{
    if (!S || (!out && count > 0)) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (!S->last_valid) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "no solve has run");
    const int m = std::min(count, (int)S->last_all.size());
    for (int i = 0; i < m; ++i) {
        const SysState &q = S->last_all[i];
        out[i].status = map_status(q.status);
        out[i].iterations = q.iter;
        out[i].residual = q.residual;
        out[i].detail = q.detail;
        out[i].history_len = q.hist_len;
        out[i].inner_iterations = q.in_total;
    }
    return MTJG_OK;
}

extern "C" int mtjg_solver_batch_history(mtjg_solver *S, int sys, double *resid, int *iters, int cap, int *len)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    if (sys < 0 || sys >= (int)S->last_all.size()) return fail(MTJG_ERR_INDEX_OUT_OF_BOUNDS, "system index");
    const int have = std::min(S->last_all[sys].hist_len, S->mon.history_cap);
    if (len) *len = have;
    return copy_history(S, sys, resid, iters, std::min(have, cap));
}

extern "C" int mtjg_solver_solve(mtjg_solver *S, mtjg_csr *A, const double *b, double *x, mtjg_result *res)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    int st = check_sizes(S, A);
    if (st != MTJG_OK) return st;
    if (S->n == 0) return run_empty(S, res);
    if (!b || !x) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL vector");
    mtjg_ctx *ctx = S->ctx;
    MTJG_CUDA(cudaSetDevice(ctx->device));
    const size_t nb = sizeof(double) * (size_t)S->n;
    MTJG_CUDA(cudaMemcpyAsync(S->vecs[V_B], b, nb, cudaMemcpyHostToDevice, ctx->stream));
    MTJG_CUDA(cudaMemcpyAsync(S->vecs[V_X], x, nb, cudaMemcpyHostToDevice, ctx->stream));
    st = batch_persistent(S, A)            ? run_batch(S, A, res)
         : S->mixed && S->kind != MTJG_CG ? run_mixed_ir(S, A, res)
                                           : run(S, A, res);
    if (st == MTJG_ERR_CUDA || st == MTJG_ERR_OUT_OF_MEMORY || st == MTJG_ERR_DEVICE_TIMEOUT) return st;
    MTJG_CUDA(cudaMemcpyAsync(x, S->vecs[V_X], nb, cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    return st;
}

extern "C" int mtjg_solver_solve_dev(mtjg_solver *S, mtjg_csr *A, const double *db, double *dx, mtjg_result *res)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    int st = check_sizes(S, A);
    if (st != MTJG_OK) return st;
    if (S->n == 0) return run_empty(S, res);
    if (!db || !dx) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL vector");
    mtjg_ctx *ctx = S->ctx;
    MTJG_CUDA(cudaSetDevice(ctx->device));
    const size_t nb = sizeof(double) * (size_t)S->n;
    MTJG_CUDA(cudaMemcpyAsync(S->vecs[V_B], db, nb, cudaMemcpyDeviceToDevice, ctx->stream));
    MTJG_CUDA(cudaMemcpyAsync(S->vecs[V_X], dx, nb, cudaMemcpyDeviceToDevice, ctx->stream));
    st = batch_persistent(S, A)            ? run_batch(S, A, res)
         : S->mixed && S->kind != MTJG_CG ? run_mixed_ir(S, A, res)
                                           : run(S, A, res);
    if (st == MTJG_ERR_CUDA || st == MTJG_ERR_OUT_OF_MEMORY || st == MTJG_ERR_DEVICE_TIMEOUT) return st;
    MTJG_CUDA(cudaMemcpyAsync(dx, S->vecs[V_X], nb, cudaMemcpyDeviceToDevice, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    return st;
}

extern "C" int mtjg_solver_history(mtjg_solver *S, double *resid, int *iters, int cap, int *len)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL solver");
    const int have = S->last_valid ? std::min(S->last.hist_len, S->mon.history_cap) : 0;
    if (len) *len = have;
    return copy_history(S, S->last_sys, resid, iters, std::min(have, cap));
}
