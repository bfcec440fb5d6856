// krylov_ext.cuh -- BiCG, CGS, QMR, Chebyshev and IR (S/BiCG.java,
// S/CGS.java, S/QMR.java, S/Chebyshev.java, S/IR.java) as fused device
// phases, in the form of the CG / BiCGstab phases of solver.cu: CSR products
// with epilogues, row kernels, and per-system scalar steps run by the
// finalize launch.  Vector updates keep MTJ's operation order and its
// short-circuits (DenseVector.add(alpha, y) skips alpha == 0, set(alpha, y)
// zeroes, M/DenseVector.java:216-264); STRICT numerics round every product
// and sum as Java does.  Scalar recurrences that add a product use explicit
// round-to-nearest operations, so the compiler cannot fuse them.  With the
// identity or the Jacobi preconditioner its apply is fused into the
// neighbouring phase; ILU and ICC run as their own sweeps between phases.
#pragma once

#include "phases.cuh"

namespace mtjg {

// mtjg_result.detail of a breakdown: the quantity that became zero
constexpr int kBdRho = 1, kBdOmega = 2, kBdXi = 3, kBdDelta = 4, kBdEp = 5, kBdBeta = 6, kBdGamma = 7;

__device__ __forceinline__ void breakdown(SysState &t, int &c, int what)
{
    c = MTJG_NOT_CONVERGED_BREAKDOWN;
    t.detail = what;
}

// z = M r for the fused preconditioners (identity: r itself)
__device__ __forceinline__ double pc_fused(int pc, double r, const double *invdiag, int i)
{
    return pc == kPcJacobi ? r * invdiag[i] : r;
}

// ================================================================== IR
// S/IR.java:57-70
template <bool S>
struct IrRes {  // r = b - A x (A.multAdd(-1, x, r.set(b)), :61, :66); the monitor's test
    const double *b;
    double *r;
    MonPtrs m;
    bool first;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm;
    __device__ bool active(int sys) const { return first || m.st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double rr = b[i] - d;
        r[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        if (first) t.iter = 0;
        else t.iter++;
        m.finish(t, m.check(t, sys, norm_finish(s.v, m.mon.norm)));
    }
};

template <bool S>
struct IrX {  // z = M r; x.add(z) (:64-65); z applied here for identity and Jacobi
    double *x;
    const double *r, *z, *invdiag;
    int pc;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int, Acc &) const
    {
        if (pc == kPcJacobi) x[i] = fmac<S>(r[i], invdiag[i], x[i]);
        else x[i] = x[i] + (pc == kPcIdentity ? r[i] : z[i]);
    }
    __device__ void scalar(int, const Acc &) {}
};

// ============================================================ Chebyshev
// S/Chebyshev.java:90-120.  c and d come from the eigenvalue bounds (host).
struct ChCfg {
    double c, d;
};

template <bool S>
struct ChInit {  // r = b - A x (:96); test; z = M r fused (:102); alpha = 2 / d (:106)
    const double *b;
    double *r, *z;
    const double *invdiag;
    int pc;
    MonPtrs m;
    ChCfg cf;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm;
    __device__ bool active(int) const { return true; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double rr = b[i] - d;
        r[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
        if (pc == kPcJacobi) z[i] = rr * invdiag[i];
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.iter = 0;
        const int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING) t.alpha = 2.0 / cf.d;
        m.finish(t, c);
    }
};

struct ChQ {  // q = A p (A.mult, :114)
    double *q;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &) const { q[i] = mtj_assign(d); }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct ChUpd {  // x += alpha p; r -= alpha q (:115-116); next test; z = M r fused; next alpha, beta (:108-110)
    double *x, *r, *z;
    const double *p, *q, *invdiag;
    int pc;
    MonPtrs m;
    ChCfg cf;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm;
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
        if (pc == kPcJacobi) z[i] = rr * invdiag[i];
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.iter++;
        const int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING) {
            double beta = __ddiv_rn(__dmul_rn(t.alpha, cf.c), 2.0);
            beta = __dmul_rn(beta, beta);
            t.beta = beta;
            t.alpha = __ddiv_rn(1.0, __dsub_rn(cf.d, beta));
        }
        m.finish(t, c);
    }
};

// ================================================================= BiCG
// S/BiCG.java:63-102
template <bool S>
struct BgInit {  // r = b - A x; rtilde = r (:69-70); test; z = M r, zt = M' rt, rho_1 = z.rt fused (:73-75)
    const double *b;
    double *r, *rt, *z, *zt;
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
        rt[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
        if (pc != kPcExternal) {
            const double zz = pc_fused(pc, rr, invdiag, i);
            if (pc == kPcJacobi) {
                z[i] = zz;
                zt[i] = zz;
            }
            a.v[2] = fmac<S>(zz, rr, a.v[2]);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.iter = 0;
        int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING && pc != kPcExternal) {
            t.rho_1 = s.v[2];
            if (t.rho_1 == 0.) breakdown(t, c, kBdRho);
        }
        m.finish(t, c);
    }
};

template <bool S>
struct BgRho {  // rho_1 = z.rtilde after external M.apply / M.transApply (:73-79); beta (:85)
    const double *z, *rt;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int, Acc &a) const { a.v[2] = fmac<S>(z[i], rt[i], a.v[2]); }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.rho_1 = s.v[2];
        int c = ST_RUNNING;
        if (t.rho_1 == 0.) breakdown(t, c, kBdRho);
        else if (t.iter > 0) t.beta = t.rho_1 / t.rho_2;
        if (c != ST_RUNNING) m.finish(t, c);
    }
};

template <bool S>
struct BgP {  // p = z, pt = zt (first) or p = beta p + z, pt = beta pt + zt (:81-88)
    double *p, *pt;
    const double *z, *zt;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &) const
    {
        const SysState &t = st[sys];
        if (t.iter == 0) {
            p[i] = z[i];
            pt[i] = zt[i];
        } else {
            p[i] = fmac<S>(p[i], t.beta, z[i]);
            pt[i] = fmac<S>(pt[i], t.beta, zt[i]);
        }
    }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct BgQt {  // qt = A' pt (A.transMult, :91); alpha = rho_1 / pt.q (:93) -- on the transpose
    double *qt;
    const double *q;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = true;  // pt_c arrives with the row's diagonal gather
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int c, int, double d, double ptc, Acc &a) const
    {
        qt[c] = d;
        a.v[2] = fmac<S>(ptc, q[c], a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.alpha = t.rho_1 / s.v[2];
    }
};

template <bool S>
struct BgUpd {  // x += alpha p; r -= alpha q; rt -= alpha qt (:94-96); test; z, zt, rho_1 fused
    double *x, *r, *rt, *z, *zt;
    const double *p, *q, *qt, *invdiag;
    int pc;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm | kSlotD2;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &a) const
    {
        const double al = m.st[sys].alpha;
        double rr = r[i], rtt = rt[i];
        if (al != 0) {
            x[i] = fmac<S>(al, p[i], x[i]);
            rr = fmac<S>(-al, q[i], rr);
            r[i] = rr;
            rtt = fmac<S>(-al, qt[i], rtt);
            rt[i] = rtt;
        }
        norm_add<S>(a, rr, m.mon.norm);
        if (pc != kPcExternal) {
            const double zz = pc_fused(pc, rr, invdiag, i);
            if (pc == kPcJacobi) {
                z[i] = zz;
                zt[i] = rtt * invdiag[i];
            }
            a.v[2] = fmac<S>(zz, rtt, a.v[2]);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.rho_2 = t.rho_1;
        t.iter++;
        int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING && pc != kPcExternal) {
            t.rho_1 = s.v[2];
            if (t.rho_1 == 0.) breakdown(t, c, kBdRho);
            else t.beta = t.rho_1 / t.rho_2;
        }
        m.finish(t, c);
    }
};

// ================================================================== CGS
// S/CGS.java:65-105
template <bool S>
struct CsInit {  // r = b - A x; rtilde = r (:71-72); test; rho_1 = rtilde.r (:75)
    const double *b;
    double *r, *rt;
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
            if (t.rho_1 == 0) breakdown(t, c, kBdRho);
        }
        m.finish(t, c);
    }
};

template <bool S>
struct CsP {  // u = r, p = u (first); u = r + beta q, sum = q + beta p, p = u + beta sum (:81-89); phat = M p fused (:91)
    double *u, *p, *phat;
    const double *r, *q, *invdiag;
    int pc;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &) const
    {
        const SysState &t = st[sys];
        const double rr = r[i];
        double uu, pp;
        if (t.iter == 0) {
            uu = rr;
            pp = uu;
        } else {
            const double be = t.beta, qq = q[i];
            uu = be != 0 ? fmac<S>(be, qq, rr) : rr;
            const double sum = be != 0 ? fmac<S>(be, p[i], qq) : qq;
            pp = be != 0 ? fmac<S>(be, sum, uu) : uu;
        }
        u[i] = uu;
        p[i] = pp;
        if (pc == kPcJacobi) phat[i] = pp * invdiag[i];
    }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct CsV {  // vhat = A phat; alpha = rho_1 / rtilde.vhat (:92-93)
    double *vhat;
    const double *rt;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double vv = mtj_assign(d);
        vhat[i] = vv;
        a.v[2] = fmac<S>(rt[i], vv, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.alpha = t.rho_1 / s.v[2];
    }
};

template <bool S>
struct CsQ {  // q = -alpha vhat + u; sum = u + q; uhat = M sum; x += alpha uhat (:94-97), M fused
    double *q, *sum, *uhat, *x;
    const double *vhat, *u, *invdiag;
    int pc;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &) const
    {
        const double al = st[sys].alpha, na = -al;
        const double uu = u[i];
        const double qq = na == 0 ? 0.0 + uu : fmac<S>(na, vhat[i], uu);
        q[i] = qq;
        const double ss = uu + qq;
        if (pc == kPcExternal) {
            sum[i] = ss;
            return;
        }
        const double uh = pc_fused(pc, ss, invdiag, i);
        uhat[i] = uh;
        if (al != 0) x[i] = fmac<S>(al, uh, x[i]);
    }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct CsX {  // x += alpha uhat after an external M.apply (:97)
    double *x;
    const double *uhat;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &) const
    {
        const double al = st[sys].alpha;
        if (al != 0) x[i] = fmac<S>(al, uhat[i], x[i]);
    }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct CsQh {  // qhat = A uhat; r -= alpha qhat (:98-99); next test; rho_1 = rtilde.r, beta (:75, :85)
    double *r;
    const double *rt;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm | kSlotD2;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int sys, double d, double, Acc &a) const
    {
        const double qh = mtj_assign(d), al = m.st[sys].alpha;
        double rr = r[i];
        if (al != 0) {
            rr = fmac<S>(-al, qh, rr);
            r[i] = rr;
        }
        norm_add<S>(a, rr, m.mon.norm);
        a.v[2] = fmac<S>(rt[i], rr, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.rho_2 = t.rho_1;
        t.iter++;
        int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (c == ST_RUNNING) {
            t.rho_1 = s.v[2];
            if (t.rho_1 == 0) breakdown(t, c, kBdRho);
            else t.beta = t.rho_1 / t.rho_2;
        }
        m.finish(t, c);
    }
};

// ================================================================== QMR
// S/QMR.java:117-213 with M1 = M2 = the solver's preconditioner.  The
// scalars live in SysState (rho, rho_1, xi, gamma, gamma_1, theta, theta_1,
// eta, delta, ep, beta); scratch[0] = 1 / rho and scratch[1] = 1 / xi of the
// running iteration.

// rho and xi are due: breakdown checks (:134-141), then the reciprocals
__device__ __forceinline__ void qmr_rho_xi(SysState &t, int &c)
{
    if (t.rho == 0) breakdown(t, c, kBdRho);
    else if (t.xi == 0) breakdown(t, c, kBdXi);
    else {
        t.scratch[0] = 1 / t.rho;
        t.scratch[1] = 1 / t.xi;
    }
}

// gamma, theta, eta after xi (:188-197); coef[0] = the d / s scale factor (:203)
__device__ __forceinline__ void qmr_gamma(SysState &t, int &c)
{
    t.gamma_1 = t.gamma;
    t.theta_1 = t.theta;
    t.theta = t.rho / __dmul_rn(t.gamma_1, t.beta);
    t.gamma = 1 / sqrt(__dadd_rn(1.0, __dmul_rn(t.theta, t.theta)));
    if (t.gamma == 0) {
        breakdown(t, c, kBdGamma);
        return;
    }
    t.eta = __dmul_rn(__dmul_rn(__dmul_rn(-t.eta, t.rho_1), t.gamma), t.gamma) /
            __dmul_rn(__dmul_rn(t.beta, t.gamma_1), t.gamma_1);
    t.coef[0] = __dmul_rn(__dmul_rn(__dmul_rn(t.theta_1, t.theta_1), t.gamma), t.gamma);
}

template <bool S>
struct QmInit {  // r = b - A x; v_tld = w_tld = r (:123-129); y = M1 v_tld, z = M2' w_tld fused;
                 // rho = |y|, xi = |z| (:126-131); the test; gamma = 1, eta = -1 (:121)
    const double *b;
    double *r, *vt, *wt, *y, *z;
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
        vt[i] = rr;
        wt[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
        if (pc != kPcExternal) {
            // M2' w_tld = M1 v_tld here: the same vector and a symmetric preconditioner
            const double yy = pc_fused(pc, rr, invdiag, i);
            y[i] = yy;
            z[i] = yy;
            a.v[2] = fmac<S>(yy, yy, a.v[2]);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.iter = 0;
        t.gamma = 1.;
        t.eta = -1.;
        t.theta = 0;
        t.ep = 0;
        int c = m.check(t, sys, norm_finish(s.v, m.mon.norm));
        if (pc != kPcExternal) {
            t.rho = sqrt(s.v[2]);
            t.xi = t.rho;
            if (c == ST_RUNNING) qmr_rho_xi(t, c);
        }
        m.finish(t, c);
    }
};

template <bool S>
struct QmNorms {  // external M: rho = |y|, xi = |z| after y = M1 v_tld, z = M2' w_tld (:126-131)
    const double *y, *z;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2 | kSlotD3;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int, Acc &a) const
    {
        a.v[2] = fmac<S>(y[i], y[i], a.v[2]);
        a.v[3] = fmac<S>(z[i], z[i], a.v[3]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.rho = sqrt(s.v[2]);
        t.xi = sqrt(s.v[3]);
        int c = ST_RUNNING;
        qmr_rho_xi(t, c);
        if (c != ST_RUNNING) m.finish(t, c);
    }
};

template <bool S>
struct QmA {  // v = v_tld / rho, y /= rho, w = w_tld / xi, z /= xi (:143-146); delta = z.y (:148-152);
              // y_tld = M2 y, z_tld = M1' z fused (:154-155)
    double *v, *y, *w, *z, *yt, *zt;
    const double *vt, *wt, *invdiag;
    int pc;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &a) const
    {
        const SysState &t = m.st[sys];
        const double ir = t.scratch[0], ix = t.scratch[1];
        v[i] = ir == 0 ? 0.0 : ir * vt[i];
        const double yy = y[i] * ir;
        y[i] = yy;
        w[i] = ix == 0 ? 0.0 : ix * wt[i];
        const double zz = z[i] * ix;
        z[i] = zz;
        a.v[2] = fmac<S>(zz, yy, a.v[2]);
        if (pc != kPcExternal) {
            yt[i] = pc_fused(pc, yy, invdiag, i);
            zt[i] = pc_fused(pc, zz, invdiag, i);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.delta = s.v[2];
        int c = ST_RUNNING;
        if (t.delta == 0) breakdown(t, c, kBdDelta);
        else if (t.iter > 0) {
            t.coef[0] = __dmul_rn(-t.xi, t.delta) / t.ep;
            t.coef[1] = __dmul_rn(-t.rho, t.delta) / t.ep;
        }
        if (c != ST_RUNNING) m.finish(t, c);
    }
};

template <bool S>
struct QmP {  // p = y_tld, q = z_tld (first) or p = c0 p + y_tld, q = c1 q + z_tld (:157-163)
    double *p, *q;
    const double *yt, *zt;
    SysState *st;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &) const
    {
        const SysState &t = st[sys];
        if (t.iter == 0) {
            p[i] = yt[i];
            q[i] = zt[i];
        } else {
            p[i] = fmac<S>(p[i], t.coef[0], yt[i]);
            q[i] = fmac<S>(q[i], t.coef[1], zt[i]);
        }
    }
    __device__ void scalar(int, const Acc &) {}
};

template <bool S>
struct QmPt {  // p_tld = A p; ep = q.p_tld; beta = ep / delta (:165-177)
    double *ptl;
    const double *q;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double d, double, Acc &a) const
    {
        const double pv = mtj_assign(d);
        ptl[i] = pv;
        a.v[2] = fmac<S>(q[i], pv, a.v[2]);
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.ep = s.v[2];
        int c = ST_RUNNING;
        if (t.ep == 0) breakdown(t, c, kBdEp);
        else {
            t.beta = t.ep / t.delta;
            if (t.beta == 0) breakdown(t, c, kBdBeta);
        }
        if (c != ST_RUNNING) m.finish(t, c);
    }
};

template <bool S>
struct QmV {  // v_tld = -beta v + p_tld (:179); y = M1 v_tld fused (:180); rho_1 = rho, rho = |y| (:181-182)
    double *vt, *y;
    const double *v, *ptl, *invdiag;
    int pc;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &a) const
    {
        const double nb = -st[sys].beta;
        const double vv = nb == 0 ? 0.0 + ptl[i] : fmac<S>(nb, v[i], ptl[i]);
        vt[i] = vv;
        if (pc != kPcExternal) {
            const double yy = pc_fused(pc, vv, invdiag, i);
            y[i] = yy;
            a.v[2] = fmac<S>(yy, yy, a.v[2]);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        if (pc == kPcExternal) return;
        SysState &t = st[sys];
        t.rho_1 = t.rho;
        t.rho = sqrt(s.v[2]);
    }
};

template <bool S>
struct QmRho {  // external M: rho_1 = rho, rho = |y| after y = M1 v_tld (:181-182)
    const double *y;
    SysState *st;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int, Acc &a) const { a.v[2] = fmac<S>(y[i], y[i], a.v[2]); }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = st[sys];
        t.rho_1 = t.rho;
        t.rho = sqrt(s.v[2]);
    }
};

template <bool S>
struct QmW {  // w_tld = A' q + (-beta w) (A.transMultAdd(q, w_tld.set(-beta, w)), :184) on the
              // transpose; z = M2' w_tld fused; xi = |z| (:185-186); gamma, theta, eta (:188-197)
    double *wt, *z;
    const double *w, *invdiag;
    int pc;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    // transMultAdd(1, q, y) scales y by 1 / 1 and by 1 again: both exact
    __device__ double init(int c, int sys) const
    {
        const double nb = -m.st[sys].beta;
        return nb == 0 ? 0.0 : nb * w[c];
    }
    __device__ void row(int c, int, double d, double, Acc &a) const
    {
        wt[c] = d;
        if (pc != kPcExternal) {
            const double zz = pc_fused(pc, d, invdiag, c);
            z[c] = zz;
            a.v[2] = fmac<S>(zz, zz, a.v[2]);
        }
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        if (pc == kPcExternal) return;
        SysState &t = m.st[sys];
        t.xi = sqrt(s.v[2]);
        int c = ST_RUNNING;
        qmr_gamma(t, c);
        if (c != ST_RUNNING) m.finish(t, c);
    }
};

template <bool S>
struct QmXi {  // external M: xi = |z| after z = M2' w_tld (:185-186); gamma, theta, eta (:188-197)
    const double *z;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotD2;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int, Acc &a) const { a.v[2] = fmac<S>(z[i], z[i], a.v[2]); }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        t.xi = sqrt(s.v[2]);
        int c = ST_RUNNING;
        qmr_gamma(t, c);
        if (c != ST_RUNNING) m.finish(t, c);
    }
};

template <bool S>
struct QmUpd {  // d = eta p, s = eta p_tld (first) or d = val d + eta p, s = val s + eta p_tld (:199-206);
                // x += d; r -= s (:208-209); the next test; rho / xi breakdown checks (:134-141)
    double *d, *s, *x, *r;
    const double *p, *ptl;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ void row(int i, int sys, Acc &a) const
    {
        const SysState &t = m.st[sys];
        const double eta = t.eta;
        double dd, ss;
        if (t.iter == 0) {
            dd = eta == 0 ? 0.0 : eta * p[i];
            ss = eta == 0 ? 0.0 : eta * ptl[i];
        } else {
            const double val = t.coef[0];
            dd = d[i] * val;
            ss = s[i] * val;
            if (eta != 0) {
                dd = fmac<S>(eta, p[i], dd);
                ss = fmac<S>(eta, ptl[i], ss);
            }
        }
        d[i] = dd;
        s[i] = ss;
        x[i] = x[i] + dd;
        const double rr = r[i] - ss;
        r[i] = rr;
        norm_add<S>(a, rr, m.mon.norm);
    }
    __device__ void scalar(int sys, const Acc &sm)
    {
        SysState &t = m.st[sys];
        t.iter++;
        int c = m.check(t, sys, norm_finish(sm.v, m.mon.norm));
        if (c == ST_RUNNING) qmr_rho_xi(t, c);
        m.finish(t, c);
    }
};

}  // namespace mtjg
