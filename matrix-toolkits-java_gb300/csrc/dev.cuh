// dev.cuh -- device helpers: rounding modes, reductions, bulk copies, the
// on-device iteration monitor.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "internal.h"

namespace mtjg {

// a*b + c.  STRICT rounds the product and the sum separately (Java's
// semantics, no contraction); FAST issues one fused multiply-add.
template <bool S>
__device__ __forceinline__ double fmac(double a, double b, double c)
{
    if constexpr (S)
        return __dadd_rn(__dmul_rn(a, b), c);
    else
        return fma(a, b, c);
}

template <bool S>
__device__ __forceinline__ float fmac(float a, float b, float c)
{
    if constexpr (S)
        return __fadd_rn(__fmul_rn(a, b), c);
    else
        return fmaf(a, b, c);
}

// the rounded product and the rounded sum of STRICT, apart
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

// MTJ assigns a row sum only when it is nonzero (CompRowMatrix.mult,
// S/CompRowMatrix.java:309-311), so a -0.0 sum leaves +0.0 behind.  Done on
// the bits: an FP64 compare would take an issue slot of the narrow FP64 pipe
// for every row.
__device__ __forceinline__ double mtj_assign(double d)
{
    return __double_as_longlong(d) == (long long)0x8000000000000000ULL ? 0.0 : d;
}

// java.lang.Math.max: NaN propagates.
__device__ __forceinline__ double jmax(double a, double b)
{
    if (a != a) return a;
    if (b != b) return b;
    return a >= b ? a : b;
}

// ----------------------------------------------------------- partial sums
// Acc slots: v[0], v[1] hold a vector norm (ONE/TWO: sum in v[0]; INFINITY:
// max in v[0]; TWO_ROBUST: (scale, ssq) in v[0], v[1]); v[2], v[3] hold
// plain sums (dot products).
// Per-thread partial sums.  f[0] / f[1] are FP32 running sums that FP32
// phases add into instead of slots 2 / 3: they reach the FP64 slots once per
// thread and group (group_partial), so an FP32 dot product costs no FP64
// conversion or add per row -- GB300's FP64 pipe is the narrow one.
struct Acc {
    double v[kParts];
    float f[2];
};

__device__ __forceinline__ void acc_zero(Acc &a)
{
#pragma unroll
    for (int i = 0; i < kParts; ++i) a.v[i] = 0.0;
    a.f[0] = a.f[1] = 0.0f;
}

template <bool S>
__device__ __forceinline__ void norm_add(Acc &a, double x, int type)
{
    if (type == MTJG_NORM_TWO) {
        a.v[0] = fmac<S>(x, x, a.v[0]);
    } else if (type == MTJG_NORM_ONE) {
        a.v[0] = a.v[0] + fabs(x);
    } else if (type == MTJG_NORM_INFINITY) {
        a.v[0] = jmax(fabs(x), a.v[0]);
    } else if (x != 0) {  // robust two-norm, scaled sum of squares
        double ax = fabs(x);
        if (a.v[0] < ax) {
            double q = a.v[0] / ax;
            a.v[1] = 1.0 + a.v[1] * q * q;
            a.v[0] = ax;
        } else {
            double q = ax / a.v[0];
            a.v[1] += q * q;
        }
    }
}

__device__ __forceinline__ void norm_merge(double &s1, double &q1, double s2, double q2, int type)
{
    if (type == MTJG_NORM_INFINITY) {
        s1 = jmax(s1, s2);
    } else if (type == MTJG_NORM_TWO_ROBUST) {
        if (s2 == 0) return;
        if (s1 == 0) { s1 = s2; q1 = q2; return; }
        if (s1 >= s2) {
            double r = s2 / s1;
            q1 = q1 + q2 * r * r;
        } else {
            double r = s1 / s2;
            q1 = q2 + q1 * r * r;
            s1 = s2;
        }
    } else {
        s1 = s1 + s2;
    }
}

__device__ __forceinline__ double norm_finish(const double *v, int type)
{
    if (type == MTJG_NORM_TWO) return sqrt(v[0]);
    if (type == MTJG_NORM_TWO_ROBUST) return v[0] * sqrt(v[1]);
    return v[0];
}

// Slot masks: bit i set = Acc slot i carries a value.  Slots 0/1 hold a norm
// (slot 1 only for TWO_ROBUST); slots 2/3 plain sums.  Reductions touch only
// the slots a phase uses: every FP64 add or compare spent on an idle slot is
// an issue slot of GB300's narrow FP64 pipe.
constexpr int kSlotNorm = 1, kSlotD2 = 4, kSlotD3 = 8;

// Op::kSlots when the op declares it, else every slot.
template <class Op, class = void>
struct OpSlots {
    static constexpr int value = kSlotNorm | kSlotD2 | kSlotD3;
};
template <class Op>
struct OpSlots<Op, decltype((void)Op::kSlots)> {
    static constexpr int value = Op::kSlots;
};

// Shared-memory rows (kBlock doubles each) a block reduction of SLOTS uses:
// two for a norm (the robust norm's scale and sum), one per plain sum.
template <int SLOTS>
constexpr int red_rows()
{
    return ((SLOTS & kSlotNorm) ? 2 : 0) + ((SLOTS & kSlotD2) ? 1 : 0) + ((SLOTS & kSlotD3) ? 1 : 0);
}

template <int SLOTS>
__device__ __forceinline__ void acc_merge_m(Acc &a, const Acc &b, int type)
{
    if constexpr ((SLOTS & kSlotNorm) != 0) {
        if (type == MTJG_NORM_ONE || type == MTJG_NORM_TWO) a.v[0] += b.v[0];
        else norm_merge(a.v[0], a.v[1], b.v[0], b.v[1], type);
    }
    if constexpr ((SLOTS & kSlotD2) != 0) a.v[2] += b.v[2];
    if constexpr ((SLOTS & kSlotD3) != 0) a.v[3] += b.v[3];
}

__device__ __forceinline__ void acc_merge(Acc &a, const Acc &b, int type)
{
    acc_merge_m<kSlotNorm | kSlotD2 | kSlotD3>(a, b, type);
}

template <int SLOTS>
__device__ __forceinline__ void acc_shfl_down(Acc &a, int off, int type)
{
    Acc o;
    if constexpr ((SLOTS & kSlotNorm) != 0) {
        o.v[0] = __shfl_down_sync(0xffffffffu, a.v[0], off);
        o.v[1] = type == MTJG_NORM_TWO_ROBUST ? __shfl_down_sync(0xffffffffu, a.v[1], off) : 0.0;
    }
    if constexpr ((SLOTS & kSlotD2) != 0) o.v[2] = __shfl_down_sync(0xffffffffu, a.v[2], off);
    if constexpr ((SLOTS & kSlotD3) != 0) o.v[3] = __shfl_down_sync(0xffffffffu, a.v[3], off);
    acc_merge_m<SLOTS>(a, o, type);
}

// Block-wide fixed-order reduction of the slots in SLOTS; result valid in
// thread 0.  Every thread parks its slots in shared memory; warp 0 alone
// then sums them (lane l takes entries l, l+32, ..., sequentially) and
// finishes with a 5-level butterfly.  That costs about a quarter of the
// FP64 instructions of a shuffle tree run in every warp.
template <int SLOTS>
__device__ __forceinline__ void block_reduce(Acc &a, int type, double *sm /* [red_rows<SLOTS>() * kBlock] */)
{
    constexpr bool kN = (SLOTS & kSlotNorm) != 0, k2 = (SLOTS & kSlotD2) != 0, k3 = (SLOTS & kSlotD3) != 0;
    // rows: norm scale, norm sum (with a norm), then slot 2, then slot 3
    constexpr int o2 = kN ? 2 * kBlock : 0, o3 = o2 + (k2 ? kBlock : 0);
    const int tid = threadIdx.x, lane = tid & 31, nt = blockDim.x;
    const bool robust = type == MTJG_NORM_TWO_ROBUST;
    if constexpr (kN) {
        sm[tid] = a.v[0];
        if (robust) sm[kBlock + tid] = a.v[1];
    }
    if constexpr (k2) sm[o2 + tid] = a.v[2];
    if constexpr (k3) sm[o3 + tid] = a.v[3];
    __syncthreads();
    if (tid < 32 && SLOTS != 0) {
        Acc o;
        if constexpr (kN) {
            a.v[0] = sm[lane];
            a.v[1] = robust ? sm[kBlock + lane] : 0.0;
        }
        if constexpr (k2) a.v[2] = sm[o2 + lane];
        if constexpr (k3) a.v[3] = sm[o3 + lane];
        for (int i = lane + 32; i < nt; i += 32) {
            if constexpr (kN) {
                o.v[0] = sm[i];
                o.v[1] = robust ? sm[kBlock + i] : 0.0;
            }
            if constexpr (k2) o.v[2] = sm[o2 + i];
            if constexpr (k3) o.v[3] = sm[o3 + i];
            acc_merge_m<SLOTS>(a, o, type);
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc_shfl_down<SLOTS>(a, off, type);
    }
    __syncthreads();
}

// Stores one group's partial: block-reduce the per-thread partials (fixed
// order) and write the used slots to the group's entry.
template <int SLOTS>
__device__ __forceinline__ void group_partial(Acc &a, int group, const RedCtx &rc, int type, double *sm)
{
    if constexpr ((SLOTS & kSlotD2) != 0) a.v[2] += (double)a.f[0];
    if constexpr ((SLOTS & kSlotD3) != 0) a.v[3] += (double)a.f[1];
    block_reduce<SLOTS>(a, type, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < kParts; ++i)
            if (SLOTS & (i < 2 ? kSlotNorm : (1 << i))) rc.part[(size_t)group * kParts + i] = a.v[i];
    }
}

// System sys's group partials summed in group order by a block of kBlock
// threads (valid in thread 0): thread t takes groups t, t+B, t+2B, ... with
// four loads in flight, then the fixed block tree.  Plain loads: a kernel
// may sum partials that its own blocks wrote before a grid barrier.
template <int SLOTS>
__device__ __forceinline__ Acc system_sum(const RedCtx &rc, int sys, int type, double *sm)
{
    const int g0 = rc.sys_group[sys], g1 = rc.sys_group[sys + 1];
    const int stride = blockDim.x;
    Acc s;
    acc_zero(s);
    for (int base = g0 + (int)threadIdx.x; base < g1; base += 4 * stride) {
        Acc o[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int g = base + u * stride;
#pragma unroll
            for (int i = 0; i < kParts; ++i)
                o[u].v[i] = (g < g1 && (SLOTS & (i < 2 ? kSlotNorm : (1 << i)))) ? rc.part[(size_t)g * kParts + i]
                                                                                  : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (base + u * stride < g1) acc_merge_m<SLOTS>(s, o[u], type);
    }
    block_reduce<SLOTS>(s, type, sm);
    return s;
}

// |x| in the monitor's norm for a MatrixIterationMonitor, by the whole block
// (thread-strided sums, the fixed block tree), into t.xnorm ahead of the
// test; sm holds kParts * kBlock doubles.
__device__ __forceinline__ void xnorm_block(SysState &t, int type, double *sm)
{
    Acc a;
    acc_zero(a);
    const double *x = t.xm_x;
    const int n = t.xm_n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (t.xm_strict) norm_add<true>(a, x[i], type);
        else norm_add<false>(a, x[i], type);
    }
    block_reduce<kSlotNorm>(a, type, sm);
    if (threadIdx.x == 0) t.xnorm = norm_finish(a.v, type);
    __syncthreads();
}

// An op with a monitor (member m) has its finalize form |x| first when a
// MatrixIterationMonitor is set (a variant of its own, k_finalize<Op, true>,
// so the default monitor's finalize carries none of it).
template <class Op, class = void>
struct OpMon {
    static constexpr bool value = false;
};
template <class Op>
struct OpMon<Op, decltype((void)std::declval<const Op &>().m.mon.xmon)> {
    static constexpr bool value = true;
};

// The reduction of a phase finishes in k_finalize (a launch of its own after
// the phase's kernel): block s forms system s's sums and thread 0 runs
// op.scalar(s, sums).  No atomics and no fences: the launch boundary orders
// the partial stores before it.  (The one-launch CG sums a phase's partials
// itself, with the same function, after a grid barrier.)
//
// Kernel templates and their launchers live in an unnamed namespace: without
// relocatable device code every translation unit carries its own device
// image, so each one instantiates (and sets attributes on) its own kernels.
namespace {
template <class Op, bool XN = false>
__global__ void __launch_bounds__(kBlock) k_finalize(Op op, RedCtx rc, int type)
{
    constexpr int SLOTS = OpSlots<Op>::value;
    __shared__ double sm[kParts * kBlock];
    const int sys = blockIdx.x;
    if (!op.active(sys)) return;
    if constexpr (XN) xnorm_block(op.m.st[sys], op.m.mon.norm, sm);
    const Acc s = system_sum<SLOTS>(rc, sys, type, sm);
    if (threadIdx.x == 0) op.scalar(sys, s);
}
}  // namespace

// ------------------------------------------------------------ monitor
// AbstractIterationMonitor.converged(double) + DefaultIterationMonitor.convergedI
// (S/AbstractIterationMonitor.java:81-93, S/DefaultIterationMonitor.java:133-156):
// record (r, iter) for the reporter, then test in MTJ's order (with a
// MatrixIterationMonitor, its convergence test, S/MatrixIterationMonitor.java
// :101-124).
__device__ __forceinline__ int monitor_check(SysState &st, const MonCfgDev &c, double r,
                                             double *hist_r, int *hist_it)
{
    if (st.hist_len < c.hist_cap) {
        hist_r[st.hist_len] = r;
        hist_it[st.hist_len] = st.iter;
    }
    st.hist_len++;
    st.residual = r;
    if (st.iter == 0) st.initR = r;
    const double tol =
        c.xmon ? jmax(c.rtol * (st.xm_normA * st.xnorm + st.xm_normb), c.atol) : jmax(c.rtol * st.initR, c.atol);
    if (r < tol) return ST_DONE;
    if (r > c.dtol * st.initR) return MTJG_NOT_CONVERGED_DIVERGENCE;
    if (st.iter >= c.max_iter) return MTJG_NOT_CONVERGED_ITERATIONS;
    if (r != r) return MTJG_NOT_CONVERGED_DIVERGENCE;
    return ST_RUNNING;
}

// AbstractIterationMonitor.converged(double) (S/AbstractIterationMonitor.java
// :88-93), GMRES's inner test: the reporter and the residual, then
// convergedI(r), which a MatrixIterationMonitor does not support
// (S/MatrixIterationMonitor.java:127-129).
__device__ __forceinline__ int monitor_check_scalar(SysState &st, const MonCfgDev &c, double r, double *hist_r,
                                                    int *hist_it)
{
    if (!c.xmon) return monitor_check(st, c, r, hist_r, hist_it);
    if (st.hist_len < c.hist_cap) {
        hist_r[st.hist_len] = r;
        hist_it[st.hist_len] = st.iter;
    }
    st.hist_len++;
    st.residual = r;
    return MTJG_ERR_UNSUPPORTED;
}

// ---------------------------------------------------- bulk copies (TMA)
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after `limit` polls and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, long long limit)
{
    for (long long i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Global -> shared bulk copy (cp.async.bulk): 16-byte aligned addresses and
// a byte count that is a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

}  // namespace mtjg
