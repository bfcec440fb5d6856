// dev.cuh -- device helpers: rounding modes, reductions, bulk copies, the
// on-device iteration monitor.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

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
struct Acc {
    double v[kParts];
};

__device__ __forceinline__ void acc_zero(Acc &a)
{
#pragma unroll
    for (int i = 0; i < kParts; ++i) a.v[i] = 0.0;
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

__device__ __forceinline__ void acc_merge(Acc &a, const Acc &b, int type)
{
    norm_merge(a.v[0], a.v[1], b.v[0], b.v[1], type);
#pragma unroll
    for (int i = 2; i < kParts; ++i) a.v[i] += b.v[i];
}

__device__ __forceinline__ void acc_shfl_down(Acc &a, int off, int type)
{
    Acc o;
#pragma unroll
    for (int i = 0; i < kParts; ++i) o.v[i] = __shfl_down_sync(0xffffffffu, a.v[i], off);
    acc_merge(a, o, type);
}

// Block-wide fixed-order reduction; result valid in thread 0.
__device__ __forceinline__ void block_reduce(Acc &a, int type, Acc *sm /* [kBlock/32] */)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc_shfl_down(a, off, type);
    if (lane == 0) sm[wid] = a;
    __syncthreads();
    if (wid == 0) {
        if (lane < (int)(blockDim.x >> 5)) a = sm[lane];
        else acc_zero(a);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc_shfl_down(a, off, type);
    }
    __syncthreads();
}

// Stores one tile's partial: block-reduce the per-thread partials (fixed
// order) and write them to the tile's slot.  No fence: see tiles_arrive.
__device__ __forceinline__ void tile_partial(Acc &a, int tile, const RedCtx &rc, int type, Acc *sm)
{
    block_reduce(a, type, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int i = 0; i < kParts; ++i) rc.part[(size_t)tile * kParts + i] = a.v[i];
    }
}

// The reduction of a phase finishes in k_finalize (a launch of its own after
// the phase's kernel): block s sums system s's tile partials in tile order
// (thread t takes tiles t, t+B, t+2B, ... with eight loads in flight, then
// the fixed block tree) and thread 0 runs op.scalar(s, sums).  No atomics
// and no fences: the launch boundary orders the partial stores before it.
template <class Op>
__global__ void __launch_bounds__(kBlock) k_finalize(Op op, RedCtx rc, int type)
{
    __shared__ Acc sm[kBlock / 32];
    const int sys = blockIdx.x;
    if (!op.active(sys)) return;
    const int t0 = rc.sys_tile[sys], t1 = rc.sys_tile[sys + 1];
    const int stride = blockDim.x;
    Acc s;
    acc_zero(s);
    for (int base = t0 + (int)threadIdx.x; base < t1; base += 8 * stride) {
        Acc o[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int t = base + u * stride;
#pragma unroll
            for (int i = 0; i < kParts; ++i) o[u].v[i] = t < t1 ? rc.part[(size_t)t * kParts + i] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (base + u * stride < t1) acc_merge(s, o[u], type);
    }
    block_reduce(s, type, sm);
    if (threadIdx.x == 0) op.scalar(sys, s);
}

// ------------------------------------------------------------ monitor
// AbstractIterationMonitor.converged(double) + DefaultIterationMonitor.convergedI
// (S/AbstractIterationMonitor.java:81-93, S/DefaultIterationMonitor.java:133-156):
// record (r, iter) for the reporter, then test in MTJ's order.
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
    if (r < jmax(c.rtol * st.initR, c.atol)) return ST_DONE;
    if (r > c.dtol * st.initR) return MTJG_NOT_CONVERGED_DIVERGENCE;
    if (st.iter >= c.max_iter) return MTJG_NOT_CONVERGED_ITERATIONS;
    if (r != r) return MTJG_NOT_CONVERGED_DIVERGENCE;
    return ST_RUNNING;
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
