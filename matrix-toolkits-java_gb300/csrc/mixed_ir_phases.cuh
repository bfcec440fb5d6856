// mixed_ir_phases.cuh -- kernels and product epilogues of the mixed-precision
// GMRES(m) and BiCGstab solves (mixed_ir.cuh drives them).
#pragma once

#include "phases.cuh"

namespace mtjg {

constexpr int kIrBlock = 256;

__device__ __forceinline__ double ir_block_sum(double v, double *sm)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sm[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < kIrBlock / 32; ++k) s += sm[k];
    return s;
}

// part[y * gridDim.x + block] = block's share of V_y . w  (grid: G x k)
__global__ void __launch_bounds__(kIrBlock) k_ir_vdot(int n, const float *V, int64_t ldv, const float *w, double *part)
{
    __shared__ double sm[kIrBlock / 32];
    const float *v = V + (int64_t)blockIdx.y * ldv;
    double acc = 0.0;
    for (int i = blockIdx.x * kIrBlock + threadIdx.x; i < n; i += gridDim.x * kIrBlock)
        acc += (double)v[i] * (double)w[i];
    acc = ir_block_sum(acc, sm);
    if (threadIdx.x == 0) part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = acc;
}

// out[slot] = sum over blocks of part[slot * G + block], in block order
// within each lane's stride and then a fixed shuffle tree (grid: k x 32)
__global__ void k_ir_final(const double *part, int G, double *out)
{
    const int slot = blockIdx.x, lane = threadIdx.x;
    double s = 0.0;
    for (int b = lane; b < G; b += 32) s += part[(size_t)slot * G + b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) out[slot] = s;
}

// out = ca a + cb b + cc c (b, c nullable; out may alias a, b or c), with
// the partials of out . out (part[block]) and of out . q (part[G + block])
// when part (and q) are given
__global__ void __launch_bounds__(kIrBlock) k_ir_lin(int n, float *out, const float *a, float ca, const float *b,
                                                     float cb, const float *c, float cc, const float *q, double *part)
{
    __shared__ double sm[kIrBlock / 32];
    double s0 = 0.0, s1 = 0.0;
    for (int i = blockIdx.x * kIrBlock + threadIdx.x; i < n; i += gridDim.x * kIrBlock) {
        float v = ca * a[i];
        if (b) v = fmaf(cb, b[i], v);
        if (c) v = fmaf(cc, c[i], v);
        out[i] = v;
        s0 += (double)v * (double)v;
        if (q) s1 += (double)v * (double)q[i];
    }
    if (!part) return;
    s0 = ir_block_sum(s0, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = s0;
    if (q) {
        __syncthreads();
        s1 = ir_block_sum(s1, sm);
        if (threadIdx.x == 0) part[gridDim.x + blockIdx.x] = s1;
    }
}

// w -= sum_t h[t] V_t  (k <= 64)
__global__ void __launch_bounds__(kIrBlock) k_ir_vupd(int n, const float *V, int64_t ldv, int k, const double *h,
                                                      float *w)
{
    __shared__ float hs[64];
    if (threadIdx.x < k) hs[threadIdx.x] = (float)h[threadIdx.x];
    __syncthreads();
    for (int i = blockIdx.x * kIrBlock + threadIdx.x; i < n; i += gridDim.x * kIrBlock) {
        float acc = w[i];
        for (int t = 0; t < k; ++t) acc = fmaf(-hs[t], V[(int64_t)t * ldv + i], acc);
        w[i] = acc;
    }
}

// out = sum_t y[t] V_t  (k <= 64)
__global__ void __launch_bounds__(kIrBlock) k_ir_vcomb(int n, const float *V, int64_t ldv, int k, const double *y,
                                                       float *out)
{
    __shared__ float ys[64];
    if (threadIdx.x < k) ys[threadIdx.x] = (float)y[threadIdx.x];
    __syncthreads();
    for (int i = blockIdx.x * kIrBlock + threadIdx.x; i < n; i += gridDim.x * kIrBlock) {
        float acc = 0.0f;
        for (int t = 0; t < k; ++t) acc = fmaf(ys[t], V[(int64_t)t * ldv + i], acc);
        out[i] = acc;
    }
}

// x += d (the FP32 correction, widened exactly), then iter.next()
__global__ void k_ir_xadd(int n, double *x, const float *d, SysState *st)
{
    if (st->status != ST_RUNNING) return;
    for (int i = blockIdx.x * kIrBlock + threadIdx.x; i < n; i += gridDim.x * kIrBlock) x[i] = x[i] + (double)d[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) st->iter++;
}

// r = b - A x in FP64, rin = (float) r, and the monitor's test on r
struct MiOuter {
    const double *b;
    float *rin;
    MonPtrs m;
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm;
    __device__ bool active(int sys) const { return m.st[sys].status == ST_RUNNING; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int i, int, double dd, double, Acc &a) const
    {
        const double rr = b[i] - dd;
        norm_add<false>(a, rr, m.mon.norm);
        rin[i] = (float)rr;
    }
    __device__ void scalar(int sys, const Acc &s)
    {
        SysState &t = m.st[sys];
        m.finish(t, m.check(t, sys, norm_finish(s.v, m.mon.norm)));
    }
};

// y = A32 x, or y = rhs - A32 x
struct Mi32Prod {
    float *y;
    const float *rhs;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int) const { return true; }
    __device__ float init(int, int) const { return 0.0f; }
    __device__ void row(int i, int, float dd, float, Acc &) const { y[i] = rhs ? rhs[i] - dd : dd; }
    __device__ void scalar(int, const Acc &) {}
};

}  // namespace mtjg
