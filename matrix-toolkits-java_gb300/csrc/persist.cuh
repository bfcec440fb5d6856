// persist.cuh -- CG (identity or Jacobi preconditioner) on one small system
// in one launch.
//
// On a system of a few hundred tiles every phase of the graph-captured loop
// (p, q = A p, its finalize, the update, its finalize) is a few dependent
// L2 round trips wide, and the iteration costs their latency plus the launch
// gaps.  Here one cooperative launch runs the iterations of the same loop
// (S/CG.java:66-87) until the monitor stops the solve, with three changes of
// schedule and none of arithmetic:
//   - each CTA copies its product tiles (row offsets, columns, values) into
//     shared memory once, so an iteration reads the matrix from there;
//   - p = z + beta p is formed where the product gathers it (both operands
//     gathered, the same fused multiply-add), into the other of two p
//     buffers, so the p phase and its grid barrier go;
//   - the update loads all of a thread's rows before its first store.
// Two grid barriers per iteration remain: after the product (alpha needs
// every p.q partial) and after the update (beta and the monitor's test need
// every partial of r).  Every CTA then sums the partials itself, in group
// order with k_finalize's block tree (system_sum), and applies the scalar
// step to its own copy of the system's state, so every copy holds the same
// alpha, beta and status; CTA 0 alone writes the residual history, the
// running count and, at the end, the state.  The tiles, the groups, the
// per-thread row order and the block trees are the graph path's, so x, the
// history and the iteration count are the graph path's bit for bit.
//
// Vectors written in the launch are read with plain loads (the read-only
// path is for data fixed for a kernel's lifetime); the matrix and the
// inverse diagonal stay on it.  Barrier waits are bounded: a CTA that gives
// up sets the error flag and the abort word, and every CTA leaves at its
// next barrier.
#pragma once

#include "spmv.cuh"

// systems of at most this many product tiles take the one-launch CG (when
// their tiles also fit the shared memory of the co-resident CTAs).  Measured
// on GB300 (CG + Jacobi): 1.4-1.5x the graph path's speed up to ~100 tiles,
// 1.2x at ~300, even at ~600 and behind it beyond.
#ifndef MTJG_PERSIST_MAX_TILES
#define MTJG_PERSIST_MAX_TILES 512
#endif
// resident CTAs per SM the one-launch CG is compiled for (its register cap):
// 2 (107 registers, no spills) measured a little faster than 3 or 4 at every
// size
#ifndef MTJG_PERSIST_MINB
#define MTJG_PERSIST_MINB 2
#endif

namespace mtjg {

constexpr int kPersistMaxTiles = MTJG_PERSIST_MAX_TILES;
constexpr long long kGridSpinLimit = 1LL << 22;
// one cached product tile: values, columns, row offsets (16-byte multiples)
constexpr int kSlotValBytes = kTileNnz * 8;
constexpr int kSlotColBytes = ((kTileNnz * 4 + 15) / 16) * 16;
constexpr int kSlotRowBytes = (((kTileRows + 1) * 4 + 15) / 16) * 16;
constexpr int kSlotBytes = kSlotValBytes + kSlotColBytes + kSlotRowBytes;

struct GridBar {
    unsigned long long *count;  // arrivals in this launch (zeroed before it)
    int *abort;                 // set by a CTA whose wait gave up
};

// What the one-launch CG reads and writes (the solver's vectors and tiles).
struct PersistCg {
    CsrArgs A;
    TileArgs pt;  // product tiles (a tile is a group)
    TileArgs rt;  // row tiles (a tile is a group)
    const double *invdiag;
    double *x, *r, *z, *q;
    double *p[2];  // p of the even / odd iterations
    int pc;
    int slots;     // product tiles cached per CTA (tile bid + k G in slot k)
    RedCtx rcq;    // the product's partials (a buffer of their own)
    RedCtx rcu;    // the update's partials
    MonPtrs m;
    GridBar gb;
    int *err;
};

namespace {

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Arrive and wait until `target` arrivals (G per barrier of the launch).
// Every write of the CTA before it is seen by every CTA after it.  Returns
// false in every thread of the CTA when the wait gave up (about a second, or
// at once when another CTA has given up).
__device__ bool grid_barrier(const GridBar &gb, unsigned long long target, int *err)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(gb.count, 1ull);
        bool ok = false;
        unsigned ns = 0;
        for (long long i = 0; i < kGridSpinLimit; ++i) {
            if (ld_acquire_u64(gb.count) >= target) {
                ok = true;
                break;
            }
            if ((i & 63) == 63) {
                if (*(volatile int *)gb.abort) break;
                ns = ns < 256 ? ns + 32 : ns;
                __nanosleep(ns);
            }
        }
        if (!ok) {
            atomicExch(gb.abort, 1);
            atomicExch(err, 1);
        }
        __threadfence();
        s_ok = ok ? 1 : 0;
    }
    __syncthreads();
    return s_ok != 0;
}

// p_j of this iteration, formed as CgP forms it: z_j (first) or beta p_j + z_j
template <bool S>
__device__ __forceinline__ double p_of(const double *po, const double *z, int j, bool first, double beta)
{
    return first ? z[j] : fmac<S>(po[j], beta, z[j]);
}

// q = A p over cached tile slot k (tile t) with CgQ's epilogue, in k_spmv's
// order: one thread per row (STRICT, or a 1-lane tile), else VEC lanes per
// row with strided entries and a butterfly.  The row's own p_r is stored
// into pn (by the thread that hands the row to the epilogue).
template <bool S, int VEC>
__device__ __forceinline__ void pcg_tile(const PersistCg &c, const CgQ<S> &qop, const unsigned char *slot, int t,
                                         const double *po, double *pn, bool first, double beta, Acc &acc)
{
    const double *sv = reinterpret_cast<const double *>(slot);
    const int *sc = reinterpret_cast<const int *>(slot + kSlotValBytes);
    const int *sr = reinterpret_cast<const int *>(slot + kSlotValBytes + kSlotColBytes);
    const double *z = c.z;
    const int tid = threadIdx.x;
    const int r0 = c.pt.tile_row[t], r1 = c.pt.tile_row_end[t];
    if constexpr (VEC == 1) {
        for (int r = r0 + tid; r < r1; r += kBlock) {
            const int b = sr[r - r0], e = sr[r - r0 + 1];
            double sum = qop.init(r, 0);
#pragma unroll 8
            for (int k = b; k < e; ++k) sum = fmac<S>(sv[k], p_of<S>(po, z, sc[k], first, beta), sum);
            const double pr = p_of<S>(po, z, r, first, beta);
            pn[r] = pr;
            qop.row(r, 0, sum, pr, acc);
        }
    } else {
        const int gg = tid / VEC, l = tid % VEC;
        for (int base = r0; base < r1; base += kBlock / VEC) {
            const int r = base + gg;
            double sum = 0.0;
            if (r < r1 && l == 0) sum = qop.init(r, 0);
            if (r < r1) {
                const int b = sr[r - r0], e = sr[r - r0 + 1];
                for (int k = b + l; k < e; k += VEC) sum = fmac<S>(sv[k], p_of<S>(po, z, sc[k], first, beta), sum);
            }
#pragma unroll
            for (int off = VEC / 2; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off, VEC);
            if (r < r1 && l == 0) {
                const double pr = p_of<S>(po, z, r, first, beta);
                pn[r] = pr;
                qop.row(r, 0, sum, pr, acc);
            }
        }
    }
}

// Row tile t of the update (CgUpd::rows with plain loads): x += alpha p,
// r -= alpha q, z = M r, the |r| and r.z partials in row order.
template <bool S>
__device__ __forceinline__ void pcg_update(const PersistCg &c, const double *p, int t, double al, int nt, Acc &acc)
{
    constexpr int U = kRowsPerThread;
    const int r0 = c.rt.tile_row[t], r1 = c.rt.tile_row_end[t];
    const bool jac = c.pc == kPcJacobi;
    for (int base = r0 + (int)threadIdx.x; base < r1; base += kRowTile) {
        double rv[U], xv[U], pv[U], qv[U], dv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = base + u * kBlock;
            const bool in = i < r1;
            rv[u] = in ? c.r[i] : 0.0;
            xv[u] = in ? c.x[i] : 0.0;
            pv[u] = in ? p[i] : 0.0;
            qv[u] = in ? c.q[i] : 0.0;
            dv[u] = in && jac ? __ldg(c.invdiag + i) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = base + u * kBlock;
            if (i >= r1) break;
            double rr = rv[u];
            if (al != 0) {
                c.x[i] = fmac<S>(al, pv[u], xv[u]);
                rr = fmac<S>(-al, qv[u], rr);
                c.r[i] = rr;
            }
            norm_add<S>(acc, rr, nt);
            if (jac) {
                const double zz = rr * dv[u];
                c.z[i] = zz;
                acc.v[2] = fmac<S>(rr, zz, acc.v[2]);
            } else {
                acc.v[2] = fmac<S>(rr, rr, acc.v[2]);
            }
        }
    }
}

template <bool S>
__global__ void __launch_bounds__(kBlock, MTJG_PERSIST_MINB) k_cg_persist(PersistCg c, int normtype)
{
    extern __shared__ __align__(16) unsigned char slots[];
    __shared__ double red_sm[kParts * kBlock];
    __shared__ SysState s_st;
    __shared__ int s_run;  // the running count of CTAs other than 0 (unused)
    const int tid = threadIdx.x, G = (int)gridDim.x, bid = (int)blockIdx.x;
    if (tid == 0) {
        s_st = c.m.st[0];
        s_run = 1;
    }
    // this CTA's product tiles into their slots (entries and rows checked
    // against the slot: a tile that does not fit stops the solve)
    int bad = 0;
    for (int k = 0; k < c.slots; ++k) {
        const int t = bid + k * G;
        if (t >= c.pt.num_tiles) break;
        unsigned char *slot = slots + (size_t)k * kSlotBytes;
        const int r0 = c.pt.tile_row[t], r1 = c.pt.tile_row_end[t];
        const int nz0 = __ldg(c.A.rowptr + r0), nz1 = __ldg(c.A.rowptr + r1);
        if (r1 - r0 > kTileRows || nz1 - nz0 > kTileNnz) {
            bad = 1;
            continue;
        }
        double *sv = reinterpret_cast<double *>(slot);
        int *sc = reinterpret_cast<int *>(slot + kSlotValBytes);
        int *sr = reinterpret_cast<int *>(slot + kSlotValBytes + kSlotColBytes);
        for (int i = tid; i <= r1 - r0; i += kBlock) sr[i] = __ldg(c.A.rowptr + r0 + i) - nz0;
        for (int e = tid; e < nz1 - nz0; e += kBlock) {
            sv[e] = __ldg(c.A.val + nz0 + e);
            sc[e] = __ldg(c.A.colind + nz0 + e);
        }
    }
    if (__syncthreads_or(bad)) {
        if (tid == 0) {
            atomicExch(c.err, 1);
            atomicExch(c.gb.abort, 1);  // the other CTAs leave at their first barrier
        }
        return;
    }
    CgQ<S> qop{nullptr, c.q, &s_st};
    MonPtrs m = c.m;
    m.st = &s_st;
    if (bid != 0) {
        m.mon.hist_cap = 0;
        m.num_running = &s_run;
    }
    CgUpd<S> uop{c.x, c.r, c.z, nullptr, c.q, c.invdiag, c.pc, m};
    const int nt = normtype;
    unsigned long long target = 0;
    int par = 0;  // p[par] holds the previous iteration's p
    while (s_st.status == ST_RUNNING) {
        const double *po = c.p[par];
        double *pn = c.p[par ^ 1];
        // p = z (first) or beta p + z, formed in the gathers; q = A p and the
        // p.q partials, one tile (group) at a time
        {
            const bool first = s_st.iter == 0;
            const double beta = s_st.beta;
            for (int k = 0; k < c.slots; ++k) {
                const int t = bid + k * G;
                if (t >= c.pt.num_tiles) break;
                const unsigned char *slot = slots + (size_t)k * kSlotBytes;
                Acc acc;
                acc_zero(acc);
                const int vec = S ? 1 : (c.pt.group_info[t] & 0xff);
                if (vec == 1)
                    pcg_tile<S, 1>(c, qop, slot, t, po, pn, first, beta, acc);
                else if (vec == 4)
                    pcg_tile<S, 4>(c, qop, slot, t, po, pn, first, beta, acc);
                else
                    pcg_tile<S, 32>(c, qop, slot, t, po, pn, first, beta, acc);
                group_partial<OpSlots<CgQ<S>>::value>(acc, t, c.rcq, nt, red_sm);
            }
        }
        target += (unsigned long long)G;
        if (!grid_barrier(c.gb, target, c.err)) break;
        {
            const Acc s = system_sum<OpSlots<CgQ<S>>::value>(c.rcq, 0, nt, red_sm);
            if (tid == 0) qop.scalar(0, s);
            __syncthreads();
        }
        // x += alpha p, r -= alpha q, z = M r with the |r| and r.z partials
        {
            const double al = s_st.alpha;
            for (int t = bid; t < c.rt.num_tiles; t += G) {
                Acc acc;
                acc_zero(acc);
                pcg_update<S>(c, pn, t, al, nt, acc);
                group_partial<OpSlots<CgUpd<S>>::value>(acc, t, c.rcu, nt, red_sm);
            }
        }
        target += (unsigned long long)G;
        if (!grid_barrier(c.gb, target, c.err)) break;
        {
            const Acc s = system_sum<OpSlots<CgUpd<S>>::value>(c.rcu, 0, nt, red_sm);
            if (tid == 0) uop.scalar(0, s);
            __syncthreads();
        }
        par ^= 1;
    }
    if (bid == 0 && tid == 0) c.m.st[0] = s_st;
}

}  // namespace
}  // namespace mtjg
