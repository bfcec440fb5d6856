// spmv.cuh -- tiled CSR product and tiled row kernels.
//
// k_spmv: persistent CTAs walk reduction groups of product tiles (up to
// kGroupTiles consecutive tiles of one system; CTA b takes groups b, b+G,
// ...).  The row pointers, values and column indices of the next tile are
// brought into shared memory by one thread with three cp.async.bulk copies
// completing on an mbarrier, while the block computes the current tile
// (kSpmvStages stages; two measured best: occupancy hides the x gathers
// better than a deeper pipeline).  Each row is summed from shared memory in ascending entry order
// (vec == 1: one thread per row, the order of CompRowMatrix.mult,
// S/CompRowMatrix.java:304-312) or by a group of `vec` lanes with a fixed
// butterfly (vec > 1).  x is gathered through the read-only path (L1/L2).
// The epilogue object gives the starting value of a row sum (init) and
// decides what a finished row sum becomes (y = Ax, y += alpha*Ax,
// r = b - Ax, fused dot products, ...).
//
// k_rows: one block per row tile (passes of kRowTile rows, kRowsPerThread
// rows per thread and pass, strided for coalescing).
//
// A phase with a reduction accumulates per thread over a whole group, then
// stores one block-reduced partial per group; k_finalize (dev.cuh) reduces
// each system's partials in group order and runs the scalar step.
#pragma once

#include "dev.cuh"

namespace mtjg {

// Shared-memory stage of one tile, per value type.  FP32 tiles may hold 1.5x
// the entries and 2x the rows of FP64 tiles in about the same bytes (tiles
// planned for FP64 always fit an FP32 stage).
// FP32 tiles: 2560 entries hold 512 five-entry rows, two per thread, and
// served the mixed stream 6.0 % faster (4 CTAs per SM) than 1728 entries
// (345 such rows: a third of the threads with two, the rest with one; 5 CTAs)
#ifndef MTJG_TILE_NNZ32
#define MTJG_TILE_NNZ32 2560
#endif
#ifndef MTJG_TILE_ROWS32
#define MTJG_TILE_ROWS32 (2 * MTJG_TILE_ROWS)
#endif
constexpr int kTileNnz32 = MTJG_TILE_NNZ32;
constexpr int kTileRows32 = MTJG_TILE_ROWS32;
static_assert(kTileNnz32 >= kTileNnz && kTileRows32 >= kTileRows, "FP64 tiles must fit an FP32 stage");
constexpr int round16(int b) { return ((b + 15) / 16) * 16; }
template <class T>
struct Stage {
    static constexpr int kNnz = sizeof(T) == 8 ? kTileNnz : kTileNnz32;
    static constexpr int kRows = sizeof(T) == 8 ? kTileRows : kTileRows32;
    // a tile's copies start and end on 16 bytes: up to 2 (16/sizeof(T) - 1) extra values
    static constexpr int kValBytes = round16((kNnz + 2 * (16 / (int)sizeof(T) - 1)) * (int)sizeof(T));
    static constexpr int kColBytes = round16((kNnz + 8) * 4);       // 16-byte rounding at both ends
    static constexpr int kRowBytes = round16((kRows + 1 + 8) * 4);  // row pointers
    static constexpr int kBytes = kValBytes + kColBytes + kRowBytes;
};
#ifndef MTJG_SPMV_STAGES
#define MTJG_SPMV_STAGES 2
#endif
#ifndef MTJG_SPMV_CTAS
#define MTJG_SPMV_CTAS 6
#endif
#ifndef MTJG_SPMV_CTAS_REDUCE
#define MTJG_SPMV_CTAS_REDUCE 5
#endif
constexpr int kSpmvStages = MTJG_SPMV_STAGES;  // tiles in shared memory per CTA (NST - 1 in flight ahead)
// How a one-thread-per-row tile gets x_r for an epilogue that needs it:
// caught from the row's own diagonal gather, or one load per row, which
// saves a compare and a select per entry (the value is the same).  Measured
// on GB300: the load made the served FP32 mix 1.5 % faster and the FP64 CG
// 1 % slower, so FP32 tiles load and FP64 tiles catch (MTJG_SPMV_XR_LOAD=1
// makes every tile load).
#ifndef MTJG_SPMV_XR_LOAD
#define MTJG_SPMV_XR_LOAD 0
#endif
template <class T>
constexpr bool xr_load() { return MTJG_SPMV_XR_LOAD != 0 || sizeof(T) == 4; }
template <class T>
constexpr int spmv_smem() { return kSpmvStages * Stage<T>::kBytes; }
// resident CTAs per SM the register budget is set for: products without a
// reduction, and products whose epilogue reduces (they hold more state)
constexpr int kSpmvCtasPerSm = MTJG_SPMV_CTAS;
constexpr int kSpmvCtasReduce = MTJG_SPMV_CTAS_REDUCE;
constexpr long long kWaitLimit = 1LL << 22;
// row pointer arrays handed to k_spmv carry this many padding entries
constexpr int kRowptrPad = 4;

// One system of a served batch: its own resident CSR (rows numbered from 0)
// and the offset of its rows in the pooled vectors.
struct SysDesc {
    const int *rowptr;
    const int *colind;
    const double *val;
    const float *val32;
    int voff;
    int pad;
};

struct TileArgs {
    int num_tiles;
    int num_groups;
    const int *tile_row;      // tile t covers rows [tile_row[t], tile_row_end[t])
    const int *tile_row_end;
    const int *tile_nz;       // and entries [tile_nz[t], tile_nz_end[t])
    const int *tile_nz_end;
    const int *tile_sys;
    const unsigned char *tile_flags;
    const int *group_tile;
    const int *group_info;  // per group: (system << 8) | lanes per row of its tiles
    const SysDesc *sd;  // nullptr: one CSR (the kernel's argument), rows = vector indices
    const double *long_sum;  // FAST: the sums of the long rows, by tile (k_long_sum), else nullptr
};

template <class T>
struct CsrArgsT {
    const int *rowptr;
    const int *colind;
    const T *val;
};
using CsrArgs = CsrArgsT<double>;

__device__ __forceinline__ int tile_system(const TileArgs &ta, int t)
{
    return ta.tile_sys ? ta.tile_sys[t] : 0;
}

// A staged tile as its copies and its rows need it: the CSR it reads (its
// system's own, for a served batch), its rows and entries, and where its
// rows sit in the vectors.
template <class T>
struct TileDesc {
    const T *val;
    const int *colind;
    const int *rowptr;
    int r0, r1;    // rows [r0, r1) of the matrix
    int nz0, nz1;  // entries [nz0, nz1)
    int voff;      // vector index of row 0
    int sys;
    int staged;
};

// Resident CTAs per SM a product kernel is compiled and launched for:
// Epi::kCtas when the epilogue declares it (it fits that many CTAs' registers
// without spilling), else kSpmvCtasPerSm, or kSpmvCtasReduce when it reduces.
template <class Epi, class = void>
struct EpiCtas {
    static constexpr int value = Epi::kReduce ? kSpmvCtasReduce : kSpmvCtasPerSm;
};
template <class Epi>
struct EpiCtas<Epi, decltype((void)Epi::kCtas)> {
    static constexpr int value = Epi::kCtas;
};

// Kernels and launchers are private to each translation unit (see k_finalize).
namespace {

template <int VEC, bool S, class T, class Epi>
__global__ void __launch_bounds__(kBlock, EpiCtas<Epi>::value)
    k_spmv(CsrArgsT<T> A, TileArgs ta, const T *__restrict__ x, Epi epi, RedCtx rc, int normtype, int *err)
{
    constexpr int kVA = 16 / (int)sizeof(T);  // values per 16 bytes
    constexpr int NST = kSpmvStages;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t bar[NST];
    // block reductions use only the epilogue's slots (and so fit more CTAs)
    constexpr int kRedRows = Epi::kReduce ? red_rows<OpSlots<Epi>::value>() : 0;
    __shared__ double red_sm[(kRedRows > 0 ? kRedRows : 1) * kBlock];
    __shared__ T s_long[kBlock / 32];
    __shared__ unsigned s_done[NST];    // warps done with the tile in stage i
    __shared__ unsigned s_issued[NST];  // copies issued into stage i
    __shared__ int s_abort;
    // s_hdr[i]: the tile whose copies were issued into stage i, written
    // before the copies (the mbarrier's completion publishes it with them);
    // s_next: the next tile to issue, prepared one issue ahead so that the
    // dependent table loads behind it (tile -> system -> its CSR) stay off
    // the path from a freed stage to its next copy
    __shared__ TileDesc<T> s_hdr[NST];
    __shared__ TileDesc<T> s_next;

    const int tid = threadIdx.x, lane = tid & 31;
    const int G = gridDim.x, NG = ta.num_groups;
    if (tid == 0) {
#pragma unroll
        for (int i = 0; i < NST; ++i) mbar_init(&bar[i], 1);
        mbar_fence_init();
    }
    __syncthreads();

    using St = Stage<T>;
    auto sval = [&](int s) { return reinterpret_cast<T *>(smem + s * St::kBytes); };
    auto scol = [&](int s) { return reinterpret_cast<int *>(smem + s * St::kBytes + St::kValBytes); };
    auto srow = [&](int s) {
        return reinterpret_cast<int *>(smem + s * St::kBytes + St::kValBytes + St::kColBytes);
    };
    // a launch takes the groups of its lanes-per-row class (STRICT: all)
    // whose system is active; one load per group, and a system's activity
    // (fixed for the launch) is read once per run of its groups
    int last_sys = -1;
    bool last_active = false;
    auto group_active = [&](int g) {
        const int info = ta.group_info[g];
        if (!S && (info & 0xff) != VEC) return false;
        const int sys = info >> 8;
        if (sys != last_sys) {
            last_sys = sys;
            last_active = epi.active(sys);
        }
        return last_active;
    };
    auto next_group = [&](int g) {
        while (g < NG && !group_active(g)) g += G;
        return g;
    };
    auto staged = [&](int t) { return !(ta.tile_flags[t] & 1); };
    // the CSR a tile reads and the vector offset of its rows
    struct MatView {
        const int *rowptr;
        const int *colind;
        const T *val;
        int voff;
    };
    auto view = [&](int t) -> MatView {
        if (ta.sd) {
            const SysDesc &d = ta.sd[tile_system(ta, t)];
            if constexpr (sizeof(T) == 8)
                return MatView{d.rowptr, d.colind, reinterpret_cast<const T *>(d.val), d.voff};
            else
                return MatView{d.rowptr, d.colind, reinterpret_cast<const T *>(d.val32), d.voff};
        }
        return MatView{A.rowptr, A.colind, A.val, 0};
    };
    // tile t from the global tables
    auto prepare = [&](int t) {
        const MatView m = view(t);
        TileDesc<T> d;
        d.val = m.val;
        d.colind = m.colind;
        d.rowptr = m.rowptr;
        d.r0 = ta.tile_row[t];
        d.r1 = ta.tile_row_end[t];
        d.nz0 = ta.tile_nz[t];
        d.nz1 = ta.tile_nz_end[t];
        d.voff = m.voff;
        d.sys = tile_system(ta, t);
        d.staged = staged(t) ? 1 : 0;
        return d;
    };
    // the staged tile d's row pointers, values and columns into stage s,
    // rounded out to 16 bytes (the arrays carry the padding this reads past
    // their ends), after its header
    auto issue = [&](const TileDesc<T> &d, int s) {
        s_hdr[s] = d;
        const int v0 = d.nz0 & ~(kVA - 1), v1 = (d.nz1 + kVA - 1) & ~(kVA - 1);
        const int c0 = d.nz0 & ~3, c1 = (d.nz1 + 3) & ~3;
        const int p0 = d.r0 & ~3, p1 = (d.r1 + 1 + 3) & ~3;
        const unsigned vb = (unsigned)(v1 - v0) * (unsigned)sizeof(T), cb = (unsigned)(c1 - c0) * 4u,
                       pb = (unsigned)(p1 - p0) * 4u;
        fence_proxy_async();
        mbar_arrive_expect_tx(&bar[s], vb + cb + pb);
        if (vb) bulk_g2s(sval(s), d.val + v0, vb, &bar[s]);
        if (cb) bulk_g2s(scol(s), d.colind + c0, cb, &bar[s]);
        bulk_g2s(srow(s), d.rowptr + p0, pb, &bar[s]);
    };

    // The k-th tile of the block's walk lives in stage k % NST.  The first
    // NST tiles are issued up front; after that the last warp to finish the
    // tile in stage s issues the tile NST further on into s (from s_next),
    // so warps never wait for each other between tiles (only at group ends,
    // for the block reduction).  The walk and staged() read global tables
    // and are uniform over the block; a staged tile's rows come from its
    // stage header.
    //
    // s_next is handed from issuer to issuer: the issuer of the tile for
    // stage s writes it before its release of the stage after s, and the
    // next issuer is the last warp to release that stage, so it sees it.
    constexpr int NW = kBlock / 32;
    auto advance = [&](int &gg, int &tt) {
        ++tt;
        if (tt >= ta.group_tile[gg + 1]) {
            gg = next_group(gg + G);
            tt = gg < NG ? ta.group_tile[gg] : 0;
        }
    };
    if (tid == 0) {
#pragma unroll
        for (int i = 0; i < NST; ++i) s_done[i] = s_issued[i] = 0u;
        s_abort = 0;
    }
    // (g, t): the current group and tile; (pg, pt): the next tile to issue
    int g = next_group(blockIdx.x);
    int t = g < NG ? ta.group_tile[g] : 0;
    int pg = g, pt = t;
    __syncthreads();
    for (int k = 0; k < NST && pg < NG; ++k) {
        if (tid == 0 && staged(pt)) {
            s_issued[k] += 1u;
            issue(prepare(pt), k);
        }
        advance(pg, pt);
    }
    if (tid == 0 && pg < NG) s_next = prepare(pt);
    // bit i: parity of the copies of stage i this thread has waited for (and
    // so of stage i's next completion).  A copy into a stage is issued only
    // after every warp is done with the stage's previous tile, so a thread is
    // at most one copy behind s_issued[i]; the parities tell which.
    unsigned phase = 0u;
    bool skip = false;  // a copy never completed: walk on without work, drain, stop
    int s = 0;
    __syncthreads();
    Acc acc;
    acc_zero(acc);
    while (g < NG) {
        // the tile after t in this block's walk
        int gn = g, tn = t;
        advance(gn, tn);
        const bool st = staged(t);
        if (!skip && st) {
            bool ok = false;
            for (long long i = 0; i < kWaitLimit; ++i) {
                if (mbar_try_wait(&bar[s], (phase >> s) & 1u)) {
                    ok = true;
                    break;
                }
                if ((i & 1023) == 1023 && *(volatile int *)&s_abort) break;
            }
            if (ok) phase ^= 1u << s;
            // the warp skips together (the lane shuffles below need all lanes)
            if (!__all_sync(0xffffffffu, ok)) {
                *(volatile int *)&s_abort = 1;
                if (lane == 0) atomicExch(err, 1);
                skip = true;
            }
        }
        if (!skip && st) {
            // rows r are the matrix's own; vectors are indexed at vgo + r
            const TileDesc<T> &h = s_hdr[s];
            const int r0 = h.r0, r1 = h.r1, sys = h.sys, vgo = h.voff, nzb = h.nz0;
            const T *xs = x + vgo;
            const T *sv = sval(s);
            const int *sc = scol(s);
            const int *sr = srow(s);
            const int vo = nzb & ~(kVA - 1), co = nzb & ~3, po = r0 & ~3;
            if constexpr (VEC == 1 && Stage<T>::kRows > kBlock) {
                // a tile may hold up to 2 kBlock rows: a thread's two rows
                // gather together (one latency round, not two); each row's
                // sum keeps its order and the rows finish in row order
                static_assert(Stage<T>::kRows <= 2 * kBlock, "at most two rows per thread");
                const int ra = r0 + tid, rb = ra + kBlock;
                if (ra < r1) {
                    const bool hb = rb < r1;
                    const int ba = sr[ra - po], la = sr[ra + 1 - po] - ba;
                    const int bb = hb ? sr[rb - po] : 0, lb = hb ? sr[rb + 1 - po] - bb : 0;
                    T suma = epi.init(vgo + ra, sys), sumb = hb ? epi.init(vgo + rb, sys) : T(0);
                    T xra = T(0), xrb = T(0);
                    bool da = false, db = false;
                    const int lm = la > lb ? la : lb;
#pragma unroll 4
                    for (int k = 0; k < lm; ++k) {
                        if (k < la) {
                            const int c = sc[ba + k - co];
                            const T xv = __ldg(xs + c);
                            if (!xr_load<T>() && c == ra) {
                                xra = xv;
                                da = true;
                            }
                            suma = fmac<S>(sv[ba + k - vo], xv, suma);
                        }
                        if (k < lb) {
                            const int c = sc[bb + k - co];
                            const T xv = __ldg(xs + c);
                            if (!xr_load<T>() && c == rb) {
                                xrb = xv;
                                db = true;
                            }
                            sumb = fmac<S>(sv[bb + k - vo], xv, sumb);
                        }
                    }
                    if constexpr (Epi::kNeedsXr) {
                        if (!da) xra = __ldg(xs + ra);
                        if (hb && !db) xrb = __ldg(xs + rb);
                    }
                    epi.row(vgo + ra, sys, suma, xra, acc);
                    if (hb) epi.row(vgo + rb, sys, sumb, xrb, acc);
                }
            } else if constexpr (VEC == 1) {
                for (int r = r0 + tid; r < r1; r += kBlock) {
                    const int b = sr[r - po], e = sr[r + 1 - po];
                    T sum = epi.init(vgo + r, sys);
                    T xr = T(0);
                    bool diag = false;
#pragma unroll 8
                    for (int k = b; k < e; ++k) {
                        const int c = sc[k - co];
                        const T xv = __ldg(xs + c);
                        if (!xr_load<T>() && c == r) {
                            xr = xv;
                            diag = true;
                        }
                        sum = fmac<S>(sv[k - vo], xv, sum);
                    }
                    if constexpr (Epi::kNeedsXr) {
                        if (!diag) xr = __ldg(xs + r);
                    }
                    epi.row(vgo + r, sys, sum, xr, acc);
                }
            } else if constexpr (Stage<T>::kRows > kBlock) {
                // up to two passes of kBlock / VEC rows: a lane group's two
                // rows gather together; each keeps its entry order and its
                // butterfly, and the rows finish in row order
                const int gg = tid / VEC, l = tid % VEC;
                const int ra = r0 + gg, rb = ra + kBlock / VEC;
                const bool ha = ra < r1, hb = rb < r1;
                T suma = T(0), sumb = T(0);
                if (ha && l == 0) suma = epi.init(vgo + ra, sys);
                if (hb && l == 0) sumb = epi.init(vgo + rb, sys);
                const int ba = ha ? sr[ra - po] : 0, la = ha ? sr[ra + 1 - po] - ba : 0;
                const int bb = hb ? sr[rb - po] : 0, lb = hb ? sr[rb + 1 - po] - bb : 0;
                const int lm = la > lb ? la : lb;
                for (int k = l; k < lm; k += VEC) {
                    if (k < la) suma = fmac<S>(sv[ba + k - vo], __ldg(xs + sc[ba + k - co]), suma);
                    if (k < lb) sumb = fmac<S>(sv[bb + k - vo], __ldg(xs + sc[bb + k - co]), sumb);
                }
#pragma unroll
                for (int off = VEC / 2; off > 0; off >>= 1) {
                    suma += __shfl_xor_sync(0xffffffffu, suma, off, VEC);
                    sumb += __shfl_xor_sync(0xffffffffu, sumb, off, VEC);
                }
                if (ha && l == 0) epi.row(vgo + ra, sys, suma, Epi::kNeedsXr ? __ldg(xs + ra) : T(0), acc);
                if (hb && l == 0) epi.row(vgo + rb, sys, sumb, Epi::kNeedsXr ? __ldg(xs + rb) : T(0), acc);
            } else {
                const int gg = tid / VEC, l = tid % VEC;
                for (int base = r0; base < r1; base += kBlock / VEC) {
                    const int r = base + gg;
                    T sum = T(0);
                    if (r < r1 && l == 0) sum = epi.init(vgo + r, sys);
                    if (r < r1) {
                        const int b = sr[r - po], e = sr[r + 1 - po];
                        for (int k = b + l; k < e; k += VEC) sum = fmac<S>(sv[k - vo], __ldg(xs + sc[k - co]), sum);
                    }
#pragma unroll
                    for (int off = VEC / 2; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off, VEC);
                    if (r < r1 && l == 0) epi.row(vgo + r, sys, sum, Epi::kNeedsXr ? __ldg(xs + r) : T(0), acc);
                }
            }
        } else if (!st && ta.long_sum) {
            // a single row longer than a stage, summed ahead by k_long_seg / k_long_sum
            const int sys = tile_system(ta, t);
            const int r = ta.tile_row[t];
            const MatView mv = view(t);
            if (tid == 0)
                epi.row(mv.voff + r, sys, epi.init(mv.voff + r, sys) + (T)ta.long_sum[t],
                        Epi::kNeedsXr ? __ldg(x + mv.voff + r) : T(0), acc);
        } else if (!st) {
            // a single row longer than a stage: straight from global memory
            const int sys = tile_system(ta, t);
            const int r = ta.tile_row[t];
            const MatView mv = view(t);
            const T *xs = x + mv.voff;
            const int vgo = mv.voff;
            const int b = mv.rowptr[r], e = mv.rowptr[r + 1];
            T sum = tid == 0 ? epi.init(vgo + r, sys) : T(0);
            if constexpr (S) {
                // Java's order: products rounded, then added one by one in
                // entry order.  Warp 0's lanes form 32 rounded products at a
                // time (the next 32 loading while lane 0 adds these), so the
                // row is bound by the add chain, not by a load per entry.
                if (tid < 32) {
                    T nxt = b + tid < e ? mul_rn(mv.val[b + tid], __ldg(xs + mv.colind[b + tid])) : T(0);
                    for (int k0 = b; k0 < e; k0 += 32) {
                        const T cur = nxt;
                        const int kn = k0 + 32 + tid;
                        nxt = kn < e ? mul_rn(mv.val[kn], __ldg(xs + mv.colind[kn])) : T(0);
                        const int cnt = e - k0 < 32 ? e - k0 : 32;
                        if (cnt == 32) {  // unrolled: the shuffles run ahead of the add chain
#pragma unroll
                            for (int u = 0; u < 32; ++u) {
                                const T pu = __shfl_sync(0xffffffffu, cur, u);
                                if (tid == 0) sum = add_rn(sum, pu);
                            }
                        } else {
                            for (int u = 0; u < cnt; ++u) {
                                const T pu = __shfl_sync(0xffffffffu, cur, u);
                                if (tid == 0) sum = add_rn(sum, pu);
                            }
                        }
                    }
                }
            } else {
                for (int k = b + tid; k < e; k += kBlock) sum = fmac<S>(mv.val[k], __ldg(xs + mv.colind[k]), sum);
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
                if ((tid & 31) == 0) s_long[tid >> 5] = sum;
                __syncthreads();
                if (tid == 0) {
                    sum = s_long[0];
                    for (int w = 1; w < kBlock / 32; ++w) sum += s_long[w];
                }
                __syncthreads();
            }
            if (tid == 0) epi.row(vgo + r, sys, sum, Epi::kNeedsXr ? __ldg(xs + r) : T(0), acc);
        }
        // release stage s: the last warp done with it issues the tile NST on
        __syncwarp();
        if (lane == 0) {
            __threadfence_block();
            const unsigned c = atomicAdd(&s_done[s], 1u);
            if (c == NW - 1) {
                s_done[s] = 0u;
                __threadfence_block();
                if (pg < NG && !*(volatile int *)&s_abort) {
                    if (s_next.staged) {
                        s_issued[s] += 1u;
                        issue(s_next, s);
                    }
                    int qg = pg, qt = pt;
                    advance(qg, qt);
                    if (qg < NG) s_next = prepare(qt);
                }
            }
        }
        if (pg < NG) advance(pg, pt);
        if (gn != g) {
            // the group is complete
            if constexpr (Epi::kReduce) {
                group_partial<OpSlots<Epi>::value>(acc, g, rc, normtype, red_sm);
                acc_zero(acc);
            }
        }
        s = s + 1 == NST ? 0 : s + 1;
        g = gn;
        t = tn;
    }
    __syncthreads();  // every thread has left the walk: s_abort and s_issued are final
    if (*(volatile int *)&s_abort) {
        // wait (bounded) for every copy this thread has not waited for, so
        // none lands in shared memory after the block has left (no copy is
        // issued once s_abort is set)
#pragma unroll
        for (int i = 0; i < NST; ++i)
            if ((s_issued[i] & 1u) != ((phase >> i) & 1u)) mbar_wait_bounded(&bar[i], (phase >> i) & 1u, kWaitLimit);
    }
}

// An Op with kBatched = true also has rows(base, end, sys, acc): the rows
// base, base + kBlock, ... (kRowsPerThread of them, those below end) with
// every load of every row issued before the first store, so a thread keeps
// all its rows' reads in flight at once (the compiler cannot hoist a later
// row's loads above an earlier row's stores to other arrays by itself).
// The arithmetic and the accumulation order are those of row() in row order.
template <class Op, class = void>
struct OpBatched {
    static constexpr bool value = false;
};
template <class Op>
struct OpBatched<Op, decltype((void)Op::kBatched)> {
    static constexpr bool value = Op::kBatched;
};
// Resident blocks per SM a row phase asks the register allocator for
// (Op::kMinBlocks; 0: no bound).
template <class Op, class = void>
struct OpMinBlocks {
    static constexpr int value = 0;
};
template <class Op>
struct OpMinBlocks<Op, decltype((void)Op::kMinBlocks)> {
    static constexpr int value = Op::kMinBlocks;
};

// Row kernel: block b handles row tile b, kRowsPerThread rows per thread
// (rows tid, tid + kBlock, ...), one partial per tile.
template <class Op>
__global__ void __launch_bounds__(kBlock, OpMinBlocks<Op>::value) k_rows(TileArgs ta, Op op, RedCtx rc, int normtype)
{
    __shared__ double red_sm[kParts * kBlock];
    const int t = blockIdx.x;
    const int sys = tile_system(ta, t);
    if (!op.active(sys)) return;
    Acc acc;
    acc_zero(acc);
    const int r0 = ta.tile_row[t], r1 = ta.tile_row_end[t];
    if constexpr (OpBatched<Op>::value) {
        for (int base = r0 + (int)threadIdx.x; base < r1; base += kRowTile) op.rows(base, r1, sys, acc);
    } else {
#pragma unroll 2
        for (int r = r0 + (int)threadIdx.x; r < r1; r += kBlock) op.row(r, sys, acc);
    }
    if constexpr (Op::kReduce) group_partial<OpSlots<Op>::value>(acc, t, rc, normtype, red_sm);
}

inline TileArgs tile_args(const TileSet &ts, bool long_sums = false)
{
    // contiguous tilings end each tile where the next one starts
    return TileArgs{ts.num_tiles,
                    ts.num_groups,
                    ts.tile_row,
                    ts.tile_row_end ? ts.tile_row_end : ts.tile_row + 1,
                    ts.tile_nz,
                    ts.tile_nz_end ? ts.tile_nz_end : (ts.tile_nz ? ts.tile_nz + 1 : nullptr),
                    ts.tile_sys,
                    ts.tile_flags,
                    ts.group_tile,
                    ts.group_info,
                    ts.sd,
                    long_sums ? ts.long_sum : nullptr};
}

// Long rows, FAST: block s sums segment s (thread-strided, then a fixed
// shuffle tree and the warps in order); then each long row's segments are
// added in segment order.  Fixed segments and orders: the sums depend on
// the matrix alone, not on the grid.
template <class T>
__global__ void __launch_bounds__(kBlock) k_long_seg(CsrArgsT<T> A, const int *seg_begin, const int *seg_end,
                                                     const T *__restrict__ x, double *part)
{
    __shared__ T s_w[kBlock / 32];
    const int sg = blockIdx.x, b = seg_begin[sg], e = seg_end[sg];
    T sum = T(0);
    for (int k = b + (int)threadIdx.x; k < e; k += kBlock) sum = fmac<false>(A.val[k], __ldg(x + A.colind[k]), sum);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, off);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        T s = s_w[0];
        for (int w = 1; w < kBlock / 32; ++w) s += s_w[w];
        part[sg] = (double)s;
    }
}

__global__ void k_long_sum(int num_long, const int *long_first, const int *long_tile, const double *part,
                           double *long_sum)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= num_long) return;
    double s = 0.0;
    for (int q = long_first[j]; q < long_first[j + 1]; ++q) s += part[q];
    long_sum[long_tile[j]] = s;
}

template <class T>
cudaError_t launch_long_rows(mtjg_ctx *ctx, CsrArgsT<T> A, const TileSet &ts, const T *x)
{
    k_long_seg<T><<<ts.num_segs, kBlock, 0, ctx->stream>>>(A, ts.seg_begin, ts.seg_end, x, ts.seg_part);
    k_long_sum<<<(ts.num_long + kBlock - 1) / kBlock, kBlock, 0, ctx->stream>>>(ts.num_long, ts.long_first,
                                                                               ts.long_tile, ts.seg_part,
                                                                               ts.long_sum);
    ctx->launches += 2;
    return cudaGetLastError();
}

template <class Op>
cudaError_t launch_finalize(mtjg_ctx *ctx, const TileSet &ts, const Op &op, const RedCtx &rc, int normtype)
{
    ctx->launches++;
    if constexpr (OpMon<Op>::value) {
        if (op.m.mon.xmon) {  // MatrixIterationMonitor: |x| first
            k_finalize<Op, true><<<ts.num_sys, kBlock, 0, ctx->stream>>>(op, rc, normtype);
            return cudaGetLastError();
        }
    }
    k_finalize<Op><<<ts.num_sys, kBlock, 0, ctx->stream>>>(op, rc, normtype);
    return cudaGetLastError();
}

template <int VEC, bool S, class T, class Epi>
cudaError_t launch_spmv_t(mtjg_ctx *ctx, CsrArgsT<T> A, const TileSet &ts, const T *x, const Epi &epi,
                          const RedCtx &rc, int normtype)
{
    auto k = k_spmv<VEC, S, T, Epi>;
    // the shared-memory opt-in is a per-device attribute of this kernel
    static std::atomic<unsigned long long> attr_set{0};
    const unsigned long long bit = 1ull << (ctx->device & 63);
    if (!(attr_set.load() & bit)) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, spmv_smem<T>());
        if (e != cudaSuccess) return e;
        attr_set.fetch_or(bit);
    }
    // the epilogue's CTAs per SM, at most as many as fit (a persistent walk:
    // a CTA that would wait for a slot only lengthens the tail)
    static std::atomic<int> fit{0};
    int per_sm = fit.load();
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBlock, spmv_smem<T>()) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        fit.store(per_sm);
    }
    const int cap = ctx->num_sms * (EpiCtas<Epi>::value < per_sm ? EpiCtas<Epi>::value : per_sm);
    const int grid = ts.num_groups < cap ? ts.num_groups : cap;
    k<<<grid, kBlock, spmv_smem<T>(), ctx->stream>>>(A, tile_args(ts, !S && ts.num_long > 0 && !ts.sd), x, epi, rc, normtype,
                                                     ctx->d_flag);
    ctx->launches++;
    return cudaGetLastError();
}

// Chooses the lanes-per-row variant of the tiles and the rounding mode of
// the context.  STRICT always sums one row per thread in entry order.
template <class T, class Epi>
cudaError_t launch_spmv(mtjg_ctx *ctx, CsrArgsT<T> A, const TileSet &ts, const T *x, const Epi &epi,
                        const RedCtx &rc, int normtype)
{
    if (ts.num_tiles == 0) return cudaSuccess;
    RedCtx r = rc;
    r.sys_group = ts.sys_group;  // partial slots are this tiling's groups
    cudaError_t e = cudaSuccess;
    // FAST: rows longer than a stage are summed ahead, over many CTAs (a
    // single CSR; served batches keep one CTA per long row)
    if (ctx->numerics != MTJG_NUMERICS_STRICT && ts.num_long > 0 && !ts.sd) e = launch_long_rows<T>(ctx, A, ts, x);
    if (e != cudaSuccess) return e;
    if (ctx->numerics == MTJG_NUMERICS_STRICT) {
        e = launch_spmv_t<1, true, T>(ctx, A, ts, x, epi, r, normtype);
    } else {
        // one launch per lanes-per-row class present (a batch may mix
        // classes; every system's tiles belong to one class)
        if (ts.vec_mask & 1) e = launch_spmv_t<1, false, T>(ctx, A, ts, x, epi, r, normtype);
        if (e == cudaSuccess && (ts.vec_mask & 4)) e = launch_spmv_t<4, false, T>(ctx, A, ts, x, epi, r, normtype);
        if (e == cudaSuccess && (ts.vec_mask & 32))
            e = launch_spmv_t<32, false, T>(ctx, A, ts, x, epi, r, normtype);
    }
    if (e == cudaSuccess && Epi::kReduce) e = launch_finalize(ctx, ts, epi, r, normtype);
    return e;
}

// Row kernels run on the row tiles (one block per tile, a tile is a group).
template <class Op>
cudaError_t launch_rows(mtjg_ctx *ctx, const TileSet &ts, const Op &op, const RedCtx &rc, int normtype)
{
    if (ts.num_tiles == 0) return cudaSuccess;
    RedCtx r = rc;
    r.sys_group = ts.sys_group;
    k_rows<Op><<<ts.num_tiles, kBlock, 0, ctx->stream>>>(tile_args(ts), op, r, normtype);
    ctx->launches++;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && Op::kReduce) e = launch_finalize(ctx, ts, op, r, normtype);
    return e;
}

}  // namespace

inline RedCtx red_ctx(const mtjg_csr *A, const TileSet &ts)
{
    return RedCtx{A->part, A->cnt, ts.sys_group, A->num_running};
}

// Appends the product tiles of rows [row_begin, row_end) of a CSR (host row
// pointers) to `tile_row` (first rows) / `tile_flags`.
void plan_tiles(const int *rowptr, int row_begin, int row_end, int vec, std::vector<int> &tile_row,
                std::vector<unsigned char> &tile_flags, int nnz_cap = kTileNnz, int rows_cap = kTileRows);
// Appends row-kernel tiles of `rows` rows (a multiple of kRowTile) of rows
// [row_begin, row_end).
void plan_row_tiles(int row_begin, int row_end, int rows, std::vector<int> &tile_row,
                    std::vector<unsigned char> &tile_flags);
int choose_vec(int64_t nnz, int64_t n);
// Uploads a host tiling (tile_row has num_tiles+1 entries, sys_tile has
// num_sys+1 tile offsets) and groups each system's tiles by group_size
// consecutive tiles; rowptr gives each tile's first entry (nullptr for row
// tiles).
int upload_tiles(TileSet &ts, const std::vector<int> &tile_row, const std::vector<unsigned char> &tile_flags,
                 const std::vector<int> *tile_sys, const std::vector<int> &sys_tile, int vec, const int *rowptr,
                 int group_size, int group_div = kGroupDiv);
void free_tiles(TileSet &ts);
// Device exclusive scan of n ints into out[0..n] (out[n] = total).
int exclusive_scan(mtjg_ctx *ctx, const int *in, int *out, int n);
// Device transpose of selected entries of a CSR: mode 0 = all entries,
// mode 1 = strictly upper entries (column > row), mode 2 = strictly lower.
// Rows of the result list their entries in ascending source row order; the
// row pointer array carries kRowptrPad padding entries.
int csr_transpose(mtjg_ctx *ctx, int n, int m, const int *rowptr, const int *colind, const double *val,
                  int mode, int **t_rowptr, int **t_colind, double **t_val, int64_t *t_nnz);

}  // namespace mtjg
