// spmv.cu -- device CSR (CompRowMatrix) handles and their products.
#include <algorithm>
#include <cstring>

#include "spmv.cuh"

namespace mtjg {

// ------------------------------------------------------------------ tiles
int choose_vec(int64_t nnz, int64_t n)
{
    if (n <= 0) return 1;
    double avg = (double)nnz / (double)n;
    if (avg <= 12.0) return 1;
    if (avg <= 48.0) return 4;
    return 32;
}

// Tiles of consecutive rows, at most rows_cap_all / lanes rows and nnz_cap
// entries.  A row of the system's lanes-per-row class `vec` that is much
// longer than its neighbours (kWideRow entries or more, over 8 per lane)
// would keep one thread busy while the rest of its tile waits: such rows
// form tiles of their own summed by a whole warp per row (class 32).  A row
// longer than a stage is a tile of its own (long-row bit).
void plan_tiles(const int *rowptr, int row_begin, int row_end, int vec, std::vector<int> &tile_row,
                std::vector<unsigned char> &tile_flags, int nnz_cap, int rows_cap_all)
{
    auto lanes_for = [&](int len) { return vec < 32 && len >= kWideRow && len > 8 * vec ? 32 : vec; };
    int r = row_begin;
    while (r < row_end) {
        tile_row.push_back(r);
        int len0 = rowptr[r + 1] - rowptr[r];
        if (len0 > nnz_cap) {
            tile_flags.push_back((unsigned char)((vec << 1) | 1));
            r += 1;
            continue;
        }
        const int tv = lanes_for(len0);
        const int rows_cap = rows_cap_all / tv;
        int nz = len0, rows = 1;
        r += 1;
        while (r < row_end && rows < rows_cap) {
            int len = rowptr[r + 1] - rowptr[r];
            if (nz + len > nnz_cap || lanes_for(len) != tv) break;
            nz += len;
            rows++;
            r++;
        }
        tile_flags.push_back((unsigned char)(tv << 1));
    }
}

void plan_row_tiles(int row_begin, int row_end, int rows, std::vector<int> &tile_row,
                    std::vector<unsigned char> &tile_flags)
{
    for (int r = row_begin; r < row_end; r += rows) {
        tile_row.push_back(r);
        tile_flags.push_back((unsigned char)(1 << 1));
    }
}

int upload_tiles(TileSet &ts, const std::vector<int> &tile_row, const std::vector<unsigned char> &tile_flags,
                 const std::vector<int> *tile_sys, const std::vector<int> &sys_tile, int vec, const int *rowptr,
                 int group_size, int group_div)
{
    free_tiles(ts);
    ts.num_tiles = (int)tile_flags.size();
    ts.num_sys = (int)sys_tile.size() - 1;
    // reduction groups: runs of consecutive tiles inside each system.  A
    // system of T tiles uses groups of min(group_size, T / kGroupDiv) tiles (at
    // least 1): large systems amortise the block reduction over several
    // tiles while keeping thousands of groups for the CTAs to share evenly;
    // the size depends on the system alone, never on the rest of a batch.  A
    // group holds tiles of one lanes-per-row class (a launch takes a class).
    std::vector<int> group_tile, sys_group = {0};
    for (int s = 0; s < ts.num_sys; ++s) {
        const int t0 = sys_tile[s], t1 = sys_tile[s + 1];
        const int gs = std::max(1, std::min(group_size, (t1 - t0) / group_div));
        for (int t = t0, g0 = t0; t < t1; ++t)
            if (t == t0 || t - g0 == gs || (tile_flags[(size_t)t] >> 1) != (tile_flags[(size_t)g0] >> 1)) {
                group_tile.push_back(t);
                g0 = t;
            }
        sys_group.push_back((int)group_tile.size());
    }
    ts.num_groups = (int)group_tile.size();
    std::vector<int> group_info(std::max<size_t>(1, group_tile.size()));
    for (int s = 0, g = 0; s < ts.num_sys; ++s)
        for (; g < sys_group[s + 1]; ++g) group_info[g] = (s << 8) | (tile_flags[group_tile[g]] >> 1);
    MTJG_CUDA(cudaMalloc(&ts.group_info, sizeof(int) * group_info.size()));
    MTJG_CUDA(cudaMemcpy(ts.group_info, group_info.data(), sizeof(int) * group_info.size(), cudaMemcpyHostToDevice));
    group_tile.push_back(ts.num_tiles);
    MTJG_CUDA(cudaMalloc(&ts.group_tile, sizeof(int) * group_tile.size()));
    MTJG_CUDA(cudaMemcpy(ts.group_tile, group_tile.data(), sizeof(int) * group_tile.size(), cudaMemcpyHostToDevice));
    MTJG_CUDA(cudaMalloc(&ts.sys_group, sizeof(int) * sys_group.size()));
    MTJG_CUDA(cudaMemcpy(ts.sys_group, sys_group.data(), sizeof(int) * sys_group.size(), cudaMemcpyHostToDevice));
    ts.vec = vec;
    ts.vec_mask = 0;
    for (unsigned char f : tile_flags) ts.vec_mask |= f >> 1;
    ts.h_tile_row = tile_row;
    MTJG_CUDA(cudaMalloc(&ts.tile_row, sizeof(int) * tile_row.size()));
    MTJG_CUDA(cudaMemcpy(ts.tile_row, tile_row.data(), sizeof(int) * tile_row.size(), cudaMemcpyHostToDevice));
    if (rowptr) {
        std::vector<int> nz(tile_row.size());
        for (size_t i = 0; i < tile_row.size(); ++i) nz[i] = rowptr[tile_row[i]];
        MTJG_CUDA(cudaMalloc(&ts.tile_nz, sizeof(int) * nz.size()));
        MTJG_CUDA(cudaMemcpy(ts.tile_nz, nz.data(), sizeof(int) * nz.size(), cudaMemcpyHostToDevice));
    }
    MTJG_CUDA(cudaMalloc(&ts.tile_flags, std::max<size_t>(1, tile_flags.size())));
    if (!tile_flags.empty())
        MTJG_CUDA(cudaMemcpy(ts.tile_flags, tile_flags.data(), tile_flags.size(), cudaMemcpyHostToDevice));
    if (rowptr) {
        // long rows (tiles of a single row longer than a stage): segments for the FAST pre-pass
        std::vector<int> sb, se, lf{0}, lt;
        for (int t = 0; t < ts.num_tiles; ++t) {
            if (!(tile_flags[(size_t)t] & 1)) continue;
            const int r = tile_row[(size_t)t], b = rowptr[r], e = rowptr[r + 1];
            for (int k = b; k < e; k += kLongSeg) {
                sb.push_back(k);
                se.push_back(std::min(e, k + kLongSeg));
            }
            lf.push_back((int)sb.size());
            lt.push_back(t);
        }
        if (!lt.empty()) {
            ts.num_long = (int)lt.size();
            ts.num_segs = (int)sb.size();
            MTJG_CUDA(cudaMalloc(&ts.seg_begin, sizeof(int) * sb.size()));
            MTJG_CUDA(cudaMalloc(&ts.seg_end, sizeof(int) * se.size()));
            MTJG_CUDA(cudaMalloc(&ts.long_first, sizeof(int) * lf.size()));
            MTJG_CUDA(cudaMalloc(&ts.long_tile, sizeof(int) * lt.size()));
            MTJG_CUDA(cudaMalloc(&ts.seg_part, sizeof(double) * sb.size()));
            MTJG_CUDA(cudaMalloc(&ts.long_sum, sizeof(double) * (size_t)ts.num_tiles));
            MTJG_CUDA(cudaMemcpy(ts.seg_begin, sb.data(), sizeof(int) * sb.size(), cudaMemcpyHostToDevice));
            MTJG_CUDA(cudaMemcpy(ts.seg_end, se.data(), sizeof(int) * se.size(), cudaMemcpyHostToDevice));
            MTJG_CUDA(cudaMemcpy(ts.long_first, lf.data(), sizeof(int) * lf.size(), cudaMemcpyHostToDevice));
            MTJG_CUDA(cudaMemcpy(ts.long_tile, lt.data(), sizeof(int) * lt.size(), cudaMemcpyHostToDevice));
        }
    }
    if (tile_sys) {
        MTJG_CUDA(cudaMalloc(&ts.tile_sys, sizeof(int) * std::max<size_t>(1, tile_sys->size())));
        if (!tile_sys->empty())
            MTJG_CUDA(cudaMemcpy(ts.tile_sys, tile_sys->data(), sizeof(int) * tile_sys->size(),
                                 cudaMemcpyHostToDevice));
    }
    return MTJG_OK;
}

void free_tiles(TileSet &ts)
{
    cudaFree(ts.tile_row);
    cudaFree(ts.tile_nz);
    cudaFree(ts.tile_sys);
    cudaFree(ts.group_tile);
    cudaFree(ts.group_info);
    cudaFree(ts.sys_group);
    cudaFree(ts.tile_flags);
    ts.tile_row = ts.tile_nz = ts.tile_sys = ts.group_tile = ts.group_info = ts.sys_group = nullptr;
    ts.tile_flags = nullptr;
    cudaFree(ts.seg_begin);
    cudaFree(ts.seg_end);
    cudaFree(ts.long_first);
    cudaFree(ts.long_tile);
    cudaFree(ts.seg_part);
    cudaFree(ts.long_sum);
    ts.seg_begin = ts.seg_end = ts.long_first = ts.long_tile = nullptr;
    ts.seg_part = ts.long_sum = nullptr;
    ts.num_long = ts.num_segs = 0;
    ts.num_tiles = 0;
    ts.num_groups = 0;
}

// ------------------------------------------------------------------- scan
constexpr int kScanChunk = 2048;

__global__ void k_scan_chunks(const int *in, int n, int *chunk_sum)
{
    __shared__ int sm[kBlock / 32];
    const int c = blockIdx.x;
    const int base = c * kScanChunk;
    int s = 0;
    for (int i = base + threadIdx.x; i < base + kScanChunk && i < n; i += blockDim.x) s += in[i];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
        chunk_sum[c] = t;
    }
}

// single block: exclusive scan of the chunk sums in place, total at [nc]
__global__ void k_scan_top(int *chunk_sum, int nc)
{
    __shared__ int carry;
    __shared__ int sm[kBlock];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nc; base += blockDim.x) {
        int i = base + threadIdx.x;
        int v = i < nc ? chunk_sum[i] : 0;
        sm[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            int add = threadIdx.x >= (unsigned)off ? sm[threadIdx.x - off] : 0;
            __syncthreads();
            sm[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < nc) chunk_sum[i] = carry + sm[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += sm[blockDim.x - 1];
        __syncthreads();
    }
    if (threadIdx.x == 0) chunk_sum[nc] = carry;
}

__global__ void k_scan_apply(const int *in, int n, const int *chunk_off, int *out)
{
    __shared__ int sm[kBlock];
    __shared__ int carry;
    const int c = blockIdx.x;
    const int base = c * kScanChunk;
    if (threadIdx.x == 0) carry = chunk_off[c];
    __syncthreads();
    for (int b = base; b < base + kScanChunk && b < n; b += blockDim.x) {
        int i = b + threadIdx.x;
        int v = i < n ? in[i] : 0;
        sm[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < (int)blockDim.x; off <<= 1) {
            int add = threadIdx.x >= (unsigned)off ? sm[threadIdx.x - off] : 0;
            __syncthreads();
            sm[threadIdx.x] += add;
            __syncthreads();
        }
        if (i < n) out[i] = carry + sm[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 0) carry += sm[blockDim.x - 1];
        __syncthreads();
    }
    if (c == (int)gridDim.x - 1 && threadIdx.x == 0) out[n] = chunk_off[gridDim.x];
}

int exclusive_scan(mtjg_ctx *ctx, const int *in, int *out, int n)
{
    if (n == 0) {
        MTJG_CUDA(cudaMemsetAsync(out, 0, sizeof(int), ctx->stream));
        return MTJG_OK;
    }
    int nc = (n + kScanChunk - 1) / kScanChunk;
    int *cs = nullptr;
    MTJG_CUDA(cudaMalloc(&cs, sizeof(int) * (nc + 1)));
    k_scan_chunks<<<nc, kBlock, 0, ctx->stream>>>(in, n, cs);
    k_scan_top<<<1, kBlock, 0, ctx->stream>>>(cs, nc);
    k_scan_apply<<<nc, kBlock, 0, ctx->stream>>>(in, n, cs, out);
    ctx->launches += 3;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    cudaFree(cs);
    if (e != cudaSuccess) return cuda_fail(e, "exclusive_scan");
    return MTJG_OK;
}

// -------------------------------------------------------------- transpose
__global__ void k_tr_count(int n, const int *rowptr, const int *colind, int mode, int *cnt)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            int c = colind[k];
            if (mode == 0 || (mode == 1 && c > i) || (mode == 2 && c < i))atomicAdd(&cnt[c], 1);
        }
}

__global__ void k_tr_fill(int n, const int *rowptr, const int *colind, const double *val, int mode,
                          const int *t_rowptr, int *cursor, int *t_colind, double *t_val)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            int c = colind[k];
            if (mode == 0 || (mode == 1 && c > i) || (mode == 2 && c < i)){
                int pos = t_rowptr[c] + atomicAdd(&cursor[c], 1);
                t_colind[pos] = i;
                t_val[pos] = val[k];
            }
        }
}

// Each transposed row sorted by source row (the fill's atomics leave it in
// any order).  Rows of up to kTrShort entries: an insertion sort by one
// thread.  Longer rows (a dense column of A) would make that quadratic:
// k_tr_sort_long gives each one a block, which sorts it with a bitonic
// network in scratch, padded to a power of two with keys above every row.
constexpr int kTrShort = 64;

__global__ void k_tr_sort(int m, const int *t_rowptr, int *t_colind, double *t_val)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m; c += gridDim.x * blockDim.x) {
        int b = t_rowptr[c], e = t_rowptr[c + 1];
        if (e - b > kTrShort) continue;
        for (int p = b + 1; p < e; ++p) {
            int key = t_colind[p];
            double v = t_val[p];
            int q = p - 1;
            while (q >= b && t_colind[q] > key) {
                t_colind[q + 1] = t_colind[q];
                t_val[q + 1] = t_val[q];
                --q;
            }
            t_colind[q + 1] = key;
            t_val[q + 1] = v;
        }
    }
}

__global__ void k_tr_sort_long(const int *rows, const int64_t *soff, const int *t_rowptr, int *t_colind,
                               double *t_val, int *skey, double *sval)
{
    const int c = rows[blockIdx.x];
    const int b = t_rowptr[c], len = t_rowptr[c + 1] - b;
    int P = 1;
    while (P < len) P <<= 1;
    int *K = skey + soff[blockIdx.x];
    double *V = sval + soff[blockIdx.x];
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        K[i] = i < len ? t_colind[b + i] : 0x7fffffff;
        V[i] = i < len ? t_val[b + i] : 0.0;
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const int ki = K[i], kl = K[l];
                    if ((ki > kl) == ((i & k) == 0)) {
                        K[i] = kl;
                        K[l] = ki;
                        const double t = V[i];
                        V[i] = V[l];
                        V[l] = t;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
        t_colind[b + i] = K[i];
        t_val[b + i] = V[i];
    }
}

int csr_transpose(mtjg_ctx *ctx, int n, int m, const int *rowptr, const int *colind, const double *val,
                  int mode, int **t_rowptr, int **t_colind, double **t_val, int64_t *t_nnz)
{
    int *cnt = nullptr, *cursor = nullptr, *trp = nullptr, *tci = nullptr;
    double *tv = nullptr;
    const int grid = std::max(1, std::min((n + kBlock - 1) / kBlock, ctx->num_sms * 8));
    MTJG_CUDA(cudaMalloc(&cnt, sizeof(int) * (size_t)std::max(1, m)));
    MTJG_CUDA(cudaMalloc(&cursor, sizeof(int) * (size_t)std::max(1, m)));
    MTJG_CUDA(cudaMalloc(&trp, sizeof(int) * (size_t)(m + 1 + kRowptrPad)));
    MTJG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int) * (size_t)std::max(1, m), ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)std::max(1, m), ctx->stream));
    if (n > 0) {
        k_tr_count<<<grid, kBlock, 0, ctx->stream>>>(n, rowptr, colind, mode, cnt);
        ctx->launches++;
    }
    int st = exclusive_scan(ctx, cnt, trp, m);
    if (st != MTJG_OK) return st;
    int total = 0;
    MTJG_CUDA(cudaMemcpy(&total, trp + m, sizeof(int), cudaMemcpyDeviceToHost));
    {
        const int pad[kRowptrPad] = {total, total, total, total};
        MTJG_CUDA(cudaMemcpy(trp + m + 1, pad, sizeof(pad), cudaMemcpyHostToDevice));
    }
    MTJG_CUDA(cudaMalloc(&tci, sizeof(int) * (size_t)(total + 4)));
    MTJG_CUDA(cudaMalloc(&tv, sizeof(double) * (size_t)(total + 2)));
    MTJG_CUDA(cudaMemsetAsync(tci, 0xff, sizeof(int) * (size_t)(total + 4), ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(tv, 0, sizeof(double) * (size_t)(total + 2), ctx->stream));
    if (n > 0) {
        k_tr_fill<<<grid, kBlock, 0, ctx->stream>>>(n, rowptr, colind, val, mode, trp, cursor, tci, tv);
        ctx->launches++;
    }
    if (m > 0) {
        const int gm = std::max(1, std::min((m + kBlock - 1) / kBlock, ctx->num_sms * 8));
        k_tr_sort<<<gm, kBlock, 0, ctx->stream>>>(m, trp, tci, tv);
        ctx->launches++;
    }
    // the long transposed rows (found from the row pointers on the host)
    std::vector<int> h_trp((size_t)m + 1);
    if (m > 0) MTJG_CUDA(cudaMemcpy(h_trp.data(), trp, sizeof(int) * ((size_t)m + 1), cudaMemcpyDeviceToHost));
    std::vector<int> lrows;
    std::vector<int64_t> loff{0};
    for (int c = 0; c < m; ++c) {
        const int len = h_trp[(size_t)c + 1] - h_trp[(size_t)c];
        if (len <= kTrShort) continue;
        int64_t P = 1;
        while (P < len) P <<= 1;
        lrows.push_back(c);
        loff.push_back(loff.back() + P);
    }
    if (!lrows.empty()) {
        int *d_rows = nullptr, *skey = nullptr;
        int64_t *d_off = nullptr;
        double *sval = nullptr;
        cudaError_t e = cudaMalloc(&d_rows, sizeof(int) * lrows.size());
        if (e == cudaSuccess) e = cudaMalloc(&d_off, sizeof(int64_t) * loff.size());
        if (e == cudaSuccess) e = cudaMalloc(&skey, sizeof(int) * (size_t)loff.back());
        if (e == cudaSuccess) e = cudaMalloc(&sval, sizeof(double) * (size_t)loff.back());
        if (e == cudaSuccess)
            e = cudaMemcpy(d_rows, lrows.data(), sizeof(int) * lrows.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(d_off, loff.data(), sizeof(int64_t) * loff.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            k_tr_sort_long<<<(unsigned)lrows.size(), 1024, 0, ctx->stream>>>(d_rows, d_off, trp, tci, tv, skey, sval);
            ctx->launches++;
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        cudaFree(d_rows);
        cudaFree(d_off);
        cudaFree(skey);
        cudaFree(sval);
        if (e != cudaSuccess) return cuda_fail(e, "sorting the long rows of a transpose");
    }
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    cudaFree(cnt);
    cudaFree(cursor);
    *t_rowptr = trp;
    *t_colind = tci;
    *t_val = tv;
    *t_nnz = total;
    return MTJG_OK;
}

// ----------------------------------------------------------- epilogues
// CompRowMatrix.mult: y = Ax, a zero sum stored as +0 (y.zero() and the
// "if (dot != 0)" test, S/CompRowMatrix.java:299,309-311).
struct EpiMult {
    double *y;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int) const { return true; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int r, int, double d, double, Acc &) const { y[r] = mtj_assign(d); }
    __device__ void scalar(int, const Acc &) {}
};

// CompRowMatrix.multAdd: y_i += alpha * dot (S/CompRowMatrix.java:343)
template <bool S>
struct EpiMultAdd {
    double *y;
    double alpha;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int) const { return true; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int r, int, double d, double, Acc &) const { y[r] = fmac<S>(alpha, d, y[r]); }
    __device__ void scalar(int, const Acc &) {}
};

// transMult on the transpose: y_c = sum over ascending source rows, from 0
// (the scatter of S/CompRowMatrix.java:359-363 in gather form).
struct EpiSet {
    double *y;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int) const { return true; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int r, int, double d, double, Acc &) const { y[r] = d; }
    __device__ void scalar(int, const Acc &) {}
};

// transMultAdd (S/CompRowMatrix.java:378-387): y scaled by 1/alpha, the
// products added onto it in ascending source row order, then scaled by alpha.
struct EpiTransMultAdd {
    double *y;
    double alpha, inv;
    static constexpr bool kReduce = false;
    static constexpr bool kNeedsXr = false;
    __device__ bool active(int) const { return true; }
    __device__ double init(int r, int) const { return y[r] * inv; }
    __device__ void row(int r, int, double d, double, Acc &) const { y[r] = d * alpha; }
    __device__ void scalar(int, const Acc &) {}
};

}  // namespace mtjg

using namespace mtjg;

// ------------------------------------------------------------- handle ops
int mtjg::csr_validate(int n, int m, const int *rowptr, const int *colind)
{
    if (n < 0 || m < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "negative matrix dimension");
    if (!rowptr) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "rowptr is NULL");
    if (rowptr[0] != 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "rowptr[0] != 0");
    for (int i = 0; i < n; ++i) {
        if (rowptr[i + 1] < rowptr[i]) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "rowptr is not nondecreasing");
        for (int k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            int c = colind[k];
            if (c < 0 || c >= m)
                return fail(MTJG_ERR_ILLEGAL_ARGUMENT,
                            "nz[" + std::to_string(i) + "][" + std::to_string(k - rowptr[i]) + "]=" +
                                std::to_string(c) + ", which is not a valid column index");
            if (k > rowptr[i] && colind[k - 1] >= c)
                return fail(MTJG_ERR_ILLEGAL_ARGUMENT,
                            "column indices of row " + std::to_string(i) + " are not strictly ascending");
        }
    }
    return MTJG_OK;
}

static int csr_finish(mtjg_csr *A, int num_sys, const int *sys_rows);

// Uploads a CSR; with sys_rows (num_sys + 1 row offsets) it is a batch of
// independent systems whose tiles are planned system by system.
static int csr_upload_impl(mtjg_ctx *ctx, int n, int m, const int *rowptr, const int *colind, const double *val,
                           int num_sys, const int *sys_rows, mtjg_csr **out)
{
    if (!ctx || !out) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    int st = csr_validate(n, m, rowptr, colind);
    if (st != MTJG_OK) return st;
    if (sys_rows) {
        if (sys_rows[0] != 0 || sys_rows[num_sys] != n)
            return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "system row offsets must run from 0 to the number of rows");
        for (int s = 0; s < num_sys; ++s) {
            const int r0 = sys_rows[s], r1 = sys_rows[s + 1];
            if (r1 < r0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "system row offsets must be nondecreasing");
            for (int i = r0; i < r1; ++i)
                if (rowptr[i + 1] > rowptr[i] && (colind[rowptr[i]] < r0 || colind[rowptr[i + 1] - 1] >= r1))
                    return fail(MTJG_ERR_ILLEGAL_ARGUMENT,
                                "system " + std::to_string(s) + " references a column outside its rows");
        }
    }
    MTJG_CUDA(cudaSetDevice(ctx->device));
    const int64_t nnz = rowptr[n];
    mtjg_csr *A = new mtjg_csr();
    A->ctx = ctx;
    ctx_retain(ctx);
    A->n = n;
    A->m = m;
    A->nnz = nnz;
    A->h_rowptr.assign(rowptr, rowptr + n + 1);
    auto bail = [&](int code) {
        mtjg_csr_destroy(A);
        return code;
    };
    if (cudaMalloc(&A->rowptr, sizeof(int) * (size_t)(n + 1 + kRowptrPad)) != cudaSuccess ||
        cudaMalloc(&A->colind, sizeof(int) * (size_t)(nnz + 4)) != cudaSuccess ||
        cudaMalloc(&A->val, sizeof(double) * (size_t)(nnz + 2)) != cudaSuccess ||
        cudaMalloc(&A->d_x, sizeof(double) * (size_t)std::max(1, std::max(n, m))) != cudaSuccess ||
        cudaMalloc(&A->d_y, sizeof(double) * (size_t)std::max(1, std::max(n, m))) != cudaSuccess)
        return bail(fail(MTJG_ERR_OUT_OF_MEMORY, "cudaMalloc failed for the CSR matrix"));
    cudaMemset(A->colind, 0xff, sizeof(int) * (size_t)(nnz + 4));
    cudaMemset(A->val, 0, sizeof(double) * (size_t)(nnz + 2));
    if (cudaMemcpy(A->rowptr, rowptr, sizeof(int) * (size_t)(n + 1), cudaMemcpyHostToDevice) != cudaSuccess ||
        (nnz && cudaMemcpy(A->colind, colind, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice) != cudaSuccess) ||
        (nnz && cudaMemcpy(A->val, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice) != cudaSuccess))
        return bail(fail(MTJG_ERR_CUDA, "copying the CSR matrix to the device failed"));
    {
        // bulk copies of a tile's row pointers may read up to 3 entries past rowptr[n]
        const int pad[kRowptrPad] = {rowptr[n], rowptr[n], rowptr[n], rowptr[n]};
        if (cudaMemcpy(A->rowptr + n + 1, pad, sizeof(pad), cudaMemcpyHostToDevice) != cudaSuccess)
            return bail(fail(MTJG_ERR_CUDA, "copying the CSR matrix to the device failed"));
    }
    st = csr_finish(A, num_sys, sys_rows);
    if (st != MTJG_OK) return bail(st);
    *out = A;
    return MTJG_OK;
}

// The tiles, reduction scratch and staging vectors of a CSR whose arrays are
// on the device and whose row pointers are in A->h_rowptr.  Tiles are
// planned system by system (they never straddle two systems); each system's
// lanes per row follow its own entries per row, so its tiles and its results
// do not depend on the rest of a batch.
static int csr_finish(mtjg_csr *A, int num_sys, const int *sys_rows)
{
    const int n = A->n, m = A->m;
    const int64_t nnz = A->nnz;
    const int *rowptr = A->h_rowptr.data();
    int st = MTJG_OK;
    if (!A->d_x && (cudaMalloc(&A->d_x, sizeof(double) * (size_t)std::max(1, std::max(n, m))) != cudaSuccess ||
                    cudaMalloc(&A->d_y, sizeof(double) * (size_t)std::max(1, std::max(n, m))) != cudaSuccess))
        return fail(MTJG_ERR_OUT_OF_MEMORY, "cudaMalloc failed for the CSR matrix");
    const int vec = choose_vec(nnz, n);
    std::vector<int> tile_row, rtile_row, tile_sys, rtile_sys, sys_tile = {0}, rsys_tile = {0};
    std::vector<unsigned char> tile_flags, rtile_flags;
    const int ns = sys_rows ? num_sys : 1;
    for (int s = 0; s < ns; ++s) {
        const int r0 = sys_rows ? sys_rows[s] : 0, r1 = sys_rows ? sys_rows[s + 1] : n;
        const int vs = choose_vec((int64_t)rowptr[r1] - rowptr[r0], r1 - r0);
        plan_tiles(rowptr, r0, r1, vs, tile_row, tile_flags);
        plan_row_tiles(r0, r1, sys_rows || n >= kRowTileLoneMin ? kRowTileRows : kRowTile, rtile_row, rtile_flags);
        tile_sys.resize(tile_flags.size(), s);
        rtile_sys.resize(rtile_flags.size(), s);
        sys_tile.push_back((int)tile_flags.size());
        rsys_tile.push_back((int)rtile_flags.size());
    }
    tile_row.push_back(n);
    rtile_row.push_back(n);
    // a batch (mtjg_batch_upload, any number of systems) spreads over its
    // systems, so its systems take larger reduction groups (product and row
    // tiles) than a lone uploaded CSR, which needs many groups to fill the
    // GPU by itself
    st = upload_tiles(A->tiles, tile_row, tile_flags, sys_rows ? &tile_sys : nullptr, sys_tile, vec, rowptr,
                      kGroupTiles, sys_rows ? kBatchGroupDiv : kGroupDiv);
    if (st != MTJG_OK) return st;
    st = upload_tiles(A->rtiles, rtile_row, rtile_flags, sys_rows ? &rtile_sys : nullptr, rsys_tile, 1, nullptr, 1);
    if (st != MTJG_OK) return st;
    const size_t nt = std::max<size_t>(1, std::max(tile_flags.size(), rtile_flags.size()));
    if (cudaMalloc(&A->part, sizeof(double) * nt * kParts) != cudaSuccess ||
        cudaMalloc(&A->cnt, sizeof(unsigned) * (size_t)std::max(4, ns)) != cudaSuccess ||
        cudaMalloc(&A->num_running, sizeof(int) * 4) != cudaSuccess)
        return fail(MTJG_ERR_OUT_OF_MEMORY, "cudaMalloc failed for reduction scratch");
    cudaMemset(A->cnt, 0, sizeof(unsigned) * (size_t)std::max(4, ns));
    cudaMemset(A->num_running, 0, sizeof(int) * 4);
    if (sys_rows) A->sys_rows.assign(sys_rows, sys_rows + num_sys + 1);
    return MTJG_OK;
}

namespace mtjg {
// A CSR handle over device arrays the caller hands over (rowptr with
// kRowptrPad padding entries, colind padded with 4 entries of -1, val with 2
// zeros), with its host row pointers.  The arrays belong to the handle from
// the call on: a failure frees them with it.
int csr_adopt(mtjg_ctx *ctx, int n, int m, std::vector<int> &&h_rowptr, int *d_rowptr, int *d_colind, double *d_val,
              mtjg_csr **out)
{
    *out = nullptr;
    mtjg_csr *A = new mtjg_csr();
    A->ctx = ctx;
    ctx_retain(ctx);
    A->n = n;
    A->m = m;
    A->nnz = h_rowptr[(size_t)n];
    A->h_rowptr = std::move(h_rowptr);
    A->rowptr = d_rowptr;
    A->colind = d_colind;
    A->val = d_val;
    const int st = csr_finish(A, 1, nullptr);
    if (st != MTJG_OK) {
        mtjg_csr_destroy(A);
        return st;
    }
    *out = A;
    return MTJG_OK;
}

// A CSR handle over device arrays owned by someone else (a served matrix):
// its tiles and scratch are its own, the arrays are not freed with it.
int csr_borrow(mtjg_ctx *ctx, int n, const int *h_rowptr, const int *d_rowptr, const int *d_colind,
               const double *d_val, const float *d_val32, mtjg_csr **out)
{
    *out = nullptr;
    mtjg_csr *A = new mtjg_csr();
    A->ctx = ctx;
    ctx_retain(ctx);
    A->borrowed = true;
    A->n = n;
    A->m = n;
    A->nnz = h_rowptr[n];
    A->h_rowptr.assign(h_rowptr, h_rowptr + n + 1);
    A->rowptr = const_cast<int *>(d_rowptr);
    A->colind = const_cast<int *>(d_colind);
    A->val = const_cast<double *>(d_val);
    A->val32 = const_cast<float *>(d_val32);
    const int st = csr_finish(A, 1, nullptr);
    if (st != MTJG_OK) {
        mtjg_csr_destroy(A);
        return st;
    }
    *out = A;
    return MTJG_OK;
}
}  // namespace mtjg

extern "C" int mtjg_csr_upload(mtjg_ctx *ctx, int n, int m, const int *rowptr, const int *colind,
                               const double *val, mtjg_csr **out)
{
    return csr_upload_impl(ctx, n, m, rowptr, colind, val, 1, nullptr, out);
}

extern "C" int mtjg_batch_upload(mtjg_ctx *ctx, int num_systems, const int *sys_rows, const int *rowptr,
                                 const int *colind, const double *val, mtjg_csr **out)
{
    if (num_systems <= 0 || !sys_rows) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "a batch needs at least one system");
    const int n = sys_rows[num_systems];
    return csr_upload_impl(ctx, n, n, rowptr, colind, val, num_systems, sys_rows, out);
}

extern "C" int mtjg_csr_update_values(mtjg_csr *A, const double *val)
{
    if (!A || (!val && A->nnz)) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (A->borrowed) return fail(MTJG_ERR_UNSUPPORTED, "the matrix's values belong to a server");
    MTJG_CUDA(cudaSetDevice(A->ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(A->ctx->stream));
    if (A->nnz) MTJG_CUDA(cudaMemcpy(A->val, val, sizeof(double) * (size_t)A->nnz, cudaMemcpyHostToDevice));
    // the transpose holds old values: rebuild on next use
    cudaFree(A->t_rowptr);
    cudaFree(A->t_colind);
    cudaFree(A->t_val);
    cudaFree(A->t_part);
    A->t_rowptr = A->t_colind = nullptr;
    A->t_val = A->t_part = nullptr;
    static std::atomic<int64_t> s_version{0};
    A->version = ++s_version;
    free_tiles(A->t_tiles);
    cudaFree(A->val32);  // the FP32 copy too
    A->val32 = nullptr;
    return MTJG_OK;
}

extern "C" int mtjg_csr_destroy(mtjg_csr *A)
{
    if (!A) return MTJG_OK;
    if (A->ctx) cudaSetDevice(A->ctx->device);
    if (A->ctx) cudaStreamSynchronize(A->ctx->stream);
    if (!A->borrowed) {
        cudaFree(A->rowptr);
        cudaFree(A->colind);
        cudaFree(A->val);
        cudaFree(A->val32);
    }
    cudaFree(A->t_rowptr);
    cudaFree(A->t_colind);
    cudaFree(A->t_val);
    cudaFree(A->t_part);
    cudaFree(A->d_sys_rows);
    cudaFree(A->part);
    cudaFree(A->cnt);
    cudaFree(A->num_running);
    cudaFree(A->d_x);
    cudaFree(A->d_y);
    free_tiles(A->tiles);
    free_tiles(A->rtiles);
    free_tiles(A->t_tiles);
    mtjg_ctx *ctx = A->ctx;
    delete A;
    ctx_release(ctx);
    return MTJG_OK;
}

extern "C" int mtjg_csr_dims(const mtjg_csr *A, int *n, int *m, int64_t *nnz)
{
    if (!A) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL matrix");
    if (n) *n = A->n;
    if (m) *m = A->m;
    if (nnz) *nnz = A->nnz;
    return MTJG_OK;
}

extern "C" int mtjg_csr_to_host(const mtjg_csr *A, int *rowptr, int *colind, double *val)
{
    if (!A) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL matrix");
    MTJG_CUDA(cudaSetDevice(A->ctx->device));
    MTJG_CUDA(cudaStreamSynchronize(A->ctx->stream));
    if (rowptr) std::memcpy(rowptr, A->h_rowptr.data(), sizeof(int) * (size_t)(A->n + 1));
    if (colind && A->nnz) MTJG_CUDA(cudaMemcpy(colind, A->colind, sizeof(int) * (size_t)A->nnz, cudaMemcpyDeviceToHost));
    if (val && A->nnz) MTJG_CUDA(cudaMemcpy(val, A->val, sizeof(double) * (size_t)A->nnz, cudaMemcpyDeviceToHost));
    return MTJG_OK;
}

namespace mtjg {
// The transpose of A (for transMult and the transposed products of BiCG and
// QMR), its tiles and its reduction scratch, built on first use.
int csr_ensure_transpose(mtjg_csr *A);
}  // namespace mtjg

static int ensure_transpose(mtjg_csr *A) { return mtjg::csr_ensure_transpose(A); }

int mtjg::csr_ensure_transpose(mtjg_csr *A)
{
    if (A->t_rowptr) return MTJG_OK;
    mtjg_ctx *ctx = A->ctx;
    int64_t tnnz = 0;
    int st = csr_transpose(ctx, A->n, A->m, A->rowptr, A->colind, A->val, 0, &A->t_rowptr, &A->t_colind,
                           &A->t_val, &tnnz);
    if (st != MTJG_OK) return st;
    std::vector<int> trp(A->m + 1);
    MTJG_CUDA(cudaMemcpy(trp.data(), A->t_rowptr, sizeof(int) * (size_t)(A->m + 1), cudaMemcpyDeviceToHost));
    const int vec = choose_vec(tnnz, A->m);
    std::vector<int> tile_row;
    std::vector<unsigned char> tile_flags;
    plan_tiles(trp.data(), 0, A->m, vec, tile_row, tile_flags);
    tile_row.push_back(A->m);
    std::vector<int> sys_tile = {0, (int)tile_flags.size()};
    st = upload_tiles(A->t_tiles, tile_row, tile_flags, nullptr, sys_tile, vec, trp.data(), kGroupTiles);
    if (st != MTJG_OK) return st;
    MTJG_CUDA(cudaMalloc(&A->t_part, sizeof(double) * (size_t)std::max(1, A->t_tiles.num_groups) * kParts));
    return MTJG_OK;
}

static int check_err_flag(mtjg_ctx *ctx)
{
    int flag = 0;
    MTJG_CUDA(cudaMemcpy(&flag, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) {
        cudaMemset(ctx->d_flag, 0, sizeof(int));
        return fail(MTJG_ERR_DEVICE_TIMEOUT, "a bounded wait in a device kernel gave up");
    }
    return MTJG_OK;
}

// op: 0 mult, 1 multAdd, 2 transMult, 3 transMultAdd.  Device pointers.
static int csr_product_dev(mtjg_csr *A, int op, double alpha, const double *dx, double *dy)
{
    mtjg_ctx *ctx = A->ctx;
    const bool strict = ctx->numerics == MTJG_NUMERICS_STRICT;
    RedCtx rc = red_ctx(A, A->tiles);
    cudaError_t e = cudaSuccess;
    if (op == 0) {
        e = launch_spmv(ctx, CsrArgs{A->rowptr, A->colind, A->val}, A->tiles, dx, EpiMult{dy}, rc, MTJG_NORM_TWO);
    } else if (op == 1) {
        if (strict)
            e = launch_spmv(ctx, CsrArgs{A->rowptr, A->colind, A->val}, A->tiles, dx, EpiMultAdd<true>{dy, alpha},
                            rc, MTJG_NORM_TWO);
        else
            e = launch_spmv(ctx, CsrArgs{A->rowptr, A->colind, A->val}, A->tiles, dx,
                            EpiMultAdd<false>{dy, alpha}, rc, MTJG_NORM_TWO);
    } else {
        int st = ensure_transpose(A);
        if (st != MTJG_OK) return st;
        RedCtx trc = red_ctx(A, A->t_tiles);
        if (op == 2)
            e = launch_spmv(ctx, CsrArgs{A->t_rowptr, A->t_colind, A->t_val}, A->t_tiles, dx, EpiSet{dy}, trc,
                            MTJG_NORM_TWO);
        else
            e = launch_spmv(ctx, CsrArgs{A->t_rowptr, A->t_colind, A->t_val}, A->t_tiles, dx,
                            EpiTransMultAdd{dy, alpha, 1. / alpha}, trc, MTJG_NORM_TWO);
    }
    if (e != cudaSuccess) return cuda_fail(e, "CSR product launch");
    return MTJG_OK;
}

static int csr_product_host(mtjg_csr *A, int op, double alpha, const double *x, double *y)
{
    if (!A || !x || !y) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    mtjg_ctx *ctx = A->ctx;
    MTJG_CUDA(cudaSetDevice(ctx->device));
    const bool trans = op >= 2;
    const int nx = trans ? A->n : A->m, ny = trans ? A->m : A->n;
    MTJG_CUDA(cudaMemcpyAsync(A->d_x, x, sizeof(double) * (size_t)nx, cudaMemcpyHostToDevice, ctx->stream));
    if (op == 1 || op == 3)
        MTJG_CUDA(cudaMemcpyAsync(A->d_y, y, sizeof(double) * (size_t)ny, cudaMemcpyHostToDevice, ctx->stream));
    int st = csr_product_dev(A, op, alpha, A->d_x, A->d_y);
    if (st != MTJG_OK) return st;
    MTJG_CUDA(cudaMemcpyAsync(y, A->d_y, sizeof(double) * (size_t)ny, cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    return check_err_flag(ctx);
}

extern "C" int mtjg_csr_mult(mtjg_csr *A, const double *x, double *y) { return csr_product_host(A, 0, 0.0, x, y); }
extern "C" int mtjg_csr_mult_add(mtjg_csr *A, double alpha, const double *x, double *y)
{
    return csr_product_host(A, 1, alpha, x, y);
}
extern "C" int mtjg_csr_trans_mult(mtjg_csr *A, const double *x, double *y)
{
    return csr_product_host(A, 2, 0.0, x, y);
}
extern "C" int mtjg_csr_trans_mult_add(mtjg_csr *A, double alpha, const double *x, double *y)
{
    return csr_product_host(A, 3, alpha, x, y);
}
extern "C" int mtjg_csr_mult_dev(mtjg_csr *A, const double *dx, double *dy)
{
    if (!A || !dx || !dy) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    MTJG_CUDA(cudaSetDevice(A->ctx->device));
    return csr_product_dev(A, 0, 0.0, dx, dy);
}
extern "C" int mtjg_csr_mult_add_dev(mtjg_csr *A, double alpha, const double *dx, double *dy)
{
    if (!A || !dx || !dy) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    MTJG_CUDA(cudaSetDevice(A->ctx->device));
    return csr_product_dev(A, 1, alpha, dx, dy);
}
extern "C" int mtjg_csr_trans_mult_dev(mtjg_csr *A, const double *dx, double *dy)
{
    if (!A || !dx || !dy) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    MTJG_CUDA(cudaSetDevice(A->ctx->device));
    return csr_product_dev(A, 2, 0.0, dx, dy);
}
