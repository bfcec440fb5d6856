// server.cu -- continuous-batching solve server.
//
// Matrices are registered once; a resident matrix holds its CSR (FP64 and
// FP32 values) and its Jacobi inverse diagonal in one device allocation.
// Requests (matrix, b, x0) queue on the host; a scheduler thread admits them
// into free slots whenever a slot and a contiguous segment of the pooled
// vector workspace are free and the request's matrix is resident (admission
// by device-memory footprint), runs chunks of the mixed-precision CG phases
// over all admitted systems at once, and retires finished systems between
// chunks, so requests that arrive while others are on the GPU join the
// running batch.
//
// With a matrix budget, the resident matrices' bytes stay within it: each
// matrix keeps a host copy, is uploaded when a request first needs it, and
// idle matrices (no system admitted) are evicted least recently used to make
// room, to be uploaded again on their next request.  A request whose matrix
// cannot be made resident (the budget is held by matrices in use) waits at
// the head of the queue.
//
// GMRES and BiCGstab requests take a second lane: a worker thread with its
// own stream solves them one at a time (mixed-precision GMRES(30) or
// BiCGstab with the Jacobi preconditioner, through the solver's own code)
// on the resident matrix, pinned for the solve under the same budget, while
// the CG batch runs on the scheduler's stream.
//
// The scheduler keeps two chunks queued on its stream: while the GPU runs
// chunk k+1, the host reads chunk k's statuses, retires finished systems,
// admits new ones and rebuilds the tile tables.  Everything the host hands
// to the device for chunk k+2 (b, x0, system states, tile tables) is staged
// in pinned memory and copied on the same stream, so stream order puts it
// after chunk k+1 without the host waiting for it.  A system admitted for
// chunk k+2 is ignored in the status snapshot of chunk k+1.
//
// Each system's product tiles are its own matrix's tiles and its reduction
// groups depend on that matrix alone, so its arithmetic -- and its result --
// is the same alone and in any mix of other systems.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

#include "phases.cuh"

namespace mtjg {
// A CSR handle over a served matrix's device arrays (spmv.cu).
int csr_borrow(mtjg_ctx *ctx, int n, const int *h_rowptr, const int *d_rowptr, const int *d_colind,
               const double *d_val, const float *d_val32, mtjg_csr **out);

namespace {

// Product tiles of one matrix (host copies).
struct ProdTiles {
    std::vector<int> row, row_end, nz, nz_end;
    std::vector<unsigned char> flags;
    void plan(const int *rowptr, int n, int vec, int nnz_cap, int rows_cap)
    {
        std::vector<int> tr;
        plan_tiles(rowptr, 0, n, vec, tr, flags, nnz_cap, rows_cap);
        tr.push_back(n);
        for (size_t t = 0; t + 1 < tr.size(); ++t) {
            row.push_back(tr[t]);
            row_end.push_back(tr[t + 1]);
            nz.push_back(rowptr[tr[t]]);
            nz_end.push_back(rowptr[tr[t + 1]]);
        }
    }
};

// Byte offsets of a served matrix's arrays in its one device allocation
// (each array starts on a 256-byte boundary).  The padding matches
// mtjg_csr_upload's: rowptr[n] repeated kRowptrPad times, colind padded with
// -1, the values with zeros, so the product kernels' bulk copies stay inside.
struct MatLayout {
    size_t rowptr = 0, colind = 0, val = 0, val32 = 0, invdiag32 = 0, bytes = 0;
    MatLayout(int n, int64_t nnz)
    {
        auto take = [&](size_t b) {
            const size_t o = bytes;
            bytes = (bytes + b + 255) & ~(size_t)255;
            return o;
        };
        rowptr = take(sizeof(int) * ((size_t)n + 1 + kRowptrPad));
        colind = take(sizeof(int) * (size_t)(nnz + 4));
        val = take(sizeof(double) * (size_t)(nnz + 2));
        val32 = take(sizeof(float) * (size_t)(nnz + 4));
        invdiag32 = take(sizeof(float) * (size_t)std::max(1, n));
    }
};

// The device copy of a served matrix: what the chunk kernels read.
struct DevMat {
    void *base = nullptr;
    int *rowptr = nullptr, *colind = nullptr;
    double *val = nullptr;
    float *val32 = nullptr, *invdiag32 = nullptr;
    void release()
    {
        cudaFree(base);  // waits for the device
        *this = DevMat();
    }
};

struct ResMat {
    int n = 0;
    int64_t nnz = 0;
    int64_t bytes = 0;                 // device bytes while resident
    DevMat dev;                        // set while resident
    std::vector<float> inv32;          // Jacobi inverse diagonal, FP32 (host)
    std::vector<int> h_rowptr, h_colind;  // host copy for uploads after an eviction
    std::vector<double> h_val;            // (kept only by servers with a matrix budget)
    ProdTiles t64, t32;  // product tiles for FP64 and FP32 values (local rows and entries)
    bool resident = false;  // dev holds the matrix
    bool loading = false;   // picked for upload, not yet attached
    int loader = 0;         // who is uploading it: 1 the scheduler, 2 the Krylov lane
    int64_t epoch = 0;      // server-unique number of the current upload (0: none)
    int busy = 0;           // systems admitted and not yet delivered: the device copy stays
    int64_t last_use = 0;   // LRU clock at the last admission or delivery
    int uses = 0;           // requests submitted and not yet delivered
    bool removed = false;   // mtjg_server_remove_matrix: freed once uses reaches 0
    // (every field but dev and the host arrays is read and written under the server lock)
};

void free_matrix(ResMat *m)
{
    m->dev.release();
    delete m;
}

// Copies a matrix into a fresh device allocation on u's stream and makes its
// FP32 values there; returns once the copy is complete.
int upload_matrix(mtjg_ctx *u, const ResMat *m, const int *rowptr, const int *colind, const double *val,
                  DevMat &d)
{
    const int n = m->n;
    const int64_t nnz = m->nnz;
    const MatLayout L(n, nnz);
    DevMat t;
    if (cudaMalloc(&t.base, L.bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(MTJG_ERR_OUT_OF_MEMORY, "no device memory for a served matrix");
    }
    char *b = static_cast<char *>(t.base);
    t.rowptr = reinterpret_cast<int *>(b + L.rowptr);
    t.colind = reinterpret_cast<int *>(b + L.colind);
    t.val = reinterpret_cast<double *>(b + L.val);
    t.val32 = reinterpret_cast<float *>(b + L.val32);
    t.invdiag32 = reinterpret_cast<float *>(b + L.invdiag32);
    int pad[kRowptrPad];
    for (int k = 0; k < kRowptrPad; ++k) pad[k] = rowptr[n];
    cudaStream_t s = u->stream;
    cudaError_t e = cudaMemcpyAsync(t.rowptr, rowptr, sizeof(int) * ((size_t)n + 1), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t.rowptr + n + 1, pad, sizeof(pad), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(t.colind + nnz, 0xff, sizeof(int) * 4, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(t.val + nnz, 0, sizeof(double) * 2, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(t.val32 + nnz, 0, sizeof(float) * 4, s);
    if (e == cudaSuccess && nnz)
        e = cudaMemcpyAsync(t.colind, colind, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nnz)
        e = cudaMemcpyAsync(t.val, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t.invdiag32, m->inv32.data(), sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && nnz) {
        k_to_f32<<<u->num_sms * 8, kBlock, 0, s>>>(nnz, t.val, t.val32);
        u->launches++;
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(s);
        t.release();
        return cuda_fail(e, "uploading a served matrix");
    }
    d = t;
    return MTJG_OK;
}

struct Req {
    int64_t ticket = 0;
    int mid = 0;
    int kind = MTJG_CG;     // MTJG_CG: the batched lane; MTJG_GMRES / MTJG_BICGSTAB: the Krylov lane
    ResMat *mat = nullptr;  // fixed at submission (the matrix table may grow meanwhile)
    std::vector<double> b, x0;
    double *x_out = nullptr;
    double t_submit = 0, t_admit = 0;
    int slot = -1;
    int voff = -1;
    int64_t first_chunk = 0;      // the first chunk the system runs in
};

// device array that grows on demand (with slack: regrowth frees, which
// waits for the device)
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;
    int ensure(size_t n)
    {
        if (n <= cap) return MTJG_OK;
        cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t c = std::max<size_t>(n + n / 2, 1024);
        MTJG_CUDA(cudaMalloc(&p, sizeof(T) * c));
        cap = c;
        return MTJG_OK;
    }
    ~DevBuf() { cudaFree(p); }
};

// pinned host array that grows on demand
template <class T>
struct PinBuf {
    T *p = nullptr;
    size_t cap = 0;
    int ensure(size_t n)
    {
        if (n <= cap) return MTJG_OK;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t c = std::max<size_t>(n + n / 2, 1024);
        MTJG_CUDA(cudaHostAlloc((void **)&p, sizeof(T) * c, cudaHostAllocDefault));
        cap = c;
        return MTJG_OK;
    }
    ~PinBuf()
    {
        if (p) cudaFreeHost(p);
    }
};

// A finished system whose x is on its way to the pinned staging area.
struct Retired {
    Req *r;
    mtjg_server_result out;
};

}  // namespace
}  // namespace mtjg

using namespace mtjg;

struct mtjg_server {
    mtjg_ctx *ctx = nullptr;   // the scheduler's own context (own stream), on the caller's device
    mtjg_ctx *uctx = nullptr;  // matrix registration (own stream, so uploads never wait for chunks)
    mtjg_ctx *lctx = nullptr;  // the scheduler's uploads of evicted matrices
    mtjg_ctx *kctx = nullptr;  // the Krylov lane (GMRES / BiCGstab requests): own stream
    std::mutex up_mu;          // registering threads share uctx
    mtjg_server_config cfg{};
    std::vector<ResMat *> mats;
    std::mutex mats_mu;
    // pooled vectors: row offsets [0, pool_rows)
    double *b64 = nullptr, *x64 = nullptr;
    float *d32 = nullptr, *rin = nullptr, *z32 = nullptr, *p32 = nullptr, *q32 = nullptr, *inv32 = nullptr;
    // pinned staging at the same row offsets: b and x0 in, x out
    double *h_b = nullptr, *h_x0 = nullptr, *h_x = nullptr;
    std::map<int, int> free_seg;  // start -> length
    // slots
    SysState *st = nullptr;       // device [max_systems]
    SysDesc *sd = nullptr;        // device [max_systems]
    std::vector<SysDesc> h_sd;    // the live table (host)
    std::vector<Req *> slot_req;
    int active = 0;
    int64_t active_rows = 0;
    // per chunk parity: status snapshot, error flag, staged uploads, events
    SysState *h_snap[2] = {nullptr, nullptr};
    int *h_flag[2] = {nullptr, nullptr};
    SysState *h_init[2] = {nullptr, nullptr};
    SysDesc *h_sdst[2] = {nullptr, nullptr};
    PinBuf<int> h_tiles[2];
    cudaEvent_t ev_start[2] = {}, ev_done[2] = {}, ev_ret[2] = {};
    // tiles of the current composition (one device blob)
    DevBuf<int> d_tiles;
    DevBuf<double> part;
    TileSet ptiles, ptiles32, rtiles;  // FP64 product tiles, FP32 product tiles, row tiles
    int *num_running = nullptr;
    unsigned *cnt = nullptr;
    bool dirty = true;
    // queue
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<Req *> pending;
    std::deque<Req *> lane_pending;  // GMRES / BiCGstab requests, FIFO
    std::condition_variable lane_cv;
    std::thread lane;
    std::deque<mtjg_server_result> done;
    int64_t next_ticket = 1;
    int64_t inflight = 0;
    bool stop = false;
    int error = MTJG_OK;
    std::string error_msg;
    std::thread th;
    std::chrono::steady_clock::time_point t0;
    // residency (under mu)
    int64_t resident_bytes = 0, use_clock = 0, uploads = 0, evictions = 0, upload_seq = 0;
    // statistics
    int64_t chunks = 0, admitted = 0, retired = 0, max_active = 0;
    double gpu_s = 0, host_s = 0, wait_s = 0, row_chunks = 0;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

namespace {

int seg_alloc(mtjg_server *S, int n)
{
    for (auto it = S->free_seg.begin(); it != S->free_seg.end(); ++it) {
        if (it->second >= n) {
            const int start = it->first, len = it->second;
            S->free_seg.erase(it);
            if (len > n) S->free_seg[start + n] = len - n;
            return start;
        }
    }
    return -1;
}

void seg_free(mtjg_server *S, int start, int n)
{
    auto it = S->free_seg.emplace(start, n).first;
    // merge with the next and the previous segment
    auto nx = std::next(it);
    if (nx != S->free_seg.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        S->free_seg.erase(nx);
    }
    if (it != S->free_seg.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            S->free_seg.erase(it);
        }
    }
}

// Host tables of one product tiling (tiles of admitted systems, slot order).
struct ProdTables {
    std::vector<int> row, rend, nz, nzend, sys, grp, ginfo, sysg{0};
    std::vector<unsigned char> flags;
    int vec_mask = 0;
    int group_div = 4096;  // a system of T tiles forms groups of clamp(T / group_div, 1, kGroupTiles) tiles
    void add(const ProdTiles &mt, int s)
    {
        const int T = (int)mt.row.size(), t0 = (int)row.size();
        const int gs = std::max(1, std::min(kGroupTiles, T / group_div));
        // groups of up to gs tiles of one lanes-per-row class
        for (int k = 0, k0 = 0; k < T; ++k) {
            if (k == 0 || k - k0 == gs || (mt.flags[k] >> 1) != (mt.flags[k0] >> 1)) {
                ginfo.push_back((s << 8) | (mt.flags[k] >> 1));
                grp.push_back(t0 + k);
                k0 = k;
            }
            vec_mask |= mt.flags[k] >> 1;
        }
        row.insert(row.end(), mt.row.begin(), mt.row.end());
        rend.insert(rend.end(), mt.row_end.begin(), mt.row_end.end());
        nz.insert(nz.end(), mt.nz.begin(), mt.nz.end());
        nzend.insert(nzend.end(), mt.nz_end.begin(), mt.nz_end.end());
        sys.insert(sys.end(), T, s);
        flags.insert(flags.end(), mt.flags.begin(), mt.flags.end());
    }
};

// Rebuilds the product tiles (FP64 and FP32 tilings) and row tiles of the
// admitted systems (slot order) into the pinned blob of parity `par`, and
// queues its upload.
int rebuild_tiles(mtjg_server *S, int par)
{
    const int ns = S->cfg.max_systems;
    ProdTables p64, p32;
    // the served batch spreads over its many systems, so the FP32 tiling (the
    // inner iterations) takes larger groups: fewer block-wide reductions
    p32.group_div = kBatchGroupDiv;
    std::vector<int> rrow, rrend, rsys, rgrp, rsysg{0};
    for (int s = 0; s < ns; ++s) {
        const Req *r = S->slot_req[s];
        if (r) {
            const ResMat *m = r->mat;
            p64.add(m->t64, s);
            p32.add(m->t32, s);
            for (int row = 0; row < m->n; row += kRowTileRows) {
                rgrp.push_back((int)rrow.size());
                rrow.push_back(r->voff + row);
                rrend.push_back(r->voff + std::min(m->n, row + kRowTileRows));
                rsys.push_back(s);
            }
        }
        p64.sysg.push_back((int)p64.grp.size());
        p32.sysg.push_back((int)p32.grp.size());
        rsysg.push_back((int)rgrp.size());
    }
    for (ProdTables *p : {&p64, &p32}) p->grp.push_back((int)p->row.size());
    rgrp.push_back((int)rrow.size());
    const int NR = (int)rrow.size();
    // one blob: the int arrays back to back, then the flag bytes
    std::vector<const std::vector<int> *> ints = {&p64.row, &p64.rend, &p64.nz,  &p64.nzend, &p64.sys,  &p64.grp,
                                                  &p64.ginfo, &p64.sysg, &p32.row, &p32.rend, &p32.nz,   &p32.nzend,
                                                  &p32.sys, &p32.grp,  &p32.ginfo, &p32.sysg, &rrow, &rrend,
                                                  &rsys,    &rgrp,     &rsysg};
    std::vector<size_t> off;
    size_t total = 0;
    for (auto *v : ints) {
        off.push_back(total);
        total += v->size();
    }
    const size_t o_flags = total;
    const size_t nflags = p64.flags.size() + p32.flags.size() + (size_t)NR;
    total += (nflags + 3) / 4 + 1;
    int st = S->h_tiles[par].ensure(total);
    if (st != MTJG_OK) return st;
    int *h = S->h_tiles[par].p;
    for (size_t i = 0; i < ints.size(); ++i)
        if (!ints[i]->empty()) std::memcpy(h + off[i], ints[i]->data(), sizeof(int) * ints[i]->size());
    unsigned char *hf = reinterpret_cast<unsigned char *>(h + o_flags);
    if (!p64.flags.empty()) std::memcpy(hf, p64.flags.data(), p64.flags.size());
    if (!p32.flags.empty()) std::memcpy(hf + p64.flags.size(), p32.flags.data(), p32.flags.size());
    std::memset(hf + p64.flags.size() + p32.flags.size(), 2, (size_t)NR);
    if ((st = S->d_tiles.ensure(total)) != MTJG_OK) return st;
    MTJG_CUDA(cudaMemcpyAsync(S->d_tiles.p, h, sizeof(int) * total, cudaMemcpyHostToDevice, S->ctx->stream));
    const int NG = std::max((int)p64.grp.size(), (int)p32.grp.size());
    if ((st = S->part.ensure((size_t)std::max(NG, NR) * kParts + kParts)) != MTJG_OK) return st;
    int *d = S->d_tiles.p;
    unsigned char *df = reinterpret_cast<unsigned char *>(d + o_flags);
    auto set_prod = [&](TileSet &P, const ProdTables &p, size_t k0, unsigned char *flags) {
        P.num_tiles = (int)p.row.size();
        P.num_groups = (int)p.grp.size() - 1;
        P.num_sys = ns;
        P.vec = 1;
        P.vec_mask = p.vec_mask;
        P.tile_row = d + off[k0];
        P.tile_row_end = d + off[k0 + 1];
        P.tile_nz = d + off[k0 + 2];
        P.tile_nz_end = d + off[k0 + 3];
        P.tile_sys = d + off[k0 + 4];
        P.group_tile = d + off[k0 + 5];
        P.group_info = d + off[k0 + 6];
        P.sys_group = d + off[k0 + 7];
        P.tile_flags = flags;
        P.sd = S->sd;
    };
    set_prod(S->ptiles, p64, 0, df);
    set_prod(S->ptiles32, p32, 8, df + p64.flags.size());
    TileSet &R = S->rtiles;
    R.num_tiles = NR;
    R.num_groups = NR;
    R.num_sys = ns;
    R.vec = 1;
    R.vec_mask = 1;
    R.tile_row = d + off[16];
    R.tile_row_end = d + off[17];
    R.tile_nz = nullptr;
    R.tile_nz_end = nullptr;
    R.tile_sys = d + off[18];
    R.group_tile = d + off[19];
    R.group_info = nullptr;
    R.sys_group = d + off[20];
    R.tile_flags = df + p64.flags.size() + p32.flags.size();
    R.sd = S->sd;
    return MTJG_OK;
}

constexpr int kServeBodies = 2;

// One chunk: kServeBodies x (outer step + kInnerPerBody inner iterations).
int run_chunk(mtjg_server *S)
{
    mtjg_ctx *ctx = S->ctx;
    const RedCtx rc{S->part.p, S->cnt, nullptr, S->num_running};
    MonCfgDev mon;
    mon.max_iter = S->cfg.max_iter;
    mon.norm = MTJG_NORM_TWO;
    mon.hist_cap = 0;
    mon.xmon = 0;
    mon.rtol = S->cfg.rtol;
    mon.atol = S->cfg.atol;
    mon.dtol = S->cfg.dtol;
    const MonPtrs mp{S->st, mon, nullptr, nullptr, S->num_running};
    const MixCfg mix{S->cfg.inner_rtol, S->cfg.inner_max_iter, 0, S->cfg.rtol, S->cfg.atol};
    const int norm = MTJG_NORM_TWO;
    const CsrArgs none64{nullptr, nullptr, nullptr};
    const CsrArgsT<float> none32{nullptr, nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    for (int bdy = 0; bdy < kServeBodies && e == cudaSuccess; ++bdy) {
        e = launch_rows(ctx, S->rtiles, MxX{S->x64, S->d32, S->st}, rc, norm);
        if (e == cudaSuccess)
            e = launch_spmv(ctx, none64, S->ptiles, (const double *)S->x64,
                            MxOuter{S->b64, S->rin, S->z32, S->d32, S->inv32, kPcJacobi, mp}, rc, norm);
        for (int k = 0; k < kInnerPerBody && e == cudaSuccess; ++k) {
            e = launch_rows(ctx, S->rtiles, MxP{S->p32, S->z32, S->st}, rc, norm);
            if (e == cudaSuccess)
                e = launch_spmv(ctx, none32, S->ptiles32, (const float *)S->p32, MxQ{S->q32, S->st}, rc, norm);
            if (e == cudaSuccess)
                e = launch_rows(ctx, S->rtiles,
                                MxUpd{S->d32, S->rin, S->z32, S->p32, S->q32, S->inv32, kPcJacobi, S->st, mix}, rc,
                                norm);
        }
    }
    if (e != cudaSuccess) return cuda_fail(e, "server chunk");
    return MTJG_OK;
}

void fail_all(mtjg_server *S, int code, const std::string &msg)
{
    std::lock_guard<std::mutex> lk(S->mu);
    S->error = code;
    S->error_msg = msg;
    S->cv_done.notify_all();
}

double since(std::chrono::steady_clock::time_point a)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
}

// Hands the finished systems staged by the previous status pass to the
// caller (their x has reached the pinned area once ev_ret[par] is done).
int deliver(mtjg_server *S, std::vector<Retired> &staged, int par)
{
    if (staged.empty()) return MTJG_OK;
    MTJG_CUDA(cudaEventSynchronize(S->ev_ret[par]));
    const double tn = S->now();
    // matrices whose last request this delivers are unlinked under the lock
    // and freed after it (cudaFree waits for the device; submit and poll
    // must not wait with it)
    std::vector<ResMat *> release;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        for (Retired &f : staged) {
            std::memcpy(f.r->x_out, S->h_x + f.r->voff, sizeof(double) * (size_t)f.r->mat->n);
            f.out.latency_s = tn - f.r->t_submit;
            S->done.push_back(f.out);
            ResMat *m = f.r->mat;
            // no queued chunk reads a delivered system's matrix: it may be
            // evicted from here on
            m->busy--;
            m->last_use = ++S->use_clock;
            if (--m->uses == 0 && m->removed) {
                release.push_back(m);
                S->mats[f.r->mid] = nullptr;
                if (m->resident) S->resident_bytes -= m->bytes;
            }
            delete f.r;
        }
        S->inflight -= (int64_t)staged.size();
        S->cv_done.notify_all();
    }
    staged.clear();
    for (ResMat *m : release) free_matrix(m);
    return MTJG_OK;
}

// Makes room in the matrix budget for `need` more bytes by evicting idle
// resident matrices, least recently used first; their device copies are
// moved to `evict` (freed by the caller outside the lock).  Evicts nothing
// and returns false when the idle matrices cannot free enough.  Under mu.
bool make_room(mtjg_server *S, int64_t need, std::vector<DevMat> &evict)
{
    const int64_t B = S->cfg.matrix_budget;
    if (B <= 0 || S->resident_bytes + need <= B) return true;
    std::vector<ResMat *> idle;
    for (ResMat *q : S->mats)
        if (q && q->resident && q->busy == 0) idle.push_back(q);
    std::sort(idle.begin(), idle.end(), [](const ResMat *a, const ResMat *b) { return a->last_use < b->last_use; });
    int64_t freed = 0;
    size_t k = 0;
    while (k < idle.size() && S->resident_bytes - freed + need > B) freed += idle[k++]->bytes;
    if (S->resident_bytes - freed + need > B) return false;
    for (size_t i = 0; i < k; ++i) {
        ResMat *q = idle[i];
        evict.push_back(q->dev);
        q->dev = DevMat();
        q->resident = false;
        S->resident_bytes -= q->bytes;
        S->evictions++;
    }
    return true;
}

void scheduler(mtjg_server *S)
{
    cudaSetDevice(S->ctx->device);
    mtjg_ctx *ctx = S->ctx;
    const int ns = S->cfg.max_systems;
    int64_t launched = 0, processed = 0;  // chunks queued / whose statuses were read
    std::vector<Retired> staged;          // retired, x on its way to the pinned area
    int staged_par = 0;
    auto fatal = [&](int code) {
        fail_all(S, code, mtjg_last_error());
        cudaStreamSynchronize(ctx->stream);
    };
    for (;;) {
        // 1. wait for the oldest queued chunk when two are queued (or when
        //    nothing else can be queued), then read its statuses
        const bool idle = S->active == 0;
        if (launched - processed == 2 || (launched > processed && idle)) {
            const int par = (int)(processed % 2);
            auto tw = std::chrono::steady_clock::now();
            cudaError_t e = cudaEventSynchronize(S->ev_done[par]);
            const double waited = since(tw);
            if (e != cudaSuccess) return fatal(cuda_fail(e, "server chunk"));
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, S->ev_start[par], S->ev_done[par]) != cudaSuccess) ms = 0.f;
            {
                std::lock_guard<std::mutex> lk(S->mu);
                S->gpu_s += 1e-3 * ms;
                S->wait_s += waited;
            }
            if (S->h_flag[par][0]) return fatal(fail(MTJG_ERR_DEVICE_TIMEOUT, "a bounded wait in a device kernel gave up"));
            auto th = std::chrono::steady_clock::now();
            if (deliver(S, staged, staged_par) != MTJG_OK) return fatal(MTJG_ERR_CUDA);
            const SysState *snap = S->h_snap[par];
            for (int s = 0; s < ns; ++s) {
                Req *r = S->slot_req[s];
                if (!r || r->first_chunk > processed || snap[s].status == ST_RUNNING) continue;
                const ResMat *m = r->mat;
                cudaMemcpyAsync(S->h_x + r->voff, S->x64 + r->voff, sizeof(double) * (size_t)m->n,
                                cudaMemcpyDeviceToHost, ctx->stream);
                const SysState &q = snap[s];
                Retired f;
                f.r = r;
                std::memset(&f.out, 0, sizeof(f.out));
                f.out.ticket = r->ticket;
                f.out.matrix = r->mid;
                f.out.result.status = q.status == ST_DONE ? MTJG_OK : q.status;
                f.out.result.iterations = q.iter;
                f.out.result.residual = q.residual;
                f.out.result.detail = q.detail;
                f.out.result.history_len = q.hist_len;
                f.out.result.inner_iterations = q.in_total;
                f.out.queue_s = r->t_admit - r->t_submit;
                staged.push_back(f);
                // the segment's D2H is queued before any later upload into it
                seg_free(S, r->voff, m->n);
                S->slot_req[s] = nullptr;
                S->h_sd[s] = SysDesc{nullptr, nullptr, nullptr, nullptr, 0, 0};
                S->active--;
                S->active_rows -= m->n;
                S->retired++;
                S->dirty = true;
            }
            staged_par = par;
            cudaEventRecord(S->ev_ret[par], ctx->stream);
            ++processed;
            const double spent = since(th);
            {
                std::lock_guard<std::mutex> lk(S->mu);
                S->host_s += spent;
            }
            continue;  // the next pass delivers, admits and queues
        }
        // 2. admission (FIFO while a slot, a workspace segment and room for
        //    the request's matrix are free)
        std::vector<Req *> admit;
        std::vector<ResMat *> load;  // matrices to upload before their systems run
        std::vector<DevMat> evict;   // device copies of evicted matrices
        {
            std::unique_lock<std::mutex> lk(S->mu);
            if (launched == processed && staged.empty())
                S->cv.wait_for(lk, std::chrono::milliseconds(2),
                               [&] { return S->stop || !S->pending.empty() || S->active > 0; });
            // destroy abandons queued and running requests between chunks
            if (S->stop || S->error != MTJG_OK) {
                lk.unlock();
                cudaStreamSynchronize(ctx->stream);
                for (Retired &f : staged) delete f.r;
                return;
            }
            while (!S->pending.empty()) {
                Req *r = S->pending.front();
                ResMat *m = r->mat;
                const int n = m->n;
                int slot = -1;
                for (int s = 0; s < ns; ++s)
                    if (!S->slot_req[s]) {
                        slot = s;
                        break;
                    }
                if (slot < 0) break;
                if (!m->resident) {
                    if (m->loading && m->loader != 1) break;  // the Krylov lane is uploading it
                    if (!m->loading) {
                        if (!make_room(S, m->bytes, evict)) break;
                        m->loading = true;
                        m->loader = 1;
                        S->resident_bytes += m->bytes;
                        load.push_back(m);
                    }
                }
                const int voff = seg_alloc(S, n);
                if (voff < 0) break;
                S->pending.pop_front();
                r->slot = slot;
                r->voff = voff;
                r->t_admit = S->now();
                r->first_chunk = launched;
                S->slot_req[slot] = r;
                S->active++;
                S->active_rows += n;
                S->admitted++;
                m->busy++;
                m->last_use = ++S->use_clock;
                admit.push_back(r);
            }
            S->max_active = std::max<int64_t>(S->max_active, S->active);
        }
        auto th = std::chrono::steady_clock::now();
        if (!staged.empty() && launched == processed) {
            if (deliver(S, staged, staged_par) != MTJG_OK) return fatal(MTJG_ERR_CUDA);
        }
        // evictions before uploads: the budget counted the freed bytes already
        for (DevMat &d : evict) d.release();
        for (ResMat *m : load) {
            DevMat d;
            int ust = upload_matrix(S->lctx, m, m->h_rowptr.data(), m->h_colind.data(), m->h_val.data(), d);
            if (ust != MTJG_OK) return fatal(ust);
            std::lock_guard<std::mutex> lk(S->mu);
            m->dev = d;
            m->resident = true;
            m->loading = false;
            m->epoch = ++S->upload_seq;
            S->uploads++;
        }
        const int par = (int)(launched % 2);  // this parity's staging was last read before chunk launched-2
        for (Req *r : admit) {
            const ResMat *m = r->mat;
            const size_t nb = sizeof(double) * (size_t)m->n;
            std::memcpy(S->h_b + r->voff, r->b.data(), nb);
            cudaMemcpyAsync(S->b64 + r->voff, S->h_b + r->voff, nb, cudaMemcpyHostToDevice, ctx->stream);
            if (r->x0.empty()) {
                cudaMemsetAsync(S->x64 + r->voff, 0, nb, ctx->stream);
            } else {
                std::memcpy(S->h_x0 + r->voff, r->x0.data(), nb);
                cudaMemcpyAsync(S->x64 + r->voff, S->h_x0 + r->voff, nb, cudaMemcpyHostToDevice, ctx->stream);
            }
            cudaMemcpyAsync(S->inv32 + r->voff, m->dev.invdiag32, sizeof(float) * (size_t)m->n,
                            cudaMemcpyDeviceToDevice, ctx->stream);
            S->h_sd[r->slot] = SysDesc{m->dev.rowptr, m->dev.colind, m->dev.val, m->dev.val32, r->voff, 0};
            SysState &init = S->h_init[par][r->slot];
            std::memset(&init, 0, sizeof(init));
            init.status = ST_RUNNING;
            init.gate = ST_RUNNING;
            init.rho_1 = init.rho_2 = init.alpha = init.beta = init.omega = 1.0;
            cudaMemcpyAsync(S->st + r->slot, &init, sizeof(SysState), cudaMemcpyHostToDevice, ctx->stream);
            S->dirty = true;
        }
        if (S->active == 0) {
            const double spent = since(th);
            std::lock_guard<std::mutex> lk(S->mu);
            S->host_s += spent;
            continue;
        }
        // 3. tile tables of a changed composition
        if (S->dirty) {
            std::memcpy(S->h_sdst[par], S->h_sd.data(), sizeof(SysDesc) * (size_t)ns);
            cudaMemcpyAsync(S->sd, S->h_sdst[par], sizeof(SysDesc) * (size_t)ns, cudaMemcpyHostToDevice,
                            ctx->stream);
            int st = rebuild_tiles(S, par);
            if (st != MTJG_OK) return fatal(st);
            S->dirty = false;
        }
        // 4. queue the chunk and its status snapshot
        cudaEventRecord(S->ev_start[par], ctx->stream);
        int st = run_chunk(S);
        if (st != MTJG_OK) return fatal(st);
        cudaMemcpyAsync(S->h_snap[par], S->st, sizeof(SysState) * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(S->h_flag[par], ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        cudaEventRecord(S->ev_done[par], ctx->stream);
        ++launched;
        const double spent = since(th);
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->chunks++;
            S->row_chunks += (double)S->active_rows;
            S->host_s += spent;
        }
    }
}

constexpr int kLaneRestart = 30;

// The Krylov lane's solver state for one upload of a matrix and one solver
// kind: a borrowed view of the resident arrays, its Jacobi preconditioner and
// the solver with its workspace.  Kept while that upload is current, so a
// matrix's later requests allocate (and free, which waits for the device)
// nothing; an entry of an evicted upload is never used again and goes when
// the cache needs its place.
struct LaneState {
    int64_t epoch = 0;
    int kind = -1;
    int64_t last = 0;
    mtjg_csr *A = nullptr;
    mtjg_precond *M = nullptr;
    mtjg_solver *sol = nullptr;
    void release()
    {
        mtjg_solver_destroy(sol);
        mtjg_precond_destroy(M);
        mtjg_csr_destroy(A);
        *this = LaneState();
    }
};
constexpr size_t kLaneCache = 4;

// One GMRES / BiCGstab request on the resident, pinned matrix: mixed
// precision with the Jacobi preconditioner and the server's monitor and
// inner settings, through the solver used by mtjg_solver_solve (so the
// result is what a lone solve with these settings gives).
int lane_solve(mtjg_server *S, const Req *r, int64_t epoch, std::vector<LaneState> &cache, int64_t &clock,
               std::vector<double> &x, mtjg_result &res)
{
    mtjg_ctx *c = S->kctx;
    const ResMat *m = r->mat;
    const int n = m->n;
    LaneState *ls = nullptr;
    for (LaneState &e : cache)
        if (e.epoch == epoch && e.kind == r->kind) ls = &e;
    int st = MTJG_OK;
    if (!ls) {
        if (cache.size() >= kLaneCache) {
            auto lru = std::min_element(cache.begin(), cache.end(),
                                        [](const LaneState &a, const LaneState &b) { return a.last < b.last; });
            lru->release();
            ls = &*lru;
        } else {
            cache.emplace_back();
            ls = &cache.back();
        }
        st = csr_borrow(c, n, m->h_rowptr.data(), m->dev.rowptr, m->dev.colind, m->dev.val, m->dev.val32, &ls->A);
        int err_row = 0;
        if (st == MTJG_OK) st = mtjg_precond_create(c, MTJG_PC_JACOBI, n, &ls->M);
        if (st == MTJG_OK) st = mtjg_precond_set_matrix(ls->M, ls->A, &err_row);
        if (st == MTJG_OK) st = mtjg_solver_create(c, r->kind, n, kLaneRestart, &ls->sol);
        if (st == MTJG_OK) st = mtjg_solver_set_precond(ls->sol, ls->M);
        mtjg_monitor mon;
        mtjg_monitor_defaults(&mon);
        mon.max_iter = S->cfg.max_iter;
        mon.rtol = S->cfg.rtol;
        mon.atol = S->cfg.atol;
        mon.dtol = S->cfg.dtol;
        if (st == MTJG_OK) st = mtjg_solver_set_monitor(ls->sol, &mon);
        if (st == MTJG_OK) st = mtjg_solver_set_mixed(ls->sol, 1, S->cfg.inner_rtol, S->cfg.inner_max_iter);
        if (st != MTJG_OK) {
            ls->release();
            return st;
        }
        ls->epoch = epoch;
        ls->kind = r->kind;
    }
    ls->last = ++clock;
    if (r->x0.empty())
        x.assign((size_t)n, 0.0);
    else
        x = r->x0;
    std::memset(&res, 0, sizeof(res));
    return mtjg_solver_solve(ls->sol, ls->A, r->b.data(), x.data(), &res);
}

// The Krylov lane: makes each request's matrix resident (evicting idle ones
// under the budget, as the scheduler does), pins it, solves, delivers.
void lane_worker(mtjg_server *S)
{
    cudaSetDevice(S->kctx->device);
    std::vector<double> x;
    std::vector<LaneState> cache;
    int64_t clock = 0;
    struct Drop {  // the cache goes with the thread, on every way out
        std::vector<LaneState> &c;
        ~Drop()
        {
            for (LaneState &e : c) e.release();
        }
    } drop{cache};
    for (;;) {
        Req *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->lane_cv.wait(lk, [&] { return S->stop || S->error != MTJG_OK || !S->lane_pending.empty(); });
            if (S->stop || S->error != MTJG_OK) return;
            r = S->lane_pending.front();
            S->lane_pending.pop_front();
        }
        ResMat *m = r->mat;
        std::vector<DevMat> evict;
        bool load = false;
        int64_t epoch = 0;
        for (;;) {
            std::unique_lock<std::mutex> lk(S->mu);
            if (S->stop || S->error != MTJG_OK) {
                delete r;
                return;
            }
            if (m->resident) {
                m->busy++;
                epoch = m->epoch;
                break;
            }
            if (!m->loading && make_room(S, m->bytes, evict)) {
                m->loading = true;
                m->loader = 2;
                m->busy++;
                S->resident_bytes += m->bytes;
                load = true;
                break;
            }
            // being uploaded by the scheduler, or the budget is held by busy matrices
            S->lane_cv.wait_for(lk, std::chrono::milliseconds(1));
        }
        r->t_admit = S->now();
        for (DevMat &d : evict) d.release();
        if (load) {
            DevMat d;
            const int ust = upload_matrix(S->kctx, m, m->h_rowptr.data(), m->h_colind.data(), m->h_val.data(), d);
            if (ust != MTJG_OK) {
                fail_all(S, ust, mtjg_last_error());
                delete r;
                return;
            }
            std::lock_guard<std::mutex> lk(S->mu);
            m->dev = d;
            m->resident = true;
            m->loading = false;
            m->loader = 0;
            m->epoch = ++S->upload_seq;
            epoch = m->epoch;
            S->uploads++;
        }
        mtjg_result res;
        const int st = lane_solve(S, r, epoch, cache, clock, x, res);
        if (st >= MTJG_ERR_CUDA) {
            fail_all(S, st, mtjg_last_error());
            std::lock_guard<std::mutex> lk(S->mu);
            m->busy--;
            delete r;
            return;
        }
        ResMat *release = nullptr;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            std::memcpy(r->x_out, x.data(), sizeof(double) * (size_t)m->n);
            mtjg_server_result out;
            std::memset(&out, 0, sizeof(out));
            out.ticket = r->ticket;
            out.matrix = r->mid;
            out.result = res;
            out.result.status = st;
            out.latency_s = S->now() - r->t_submit;
            out.queue_s = r->t_admit - r->t_submit;
            S->done.push_back(out);
            m->busy--;
            m->last_use = ++S->use_clock;
            if (--m->uses == 0 && m->removed) {
                release = m;
                S->mats[r->mid] = nullptr;
                if (m->resident) S->resident_bytes -= m->bytes;
            }
            S->admitted++;
            S->inflight--;
            S->cv_done.notify_all();
        }
        if (release) free_matrix(release);
        delete r;
    }
}

}  // namespace

extern "C" void mtjg_server_config_defaults(mtjg_server_config *cfg)
{
    if (!cfg) return;
    cfg->max_systems = 256;
    cfg->pool_rows = 1 << 24;
    cfg->max_iter = 100;
    cfg->rtol = 1e-10;
    cfg->atol = 1e-50;
    cfg->dtol = 1e+5;
    cfg->inner_rtol = 1e-6;
    cfg->inner_max_iter = 2000;
    cfg->matrix_budget = 0;
}

extern "C" int mtjg_server_create(mtjg_ctx *ctx, const mtjg_server_config *cfg, mtjg_server **out)
{
    if (!ctx || !cfg || !out) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (cfg->max_systems <= 0 || cfg->pool_rows <= 0 || cfg->pool_rows >= (1LL << 31) || cfg->max_iter < 0 ||
        !(cfg->inner_rtol > 0 && cfg->inner_rtol < 1) || cfg->inner_max_iter <= 0 || cfg->matrix_budget < 0)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "bad server configuration");
    MTJG_CUDA(cudaSetDevice(ctx->device));
    // the scheduler thread and matrix registration work on streams of their
    // own, so the caller's context stays free for other work
    mtjg_ctx *own = nullptr, *up = nullptr, *ld = nullptr, *kr = nullptr;
    int cst = mtjg_ctx_create(ctx->device, &own);
    if (cst != MTJG_OK) return cst;
    cst = mtjg_ctx_create(ctx->device, &up);
    if (cst == MTJG_OK) cst = mtjg_ctx_create(ctx->device, &ld);
    if (cst == MTJG_OK) cst = mtjg_ctx_create(ctx->device, &kr);
    if (cst != MTJG_OK) {
        mtjg_ctx_destroy(own);
        if (up) mtjg_ctx_destroy(up);
        if (ld) mtjg_ctx_destroy(ld);
        return cst;
    }
    mtjg_server *S = new mtjg_server();
    S->ctx = own;
    S->uctx = up;
    S->lctx = ld;
    S->kctx = kr;
    S->cfg = *cfg;
    S->t0 = std::chrono::steady_clock::now();
    const size_t P = (size_t)cfg->pool_rows, ns = (size_t)cfg->max_systems;
    bool ok = cudaMalloc(&S->b64, 8 * P) == cudaSuccess && cudaMalloc(&S->x64, 8 * P) == cudaSuccess &&
              cudaMalloc(&S->d32, 4 * P) == cudaSuccess && cudaMalloc(&S->rin, 4 * P) == cudaSuccess &&
              cudaMalloc(&S->z32, 4 * P) == cudaSuccess && cudaMalloc(&S->p32, 4 * P) == cudaSuccess &&
              cudaMalloc(&S->q32, 4 * P) == cudaSuccess && cudaMalloc(&S->inv32, 4 * P) == cudaSuccess &&
              cudaMalloc(&S->st, sizeof(SysState) * ns) == cudaSuccess &&
              cudaMalloc(&S->sd, sizeof(SysDesc) * ns) == cudaSuccess &&
              cudaMalloc(&S->num_running, sizeof(int) * 4) == cudaSuccess &&
              cudaMalloc(&S->cnt, sizeof(unsigned) * ns) == cudaSuccess &&
              cudaHostAlloc((void **)&S->h_b, 8 * P, cudaHostAllocDefault) == cudaSuccess &&
              cudaHostAlloc((void **)&S->h_x0, 8 * P, cudaHostAllocDefault) == cudaSuccess &&
              cudaHostAlloc((void **)&S->h_x, 8 * P, cudaHostAllocDefault) == cudaSuccess;
    for (int p = 0; p < 2 && ok; ++p) {
        ok = cudaHostAlloc((void **)&S->h_snap[p], sizeof(SysState) * ns, cudaHostAllocDefault) == cudaSuccess &&
             cudaHostAlloc((void **)&S->h_flag[p], sizeof(int) * 4, cudaHostAllocDefault) == cudaSuccess &&
             cudaHostAlloc((void **)&S->h_init[p], sizeof(SysState) * ns, cudaHostAllocDefault) == cudaSuccess &&
             cudaHostAlloc((void **)&S->h_sdst[p], sizeof(SysDesc) * ns, cudaHostAllocDefault) == cudaSuccess &&
             cudaEventCreate(&S->ev_start[p]) == cudaSuccess && cudaEventCreate(&S->ev_done[p]) == cudaSuccess &&
             cudaEventCreate(&S->ev_ret[p]) == cudaSuccess;
    }
    if (!ok) {
        mtjg_server_destroy(S);
        return fail(MTJG_ERR_OUT_OF_MEMORY, "server workspace does not fit in device or pinned host memory");
    }
    std::vector<SysState> empty(ns);
    std::memset(empty.data(), 0, sizeof(SysState) * ns);
    for (auto &q : empty) q.status = ST_DONE;  // empty slots are not running
    S->h_sd.assign(ns, SysDesc{nullptr, nullptr, nullptr, nullptr, 0, 0});
    S->slot_req.assign(ns, nullptr);
    cudaMemcpy(S->st, empty.data(), sizeof(SysState) * ns, cudaMemcpyHostToDevice);
    cudaMemset(S->num_running, 0, sizeof(int) * 4);
    S->free_seg[0] = (int)cfg->pool_rows;
    S->th = std::thread(scheduler, S);
    S->lane = std::thread(lane_worker, S);
    *out = S;
    return MTJG_OK;
}

extern "C" int mtjg_server_add_matrix(mtjg_server *S, int n, const int *rowptr, const int *colind, const double *val,
                                      int *matrix_id)
{
    if (!S || !matrix_id || !rowptr || (!val && n > 0 && rowptr[n] > 0))
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (n <= 0 || n > S->cfg.pool_rows)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "matrix larger than the server's vector pool");
    int st = csr_validate(n, n, rowptr, colind);
    if (st != MTJG_OK) return st;
    MTJG_CUDA(cudaSetDevice(S->ctx->device));
    ResMat *m = new ResMat();
    m->n = n;
    m->nnz = rowptr[n];
    m->bytes = (int64_t)MatLayout(n, m->nnz).bytes;
    const int64_t B = S->cfg.matrix_budget;
    if (B > 0 && m->bytes > B) {
        delete m;
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "matrix larger than the server's matrix budget (" +
                                                   std::to_string(m->bytes) + " > " + std::to_string(B) + " bytes)");
    }
    // DiagonalPreconditioner.setMatrix (S/DiagonalPreconditioner.java:64-76):
    // 1 / A.get(i,i), the first zero diagonal an error; kept in FP32
    m->inv32.resize((size_t)n);
    for (int i = 0; i < n; ++i) {
        const int *c0 = colind + rowptr[i], *c1 = colind + rowptr[i + 1];
        const int *p = std::lower_bound(c0, c1, i);
        const double d = (p != c1 && *p == i) ? val[p - colind] : 0.0;
        if (d == 0) {
            delete m;
            return fail(MTJG_ERR_ZERO_DIAGONAL, "Zero diagonal on row " + std::to_string(i + 1));
        }
        m->inv32[(size_t)i] = (float)(1 / d);
    }
    m->h_rowptr.assign(rowptr, rowptr + n + 1);  // the Krylov lane's tiles
    if (B > 0) {
        m->h_colind.assign(colind, colind + m->nnz);
        m->h_val.assign(val, val + m->nnz);
    }
    // uploaded now if it fits the budget without evicting, else on its first request
    bool now;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        now = B == 0 || S->resident_bytes + m->bytes <= B;
        if (now) S->resident_bytes += m->bytes;
    }
    if (now) {
        std::lock_guard<std::mutex> ul(S->up_mu);
        st = upload_matrix(S->uctx, m, rowptr, colind, val, m->dev);
        if (st != MTJG_OK) {
            std::lock_guard<std::mutex> lk(S->mu);
            S->resident_bytes -= m->bytes;
            delete m;
            return st;
        }
        m->resident = true;
    }
    // the matrix's own product tiles: FP64 as mtjg_csr_upload plans them,
    // and larger FP32 tiles for the inner products
    const int vec = choose_vec(m->nnz, n);
    m->t64.plan(rowptr, n, vec, kTileNnz, kTileRows);
    m->t32.plan(rowptr, n, vec, kTileNnz32, kTileRows32);
    std::lock_guard<std::mutex> lk(S->mats_mu);
    std::lock_guard<std::mutex> lk2(S->mu);
    *matrix_id = (int)S->mats.size();
    if (now) {
        S->uploads++;
        m->epoch = ++S->upload_seq;
    }
    S->mats.push_back(m);
    return MTJG_OK;
}

extern "C" int mtjg_server_submit(mtjg_server *S, int matrix_id, const double *b, const double *x0, double *x_out,
                                  int64_t *ticket)
{
    return mtjg_server_submit_solver(S, matrix_id, MTJG_CG, b, x0, x_out, ticket);
}

extern "C" int mtjg_server_submit_solver(mtjg_server *S, int matrix_id, int solver, const double *b,
                                         const double *x0, double *x_out, int64_t *ticket)
{
    if (!S || !b || !x_out || !ticket) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (solver != MTJG_CG && solver != MTJG_GMRES && solver != MTJG_BICGSTAB)
        return fail(MTJG_ERR_UNSUPPORTED, "the server solves with CG, GMRES or BiCGstab");
    Req *r = new Req();
    r->kind = solver;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->error != MTJG_OK) {
            delete r;
            return fail(S->error, S->error_msg);
        }
        if (matrix_id < 0 || matrix_id >= (int)S->mats.size() || !S->mats[matrix_id] ||
            S->mats[matrix_id]->removed) {
            delete r;
            return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "unknown or removed matrix id");
        }
        r->mid = matrix_id;
        r->mat = S->mats[matrix_id];
        S->mats[matrix_id]->uses++;
        const int n = r->mat->n;
        r->b.assign(b, b + n);
        if (x0) r->x0.assign(x0, x0 + n);
        r->x_out = x_out;
        r->t_submit = S->now();
        r->ticket = S->next_ticket++;
        *ticket = r->ticket;
        (solver == MTJG_CG ? S->pending : S->lane_pending).push_back(r);
        S->inflight++;
    }
    if (solver == MTJG_CG)
        S->cv.notify_one();
    else
        S->lane_cv.notify_one();
    return MTJG_OK;
}

extern "C" int mtjg_server_remove_matrix(mtjg_server *S, int matrix_id)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL server");
    ResMat *release = nullptr;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (matrix_id < 0 || matrix_id >= (int)S->mats.size() || !S->mats[matrix_id] ||
            S->mats[matrix_id]->removed)
            return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "unknown or removed matrix id");
        ResMat *m = S->mats[matrix_id];
        m->removed = true;
        if (m->uses == 0) {
            release = m;
            S->mats[matrix_id] = nullptr;
            if (m->resident) S->resident_bytes -= m->bytes;
        }
    }
    // freed outside the lock: cudaFree waits for the device
    if (release) free_matrix(release);
    return MTJG_OK;
}

extern "C" int mtjg_server_poll(mtjg_server *S, mtjg_server_result *out, int cap, int *count)
{
    if (!S || !count || (cap > 0 && !out)) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    std::lock_guard<std::mutex> lk(S->mu);
    int k = 0;
    while (k < cap && !S->done.empty()) {
        out[k++] = S->done.front();
        S->done.pop_front();
    }
    *count = k;
    if (S->error != MTJG_OK) return fail(S->error, S->error_msg);
    return MTJG_OK;
}

extern "C" int mtjg_server_drain(mtjg_server *S, double timeout_s)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL server");
    std::unique_lock<std::mutex> lk(S->mu);
    const bool ok = S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [&] { return S->inflight == 0 || S->error != MTJG_OK; });
    if (S->error != MTJG_OK) return fail(S->error, S->error_msg);
    if (!ok) return fail(MTJG_ERR_DEVICE_TIMEOUT, "requests still running after the timeout");
    return MTJG_OK;
}

extern "C" int mtjg_server_stats(mtjg_server *S, int64_t *chunks, int64_t *admitted, int64_t *max_active,
                                 double *clock_s)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> lk(S->mu);
    if (chunks) *chunks = S->chunks;
    if (admitted) *admitted = S->admitted;
    if (max_active) *max_active = S->max_active;
    if (clock_s) *clock_s = S->now();
    return MTJG_OK;
}

extern "C" int mtjg_server_residency(mtjg_server *S, int64_t *resident_bytes, int64_t *resident_matrices,
                                     int64_t *uploads, int64_t *evictions)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> lk(S->mu);
    int64_t k = 0;
    for (const ResMat *m : S->mats)
        if (m && (m->resident || m->loading)) ++k;
    if (resident_bytes) *resident_bytes = S->resident_bytes;
    if (resident_matrices) *resident_matrices = k;
    if (uploads) *uploads = S->uploads;
    if (evictions) *evictions = S->evictions;
    return MTJG_OK;
}

extern "C" int mtjg_server_timing(mtjg_server *S, double *gpu_s, double *host_s, double *wait_s,
                                  double *mean_rows)
{
    if (!S) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL server");
    std::lock_guard<std::mutex> lk(S->mu);
    if (gpu_s) *gpu_s = S->gpu_s;
    if (host_s) *host_s = S->host_s;
    if (wait_s) *wait_s = S->wait_s;
    if (mean_rows) *mean_rows = S->chunks ? S->row_chunks / (double)S->chunks : 0.0;
    return MTJG_OK;
}

extern "C" int mtjg_server_context(mtjg_server *S, mtjg_ctx **ctx)
{
    if (!S || !ctx) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *ctx = S->ctx;
    return MTJG_OK;
}

extern "C" int mtjg_server_destroy(mtjg_server *S)
{
    if (!S) return MTJG_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    S->lane_cv.notify_all();
    if (S->th.joinable()) S->th.join();
    if (S->lane.joinable()) S->lane.join();
    cudaSetDevice(S->ctx->device);
    cudaStreamSynchronize(S->ctx->stream);
    for (Req *r : S->pending) delete r;
    for (Req *r : S->lane_pending) delete r;
    for (Req *r : S->slot_req) delete r;
    for (ResMat *m : S->mats)
        if (m) free_matrix(m);
    cudaFree(S->b64);
    cudaFree(S->x64);
    cudaFree(S->d32);
    cudaFree(S->rin);
    cudaFree(S->z32);
    cudaFree(S->p32);
    cudaFree(S->q32);
    cudaFree(S->inv32);
    cudaFree(S->st);
    cudaFree(S->sd);
    cudaFree(S->num_running);
    cudaFree(S->cnt);
    cudaFreeHost(S->h_b);
    cudaFreeHost(S->h_x0);
    cudaFreeHost(S->h_x);
    for (int p = 0; p < 2; ++p) {
        cudaFreeHost(S->h_snap[p]);
        cudaFreeHost(S->h_flag[p]);
        cudaFreeHost(S->h_init[p]);
        cudaFreeHost(S->h_sdst[p]);
        if (S->ev_start[p]) cudaEventDestroy(S->ev_start[p]);
        if (S->ev_done[p]) cudaEventDestroy(S->ev_done[p]);
        if (S->ev_ret[p]) cudaEventDestroy(S->ev_ret[p]);
    }
    mtjg_ctx *ctx = S->ctx, *u = S->uctx, *ld = S->lctx, *kr = S->kctx;
    delete S;
    mtjg_ctx_destroy(ctx);
    mtjg_ctx_destroy(u);
    mtjg_ctx_destroy(ld);
    mtjg_ctx_destroy(kr);
    return MTJG_OK;
}
