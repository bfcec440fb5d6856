// server.cu -- continuous-batching solve server.
//
// Matrices are registered once and stay resident on the device (CSR, FP32
// values, Jacobi inverse diagonals).  Requests (matrix, b, x0) queue on the
// host; a scheduler thread admits them into free slots whenever a slot and
// a contiguous segment of the pooled vector workspace are free (admission
// by HBM footprint), runs a chunk of the mixed-precision CG phases over all
// admitted systems at once, and retires finished systems between chunks, so
// requests that arrive while others are on the GPU join the running batch.
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

int precond_apply_dev(mtjg_precond *M, const double *b, double *x, const int *status);

namespace {

struct ResMat {
    int n = 0;
    int64_t nnz = 0;
    mtjg_csr *A = nullptr;          // resident CSR (rows 0..n-1), FP32 values in A->val32
    mtjg_precond *J = nullptr;      // Jacobi (its invdiag)
    float *invdiag32 = nullptr;
    // product tiles of this matrix (local rows and entries), host copies
    std::vector<int> t_row, t_row_end, t_nz, t_nz_end;
    std::vector<unsigned char> t_flags;
};

struct Req {
    int64_t ticket = 0;
    int mid = 0;
    const ResMat *mat = nullptr;  // fixed at submission (the matrix table may grow meanwhile)
    std::vector<double> b, x0;
    double *x_out = nullptr;
    double t_submit = 0, t_admit = 0;
    int slot = -1;
    int voff = -1;
};

// device array that grows on demand
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
        MTJG_CUDA(cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 16)));
        cap = std::max<size_t>(n, 16);
        return MTJG_OK;
    }
    ~DevBuf() { cudaFree(p); }
};

}  // namespace
}  // namespace mtjg

using namespace mtjg;

struct mtjg_server {
    mtjg_ctx *ctx = nullptr;  // the server's own context (own stream), on the caller's device
    mtjg_server_config cfg{};
    std::vector<ResMat *> mats;
    std::mutex mats_mu;
    // pooled vectors: row offsets [0, pool_rows)
    double *b64 = nullptr, *x64 = nullptr;
    float *d32 = nullptr, *rin = nullptr, *z32 = nullptr, *p32 = nullptr, *q32 = nullptr, *inv32 = nullptr;
    std::map<int, int> free_seg;  // start -> length
    // slots
    SysState *st = nullptr;       // device [max_systems]
    SysDesc *sd = nullptr;        // device [max_systems]
    std::vector<SysState> h_st;
    std::vector<SysDesc> h_sd;
    std::vector<Req *> slot_req;
    int active = 0;
    // tiles of the current composition
    DevBuf<int> pt_row, pt_row_end, pt_nz, pt_nz_end, pt_sys, pt_group, pt_sysg;
    DevBuf<unsigned char> pt_flags;
    DevBuf<int> rt_row, rt_row_end, rt_sys, rt_group, rt_sysg;
    DevBuf<unsigned char> rt_flags;
    DevBuf<double> part;
    TileSet ptiles, rtiles;
    int *num_running = nullptr;
    unsigned *cnt = nullptr;
    bool dirty = true;
    // queue
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::deque<Req *> pending;
    std::deque<mtjg_server_result> done;
    int64_t next_ticket = 1;
    int64_t inflight = 0;
    bool stop = false;
    int error = MTJG_OK;
    std::string error_msg;
    std::thread th;
    std::chrono::steady_clock::time_point t0;
    // statistics
    int64_t chunks = 0, admitted = 0, retired = 0, max_active = 0;

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

// Rebuilds the product and row tiles of the admitted systems (slot order).
int rebuild_tiles(mtjg_server *S)
{
    const int ns = S->cfg.max_systems;
    std::vector<int> row, row_end, nz, nz_end, sys, group, sysg = {0};
    std::vector<unsigned char> flags;
    std::vector<int> rrow, rrow_end, rsys, rgroup, rsysg = {0};
    std::vector<unsigned char> rflags;
    int vec_mask = 0;
    for (int s = 0; s < ns; ++s) {
        Req *r = S->slot_req[s];
        if (r) {
            const ResMat *m = r->mat;
            const int t0 = (int)row.size(), T = (int)m->t_row.size();
            row.insert(row.end(), m->t_row.begin(), m->t_row.end());
            row_end.insert(row_end.end(), m->t_row_end.begin(), m->t_row_end.end());
            nz.insert(nz.end(), m->t_nz.begin(), m->t_nz.end());
            nz_end.insert(nz_end.end(), m->t_nz_end.begin(), m->t_nz_end.end());
            flags.insert(flags.end(), m->t_flags.begin(), m->t_flags.end());
            sys.insert(sys.end(), T, s);
            for (unsigned char f : m->t_flags) vec_mask |= f >> 1;
            const int gs = std::max(1, std::min(kGroupTiles, T / 4096));  // as for an uploaded CSR
            for (int t = t0; t < t0 + T; t += gs) group.push_back(t);
            for (int q = 0; q < m->n; q += kRowTile) {
                rrow.push_back(r->voff + q);
                rrow_end.push_back(r->voff + std::min(m->n, q + kRowTile));
                rsys.push_back(s);
                rflags.push_back(2);
                rgroup.push_back((int)rgroup.size());
            }
        }
        sysg.push_back((int)group.size());
        rsysg.push_back((int)rgroup.size());
    }
    const int NT = (int)row.size(), NG = (int)group.size(), NR = (int)rrow.size();
    group.push_back(NT);
    rgroup.push_back(NR);
    auto up_i = [&](DevBuf<int> &d, const std::vector<int> &h) -> int {
        int st = d.ensure(h.size());
        if (st != MTJG_OK) return st;
        if (!h.empty())
            MTJG_CUDA(cudaMemcpyAsync(d.p, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, S->ctx->stream));
        return MTJG_OK;
    };
    auto up_u = [&](DevBuf<unsigned char> &d, const std::vector<unsigned char> &h) -> int {
        int st = d.ensure(h.size());
        if (st != MTJG_OK) return st;
        if (!h.empty()) MTJG_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size(), cudaMemcpyHostToDevice, S->ctx->stream));
        return MTJG_OK;
    };
    int st = MTJG_OK;
    if ((st = up_i(S->pt_row, row)) || (st = up_i(S->pt_row_end, row_end)) || (st = up_i(S->pt_nz, nz)) ||
        (st = up_i(S->pt_nz_end, nz_end)) || (st = up_i(S->pt_sys, sys)) || (st = up_i(S->pt_group, group)) ||
        (st = up_i(S->pt_sysg, sysg)) || (st = up_u(S->pt_flags, flags)) || (st = up_i(S->rt_row, rrow)) ||
        (st = up_i(S->rt_row_end, rrow_end)) || (st = up_i(S->rt_sys, rsys)) || (st = up_i(S->rt_group, rgroup)) ||
        (st = up_i(S->rt_sysg, rsysg)) || (st = up_u(S->rt_flags, rflags)))
        return st;
    st = S->part.ensure((size_t)std::max(NG, NR) * kParts + kParts);
    if (st != MTJG_OK) return st;
    TileSet &P = S->ptiles;
    P.num_tiles = NT;
    P.num_groups = NG;
    P.num_sys = ns;
    P.vec = 1;
    P.vec_mask = vec_mask;
    P.tile_row = S->pt_row.p;
    P.tile_row_end = S->pt_row_end.p;
    P.tile_nz = S->pt_nz.p;
    P.tile_nz_end = S->pt_nz_end.p;
    P.tile_sys = S->pt_sys.p;
    P.tile_flags = S->pt_flags.p;
    P.group_tile = S->pt_group.p;
    P.sys_group = S->pt_sysg.p;
    P.sd = S->sd;
    TileSet &R = S->rtiles;
    R.num_tiles = NR;
    R.num_groups = NR;
    R.num_sys = ns;
    R.vec = 1;
    R.vec_mask = 1;
    R.tile_row = S->rt_row.p;
    R.tile_row_end = S->rt_row_end.p;
    R.tile_nz = nullptr;
    R.tile_nz_end = nullptr;
    R.tile_sys = S->rt_sys.p;
    R.tile_flags = S->rt_flags.p;
    R.group_tile = S->rt_group.p;
    R.sys_group = S->rt_sysg.p;
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
    mon.pad = 0;
    mon.rtol = S->cfg.rtol;
    mon.atol = S->cfg.atol;
    mon.dtol = S->cfg.dtol;
    const MonPtrs mp{S->st, mon, nullptr, nullptr, S->num_running};
    const MixCfg mix{S->cfg.inner_rtol, S->cfg.inner_max_iter};
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
                e = launch_spmv(ctx, none32, S->ptiles, (const float *)S->p32, MxQ{S->q32, S->st}, rc, norm);
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
}

void scheduler(mtjg_server *S)
{
    cudaSetDevice(S->ctx->device);
    mtjg_ctx *ctx = S->ctx;
    const int ns = S->cfg.max_systems;
    for (;;) {
        std::vector<Req *> admit;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv.wait_for(lk, std::chrono::milliseconds(2),
                           [&] { return S->stop || !S->pending.empty() || S->active > 0; });
            // destroy abandons queued and running requests between chunks
            if (S->stop || S->error != MTJG_OK) return;
            // admission: FIFO while a slot and a workspace segment are free
            while (!S->pending.empty()) {
                Req *r = S->pending.front();
                const int n = r->mat->n;
                int slot = -1;
                for (int s = 0; s < ns; ++s)
                    if (!S->slot_req[s]) {
                        slot = s;
                        break;
                    }
                if (slot < 0) break;
                const int voff = seg_alloc(S, n);
                if (voff < 0) break;
                S->pending.pop_front();
                r->slot = slot;
                r->voff = voff;
                r->t_admit = S->now();
                S->slot_req[slot] = r;
                S->active++;
                S->admitted++;
                admit.push_back(r);
            }
            S->max_active = std::max<int64_t>(S->max_active, S->active);
        }
        for (Req *r : admit) {
            const ResMat *m = r->mat;
            const size_t nb = sizeof(double) * (size_t)m->n;
            cudaMemcpyAsync(S->b64 + r->voff, r->b.data(), nb, cudaMemcpyHostToDevice, ctx->stream);
            cudaMemcpyAsync(S->x64 + r->voff, r->x0.data(), nb, cudaMemcpyHostToDevice, ctx->stream);
            cudaMemcpyAsync(S->inv32 + r->voff, m->invdiag32, sizeof(float) * (size_t)m->n, cudaMemcpyDeviceToDevice,
                            ctx->stream);
            SysDesc d{m->A->rowptr, m->A->colind, m->A->val, m->A->val32, r->voff, 0};
            S->h_sd[r->slot] = d;
            SysState init;
            std::memset(&init, 0, sizeof(init));
            init.status = ST_RUNNING;
            init.gate = ST_RUNNING;
            init.rho_1 = init.rho_2 = init.alpha = init.beta = init.omega = 1.0;
            S->h_st[r->slot] = init;
            cudaMemcpyAsync(S->st + r->slot, &S->h_st[r->slot], sizeof(SysState), cudaMemcpyHostToDevice,
                            ctx->stream);
            S->dirty = true;
        }
        if (S->active == 0) continue;
        if (S->dirty) {
            cudaMemcpyAsync(S->sd, S->h_sd.data(), sizeof(SysDesc) * (size_t)ns, cudaMemcpyHostToDevice, ctx->stream);
            int st = rebuild_tiles(S);
            if (st != MTJG_OK) {
                fail_all(S, st, mtjg_last_error());
                return;
            }
            S->dirty = false;
        }
        int st = run_chunk(S);
        if (st != MTJG_OK) {
            fail_all(S, st, mtjg_last_error());
            return;
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->chunks++;
        }
        cudaMemcpyAsync(S->h_st.data(), S->st, sizeof(SysState) * (size_t)ns, cudaMemcpyDeviceToHost, ctx->stream);
        cudaMemcpyAsync(ctx->h_pinned, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            fail_all(S, cuda_fail(e, "server chunk"), mtjg_last_error());
            return;
        }
        if (ctx->h_pinned[0]) {
            fail_all(S, MTJG_ERR_DEVICE_TIMEOUT, "a bounded wait in a device kernel gave up");
            return;
        }
        // retire finished systems
        std::vector<mtjg_server_result> fin;
        for (int s = 0; s < ns; ++s) {
            Req *r = S->slot_req[s];
            if (!r || S->h_st[s].status == ST_RUNNING) continue;
            const ResMat *m = r->mat;
            cudaMemcpy(r->x_out, S->x64 + r->voff, sizeof(double) * (size_t)m->n, cudaMemcpyDeviceToHost);
            const SysState &q = S->h_st[s];
            mtjg_server_result out;
            std::memset(&out, 0, sizeof(out));
            out.ticket = r->ticket;
            out.matrix = r->mid;
            out.result.status = q.status == ST_DONE ? MTJG_OK : q.status;
            out.result.iterations = q.iter;
            out.result.residual = q.residual;
            out.result.detail = q.detail;
            out.result.history_len = q.hist_len;
            out.result.inner_iterations = q.in_total;
            const double tn = S->now();
            out.latency_s = tn - r->t_submit;
            out.queue_s = r->t_admit - r->t_submit;
            fin.push_back(out);
            seg_free(S, r->voff, m->n);
            S->slot_req[s] = nullptr;
            S->h_sd[s] = SysDesc{nullptr, nullptr, nullptr, nullptr, 0, 0};
            S->active--;
            S->retired++;
            S->dirty = true;
            delete r;
        }
        if (!fin.empty()) {
            std::lock_guard<std::mutex> lk(S->mu);
            for (auto &f : fin) S->done.push_back(f);
            S->inflight -= (int64_t)fin.size();
            S->cv_done.notify_all();
        }
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
    cfg->inner_rtol = 1e-4;
    cfg->inner_max_iter = 2000;
}

extern "C" int mtjg_server_create(mtjg_ctx *ctx, const mtjg_server_config *cfg, mtjg_server **out)
{
    if (!ctx || !cfg || !out) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (cfg->max_systems <= 0 || cfg->pool_rows <= 0 || cfg->pool_rows >= (1LL << 31) || cfg->max_iter < 0 ||
        !(cfg->inner_rtol > 0 && cfg->inner_rtol < 1) || cfg->inner_max_iter <= 0)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "bad server configuration");
    MTJG_CUDA(cudaSetDevice(ctx->device));
    // the scheduler thread works on a stream of its own, so the caller's
    // context stays free for other work while requests run
    mtjg_ctx *own = nullptr;
    int cst = mtjg_ctx_create(ctx->device, &own);
    if (cst != MTJG_OK) return cst;
    mtjg_server *S = new mtjg_server();
    S->ctx = own;
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
              cudaMalloc(&S->cnt, sizeof(unsigned) * ns) == cudaSuccess;
    if (!ok) {
        mtjg_server_destroy(S);
        return fail(MTJG_ERR_OUT_OF_MEMORY, "server workspace does not fit in device memory");
    }
    S->h_st.assign(ns, SysState{});
    for (auto &q : S->h_st) q.status = ST_DONE;  // empty slots are not running
    S->h_sd.assign(ns, SysDesc{nullptr, nullptr, nullptr, nullptr, 0, 0});
    S->slot_req.assign(ns, nullptr);
    cudaMemcpy(S->st, S->h_st.data(), sizeof(SysState) * ns, cudaMemcpyHostToDevice);
    cudaMemset(S->num_running, 0, sizeof(int) * 4);
    S->free_seg[0] = (int)cfg->pool_rows;
    S->th = std::thread(scheduler, S);
    *out = S;
    return MTJG_OK;
}

extern "C" int mtjg_server_add_matrix(mtjg_server *S, int n, const int *rowptr, const int *colind, const double *val,
                                      int *matrix_id)
{
    if (!S || !matrix_id) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    if (n <= 0 || n > S->cfg.pool_rows)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "matrix larger than the server's vector pool");
    ResMat *m = new ResMat();
    m->n = n;
    int st = mtjg_csr_upload(S->ctx, n, n, rowptr, colind, val, &m->A);
    if (st == MTJG_OK) st = mtjg_precond_create(S->ctx, MTJG_PC_JACOBI, n, &m->J);
    if (st == MTJG_OK) st = mtjg_precond_set_matrix(m->J, m->A, nullptr);
    if (st != MTJG_OK) {
        mtjg_precond_destroy(m->J);
        mtjg_csr_destroy(m->A);
        delete m;
        return st;
    }
    m->nnz = m->A->nnz;
    const int grid = S->ctx->num_sms * 8;
    MTJG_CUDA(cudaMalloc(&m->A->val32, sizeof(float) * (size_t)(m->nnz + 4)));
    MTJG_CUDA(cudaMemset(m->A->val32, 0, sizeof(float) * (size_t)(m->nnz + 4)));
    MTJG_CUDA(cudaMalloc(&m->invdiag32, sizeof(float) * (size_t)n));
    k_to_f32<<<grid, kBlock, 0, S->ctx->stream>>>(m->nnz, m->A->val, m->A->val32);
    k_to_f32<<<grid, kBlock, 0, S->ctx->stream>>>(n, m->J->invdiag, m->invdiag32);
    MTJG_CUDA(cudaStreamSynchronize(S->ctx->stream));
    // the matrix's own product tiles (as mtjg_csr_upload plans them)
    const int vec = choose_vec(m->nnz, n);
    std::vector<int> tr;
    plan_tiles(rowptr, 0, n, vec, tr, m->t_flags);
    tr.push_back(n);
    for (size_t t = 0; t + 1 < tr.size(); ++t) {
        m->t_row.push_back(tr[t]);
        m->t_row_end.push_back(tr[t + 1]);
        m->t_nz.push_back(rowptr[tr[t]]);
        m->t_nz_end.push_back(rowptr[tr[t + 1]]);
    }
    std::lock_guard<std::mutex> lk(S->mats_mu);
    std::lock_guard<std::mutex> lk2(S->mu);
    *matrix_id = (int)S->mats.size();
    S->mats.push_back(m);
    return MTJG_OK;
}

extern "C" int mtjg_server_submit(mtjg_server *S, int matrix_id, const double *b, const double *x0, double *x_out,
                                  int64_t *ticket)
{
    if (!S || !b || !x_out || !ticket) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    Req *r = new Req();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->error != MTJG_OK) {
            delete r;
            return fail(S->error, S->error_msg);
        }
        if (matrix_id < 0 || matrix_id >= (int)S->mats.size()) {
            delete r;
            return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "unknown matrix id");
        }
        r->mid = matrix_id;
        r->mat = S->mats[matrix_id];
        const int n = r->mat->n;
        r->b.assign(b, b + n);
        if (x0) r->x0.assign(x0, x0 + n);
        else r->x0.assign(n, 0.0);
        r->x_out = x_out;
        r->t_submit = S->now();
        r->ticket = S->next_ticket++;
        *ticket = r->ticket;
        S->pending.push_back(r);
        S->inflight++;
    }
    S->cv.notify_one();
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

extern "C" int mtjg_server_destroy(mtjg_server *S)
{
    if (!S) return MTJG_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv.notify_all();
    if (S->th.joinable()) S->th.join();
    cudaSetDevice(S->ctx->device);
    cudaStreamSynchronize(S->ctx->stream);
    for (Req *r : S->pending) delete r;
    for (Req *r : S->slot_req) delete r;
    for (ResMat *m : S->mats) {
        mtjg_precond_destroy(m->J);
        mtjg_csr_destroy(m->A);
        cudaFree(m->invdiag32);
        delete m;
    }
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
    mtjg_ctx *ctx = S->ctx;
    delete S;
    mtjg_ctx_destroy(ctx);
    return MTJG_OK;
}
