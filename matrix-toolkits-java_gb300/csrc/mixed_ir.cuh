// mixed_ir.cuh -- mixed-precision GMRES(m) and BiCGstab (included by solver.cu).
//
// Iterative refinement in the shape of IR.solve (S/IR.java:57-70): r = b - A x
// in FP64, the monitor's test on it, then a correction d from an FP32 inner
// Krylov solve of A d = r in the role of IR's preconditioner, x += d in FP64.
// The inner solve is right-preconditioned GMRES(m) (CGS2 orthogonalisation,
// FP64 Hessenberg and Givens rotations on the host) or BiCGstab, both on FP32
// vectors, the FP32 matrix values and an FP32 copy of the preconditioner
// (identity, Jacobi, ILU or ILUT; triangular solves by the one-launch level
// sweeps).  Dot products accumulate FP32 products in FP64, per block in a
// fixed grid and then in block order, so they do not depend on timing.
//
// The host drives the inner iterations and reads each iteration's scalars:
// with an ILU preconditioner an inner iteration costs a millisecond or more
// of level-scheduled sweeps, against a few microseconds per read.
//
// Included by solver.cu inside its file-local namespace, after run(); the
// kernels and epilogues are in mixed_ir_phases.cuh.
#pragma once

// The inner solve's device work and the host's reads of its scalars.
struct IrInner {
    mtjg_solver *S;
    mtjg_csr *A;
    int n = 0, G = 0;
    int64_t ld = 0;
    double *part = nullptr, *dev = nullptr;  // partials and reduced scalars (device)
    double *pin = nullptr;                   // reduced scalars (pinned host)
    int total = 0;                           // inner iterations of the whole solve

    cudaStream_t stream() const { return S->ctx->stream; }
    void count() { S->ctx->launches++; }

    int lin(float *out, const float *a, float ca, const float *b, float cb, const float *c, float cc,
            const float *q, bool reduce)
    {
        k_ir_lin<<<G, kIrBlock, 0, stream()>>>(n, out, a, ca, b, cb, c, cc, q, reduce ? part : nullptr);
        count();
        return MTJG_OK;
    }
    // reduces `k` partial slots into dev[0..k) and copies them to pin (no wait)
    void finish(int k)
    {
        k_ir_final<<<k, 32, 0, stream()>>>(part, G, dev);
        count();
        cudaMemcpyAsync(pin, dev, sizeof(double) * (size_t)k, cudaMemcpyDeviceToHost, stream());
    }
    // waits for the queued work; a sweep whose bounded wait gave up ends the solve
    int wait()
    {
        MTJG_CUDA(cudaGetLastError());
        int *flag = S->ctx->h_pinned + 2;
        MTJG_CUDA(cudaMemcpyAsync(flag, S->ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, stream()));
        MTJG_CUDA(cudaStreamSynchronize(stream()));
        if (*flag) {
            cudaMemset(S->ctx->d_flag, 0, sizeof(int));
            return fail(MTJG_ERR_DEVICE_TIMEOUT, "a bounded wait in a device kernel gave up during the solve");
        }
        return MTJG_OK;
    }
    int prod(const float *x, float *y, const float *rhs)
    {
        cudaError_t e = launch_spmv(S->ctx, CsrArgsT<float>{A->rowptr, A->colind, A->val32}, A->tiles, x,
                                    Mi32Prod{y, rhs}, red_ctx(A, A->tiles), MTJG_NORM_TWO);
        if (e != cudaSuccess) return cuda_fail(e, "FP32 product");
        return MTJG_OK;
    }
    // x = M \ b in FP32; with the identity the result is b itself
    int pc(const float *b, float *x, const float **out)
    {
        if (!S->M || S->M->kind == MTJG_PC_IDENTITY) {
            *out = b;
            return MTJG_OK;
        }
        *out = x;
        return precond_apply32(S->M, b, x, nullptr);
    }

    // BiCGstab (right preconditioned) on A d = rin from d = 0 to residual tol.
    int bicgstab(const float *rin, float *d, double rn0, double tol, int in_max, float *w)
    {
        float *r = w, *p = w + ld, *v = w + 2 * ld, *ph = w + 3 * ld, *s = w + 4 * ld, *sh = w + 5 * ld,
              *t = w + 6 * ld;
        MTJG_CUDA(cudaMemsetAsync(d, 0, sizeof(float) * (size_t)n, stream()));
        lin(r, rin, 1.0f, nullptr, 0, nullptr, 0, nullptr, false);
        double rho = rn0 * rn0, rho_1 = 1.0, alpha = 1.0, omega = 1.0;
        for (int it = 0; it < in_max; ++it) {
            if (!(rho != 0.0) || !std::isfinite(rho)) break;
            if (it == 0) {
                lin(p, r, 1.0f, nullptr, 0, nullptr, 0, nullptr, false);
            } else {
                const double beta = (rho / rho_1) * (alpha / omega);
                lin(p, r, 1.0f, p, (float)beta, v, (float)(-beta * omega), nullptr, false);
            }
            const float *php;
            int st = pc(p, ph, &php);
            if (st != MTJG_OK) return st;
            if ((st = prod(php, v, nullptr)) != MTJG_OK) return st;
            k_ir_vdot<<<dim3(G, 1), kIrBlock, 0, stream()>>>(n, rin, 0, v, part);
            count();
            finish(1);
            if ((st = wait()) != MTJG_OK) return st;
            const double rtv = pin[0];
            if (!(rtv != 0.0) || !std::isfinite(rtv)) break;
            alpha = rho / rtv;
            lin(s, r, 1.0f, v, (float)-alpha, nullptr, 0, nullptr, true);
            finish(1);
            if ((st = wait()) != MTJG_OK) return st;
            ++total;
            if (!(sqrt(pin[0]) > tol)) {
                lin(d, d, 1.0f, php, (float)alpha, nullptr, 0, nullptr, false);
                break;
            }
            const float *shp;
            if ((st = pc(s, sh, &shp)) != MTJG_OK) return st;
            if ((st = prod(shp, t, nullptr)) != MTJG_OK) return st;
            k_ir_lin<<<G, kIrBlock, 0, stream()>>>(n, t, t, 1.0f, nullptr, 0, nullptr, 0, s, part);  // t.t, t.s
            count();
            finish(2);
            if ((st = wait()) != MTJG_OK) return st;
            omega = pin[0] > 0.0 ? pin[1] / pin[0] : 0.0;
            lin(d, d, 1.0f, php, (float)alpha, shp, (float)omega, nullptr, false);
            if (omega == 0.0 || !std::isfinite(omega)) break;
            lin(r, s, 1.0f, t, (float)-omega, nullptr, 0, rin, true);  // r.r, rt.r (rt = rin)
            finish(2);
            if ((st = wait()) != MTJG_OK) return st;
            rho_1 = rho;
            rho = pin[1];
            if (!(sqrt(pin[0]) > tol)) break;
        }
        return MTJG_OK;
    }

    // GMRES(m) (right preconditioned, CGS2) on A d = rin from d = 0 to residual tol.
    int gmres(const float *rin, float *d, double rn0, double tol, int in_max, int m, float *w)
    {
        float *V = w, *ww = w + (int64_t)(m + 1) * ld, *z = ww + ld, *r = z + ld;
        MTJG_CUDA(cudaMemsetAsync(d, 0, sizeof(float) * (size_t)n, stream()));
        std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m);
        const float *rv = rin;
        double beta = rn0;
        int st = MTJG_OK;
        while (beta > tol && total < in_max) {
            lin(V, rv, (float)(1.0 / beta), nullptr, 0, nullptr, 0, nullptr, false);
            std::fill(g.begin(), g.end(), 0.0);
            g[0] = beta;
            int k = 0;
            double res = beta, hn = 0.0;
            for (int j = 0; j < m; ++j) {
                const float *zp;
                if ((st = pc(V + (int64_t)j * ld, z, &zp)) != MTJG_OK) return st;
                if ((st = prod(zp, ww, nullptr)) != MTJG_OK) return st;
                // classical Gram-Schmidt, twice; the coefficients of both passes
                // land in dev[0..j] and dev[j+1..2j+1], ||w||^2 in dev[2j+2]
                for (int pass = 0; pass < 2; ++pass) {
                    k_ir_vdot<<<dim3(G, j + 1), kIrBlock, 0, stream()>>>(n, V, ld, ww, part);
                    count();
                    k_ir_final<<<j + 1, 32, 0, stream()>>>(part, G, dev + pass * (j + 1));
                    count();
                    k_ir_vupd<<<G, kIrBlock, 0, stream()>>>(n, V, ld, j + 1, dev + pass * (j + 1), ww);
                    count();
                }
                k_ir_lin<<<G, kIrBlock, 0, stream()>>>(n, ww, ww, 1.0f, nullptr, 0, nullptr, 0, nullptr, part);
                count();
                k_ir_final<<<1, 32, 0, stream()>>>(part, G, dev + 2 * (j + 1));
                count();
                cudaMemcpyAsync(pin, dev, sizeof(double) * (size_t)(2 * j + 3), cudaMemcpyDeviceToHost, stream());
                if ((st = wait()) != MTJG_OK) return st;
                for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = pin[i] + pin[j + 1 + i];
                hn = sqrt(pin[2 * j + 2]);
                H[(size_t)(j + 1) * m + j] = hn;
                for (int i = 0; i < j; ++i) {  // the earlier rotations
                    const double a = H[(size_t)i * m + j], b = H[(size_t)(i + 1) * m + j];
                    H[(size_t)i * m + j] = cs[i] * a + sn[i] * b;
                    H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * b;
                }
                const double a = H[(size_t)j * m + j], b = hn, h = std::hypot(a, b);
                cs[j] = h > 0 ? a / h : 1.0;
                sn[j] = h > 0 ? b / h : 0.0;
                H[(size_t)j * m + j] = h;
                H[(size_t)(j + 1) * m + j] = 0.0;
                g[j + 1] = -sn[j] * g[j];
                g[j] = cs[j] * g[j];
                res = std::fabs(g[j + 1]);
                k = j + 1;
                ++total;
                if (!(res > tol) || !(hn > 0.0) || total >= in_max || !std::isfinite(res)) break;
                lin(V + (int64_t)(j + 1) * ld, ww, (float)(1.0 / hn), nullptr, 0, nullptr, 0, nullptr, false);
            }
            // y = H(0:k, 0:k) \ g(0:k); a zero pivot ends the cycle early
            int kk = k;
            for (int i = 0; i < k; ++i)
                if (!(std::fabs(H[(size_t)i * m + i]) > 0.0)) {
                    kk = i;
                    break;
                }
            for (int i = kk - 1; i >= 0; --i) {
                double sacc = g[i];
                for (int c = i + 1; c < kk; ++c) sacc -= H[(size_t)i * m + c] * y[c];
                y[i] = sacc / H[(size_t)i * m + i];
            }
            if (kk > 0) {
                MTJG_CUDA(cudaMemcpyAsync(dev, y.data(), sizeof(double) * (size_t)kk, cudaMemcpyHostToDevice,
                                          stream()));
                k_ir_vcomb<<<G, kIrBlock, 0, stream()>>>(n, V, ld, kk, dev, ww);
                count();
                const float *zp;
                if ((st = pc(ww, z, &zp)) != MTJG_OK) return st;
                lin(d, d, 1.0f, zp, 1.0f, nullptr, 0, nullptr, false);
            }
            if (!(res > tol) || total >= in_max || !(hn > 0.0) || kk < k || !std::isfinite(res)) break;
            // restart on the FP32 residual of the correction so far
            if ((st = prod(d, r, rin)) != MTJG_OK) return st;
            lin(r, r, 1.0f, nullptr, 0, nullptr, 0, nullptr, true);
            finish(1);
            if ((st = wait()) != MTJG_OK) return st;
            beta = sqrt(pin[0]);
            rv = r;
        }
        return MTJG_OK;
    }
};

// FP32 and FP64 scratch of the mixed GMRES / BiCGstab solve, grown on demand
int ir_buffers(mtjg_solver *S, int64_t floats, int64_t doubles, int64_t pinned)
{
    if (floats > S->ir_fcap) {
        cudaFree(S->ir_f);
        S->ir_f = nullptr;
        S->ir_fcap = 0;
        MTJG_CUDA(cudaMalloc(&S->ir_f, sizeof(float) * (size_t)floats));
        S->ir_fcap = floats;
    }
    if (doubles > S->ir_dcap) {
        cudaFree(S->ir_d);
        S->ir_d = nullptr;
        S->ir_dcap = 0;
        MTJG_CUDA(cudaMalloc(&S->ir_d, sizeof(double) * (size_t)doubles));
        S->ir_dcap = doubles;
    }
    if (pinned > S->ir_hcap) {
        if (S->ir_h) cudaFreeHost(S->ir_h);
        S->ir_h = nullptr;
        S->ir_hcap = 0;
        MTJG_CUDA(cudaHostAlloc((void **)&S->ir_h, sizeof(double) * (size_t)pinned, cudaHostAllocDefault));
        S->ir_hcap = pinned;
    }
    return MTJG_OK;
}

// The refinement loop; b and x are in the solver's buffers.
int run_mixed_ir(mtjg_solver *S, mtjg_csr *A, mtjg_result *res)
{
    mtjg_ctx *ctx = S->ctx;
    const int n = S->n;
    int st = ensure_state(S, 1);
    if (st != MTJG_OK) return st;
    S->num_sys = 1;
    if ((st = mixed_prepare(S, A)) != MTJG_OK) return st;
    if (S->M && (st = precond_prepare32(S->M)) != MTJG_OK) return st;
    const bool gm = S->kind == MTJG_GMRES;
    const int m = gm ? S->restart : 0;
    const int64_t ld = ((int64_t)n + 63) / 64 * 64;
    const int G = ctx->num_sms * 2;
    const int64_t nvec = 2 + (gm ? (m + 1) + 3 : 7);
    const int slots = gm ? 2 * (m + 1) + 1 : 2;
    if ((st = ir_buffers(S, nvec * ld, (int64_t)G * std::max(slots, 2) + slots + 64, slots + 64)) != MTJG_OK)
        return st;
    float *rin = S->ir_f, *d = S->ir_f + ld, *work = S->ir_f + 2 * ld;
    IrInner in{S, A, n, G, ld, S->ir_d + slots + 64, S->ir_d, S->ir_h, 0};

    SysState init;
    std::memset(&init, 0, sizeof(init));
    init.status = ST_RUNNING;
    init.gate = ST_RUNNING;
    init.rho_1 = init.rho_2 = init.alpha = init.beta = init.omega = 1.0;
    S->last_all.assign(1, init);
    MTJG_CUDA(cudaMemcpyAsync(S->st, &S->last_all[0], sizeof(SysState), cudaMemcpyHostToDevice, ctx->stream));
    MTJG_CUDA(cudaMemcpyAsync(A->num_running, &S->num_sys, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(A->cnt, 0, sizeof(unsigned), ctx->stream));
    MTJG_CUDA(cudaMemsetAsync(ctx->d_flag, 0, sizeof(int), ctx->stream));
    const MonPtrs mp{S->st, mon_dev(S), S->hist_r, S->hist_it, A->num_running};
    SysState *pst = reinterpret_cast<SysState *>(S->ir_h + slots + 8);
    const double rtol = S->mon.rtol, atol = S->mon.atol;
    int *flagp = ctx->h_pinned + 2;
    for (int outer = 0;; ++outer) {
        cudaError_t e = launch_spmv(ctx, CsrArgs{A->rowptr, A->colind, A->val}, A->tiles,
                                    (const double *)S->vecs[V_X], MiOuter{S->vecs[V_B], rin, mp}, red_ctx(A, A->tiles),
                                    S->mon.norm);
        if (e != cudaSuccess) return cuda_fail(e, "mixed-precision outer step");
        MTJG_CUDA(cudaMemcpyAsync(pst, S->st, sizeof(SysState), cudaMemcpyDeviceToHost, ctx->stream));
        MTJG_CUDA(cudaMemcpyAsync(flagp, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (*flagp) break;
        if (pst->status != ST_RUNNING) break;
        if (outer > std::max(0, S->mon.max_iter) + 2)
            return fail(MTJG_ERR_DEVICE_TIMEOUT, "mixed-precision solve did not stop within maxIter steps");
        // the inner solve's target: its own decrease, and not below the monitor's
        in.lin(rin, rin, 1.0f, nullptr, 0, nullptr, 0, nullptr, true);
        in.finish(1);
        if ((st = in.wait()) != MTJG_OK) return st;
        const double rn0 = sqrt(in.pin[0]);
        const double tol = std::max(S->mix.in_rtol * rn0, std::max(rtol * pst->initR, atol));
        st = gm ? in.gmres(rin, d, rn0, tol, in.total + S->mix.in_max, m, work)
                : in.bicgstab(rin, d, rn0, tol, S->mix.in_max, work);
        if (st != MTJG_OK) return st;
        k_ir_xadd<<<G, kIrBlock, 0, ctx->stream>>>(n, S->vecs[V_X], d, S->st);
        ctx->launches++;
        MTJG_CUDA(cudaGetLastError());
    }
    MTJG_CUDA(cudaMemcpyAsync(S->last_all.data(), S->st, sizeof(SysState), cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaMemcpyAsync(flagp, ctx->d_flag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MTJG_CUDA(cudaStreamSynchronize(ctx->stream));
    S->last_all[0].in_total = in.total;
    S->last = S->last_all[0];
    S->last_valid = 1;
    S->last_empty = false;
    S->last_sys = 0;
    if (*flagp) {
        cudaMemset(ctx->d_flag, 0, sizeof(int));
        return fail(MTJG_ERR_DEVICE_TIMEOUT, "a bounded wait in a device kernel gave up during the solve");
    }
    return report(S, res);
}
