// convert.cu -- non-CSR matrices to a device CompRowMatrix, converted on the
// device: new CompRowMatrix(Matrix A) (S/CompRowMatrix.java:210-243) for
//   * CompColMatrix (S/CompColMatrix.java): its CSC arrays are the CSR of
//     A', uploaded as they are and transposed on the device (the rows of
//     the result list their entries in ascending column order);
//   * FlexCompRowMatrix (S/FlexCompRowMatrix.java): one SparseVector per
//     row (S/SparseVector.java: sorted indices index[0, used) in storage
//     of some capacity), handed over as one slab of all rows' storage with
//     each row's start and used count; the device scans the counts into row
//     pointers and gathers each row's used entries, checking order and range.
// new CompRowMatrix(A) keeps A's stored entries (explicit zeros included)
// with their values; from then on the matrix is a CompRowMatrix, so its
// products follow CompRowMatrix's operation order (CompColMatrix's own
// multAdd, S/CompColMatrix.java:285-305, rounds differently).
#include <algorithm>
#include <cstring>

#include "spmv.cuh"

namespace mtjg {

int csr_adopt(mtjg_ctx *ctx, int n, int m, std::vector<int> &&h_rowptr, int *d_rowptr, int *d_colind, double *d_val,
              mtjg_csr **out);

namespace {

// row i's used count (checked against its storage) into cnt[i]
__global__ void k_flex_counts(int n, const long long *start, const int *used, long long slab, int *cnt, int *err)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int u = used[i];
        const long long s = start[i];
        const bool ok = u >= 0 && s >= 0 && s + u <= slab;
        cnt[i] = ok ? u : 0;
        if (!ok) atomicMin(err, i);
    }
}

// one warp per row: copy the row's used entries; indices must lie in
// [0, m) and ascend strictly (a SparseVector's invariant)
__global__ void k_flex_gather(int n, int m, const long long *start, const int *rowptr, const int *index,
                              const double *data, int *colind, double *val, int *err)
{
    const int lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = w; i < n; i += nw) {
        const int b = rowptr[i], len = rowptr[i + 1] - b;
        const long long s = start[i];
        bool bad = false;
        for (int k = lane; k < len; k += 32) {
            const int c = index[s + k];
            colind[b + k] = c;
            val[b + k] = data[s + k];
            if (c < 0 || c >= m || (k > 0 && index[s + k - 1] >= c)) bad = true;
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) atomicMin(err, i);
    }
}

int grid_for(mtjg_ctx *ctx, int n) { return std::max(1, std::min((n + kBlock - 1) / kBlock, ctx->num_sms * 8)); }

}  // namespace
}  // namespace mtjg

using namespace mtjg;

extern "C" int mtjg_csr_upload_csc(mtjg_ctx *ctx, int num_rows, int num_cols, const int *colptr, const int *rowind,
                                   const double *val, mtjg_csr **out)
{
    if (!ctx || !out || !colptr) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (num_rows < 0 || num_cols < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "negative matrix dimension");
    // CompColMatrix's structure (S/CompColMatrix.java:190-215): column
    // pointers from 0, row indices in range and ascending within a column
    if (colptr[0] != 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "colptr[0] != 0");
    for (int j = 0; j < num_cols; ++j) {
        if (colptr[j + 1] < colptr[j]) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "colptr is not nondecreasing");
        for (int k = colptr[j]; k < colptr[j + 1]; ++k) {
            if (rowind[k] < 0 || rowind[k] >= num_rows)
                return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "nz[" + std::to_string(j) + "][" +
                                                           std::to_string(k - colptr[j]) + "]=" +
                                                           std::to_string(rowind[k]) +
                                                           ", which is not a valid row index");
            if (k > colptr[j] && rowind[k - 1] >= rowind[k])
                return fail(MTJG_ERR_ILLEGAL_ARGUMENT,
                            "row indices of column " + std::to_string(j) + " are not strictly ascending");
        }
    }
    MTJG_CUDA(cudaSetDevice(ctx->device));
    const int64_t nnz = colptr[num_cols];
    int *cp = nullptr, *ri = nullptr;
    double *cv = nullptr;
    auto release = [&]() {
        cudaFree(cp);
        cudaFree(ri);
        cudaFree(cv);
    };
    if (cudaMalloc(&cp, sizeof(int) * (size_t)(num_cols + 1)) != cudaSuccess ||
        cudaMalloc(&ri, sizeof(int) * (size_t)std::max<int64_t>(1, nnz)) != cudaSuccess ||
        cudaMalloc(&cv, sizeof(double) * (size_t)std::max<int64_t>(1, nnz)) != cudaSuccess) {
        release();
        return fail(MTJG_ERR_OUT_OF_MEMORY, "cudaMalloc failed for the CSC matrix");
    }
    cudaError_t e = cudaMemcpyAsync(cp, colptr, sizeof(int) * (size_t)(num_cols + 1), cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e == cudaSuccess && nnz)
        e = cudaMemcpyAsync(ri, rowind, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && nnz)
        e = cudaMemcpyAsync(cv, val, sizeof(double) * (size_t)nnz, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) {
        release();
        return cuda_fail(e, "copying the CSC matrix to the device");
    }
    // the CSC of A is the CSR of A' (num_cols rows): its transpose is A's CSR
    int *trp = nullptr, *tci = nullptr;
    double *tv = nullptr;
    int64_t tn = 0;
    int st = csr_transpose(ctx, num_cols, num_rows, cp, ri, cv, 0, &trp, &tci, &tv, &tn);
    release();
    if (st != MTJG_OK) return st;
    std::vector<int> h((size_t)num_rows + 1);
    e = cudaMemcpy(h.data(), trp, sizeof(int) * h.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        cudaFree(trp);
        cudaFree(tci);
        cudaFree(tv);
        return cuda_fail(e, "reading the converted row pointers");
    }
    // the handle owns the arrays from here on, also when it fails
    return csr_adopt(ctx, num_rows, num_cols, std::move(h), trp, tci, tv, out);
}

extern "C" int mtjg_csr_upload_rows(mtjg_ctx *ctx, int num_rows, int num_cols, const int64_t *row_start,
                                    const int *row_used, const int *index, const double *data, int64_t slab,
                                    mtjg_csr **out)
{
    if (!ctx || !out || (num_rows > 0 && (!row_start || !row_used)) || (slab > 0 && (!index || !data)))
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    *out = nullptr;
    if (num_rows < 0 || num_cols < 0 || slab < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "negative size");
    MTJG_CUDA(cudaSetDevice(ctx->device));
    const int n = num_rows;
    long long *d_start = nullptr;
    int *d_used = nullptr, *d_cnt = nullptr, *d_idx = nullptr, *rp = nullptr, *ci = nullptr;
    double *d_data = nullptr, *v = nullptr;
    int *err = ctx->d_flag + 1;
    auto release = [&](bool all) {
        cudaFree(d_start);
        cudaFree(d_used);
        cudaFree(d_cnt);
        cudaFree(d_idx);
        cudaFree(d_data);
        if (all) {
            cudaFree(rp);
            cudaFree(ci);
            cudaFree(v);
        }
    };
    auto cuda = [&](cudaError_t e, const char *what) {
        release(true);
        return cuda_fail(e, what);
    };
    cudaError_t e = cudaSuccess;
    const size_t ns = (size_t)std::max(1, n), sl = (size_t)std::max<int64_t>(1, slab);
    if ((e = cudaMalloc(&d_start, sizeof(long long) * ns)) != cudaSuccess ||
        (e = cudaMalloc(&d_used, sizeof(int) * ns)) != cudaSuccess ||
        (e = cudaMalloc(&d_cnt, sizeof(int) * ns)) != cudaSuccess ||
        (e = cudaMalloc(&d_idx, sizeof(int) * sl)) != cudaSuccess ||
        (e = cudaMalloc(&d_data, sizeof(double) * sl)) != cudaSuccess ||
        (e = cudaMalloc(&rp, sizeof(int) * (size_t)(n + 1 + kRowptrPad))) != cudaSuccess)
        return cuda(e, "cudaMalloc for the row slab");
    const int big = 0x7fffffff;
    if ((n && ((e = cudaMemcpyAsync(d_start, row_start, sizeof(long long) * (size_t)n, cudaMemcpyHostToDevice,
                                    ctx->stream)) != cudaSuccess ||
               (e = cudaMemcpyAsync(d_used, row_used, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                                    ctx->stream)) != cudaSuccess)) ||
        (slab && ((e = cudaMemcpyAsync(d_idx, index, sizeof(int) * (size_t)slab, cudaMemcpyHostToDevice,
                                       ctx->stream)) != cudaSuccess ||
                  (e = cudaMemcpyAsync(d_data, data, sizeof(double) * (size_t)slab, cudaMemcpyHostToDevice,
                                       ctx->stream)) != cudaSuccess)) ||
        (e = cudaMemcpyAsync(err, &big, sizeof(int), cudaMemcpyHostToDevice, ctx->stream)) != cudaSuccess)
        return cuda(e, "copying the row slab to the device");
    if (n) {
        k_flex_counts<<<grid_for(ctx, n), kBlock, 0, ctx->stream>>>(n, d_start, d_used, (long long)slab, d_cnt, err);
        ctx->launches++;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda(e, "row counts");
    }
    int st = exclusive_scan(ctx, d_cnt, rp, n);
    if (st != MTJG_OK) {
        release(true);
        return st;
    }
    std::vector<int> h((size_t)n + 1);
    int bad = big;
    if ((e = cudaMemcpy(h.data(), rp, sizeof(int) * h.size(), cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (e = cudaMemcpy(&bad, err, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda(e, "reading the row pointers");
    if (bad != big) {
        release(true);
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "row " + std::to_string(bad) + " lies outside the slab");
    }
    const int64_t nnz = h[(size_t)n];
    {
        const int pad[kRowptrPad] = {(int)nnz, (int)nnz, (int)nnz, (int)nnz};
        if ((e = cudaMemcpy(rp + n + 1, pad, sizeof(pad), cudaMemcpyHostToDevice)) != cudaSuccess)
            return cuda(e, "row pointer padding");
    }
    if ((e = cudaMalloc(&ci, sizeof(int) * (size_t)(nnz + 4))) != cudaSuccess ||
        (e = cudaMalloc(&v, sizeof(double) * (size_t)(nnz + 2))) != cudaSuccess ||
        (e = cudaMemsetAsync(ci, 0xff, sizeof(int) * (size_t)(nnz + 4), ctx->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(v, 0, sizeof(double) * (size_t)(nnz + 2), ctx->stream)) != cudaSuccess)
        return cuda(e, "cudaMalloc for the converted CSR");
    if (n) {
        k_flex_gather<<<std::max(1, std::min((n + 7) / 8, ctx->num_sms * 16)), kBlock, 0, ctx->stream>>>(
            n, num_cols, d_start, rp, d_idx, d_data, ci, v, err);
        ctx->launches++;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda(e, "row gather");
    }
    // the context's stream does not block with plain copies: wait for the gather
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess ||
        (e = cudaMemcpy(&bad, err, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda(e, "reading the conversion status");
    if (bad != big) {
        release(true);
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT,
                    "row " + std::to_string(bad) + " holds a column index out of range or not strictly ascending");
    }
    release(false);
    // the handle owns rp, ci and v from here on, also when it fails
    return csr_adopt(ctx, n, num_cols, std::move(h), rp, ci, v, out);
}
