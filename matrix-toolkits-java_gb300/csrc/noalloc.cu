// noalloc.cu -- y = alpha A x + y together with the two-norm of the updated
// y, computed on scratch memory that the library never allocates.
//
// The norm is a reduction: the product kernel (k_spmv) leaves one partial
// sum per reduction group and k_finalize adds them up in group order.  The
// other entry points keep those partials in memory cudaMalloc'd with the
// matrix; this one keeps them in a fixed array in the library's own device
// image (g_noalloc_part below), so the call itself allocates nothing.
//
// Scratch rules:
//   * size: kNoAllocMaxGroups groups of kParts doubles (512 KB).  A group is
//     at most kGroupTiles (8) product tiles of at most kTileNnz (1152)
//     entries, so one system fits up to 16384 * 8 * 1152 = 151 million
//     entries (about 21 million rows at 7 entries per row), and a batch up to
//     16384 systems.  A matrix whose product tiling has more groups is
//     rejected with MTJG_ERR_ILLEGAL_ARGUMENT.
//   * nothing has to start at zero: every group partial is written by the
//     product kernel before k_finalize reads it within the same call, and
//     each norm is stored, not accumulated.
//   * there is one scratch array per device, shared by every context and
//     thread of the process: two calls that overlap on one device (two
//     streams, two contexts or two host threads) overwrite each other's
//     partials and return wrong norms.  Calls made one after another on one
//     context's stream are ordered and safe.
//   * set-up: the first call on each device looks the array's device address
//     up once (cudaGetSymbolAddress, with that device current) and keeps it.
//     A caller that captures streams makes one call before capture begins,
//     so that this first-call set-up does not fall inside the capture.  A
//     cudaDeviceReset ends every handle of the library on that device, the
//     saved address included; callers make new handles after a reset.
#include <mutex>

#include "spmv.cuh"

namespace mtjg {
namespace {

constexpr int kNoAllocMaxGroups = 16384;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_part[kNoAllocMaxGroups * kParts];

std::mutex g_noalloc_mu;
double *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// The scratch's address on device `dev` (current): looked up on first use.
int noalloc_scratch(int dev, double **out)
{
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_part);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the no-allocation scratch");
        g_noalloc_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_noalloc_ptr[dev];
    return MTJG_OK;
}

// CompRowMatrix.multAdd's row update (S/CompRowMatrix.java:343), plus the
// updated entry's square into the group partial.
template <bool S>
struct EpiMultAddNorm {
    double *y;
    double alpha;
    double *norm;  // one per system
    static constexpr bool kReduce = true;
    static constexpr bool kNeedsXr = false;
    static constexpr int kSlots = kSlotNorm;
    __device__ bool active(int) const { return true; }
    __device__ double init(int, int) const { return 0.0; }
    __device__ void row(int r, int, double d, double, Acc &a) const
    {
        const double v = fmac<S>(alpha, d, y[r]);
        y[r] = v;
        norm_add<S>(a, v, MTJG_NORM_TWO);
    }
    __device__ void scalar(int sys, const Acc &s) { norm[sys] = norm_finish(s.v, MTJG_NORM_TWO); }
};

}  // namespace
}  // namespace mtjg

using namespace mtjg;

extern "C" int mtjg_csr_mult_add_norm_noalloc(mtjg_csr *A, double alpha, const double *dx, double *dy,
                                              double *dnorm)
{
    if (!A || !dx || !dy || !dnorm) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL argument");
    mtjg_ctx *ctx = A->ctx;
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return fail(MTJG_ERR_UNSUPPORTED, "device index beyond the no-allocation scratch table");
    if (A->tiles.num_groups > kNoAllocMaxGroups)
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT,
                    "matrix needs " + std::to_string(A->tiles.num_groups) +
                        " reduction groups; the no-allocation scratch holds " + std::to_string(kNoAllocMaxGroups));
    MTJG_CUDA(cudaSetDevice(ctx->device));
    double *part = nullptr;
    int st = noalloc_scratch(ctx->device, &part);
    if (st != MTJG_OK) return st;
    const int num_sys = A->tiles.num_sys > 0 ? A->tiles.num_sys : 1;
    if (A->tiles.num_tiles == 0) {  // no rows: every norm is zero
        MTJG_CUDA(cudaMemsetAsync(dnorm, 0, sizeof(double) * (size_t)num_sys, ctx->stream));
        return MTJG_OK;
    }
    const RedCtx rc{part, nullptr, A->tiles.sys_group, nullptr};
    const CsrArgs csr{A->rowptr, A->colind, A->val};
    cudaError_t e;
    if (ctx->numerics == MTJG_NUMERICS_STRICT)
        e = launch_spmv(ctx, csr, A->tiles, dx, EpiMultAddNorm<true>{dy, alpha, dnorm}, rc, MTJG_NORM_TWO);
    else
        e = launch_spmv(ctx, csr, A->tiles, dx, EpiMultAddNorm<false>{dy, alpha, dnorm}, rc, MTJG_NORM_TWO);
    if (e != cudaSuccess) return cuda_fail(e, "multAdd-with-norm launch");
    return MTJG_OK;
}
