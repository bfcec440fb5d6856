// abi.cpp -- library-wide entry points: errors, contexts, device memory,
// timing events.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "internal.h"

namespace mtjg {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg)
{
    set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what)
{
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    return e == cudaErrorMemoryAllocation ? MTJG_ERR_OUT_OF_MEMORY : MTJG_ERR_CUDA;
}

static void ctx_free(mtjg_ctx *c)
{
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto &ev : c->events)
        if (ev) cudaEventDestroy(ev);
    if (c->d_flag) cudaFree(c->d_flag);
    if (c->h_pinned) cudaFreeHost(c->h_pinned);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

void ctx_retain(mtjg_ctx *c)
{
    if (c) c->refs.fetch_add(1);
}

void ctx_release(mtjg_ctx *c)
{
    if (c && c->refs.fetch_sub(1) == 1) ctx_free(c);
}

}  // namespace mtjg

using namespace mtjg;

extern "C" const char *mtjg_last_error(void) { return g_last_error.c_str(); }

extern "C" const char *mtjg_version(void) { return "mtjg 0.1 (sm_103a)"; }

extern "C" void mtjg_monitor_defaults(mtjg_monitor *mon)
{
    if (!mon) return;
    mon->max_iter = 100000;
    mon->rtol = 1e-5;
    mon->atol = 1e-50;
    mon->dtol = 1e+5;
    mon->norm = MTJG_NORM_TWO;
    mon->history_cap = 0;
}

extern "C" int mtjg_ctx_create(int device, mtjg_ctx **out)
{
    if (!out) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL out");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) return fail(MTJG_ERR_CUDA, "no CUDA device available");
    if (device < 0 || device >= count) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "device index out of range");
    MTJG_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    MTJG_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) return fail(MTJG_ERR_UNSUPPORTED, "this library is built for sm_103a (Blackwell) only");
    mtjg_ctx *c = new mtjg_ctx();
    c->device = device;
    c->num_sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return fail(MTJG_ERR_CUDA, "cudaStreamCreate failed");
    }
    for (auto &ev : c->events) cudaEventCreate(&ev);
    if (cudaMalloc(&c->d_flag, sizeof(int) * 4) != cudaSuccess ||
        cudaHostAlloc(&c->h_pinned, sizeof(int) * 64, cudaHostAllocDefault) != cudaSuccess) {
        mtjg_ctx_destroy(c);
        return fail(MTJG_ERR_OUT_OF_MEMORY, "context allocation failed");
    }
    cudaMemset(c->d_flag, 0, sizeof(int) * 4);
    // a failed launch of a kernel image built for another GPU shows up here
    cudaError_t le = cudaDeviceSynchronize();
    if (le != cudaSuccess) {
        mtjg_ctx_destroy(c);
        return cuda_fail(le, "context initialisation");
    }
    *out = c;
    return MTJG_OK;
}

extern "C" int mtjg_ctx_destroy(mtjg_ctx *c)
{
    if (!c || c->closed) return MTJG_OK;
    c->closed = true;
    ctx_release(c);
    return MTJG_OK;
}

extern "C" int mtjg_ctx_set_numerics(mtjg_ctx *c, int numerics)
{
    if (!c || (numerics != MTJG_NUMERICS_FAST && numerics != MTJG_NUMERICS_STRICT))
        return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "bad numerics mode");
    c->numerics = numerics;
    return MTJG_OK;
}

extern "C" int mtjg_ctx_synchronize(mtjg_ctx *c)
{
    if (!c) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL context");
    MTJG_CUDA(cudaSetDevice(c->device));
    MTJG_CUDA(cudaStreamSynchronize(c->stream));
    return MTJG_OK;
}

extern "C" int64_t mtjg_ctx_launch_count(mtjg_ctx *c) { return c ? c->launches.load() : 0; }

extern "C" int mtjg_ctx_event_record(mtjg_ctx *c, int slot)
{
    if (!c || slot < 0 || slot >= 16) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "bad event slot");
    MTJG_CUDA(cudaEventRecord(c->events[slot], c->stream));
    return MTJG_OK;
}

extern "C" int mtjg_ctx_event_elapsed(mtjg_ctx *c, int a, int b, float *ms)
{
    if (!c || a < 0 || a >= 16 || b < 0 || b >= 16 || !ms) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "bad event slot");
    MTJG_CUDA(cudaEventSynchronize(c->events[b]));
    MTJG_CUDA(cudaEventElapsedTime(ms, c->events[a], c->events[b]));
    return MTJG_OK;
}

extern "C" int mtjg_dev_alloc(mtjg_ctx *c, int64_t bytes, void **dptr)
{
    if (!c || !dptr || bytes < 0) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "bad allocation request");
    MTJG_CUDA(cudaSetDevice(c->device));
    MTJG_CUDA(cudaMalloc(dptr, (size_t)(bytes > 0 ? bytes : 16)));
    return MTJG_OK;
}

extern "C" int mtjg_dev_free(mtjg_ctx *c, void *dptr)
{
    if (!c) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL context");
    MTJG_CUDA(cudaSetDevice(c->device));
    MTJG_CUDA(cudaStreamSynchronize(c->stream));
    MTJG_CUDA(cudaFree(dptr));
    return MTJG_OK;
}

extern "C" int mtjg_memcpy_h2d(mtjg_ctx *c, void *dst, const void *src, int64_t bytes)
{
    if (!c) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL context");
    MTJG_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyHostToDevice, c->stream));
    MTJG_CUDA(cudaStreamSynchronize(c->stream));
    return MTJG_OK;
}

extern "C" int mtjg_memcpy_d2h(mtjg_ctx *c, void *dst, const void *src, int64_t bytes)
{
    if (!c) return fail(MTJG_ERR_ILLEGAL_ARGUMENT, "NULL context");
    MTJG_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost, c->stream));
    MTJG_CUDA(cudaStreamSynchronize(c->stream));
    return MTJG_OK;
}
