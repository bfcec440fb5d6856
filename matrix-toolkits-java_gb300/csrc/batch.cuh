// batch.cuh -- the persistent batched CG (batch.cu): its arguments and entry points.
#pragma once

#include <functional>
#include <vector>

#include "phases.cuh"

namespace mtjg {

// One launch of the persistent batched CG over the systems in `order`.
struct BatchCg {
    const int *rowptr;
    const int *colind;
    const double *val;
    const float *val32;
    const int *sys_rows;        // [num_sys + 1]
    const int *order;           // [count]: the systems, in the order CTAs take them
    const unsigned char *vec;   // [num_sys]: lanes per row
    unsigned *ticket;           // zero at launch
    int count;
    int pc;                     // kPcIdentity or kPcJacobi
    const double *invdiag;
    const float *invdiag32;
    const double *b;
    double *x, *r, *z, *p, *q;  // FP64 solve
    float *d32, *r32, *z32, *p32, *q32;  // FP32 inner vectors (mixed)
    SysState *st;
    MonCfgDev mon;
    double *hist_r;
    int *hist_it;
    MixCfg mix;
};

cudaError_t batch_launch(mtjg_ctx *ctx, const BatchCg &a, bool mixed);
int batch_class(int64_t rows, int64_t nnz);
int batch_tuned(int cls);
// Lanes per row of each system (tuned per class, probing classes not seen
// before); probe(systems, lanes, iterations) returns milliseconds.
int batch_vec(int num_sys, const int *sys_rows, const int *h_rowptr, std::vector<unsigned char> &vec,
              const std::function<double(const std::vector<int> &, int, int)> &probe);

}  // namespace mtjg
