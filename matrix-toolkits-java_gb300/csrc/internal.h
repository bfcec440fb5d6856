// internal.h -- shared declarations of the GB300 Krylov library (host side).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mtjg.h"

namespace mtjg {

// ----------------------------------------------------------------- errors
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);

// Checks a host CSR (0-based, sorted columns in range), as CompRowMatrix's
// constructor does; MTJG_ERR_ILLEGAL_ARGUMENT names the offending entry.
int csr_validate(int n, int m, const int *rowptr, const int *colind);

}  // namespace mtjg
struct mtjg_ctx;
namespace mtjg {
// Objects made with a context keep it alive: the context is freed when its
// handle has been destroyed and the last object made with it is gone.
void ctx_retain(mtjg_ctx *ctx);
void ctx_release(mtjg_ctx *ctx);

#define MTJG_CUDA(call)                                       \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return ::mtjg::cuda_fail(e_, #call); \
    } while (0)

// ------------------------------------------------------------ tiling
// For CSR products, rows are cut into tiles of at most kTileRows/vec rows
// and kTileNnz entries (one long row may exceed kTileNnz; it forms a tile of
// its own).  Row kernels use row tiles of kRowTile or kRowTileRows rows
// (below).  Tiles never straddle two
// systems of a batch, and reductions are sums of per-tile partials in tile
// order, so no result depends on the grid size or on the other systems of a
// batch.
// Tile shape and pipeline depth can be set at build time (-DMTJG_TILE_ROWS=...)
// to tune them, as can the row-tile passes and group sizes below and, beside
// their kernels, the resident blocks of the CG and FP32 inner-solve phases
// (MTJG_CGQ_CTAS, MTJG_CGUPD_MINB, MTJG_MXQ_CTAS, MTJG_MXUPD_MINB).  The defaults were measured on GB300: 1152-entry tiles with
// 6 (plain) / 5 (reducing) resident product CTAs per SM served the mixed
// request stream 11% faster than 1792-entry tiles with 4, at 4% more time
// per 3D Poisson 128^3 CG solve.
#ifndef MTJG_TILE_ROWS
#define MTJG_TILE_ROWS 256
#endif
#ifndef MTJG_TILE_NNZ
#define MTJG_TILE_NNZ 1152
#endif
constexpr int kBlock = 256;
constexpr int kTileRows = MTJG_TILE_ROWS;
constexpr int kTileNnz = MTJG_TILE_NNZ;
constexpr int kLongSeg = 4096;        // entries per segment of a long row (FAST pre-pass)
constexpr int kWideRow = 64;          // rows this long among shorter ones get a warp each (plan_tiles)
constexpr int kParts = 4;             // partial-sum slots per group
// A reduction group is what one block sums before a block-wide reduction:
// up to kGroupTiles consecutive product tiles of one system, or one row
// tile.  Few block-wide reductions matter on
// GB300, whose FP64 pipe is narrow: a tree over 256 threads costs more FP64
// issue slots than the vector work of 256 rows.
#ifndef MTJG_GROUP_TILES
#define MTJG_GROUP_TILES 8
#endif
constexpr int kGroupTiles = MTJG_GROUP_TILES;  // at most
#ifndef MTJG_GROUP_DIV
#define MTJG_GROUP_DIV 4096
#endif
// A system of T product tiles forms groups of clamp(T / kGroupDiv, 1,
// kGroupTiles) tiles: a function of the system alone, so its sums are the
// same alone and in any batch.
constexpr int kGroupDiv = MTJG_GROUP_DIV;
// Systems of a batch (mtjg_batch_upload) and of the server's FP32 tiling
// divide by this instead: a batch fills the GPU with many systems, so fewer,
// larger groups (fewer block-wide reductions) cost it no parallelism.  A
// system's sums are then the same in any batch, and in a batch of one.
constexpr int kBatchGroupDiv = 64;
constexpr int kRowsPerThread = 4;
constexpr int kRowTile = kBlock * kRowsPerThread;
// A row tile of the vector phases (one block, one partial) of a batched or
// served system is kRowPasses passes of kRowTile rows: more passes spread one
// block-wide reduction over more rows.  A lone uploaded CSR takes them from
// kRowTileLoneMin rows on; below that it keeps one pass, so a small system
// still spreads over many blocks.
#ifndef MTJG_ROW_PASSES
#define MTJG_ROW_PASSES 2
#endif
constexpr int kRowPasses = MTJG_ROW_PASSES;
constexpr int kRowTileRows = kRowTile * kRowPasses;
constexpr int kRowTileLoneMin = 1 << 20;

// device status of a system (SysState::status)
enum : int {
    ST_RUNNING = 0,
    ST_DONE = 100  // converged
    // otherwise an MTJG_* code
};

// Per-system scalars of a solve, in device memory.
struct SysState {
    int status;
    int iter;
    int detail;
    int hist_len;
    int inner;      // GMRES: inner index i of the running cycle
    int inner_done; // GMRES: inner loop left (converged or exception)
    int gate;       // ST_RUNNING while inner-step kernels must run (GMRES), else 1
    int pad1;
    double initR;
    double residual;
    double rho, rho_1, rho_2;
    double alpha, beta, omega;
    double normr;   // GMRES: ||r||2 of the running cycle
    double scratch[3];
    // mixed precision (FP64 refinement around an FP32 inner CG)
    int phase;      // 0: the outer step is due, 1: inner iterations run
    int pending;    // 1: the FP32 correction still has to be added to x
    int in_iter;    // iterations of the running inner solve
    int in_total;   // FP32 iterations of the whole solve
    int in_fresh;   // 1: the next inner direction is p = z
    int pad2;
    double in_rho, in_rho_1, in_alpha, in_beta, in_r0;
    // QMR (S/QMR.java:120-121): xi, gamma, theta, eta, delta, ep, the
    // previous gamma / theta, and coef: the direction scale factors
    // (coef[0], coef[1]) or the d / s scale factor (coef[0])
    double xi, gamma, gamma_1, theta, theta_1, eta, delta, ep;
    double coef[2];
    // MatrixIterationMonitor (MonCfgDev::xmon): the iterate, its length, the
    // numerics its norm is formed in, normA, normb and |x| at the coming test
    const double *xm_x;
    int xm_n, xm_strict;
    double xm_normA, xm_normb;
    double xnorm;
};

struct MonCfgDev {
    int max_iter;
    int norm;
    int hist_cap;
    // MatrixIterationMonitor (S/MatrixIterationMonitor.java:101-124): a test
    // converges iff r < max(rtol (normA |x| + normb), atol), with normA,
    // normb, the iterate and |x| (formed just before the test) in SysState
    int xmon;
    double rtol, atol, dtol;
};

// Reduction context: per-group partial sums and the group ranges of the
// systems (groups of system s are [sys_group[s], sys_group[s+1])).
struct RedCtx {
    double *part;          // [num_groups * kParts]
    unsigned *cnt;         // [num_sys] (unused on the hot path)
    const int *sys_group;  // [num_sys + 1]
    int *num_running;      // number of systems with status RUNNING
};

struct TileSet {
    int num_tiles = 0;
    int num_groups = 0;
    int num_sys = 1;
    int vec = 1;
    int *tile_row = nullptr;   // device [num_tiles + 1]
    int *tile_nz = nullptr;    // device [num_tiles + 1]: rowptr at each tile's first row
    int *tile_row_end = nullptr;  // device [num_tiles], served batches only (else tile_row + 1)
    int *tile_nz_end = nullptr;   // device [num_tiles], served batches only (else tile_nz + 1)
    int *tile_sys = nullptr;   // device [num_tiles] (nullptr: all system 0)
    int *group_tile = nullptr; // device [num_groups + 1]: first tile of each reduction group
    int *group_info = nullptr; // device [num_groups]: (system << 8) | lanes per row
    int *sys_group = nullptr;  // device [num_sys + 1]
    const struct SysDesc *sd = nullptr;  // device per-system matrices (served batches), else nullptr
    // device [num_tiles]: (lanes per row << 1) | 1 if the tile is a single long row
    unsigned char *tile_flags = nullptr;
    int vec_mask = 0;          // OR of the lanes-per-row classes of the tiles
    // rows longer than a stage (tiles of their own), summed ahead of a FAST
    // product by many CTAs: fixed segments of kLongSeg entries, then the
    // segments of each row in order (k_long_seg, k_long_sum)
    int num_long = 0, num_segs = 0;
    int *seg_begin = nullptr, *seg_end = nullptr;  // device [num_segs]: entries of each segment
    int *long_first = nullptr;                     // device [num_long + 1]: first segment of each long row
    int *long_tile = nullptr;                      // device [num_long]: its tile
    double *seg_part = nullptr;                    // device [num_segs]: segment sums
    double *long_sum = nullptr;                    // device [num_tiles]: row sums, by tile
    std::vector<int> h_tile_row;
};

// A row-ordered triangular operator and its dependency levels.  A sweep
// (one launch) hands out chunks of at most 32 rows of one level, in level
// order, from a ticket counter.
struct LevelSchedule {
    int n = 0;
    int num_levels = 0;
    int num_chunks = 0;
    int *perm = nullptr;               // device: rows ordered by level (stable in row index)
    int *chunk = nullptr;              // device [num_chunks + 1]: first perm position of each chunk
    unsigned *ticket = nullptr;        // device: next chunk of the running sweep
    std::vector<int> level_ptr;        // host: [num_levels + 1]
};

}  // namespace mtjg

// --------------------------------------------------------------- handles
struct mtjg_ctx {
    std::atomic<int> refs{1};       // the handle itself + every object made with it
    bool closed = false;            // mtjg_ctx_destroy was called
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t events[16] = {};
    int numerics = MTJG_NUMERICS_FAST;
    int num_sms = 0;
    std::atomic<int64_t> launches{0};  // kernels launched (a serving thread counts here too)
    int *d_flag = nullptr;          // device error flag (bounded waits)
    int *h_pinned = nullptr;        // pinned host words for status polling
};

struct mtjg_csr {
    mtjg_ctx *ctx = nullptr;
    int n = 0, m = 0;
    int64_t nnz = 0;
    int *rowptr = nullptr;     // device [n+1]
    int *colind = nullptr;     // device [nnz + 4] (padded for 16-byte bulk copies)
    double *val = nullptr;     // device [nnz + 2]
    std::vector<int> h_rowptr; // host copy (tiling, validation)
    std::vector<int> sys_rows; // batch: first row of each system (+ end); empty for one system
    int *d_sys_rows = nullptr; // the same on the device (persistent batched CG), made on first use
    mtjg::TileSet tiles;       // product tiles
    mtjg::TileSet rtiles;      // row-kernel tiles (kBlock rows)
    // transpose (built on first transMult): CSR of A'
    int *t_rowptr = nullptr, *t_colind = nullptr;
    double *t_val = nullptr;
    mtjg::TileSet t_tiles;
    double *t_part = nullptr;  // reduction scratch of the transposed tiling
    int64_t version = 0;       // changes whenever the values (and so the transpose) change
    // FP32 copy of the values (mixed precision), built on first use
    float *val32 = nullptr;
    // reduction scratch sized for this matrix's tiles
    double *part = nullptr;
    unsigned *cnt = nullptr;
    int *num_running = nullptr;
    // staging vectors for host-pointer calls
    double *d_x = nullptr, *d_y = nullptr;
    bool borrowed = false;     // rowptr, colind, val, val32 belong to someone else (csr_borrow)
};

struct mtjg_precond {
    mtjg_ctx *ctx = nullptr;
    int kind = MTJG_PC_IDENTITY;
    int n = 0;
    bool ready = false;
    int64_t version = 0;               // changes whenever setMatrix reallocates
    double *invdiag = nullptr;         // Jacobi
    // ILU / ICC factor: private CSR copy with A's pattern
    int64_t nnz = 0;
    int *rowptr = nullptr, *colind = nullptr, *diag = nullptr;
    double *data = nullptr;
    // ICC: transpose of the strict upper part (gather form of R'\b)
    int *rt_rowptr = nullptr, *rt_colind = nullptr;
    double *rt_val = nullptr;
    double *diagv = nullptr;            // R_ii
    mtjg::LevelSchedule lo;             // ILU: L solve; ICC: R' solve
    mtjg::LevelSchedule up;             // U / R solve (rows descending)
    double *y = nullptr;                // temporary of apply
    double *d_b = nullptr, *d_x = nullptr;  // host-call staging
    void *trans = nullptr;              // ILU / ILUT transApply operators, built on first use
    // SSOR(F, reverse, omegaF, omegaR) (S/SSOR.java:62-73) and ILUT(LU, tau, p)
    // (S/ILUT.java:68-85), with MTJ's defaults
    bool reverse = true;
    double omega_f = 1, omega_r = 1;
    double tau = 1e-6;
    int p = 25;
    // FP32 copies for the mixed-precision inner solves (built on first use)
    float *data32 = nullptr, *invdiag32 = nullptr, *y32 = nullptr;
    int64_t v32 = -1;                   // version the copies were made from
};

struct mtjg_solver;
