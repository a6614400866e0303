// C-ABI of batched independent solves (many grids, one launch per RK stage).
//
// The grids keep their own element tables and coefficients; the batch copies
// them into one concatenated device state, builds one neighbour list over all
// elements, and advances every solve with one fused launch per SSP-RK3 stage.
// A step's launches can be captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "amdg.h"
#include "amdg_internal.hpp"
#include "kernels.cuh"
#include "kernels_mlp.cuh"
#include "device_alloc.cuh"

using namespace amdg;

#define AMDG_CK(...)                                                                                    \
    do {                                                                                                \
        cudaError_t amdg_err_ = (__VA_ARGS__);                                                          \
        if (amdg_err_ != cudaSuccess)                                                                   \
            return fail(AMDG_ERR_CUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(amdg_err_)); \
    } while (0)

#define AMDG_REQUIRE(cond, code, msg)        \
    do {                                     \
        if (!(cond)) return fail(code, msg); \
    } while (0)

namespace {

template <class T>
amdg_status alloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) return AMDG_OK;
    cudaError_t e = amdg::device_malloc(reinterpret_cast<void**>(p), n * sizeof(T));
    if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return AMDG_OK;
}

template <class T>
amdg_status put(T** p, const std::vector<T>& h) {
    amdg_status s = alloc(p, h.size());
    if (s != AMDG_OK || h.empty()) return s;
    AMDG_CK(cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return AMDG_OK;
}

cudaStream_t stream_of(const amdg_batch* b) { return static_cast<cudaStream_t>(b->ctx->stream); }

StageCoef coef_of(int stage) {
    switch (stage) {
        case 0: return StageCoef{1, 0.0, 1.0, 0.0};
        case 1: return StageCoef{1, 3. / 4., 1. / 4., 0.0};
        default: return StageCoef{1, 1. / 3., 2. / 3., 0.0};
    }
}

// mixed-mode candidates: [kBatchTileCount, 2 kBatchTileCount) the column kernel on the FP32-pair
// state, from 2 kBatchTileCount the bulk-copy ring kernel (on the same state)
constexpr int kRingFirst = 2 * kBatchTileCount;
// then the column kernel on the same state with a persistent grid, (CTA size, schedule) per
// configuration (schedule 1: static tile order, 2: tiles from a device counter), then the
// warp-per-element kernel
constexpr int kPersistFirst = kRingFirst + kBatchRingConfigs;
constexpr int kPersistConfigs = 3;
constexpr int kPersist[kPersistConfigs][2] = {{64, 1}, {128, 1}, {64, 2}};
constexpr int kWarpFirst = kPersistFirst + kPersistConfigs;
static_assert(kWarpFirst + kBatchWarpConfigs == AMDG_BATCH_KERNELS, "candidate numbering");
bool df_state(const amdg_batch* b, int pi) { return pi == 1 && b->kernel[1] >= kBatchTileCount; }
bool ring_kernel(const amdg_batch* b, int pi) { return pi == 1 && b->kernel[1] >= kRingFirst && b->kernel[1] < kPersistFirst; }
bool persist_kernel(const amdg_batch* b, int pi) {
    return pi == 1 && b->kernel[1] >= kPersistFirst && b->kernel[1] < kWarpFirst;
}
bool warp_kernel(const amdg_batch* b, int pi) { return pi == 1 && b->kernel[1] >= kWarpFirst; }

// one launch of the column kernel on the FP32-pair state: stage `stage`, slot in -> out; schedule
// 1 / 2 persistent (the counter schedule takes its tiles from counter `stage`, zeroed by the caller)
amdg_status df_col_stage(amdg_batch* b, int threads, int stage, int in, int out, cudaStream_t st, int schedule = 0);

// the stage-state arrays of the mixed mode: high and low parts of slot i
float* hi_of(amdg_batch* b, int i) { return b->d_shadow + i * b->sstride; }
float* lo_of(amdg_batch* b, int i) { return b->d_lo + i * b->sstride; }

// one launch of the bulk-copy ring kernel: stage `stage` of the FP32-pair state, slot in -> out
amdg_status ring_stage(amdg_batch* b, int cfg, int stage, int in, int out, cudaStream_t st) {
    const StageCoef c = coef_of(stage);
    BatchRingLaunch L{};
    L.dim = b->dim; L.np = b->k + 1; L.cfg = cfg;
    L.num_elements = b->num_elements; L.num_blocks = b->num_blocks;
    L.row_ptr = b->d_row_ptr; L.pairs = reinterpret_cast<const int2*>(b->d_pairs); L.blocks = b->d_blocks32p;
    L.coef = b->d_coef32; L.dt = b->d_dt32; L.solve_of = b->d_solve;
    L.xs = hi_of(b, in);
    L.df = df_stage(c);
    L.df.us_hi = hi_of(b, in); L.df.us_lo = lo_of(b, in);
    L.df.un_hi = hi_of(b, 0); L.df.un_lo = lo_of(b, 0);
    L.df.out_hi = hi_of(b, out); L.df.out_lo = lo_of(b, out);
    L.err = b->d_err;
    L.wait_limit = 1u << 22;
    AMDG_CK(launch_batch_ring(L, st));
    return AMDG_OK;
}

// one launch of the warp-per-element kernel: stage `stage` of the FP32-pair state, slot in -> out
amdg_status warp_stage(amdg_batch* b, int cfg, int stage, int in, int out, cudaStream_t st) {
    const StageCoef c = coef_of(stage);
    BatchWarpLaunch L{};
    L.dim = b->dim; L.np = b->k + 1; L.cfg = cfg;
    L.num_elements = b->num_elements; L.num_blocks = b->num_blocks;
    L.row_ptr = b->d_row_ptr; L.pairs = reinterpret_cast<const int2*>(b->d_pairs); L.blocks = b->d_blocks32p;
    L.coef = b->d_coef32; L.dt = b->d_dt32; L.solve_of = b->d_solve;
    L.xs = hi_of(b, in);
    L.df = df_stage(c);
    L.df.us_hi = hi_of(b, in); L.df.us_lo = lo_of(b, in);
    L.df.un_hi = hi_of(b, 0); L.df.un_lo = lo_of(b, 0);
    L.df.out_hi = hi_of(b, out); L.df.out_lo = lo_of(b, out);
    AMDG_CK(launch_batch_warp(L, st));
    return AMDG_OK;
}

amdg_status df_col_stage(amdg_batch* b, int threads, int stage, int in, int out, cudaStream_t st, int schedule) {
    const StageCoef c = coef_of(stage);
    BatchLaunch<float, float> L{};
    L.dim = b->dim; L.np = b->k + 1; L.mode = 1; L.a = c.a; L.b = c.b; L.threads = threads;
    L.num_elements = b->num_elements; L.num_blocks = b->num_blocks;
    L.xs = hi_of(b, in);
    L.row_ptr = b->d_row_ptr; L.src = b->d_src; L.blk = b->d_blk; L.blocks = b->d_blocks32;
    L.pairs = reinterpret_cast<const int2*>(b->d_pairs); L.blocks_p = b->d_blocks32p;
    L.coef = b->d_coef32; L.dt = b->d_dt; L.solve_of = b->d_solve;
    L.df = df_stage(c);
    L.df.us_hi = hi_of(b, in); L.df.us_lo = lo_of(b, in);
    L.df.un_hi = hi_of(b, 0); L.df.un_lo = lo_of(b, 0);
    L.df.out_hi = hi_of(b, out); L.df.out_lo = lo_of(b, out);
    L.dt32 = b->d_dt32;
    L.schedule = schedule;
    L.queue = b->d_queue + stage;
    L.sms = b->sms;
    AMDG_CK(launch_batch<float, float>(L, st));
    return AMDG_OK;
}

// one SSP-RK3 step of every solve: three fused launches.  The ring kernel steps the FP32-pair
// state (slots 0 -> 1 -> 2 -> 0, split from and merged into d_u by amdg_batch_rk3_steps); the
// column kernel steps the FP64 state with FP32 shadows of the stage inputs (mixed) or in FP64.
amdg_status batch_step(amdg_batch* b, amdg_precision prec, cudaStream_t st) {
    const int pi = prec == AMDG_PREC_MIXED ? 1 : 0;
    if (df_state(b, pi)) {
        const int in_i[3] = {0, 1, 2}, out_i[3] = {1, 2, 0};
        const int pc = b->kernel[1] - kPersistFirst;
        if (persist_kernel(b, pi) && kPersist[pc][1] == 2)
            AMDG_CK(cudaMemsetAsync(b->d_queue, 0, 3 * sizeof(unsigned long long), st));
        for (int stage = 0; stage < 3; ++stage) {
            amdg_status r = warp_kernel(b, pi)
                                ? warp_stage(b, b->kernel[1] - kWarpFirst, stage, in_i[stage], out_i[stage], st)
                            : persist_kernel(b, pi)
                                ? df_col_stage(b, kPersist[pc][0], stage, in_i[stage], out_i[stage], st, kPersist[pc][1])
                            : ring_kernel(b, pi)
                                ? ring_stage(b, b->kernel[1] - kRingFirst, stage, in_i[stage], out_i[stage], st)
                                : df_col_stage(b, kBatchTiles[b->kernel[1] - kBatchTileCount], stage, in_i[stage],
                                               out_i[stage], st);
            if (r != AMDG_OK) return r;
        }
        return AMDG_OK;
    }
    double* in[3] = {b->d_u, b->d_u1, b->d_u2};
    double* out[3] = {b->d_u1, b->d_u2, b->d_u};
    float* sh[3] = {hi_of(b, 0), hi_of(b, 1), hi_of(b, 2)};
    const int sout[3] = {1, 2, 0};
    const int threads = kBatchTiles[b->kernel[pi]];
    for (int stage = 0; stage < 3; ++stage) {
        const StageCoef c = coef_of(stage);
        if (prec == AMDG_PREC_MIXED) {
            BatchLaunch<float, float> L{};
            L.dim = b->dim; L.np = b->k + 1; L.mode = 1; L.a = c.a; L.b = c.b; L.threads = threads;
            L.num_elements = b->num_elements; L.num_blocks = b->num_blocks;
            L.us = in[stage]; L.xs = sh[stage]; L.un = b->d_u; L.out = out[stage]; L.shadow_out = sh[sout[stage]];
            L.row_ptr = b->d_row_ptr; L.src = b->d_src; L.blk = b->d_blk; L.blocks = b->d_blocks32;
            L.pairs = reinterpret_cast<const int2*>(b->d_pairs); L.blocks_p = b->d_blocks32p;
            L.coef = b->d_coef32; L.dt = b->d_dt; L.solve_of = b->d_solve;
            AMDG_CK(launch_batch<float, float>(L, st));
        } else {
            BatchLaunch<double, double> L{};
            L.dim = b->dim; L.np = b->k + 1; L.mode = 1; L.a = c.a; L.b = c.b; L.threads = threads;
            L.num_elements = b->num_elements; L.num_blocks = b->num_blocks;
            L.us = in[stage]; L.xs = in[stage]; L.un = b->d_u; L.out = out[stage]; L.shadow_out = nullptr;
            L.row_ptr = b->d_row_ptr; L.src = b->d_src; L.blk = b->d_blk; L.blocks = b->d_blocks64;
            L.pairs = reinterpret_cast<const int2*>(b->d_pairs); L.blocks_p = b->d_blocks64p;
            L.coef = b->d_coef64; L.dt = b->d_dt; L.solve_of = b->d_solve;
            AMDG_CK(launch_batch<double, double>(L, st));
        }
    }
    return AMDG_OK;
}

// a bulk-copy wait of the ring kernel gave up: report it and clear the flag (synchronises)
amdg_status check_ring_waits(amdg_batch* b, cudaStream_t st) {
    int h = 0;
    AMDG_CK(cudaMemcpyAsync(&h, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    if (h == 0) return AMDG_OK;
    AMDG_CK(cudaMemsetAsync(b->d_err, 0, sizeof(int), st));
    return fail(AMDG_ERR_TIMEOUT, "batch stage: a bulk copy did not complete within its wait limit; results are invalid");
}

// The concatenated element tables, neighbour lists and state of the batch's grids (as they are
// now), replacing any earlier ones; captured step graphs are dropped.
amdg_status batch_build(amdg_batch* b) {
    const int n = b->nsolves;
    std::vector<const HostGrid*> hg(n);
    for (int i = 0; i < n; ++i) {
        if (amdg_status s = grid_ensure_host(b->grids[i]); s != AMDG_OK) return s;
        hg[i] = &b->grids[i]->host;
    }
    if (b->tables.rel1d.empty()) {
        Basis1D basis{b->k, b->nmax};
        Oper1D op;
        build_oper1d(basis, &op, false);
        build_batch_tables(op, b->nmax, b->k + 1, &b->tables);
    }
    BatchTopology topo;
    build_batch_topology(hg, b->tables, &topo);
    for (int p = 0; p < 2; ++p)
        if (b->graph_exec[p]) {
            cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(b->graph_exec[p]));
            b->graph_exec[p] = nullptr;
        }
    void* old[] = {b->d_row_ptr, b->d_src, b->d_blk, b->d_solve, b->d_blocks64, b->d_blocks32,
                   b->d_u, b->d_u1, b->d_u2, b->d_shadow, b->d_lo, b->d_pairs, b->d_blocks32p, b->d_blocks64p};
    for (void* p : old) cudaFree(p);
    b->d_row_ptr = b->d_src = nullptr;
    b->d_blk = b->d_solve = nullptr;
    b->d_blocks64 = b->d_u = b->d_u1 = b->d_u2 = nullptr;
    b->d_blocks32 = b->d_shadow = b->d_lo = b->d_blocks32p = nullptr;
    b->d_blocks64p = nullptr;
    b->d_pairs = nullptr;
    b->elem_offset = topo.elem_offset;
    b->num_elements = topo.elem_offset[n];
    b->dof = b->num_elements * b->block;
    b->pairs = int64_t(topo.src.size());
    b->num_blocks = topo.num_blocks;
    std::vector<float> b32(topo.blocks.begin(), topo.blocks.end());
    // the ring kernel's tables padded to 16-byte blocks and its interleaved (src, blk) pairs
    const int np = b->k + 1, bs = (np * np + 3) / 4 * 4;
    std::vector<float> b32p(size_t(2) * b->num_blocks * bs, 0.f);
    std::vector<double> b64p(size_t(2) * b->num_blocks * bs, 0.0);
    for (int64_t j = 0; j < int64_t(2) * b->num_blocks; ++j)
        for (int i = 0; i < np * np; ++i) {
            b32p[size_t(j) * bs + i] = b32[size_t(j) * np * np + i];
            b64p[size_t(j) * bs + i] = topo.blocks[size_t(j) * np * np + i];
        }
    AMDG_REQUIRE(b->num_elements < (int64_t(1) << 31), AMDG_ERR_CAPACITY, "more than 2^31-1 elements in the batch");
    std::vector<int32_t> pairs(2 * topo.src.size());
    for (size_t i = 0; i < topo.src.size(); ++i) {
        pairs[2 * i] = int32_t(topo.src[i]);
        pairs[2 * i + 1] = topo.blk[i];
    }
    b->sstride = (b->dof + 3) / 4 * 4 + 4;
    amdg_status s;
    if ((s = put(&b->d_row_ptr, topo.row_ptr)) != AMDG_OK || (s = put(&b->d_src, topo.src)) != AMDG_OK ||
        (s = put(&b->d_blk, topo.blk)) != AMDG_OK || (s = put(&b->d_solve, topo.solve_of)) != AMDG_OK ||
        (s = put(&b->d_blocks64, topo.blocks)) != AMDG_OK || (s = put(&b->d_blocks32, b32)) != AMDG_OK ||
        (s = put(&b->d_blocks32p, b32p)) != AMDG_OK || (s = put(&b->d_blocks64p, b64p)) != AMDG_OK ||
        (s = put(&b->d_pairs, pairs)) != AMDG_OK ||
        (s = alloc(&b->d_u, size_t(b->dof))) != AMDG_OK || (s = alloc(&b->d_u1, size_t(b->dof))) != AMDG_OK ||
        (s = alloc(&b->d_u2, size_t(b->dof))) != AMDG_OK ||
        (s = alloc(&b->d_shadow, size_t(b->sstride) * 3)) != AMDG_OK ||
        (s = alloc(&b->d_lo, size_t(b->sstride) * 3)) != AMDG_OK)
        return s;
    cudaStream_t st = stream_of(b);
    for (int i = 0; i < n; ++i)
        AMDG_CK(cudaMemcpyAsync(b->d_u + b->elem_offset[i] * b->block, b->grids[i]->d_u,
                                size_t(b->grids[i]->dof) * sizeof(double), cudaMemcpyDeviceToDevice, st));
    AMDG_CK(cudaStreamSynchronize(st));
    return AMDG_OK;
}

// Autotuner of the stage kernel: for each precision, time one stage (the first RK stage from the
// current state into the scratch vectors, best of three after a warm-up) with every candidate the
// dimension supports -- the column kernel at each CTA size of kBatchTiles and, mixed only, the
// bulk-copy ring kernel in each configuration -- and keep the fastest.  Batches under 100,000 DOF
// keep the column kernel with 256 threads.
amdg_status autotune_batch(amdg_batch* b, cudaStream_t st) {
    if (b->dof < 100000) return AMDG_OK;
    cudaEvent_t e0, e1;
    AMDG_CK(cudaEventCreate(&e0));
    AMDG_CK(cudaEventCreate(&e1));
    amdg_status status = AMDG_OK;
    AMDG_CK(launch_split(b->d_u, hi_of(b, 0), lo_of(b, 0), b->dof, st));
    const StageCoef c = coef_of(0);
    for (int pi = 0; pi < 2 && status == AMDG_OK; ++pi) {
        float best = 0.f;
        const int ncand = pi == 1 ? AMDG_BATCH_KERNELS : kBatchTileCount;
        for (int ci = 0; ci < ncand; ++ci) {
            const bool warp = ci >= kWarpFirst, persist = ci >= kPersistFirst && !warp;
            const bool ring = ci >= kRingFirst && ci < kPersistFirst;
            const bool dfcol = ci >= kBatchTileCount && ci < kRingFirst;
            const int tile = persist ? kPersist[ci - kPersistFirst][0] : (ring || warp) ? 0 : kBatchTiles[ci % kBatchTileCount];
            if (warp ? !batch_warp_supported(b->dim, b->k + 1, ci - kWarpFirst)
                : ring ? !batch_ring_supported(b->dim, b->k + 1, ci - kRingFirst)
                       : !batch_tile_supported(b->dim, b->k + 1, tile))
                continue;
            float t_min = 0.f;
            for (int rep = 0; rep < 4 && status == AMDG_OK; ++rep) {
                cudaError_t e = cudaEventRecord(e0, st);
                if (warp) {
                    if (e == cudaSuccess && warp_stage(b, ci - kWarpFirst, 0, 0, 1, st) != AMDG_OK)
                        e = cudaErrorLaunchFailure;
                } else if (persist) {
                    const int sched = kPersist[ci - kPersistFirst][1];
                    if (e == cudaSuccess && sched == 2)
                        e = cudaMemsetAsync(b->d_queue, 0, 3 * sizeof(unsigned long long), st);
                    if (e == cudaSuccess && df_col_stage(b, tile, 0, 0, 1, st, sched) != AMDG_OK)
                        e = cudaErrorLaunchFailure;
                } else if (ring) {
                    if (e == cudaSuccess && ring_stage(b, ci - kRingFirst, 0, 0, 1, st) != AMDG_OK)
                        e = cudaErrorLaunchFailure;
                } else if (dfcol) {
                    if (e == cudaSuccess && df_col_stage(b, tile, 0, 0, 1, st) != AMDG_OK) e = cudaErrorLaunchFailure;
                } else if (pi == 1) {
                    BatchLaunch<float, float> L{};
                    L.dim = b->dim; L.np = b->k + 1; L.mode = 1; L.a = c.a; L.b = c.b; L.threads = tile;
                    L.num_elements = b->num_elements; L.num_blocks = b->num_blocks;
                    L.us = b->d_u; L.xs = hi_of(b, 0); L.un = b->d_u; L.out = b->d_u1; L.shadow_out = hi_of(b, 1);
                    L.row_ptr = b->d_row_ptr; L.src = b->d_src; L.blk = b->d_blk; L.blocks = b->d_blocks32;
                    L.pairs = reinterpret_cast<const int2*>(b->d_pairs); L.blocks_p = b->d_blocks32p;
                    L.coef = b->d_coef32; L.dt = b->d_dt; L.solve_of = b->d_solve;
                    if (e == cudaSuccess) e = launch_batch<float, float>(L, st);
                } else {
                    BatchLaunch<double, double> L{};
                    L.dim = b->dim; L.np = b->k + 1; L.mode = 1; L.a = c.a; L.b = c.b; L.threads = tile;
                    L.num_elements = b->num_elements; L.num_blocks = b->num_blocks;
                    L.us = b->d_u; L.xs = b->d_u; L.un = b->d_u; L.out = b->d_u1; L.shadow_out = nullptr;
                    L.row_ptr = b->d_row_ptr; L.src = b->d_src; L.blk = b->d_blk; L.blocks = b->d_blocks64;
                    L.pairs = reinterpret_cast<const int2*>(b->d_pairs); L.blocks_p = b->d_blocks64p;
                    L.coef = b->d_coef64; L.dt = b->d_dt; L.solve_of = b->d_solve;
                    if (e == cudaSuccess) e = launch_batch<double, double>(L, st);
                }
                if (e == cudaSuccess) e = cudaEventRecord(e1, st);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess) {
                    status = fail(AMDG_ERR_CUDA, std::string("batch autotune: ") + cudaGetErrorString(e));
                    break;
                }
                if (rep > 0 && (t_min == 0.f || ms < t_min)) t_min = ms;  // rep 0 warms up
            }
            b->kernel_ms[pi][ci] = t_min;
            if (status == AMDG_OK && (best == 0.f || t_min < best)) {
                best = t_min;
                b->kernel[pi] = ci;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status == AMDG_OK) status = check_ring_waits(b, st);
    return status;
}

}  // namespace

extern "C" {

amdg_status amdg_batch_create(amdg_context* ctx, int n, amdg_grid* const* grids, const double* coef, amdg_batch** out) {
    AMDG_REQUIRE(ctx && grids && coef && out && n > 0, AMDG_ERR_ARG, "bad arguments");
    *out = nullptr;
    const int dim = grids[0]->host.dim, nmax = grids[0]->host.nmax, k = grids[0]->host.k;
    std::vector<const HostGrid*> hg(n);
    for (int i = 0; i < n; ++i) {
        AMDG_REQUIRE(grids[i] && grids[i]->ctx == ctx, AMDG_ERR_ARG, "every grid must belong to the context");
        AMDG_REQUIRE(grids[i]->host.dim == dim && grids[i]->host.nmax == nmax && grids[i]->host.k == k, AMDG_ERR_ARG,
                     "grids must share dim, nmax and k");
        if (amdg_status s = grid_ensure_host(grids[i]); s != AMDG_OK) return s;
        hg[i] = &grids[i]->host;
    }
    for (int i = 0; i < n * dim; ++i) AMDG_REQUIRE(std::isfinite(coef[i]), AMDG_ERR_ARG, "non-finite velocity");
    AMDG_CK(cudaSetDevice(ctx->device));
    amdg_batch* b = new (std::nothrow) amdg_batch;
    AMDG_REQUIRE(b, AMDG_ERR_NOMEM, "host allocation failed");
    b->ctx = ctx;
    b->device = ctx->device;
    b->dim = dim; b->nmax = nmax; b->k = k; b->nsolves = n;
    b->block = grids[0]->block;
    b->grids.assign(grids, grids + n);
    std::vector<double> c64(coef, coef + size_t(n) * dim);
    std::vector<float> c32(c64.begin(), c64.end());
    std::vector<double> dt(n, 0.0);
    std::vector<float> dt32(n, 0.f);
    std::vector<int> err0(1, 0);
    std::vector<unsigned long long> queue0(3, 0);
    if (cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess) b->sms = 0;
    amdg_status s;
    if ((s = put(&b->d_coef64, c64)) != AMDG_OK || (s = put(&b->d_coef32, c32)) != AMDG_OK ||
        (s = put(&b->d_dt, dt)) != AMDG_OK || (s = put(&b->d_dt32, dt32)) != AMDG_OK ||
        (s = put(&b->d_err, err0)) != AMDG_OK || (s = put(&b->d_queue, queue0)) != AMDG_OK ||
        (s = batch_build(b)) != AMDG_OK) {
        amdg_batch_destroy(b);
        return s;
    }
    if (cudaError_t e = batch_prepare_persistent(dim, k + 1); e != cudaSuccess) {
        amdg_batch_destroy(b);
        return fail(AMDG_ERR_CUDA, std::string("persistent batch kernel occupancy: ") + cudaGetErrorString(e));
    }
    cudaStream_t st = stream_of(b);
    if ((s = autotune_batch(b, st)) != AMDG_OK) {
        amdg_batch_destroy(b);
        return s;
    }
    *out = b;
    return AMDG_OK;
}

amdg_status amdg_batch_tuning(const amdg_batch* b, int* kernel, float* stage_ms) {
    AMDG_REQUIRE(b, AMDG_ERR_ARG, "batch is null");
    if (kernel) {
        kernel[0] = b->kernel[0];
        kernel[1] = b->kernel[1];
    }
    if (stage_ms)
        for (int p = 0; p < 2; ++p)
            for (int c = 0; c < AMDG_BATCH_KERNELS; ++c) stage_ms[p * AMDG_BATCH_KERNELS + c] = b->kernel_ms[p][c];
    return AMDG_OK;
}

amdg_status amdg_batch_set_kernel(amdg_batch* b, amdg_precision prec, int kernel) {
    AMDG_REQUIRE(b, AMDG_ERR_ARG, "batch is null");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    bool ok = kernel >= 0 && kernel < AMDG_BATCH_KERNELS && (kernel < kBatchTileCount || prec == AMDG_PREC_MIXED);
    if (ok)
        ok = kernel < kRingFirst     ? batch_tile_supported(b->dim, b->k + 1, kBatchTiles[kernel % kBatchTileCount])
             : kernel < kPersistFirst ? batch_ring_supported(b->dim, b->k + 1, kernel - kRingFirst)
             : kernel < kWarpFirst    ? batch_tile_supported(b->dim, b->k + 1, kPersist[kernel - kPersistFirst][0])
                                      : batch_warp_supported(b->dim, b->k + 1, kernel - kWarpFirst);
    AMDG_REQUIRE(ok, AMDG_ERR_ARG, "unsupported stage kernel for this dimension and precision");
    const int pi = prec == AMDG_PREC_MIXED ? 1 : 0;
    if (b->kernel[pi] != kernel && b->graph_exec[pi]) {
        AMDG_CK(cudaSetDevice(b->device));
        cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(b->graph_exec[pi]));
        b->graph_exec[pi] = nullptr;
    }
    b->kernel[pi] = kernel;
    return AMDG_OK;
}

amdg_status amdg_batch_set_tile(amdg_batch* b, amdg_precision prec, int threads) {
    AMDG_REQUIRE(b, AMDG_ERR_ARG, "batch is null");
    for (int c = 0; c < kBatchTileCount; ++c)
        if (kBatchTiles[c] == threads) return amdg_batch_set_kernel(b, prec, c);
    return fail(AMDG_ERR_ARG, "unsupported CTA size");
}

amdg_status amdg_batch_destroy(amdg_batch* b) {
    if (!b) return AMDG_OK;
    cudaSetDevice(b->device);
    for (int p = 0; p < 2; ++p)
        if (b->graph_exec[p]) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(b->graph_exec[p]));
    void* ptrs[] = {b->d_row_ptr, b->d_src, b->d_blk, b->d_solve, b->d_blocks64, b->d_blocks32, b->d_coef64,
                    b->d_coef32, b->d_dt, b->d_u, b->d_u1, b->d_u2, b->d_shadow, b->d_lo, b->d_pairs,
                    b->d_blocks32p, b->d_blocks64p, b->d_dt32, b->d_err, b->d_queue, b->d_pg, b->d_feat, b->d_prob, b->d_norms};
    for (void* p : ptrs) cudaFree(p);
    delete b;
    return AMDG_OK;
}

amdg_status amdg_batch_size(const amdg_batch* b, int64_t* num_elements, int64_t* dof, int64_t* pairs) {
    AMDG_REQUIRE(b, AMDG_ERR_ARG, "batch is null");
    if (num_elements) *num_elements = b->num_elements;
    if (dof) *dof = b->dof;
    if (pairs) *pairs = b->pairs;
    return AMDG_OK;
}

amdg_status amdg_batch_set_dt(amdg_batch* b, const double* dt) {
    AMDG_REQUIRE(b && dt, AMDG_ERR_ARG, "null argument");
    for (int i = 0; i < b->nsolves; ++i) AMDG_REQUIRE(std::isfinite(dt[i]), AMDG_ERR_ARG, "non-finite dt");
    AMDG_CK(cudaSetDevice(b->device));
    std::vector<float> dt32(dt, dt + b->nsolves);
    AMDG_CK(cudaMemcpyAsync(b->d_dt, dt, size_t(b->nsolves) * sizeof(double), cudaMemcpyHostToDevice, stream_of(b)));
    AMDG_CK(cudaMemcpyAsync(b->d_dt32, dt32.data(), size_t(b->nsolves) * sizeof(float), cudaMemcpyHostToDevice,
                            stream_of(b)));
    AMDG_CK(cudaStreamSynchronize(stream_of(b)));
    return AMDG_OK;
}

amdg_status amdg_batch_rk3_steps(amdg_batch* b, int nsteps, amdg_precision prec, int use_graph) {
    AMDG_REQUIRE(b && nsteps >= 0, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(b->device));
    cudaStream_t st = stream_of(b);
    const int pi = prec == AMDG_PREC_MIXED ? 1 : 0;
    if (nsteps == 0) return AMDG_OK;
    const bool ring = ring_kernel(b, pi), pairs_state = df_state(b, pi);
    if (pairs_state) {  // the FP32-pair state for the whole call: split once here, merged once at the end
        AMDG_CK(launch_split(b->d_u, hi_of(b, 0), lo_of(b, 0), b->dof, st));
        b->ctx->launches++;
    } else if (prec == AMDG_PREC_MIXED) {
        AMDG_CK(launch_to_float(b->d_u, hi_of(b, 0), b->dof, st));
        b->ctx->launches++;
    }
    // after the steps: the ring kernel's wait check, then the merge (a wait that gave up leaves d_u)
    auto finish = [&]() -> amdg_status {
        if (!pairs_state) return AMDG_OK;
        if (ring)
            if (amdg_status r = check_ring_waits(b, st); r != AMDG_OK) return r;
        AMDG_CK(launch_merge(hi_of(b, 0), lo_of(b, 0), b->d_u, b->dof, st));
        b->ctx->launches++;
        return AMDG_OK;
    };
    if (!use_graph) {
        for (int s = 0; s < nsteps; ++s) {
            amdg_status r = batch_step(b, prec, st);
            if (r != AMDG_OK) return r;
            b->ctx->launches += 3;
        }
        return finish();
    }
    if (!b->graph_exec[pi]) {
        // capture one step (three launches) once; pointers and the dt array are fixed
        cudaGraph_t graph = nullptr;
        AMDG_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        amdg_status r = batch_step(b, prec, st);
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        if (r != AMDG_OK) return r;
        if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        cudaGraphExec_t exec = nullptr;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        b->graph_exec[pi] = exec;
    }
    for (int s = 0; s < nsteps; ++s) {
        AMDG_CK(cudaGraphLaunch(static_cast<cudaGraphExec_t>(b->graph_exec[pi]), st));
        b->ctx->launches += 3;
    }
    return finish();
}

amdg_status amdg_batch_store(amdg_batch* b, int solve) {
    AMDG_REQUIRE(b && solve >= 0 && solve < b->nsolves, AMDG_ERR_ARG, "bad arguments");
    amdg_grid* g = b->grids[solve];
    AMDG_REQUIRE(g->host.num_elements == b->elem_offset[solve + 1] - b->elem_offset[solve], AMDG_ERR_STATE,
                 "the grid changed since the batch was built");
    AMDG_CK(cudaSetDevice(b->device));
    AMDG_CK(cudaMemcpyAsync(g->d_u, b->d_u + b->elem_offset[solve] * b->block, size_t(g->dof) * sizeof(double),
                            cudaMemcpyDeviceToDevice, stream_of(b)));
    AMDG_CK(cudaStreamSynchronize(stream_of(b)));
    return AMDG_OK;
}

amdg_status amdg_batch_adapt(amdg_batch* b, amdg_mlp* mlp, double eps, double eta, double tau, int64_t* stats) {
    AMDG_REQUIRE(b && std::isfinite(eps) && std::isfinite(eta) && std::isfinite(tau), AMDG_ERR_ARG, "bad arguments");
    AMDG_CK(cudaSetDevice(b->device));
    cudaStream_t st = stream_of(b);
    const int F = b->block * (1 + 2 * b->dim);
    if (mlp) {
        int n_in = 0, n_out = 0;
        mlp_shape(mlp, &n_in, &n_out);
        AMDG_REQUIRE(n_in == F && n_out == 3, AMDG_ERR_ARG,
                     "classifier must take " + std::to_string(F) + " features and give 3 classes");
    }
    const int n = b->nsolves;
    const int64_t T = b->num_elements;
    std::vector<const HostGrid*> hg(n);
    for (int i = 0; i < n; ++i) {
        if (amdg_status s = grid_ensure_host(b->grids[i]); s != AMDG_OK) return s;
        hg[i] = &b->grids[i]->host;
        AMDG_REQUIRE(hg[i]->num_elements == b->elem_offset[i + 1] - b->elem_offset[i], AMDG_ERR_STATE,
                     "a grid changed since the batch was built");
    }
    amdg_status s;
    AMDG_CK(cudaStreamSynchronize(st));  // steps still in flight finish outside the phase timers
    // element norms of the whole batch state: one launch, one read
    std::vector<double> norms(T);
    {
        PhaseTimer timer(b->ctx, AMDG_PHASE_NORMS);
        if (T > b->norms_elems) {
            cudaFree(b->d_norms);
            b->d_norms = nullptr;
            b->norms_elems = 0;
            if ((s = alloc(&b->d_norms, size_t(T + T / 4))) != AMDG_OK) return s;
            b->norms_elems = T + T / 4;
        }
        AMDG_CK(launch_element_norms(b->d_u, b->block, T, b->d_norms, st));
        b->ctx->launches++;
        if (T > 0) AMDG_CK(cudaMemcpyAsync(norms.data(), b->d_norms, size_t(T) * sizeof(double), cudaMemcpyDeviceToHost, st));
        AMDG_CK(cudaStreamSynchronize(st));
        for (double v : norms) AMDG_REQUIRE(std::isfinite(v), AMDG_ERR_NONFINITE, "element indicator is not finite");
    }
    // classifier over the whole batch state (parent indices into the concatenation); the
    // criterion decides where it is unsure
    int64_t n_net = 0, n_unsure = 0;
    std::vector<uint8_t> force;
    if (mlp) {
        PhaseTimer timer(b->ctx, AMDG_PHASE_CLASSIFIER);
        AMDG_REQUIRE(T < (int64_t(1) << 31), AMDG_ERR_CAPACITY, "more than 2^31-1 elements in the batch");
        if (T > b->scratch_elems) {
            cudaFree(b->d_pg);
            cudaFree(b->d_feat);
            cudaFree(b->d_prob);
            b->d_pg = nullptr;
            b->d_feat = b->d_prob = nullptr;
            b->scratch_elems = 0;
            const int64_t cap = T + T / 4;
            if ((s = alloc(&b->d_pg, size_t(cap) * b->dim * 2)) != AMDG_OK ||
                (s = alloc(&b->d_feat, size_t(cap) * F)) != AMDG_OK || (s = alloc(&b->d_prob, size_t(cap) * 3)) != AMDG_OK)
                return s;
            b->scratch_elems = cap;
        }
        std::vector<int32_t> pg;
        batch_parent_table(hg, b->elem_offset, &pg);
        AMDG_CK(cudaMemcpyAsync(b->d_pg, pg.data(), pg.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
        AMDG_CK(launch_element_features(b->d_u, nullptr, b->d_pg, T, b->dim, b->block, b->d_feat, st));
        b->ctx->launches++;
        if ((s = amdg_mlp_predict(mlp, b->d_feat, T, b->d_prob)) != AMDG_OK) return s;
        std::vector<float> prob(size_t(T) * 3);
        AMDG_CK(cudaMemcpyAsync(prob.data(), b->d_prob, prob.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
        AMDG_CK(cudaStreamSynchronize(st));  // pg and prob are host vectors of this scope
        force.assign(T, 0);
        for (int64_t e = 0; e < T; ++e) {
            const float* p = &prob[size_t(e) * 3];
            int arg = 0;  // classes: 0 refine, 1 keep, 2 coarsen
            for (int q = 1; q < 3; ++q)
                if (p[q] > p[arg]) arg = q;
            if (p[arg] < float(tau)) {
                ++n_unsure;
                force[e] = norms[e] > eps ? 1 : 0;
            } else if (arg == 0) {
                force[e] = 1;
                ++n_net;
            }
        }
    }
    // every solve's state back into its grid
    for (int i = 0; i < n; ++i) {
        amdg_grid* g = b->grids[i];
        AMDG_CK(cudaMemcpyAsync(g->d_u, b->d_u + b->elem_offset[i] * b->block, size_t(g->dof) * sizeof(double),
                                cudaMemcpyDeviceToDevice, st));
    }
    AMDG_CK(cudaStreamSynchronize(st));
    // coarsen, then refine the chosen elements that the coarsening kept, on the host key sets of
    // all solves in parallel; then one element-set replacement per changed solve, in which the
    // coarsened elements that the refinement adds back start at zero (as after a separate
    // coarsen and refine)
    std::vector<std::vector<uint64_t>> keys;
    std::vector<std::vector<uint8_t>> carry;
    {
        PhaseTimer timer(b->ctx, AMDG_PHASE_ADAPT_HOST);
        batch_adapt_keys(hg, b->elem_offset, norms.data(), mlp ? force.data() : nullptr, eps, eta, &keys, &carry);
    }
    for (int i = 0; i < n; ++i) {
        const bool same = int64_t(keys[i].size()) == hg[i]->num_elements &&
                          std::all_of(carry[i].begin(), carry[i].end(), [](uint8_t c) { return c != 0; });
        if (!same && (s = grid_set_keys(b->grids[i], std::move(keys[i]), &carry[i])) != AMDG_OK) {
            // solves before i already have their new element sets: rebuild the batch on the sets the
            // grids now hold, so it stays usable, and report the failure
            const std::string msg = amdg_last_error();
            if (batch_build(b) != AMDG_OK) return s;
            return fail(s, msg);
        }
    }
    {
        PhaseTimer timer(b->ctx, AMDG_PHASE_TOPOLOGY);
        if ((s = batch_build(b)) != AMDG_OK) return s;
    }
    if (stats) {
        stats[0] = n_net;
        stats[1] = n_unsure;
        stats[2] = b->num_elements;
    }
    return AMDG_OK;
}

amdg_status amdg_batch_coefficients_device(amdg_batch* b, double** device_ptr, int64_t* elem_offsets) {
    AMDG_REQUIRE(b && device_ptr, AMDG_ERR_ARG, "null argument");
    *device_ptr = b->d_u;
    if (elem_offsets)
        for (int i = 0; i <= b->nsolves; ++i) elem_offsets[i] = b->elem_offset[i];
    return AMDG_OK;
}

}  // extern "C"
