// C-ABI of libamdg_gb300 (declared in include/amdg.h).  Host-side handle
// management, set-up (1D matrices, element table, neighbour lists) and the
// launch sequences of the device kernels.  No CPU fallback: every compute
// entry point runs on the device or fails with a status.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <unordered_map>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "amdg.h"
#include "amdg_internal.hpp"
#include "kernels.cuh"
#include "device_alloc.cuh"

namespace amdg {

// test hook of amdg_debug_fail_device_allocations: allocations left before one fails (-1: none)
static std::atomic<int64_t> g_fail_after{-1};

cudaError_t device_malloc_raw(void** p, size_t bytes) {
    int64_t left = g_fail_after.load();
    while (left >= 0) {
        if (left == 0) {
            *p = nullptr;
            return cudaErrorMemoryAllocation;
        }
        if (g_fail_after.compare_exchange_weak(left, left - 1)) break;
    }
    return cudaMalloc(p, bytes);
}

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

amdg_status fail(amdg_status s, const std::string& msg) {
    set_error(msg);
    return s;
}

}  // namespace amdg

using namespace amdg;

#define AMDG_CK(...)                                                                                   \
    do {                                                                                                \
        cudaError_t amdg_err_ = (__VA_ARGS__);                                                                 \
        if (amdg_err_ != cudaSuccess)                                                                   \
            return fail(AMDG_ERR_CUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(amdg_err_));      \
    } while (0)

#define AMDG_REQUIRE(cond, code, msg) \
    do {                              \
        if (!(cond)) return fail(code, msg); \
    } while (0)

namespace {

cudaStream_t stream_of(const amdg_context* ctx) { return static_cast<cudaStream_t>(ctx->stream); }

template <class T>
amdg_status dev_alloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return AMDG_OK;
    cudaError_t e = amdg::device_malloc(reinterpret_cast<void**>(p), count * sizeof(T));
    if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return AMDG_OK;
}

template <class T>
amdg_status upload(T** p, const std::vector<T>& host, cudaStream_t st) {
    amdg_status s = dev_alloc(p, host.size());
    if (s != AMDG_OK) return s;
    if (!host.empty()) AMDG_CK(cudaMemcpyAsync(*p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    return AMDG_OK;
}

int ipow(int b, int e) {
    int r = 1;
    while (e-- > 0) r *= b;
    return r;
}

amdg_status set_device(const amdg_context* ctx) {
    AMDG_CK(cudaSetDevice(ctx->device));
    return AMDG_OK;
}

// 1D separable projections of nterms terms: [term][d][nb1]
amdg_status project_terms(const amdg_grid* g, int nterms, const Fn1d& f, std::vector<double>* out) {
    Basis1D b{g->host.k, g->host.nmax};
    const int nb1 = b.num_basis(), dim = g->host.dim;
    out->assign(size_t(nterms) * dim * nb1, 0.0);
    for (int t = 0; t < nterms; ++t)
        for (int d = 0; d < dim; ++d) project_1d(b, f, d, t, out->data() + (size_t(t) * dim + d) * nb1);
    for (double v : *out)
        if (!std::isfinite(v)) return fail(AMDG_ERR_NONFINITE, "separable projection produced a non-finite value");
    return AMDG_OK;
}


}  // namespace

namespace amdg {

static double wall_seconds() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

PhaseTimer::PhaseTimer(amdg_context* ctx, int phase)
    : ctx_(ctx), phase_(phase), t0_(ctx && ctx->profile ? wall_seconds() : 0.0) {}

PhaseTimer::~PhaseTimer() {
    if (ctx_ && ctx_->profile) {
        ctx_->phase_sec[phase_] += wall_seconds() - t0_;
        ctx_->phase_calls[phase_]++;
    }
}

}  // namespace amdg

namespace amdg {

// Replace the grid's element set by `keys` (sorted, unique), carrying the
// coefficients of surviving elements over and zeroing new ones.
amdg_status grid_set_keys(amdg_grid* g, std::vector<uint64_t> keys, const std::vector<uint8_t>* carry) {
    PhaseTimer timer(g->ctx, AMDG_PHASE_SET_KEYS);
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    HostGrid ng;
    ng.sparse = g->host.sparse;
    grid_from_keys(g->host.dim, g->host.nmax, g->host.k, std::move(keys), &ng);
    if (ng.num_elements > (int64_t(1) << 31) - 1) return fail(AMDG_ERR_CAPACITY, "more than 2^31-1 elements");
    // old index of every new element (-1: new), by a merge of the two ascending key lists
    std::vector<int32_t> map(ng.num_elements);
    {
        const std::vector<uint64_t>& ok = g->host.key;
        size_t j = 0;
        for (int64_t e = 0; e < ng.num_elements; ++e) {
            while (j < ok.size() && ok[j] < ng.key[e]) ++j;
            map[e] = (j < ok.size() && ok[j] == ng.key[e] && (!carry || (*carry)[j])) ? int32_t(j) : -1;
        }
    }
    cudaStream_t st = stream_of(g->ctx);
    const int64_t E = ng.num_elements;
    const int64_t grown = E + E / 4 + 16;
    amdg_status s;
    // every allocation before the first change, so a failure leaves the element set as it was
    if ((s = grid_reserve_remap(g, E)) != AMDG_OK) return s;
    if (E > g->map_capacity) {
        cudaFree(g->d_map);  // scratch: no contents to keep
        g->d_map = nullptr;
        g->map_capacity = 0;
        if ((s = dev_alloc(&g->d_map, size_t(grown))) != AMDG_OK) return s;
        g->map_capacity = grown;
    }
    if (E > g->order_capacity) {
        int32_t* p = nullptr;
        if ((s = dev_alloc(&p, size_t(grown) * g->host.dim)) != AMDG_OK) return s;
        cudaFree(g->d_order);
        g->d_order = p;
        g->order_capacity = grown;
    }
    if (E > 0) AMDG_CK(cudaMemcpyAsync(g->d_map, map.data(), size_t(E) * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    // u (and u_t, the prediction) through the map into spare arrays, swapped in; new elements zero
    if ((s = grid_apply_remap(g, E)) != AMDG_OK) return s;
    AMDG_CK(cudaMemcpyAsync(g->d_order, ng.order.data(), ng.order.size() * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    AMDG_CK(cudaStreamSynchronize(st));  // the host map and orders are released on return
    g->host = std::move(ng);
    return grid_upload_keys(g);
}

// indicator norms of a device coefficient vector on the grid's current element set
amdg_status grid_norms(amdg_grid* g, const double* d_u, std::vector<double>* norms, const double* d_u2) {
    if (d_u2) {  // ||u_e|| + ||u2_e||, added in that order (DGAdapt::indicator_norm, DGAdapt.cpp:1018-1030)
        std::vector<double> second;
        if (amdg_status s = grid_norms(g, d_u2, &second); s != AMDG_OK) return s;
        if (amdg_status s = grid_norms(g, d_u, norms); s != AMDG_OK) return s;
        for (size_t e = 0; e < norms->size(); ++e) (*norms)[e] += second[e];
        return AMDG_OK;
    }
    PhaseTimer timer(g->ctx, AMDG_PHASE_NORMS);
    cudaStream_t st = stream_of(g->ctx);
    const int64_t E = g->host.num_elements;
    if (E > g->norms_capacity) {
        cudaFree(g->d_norms);
        g->d_norms = nullptr;
        g->norms_capacity = 0;
        const int64_t cap = E + E / 4 + 16;
        if (amdg_status s = dev_alloc(&g->d_norms, size_t(cap)); s != AMDG_OK) return s;
        g->norms_capacity = cap;
    }
    cudaError_t e = launch_element_norms(d_u, g->block, E, g->d_norms, st);
    g->ctx->launches++;
    norms->assign(E, 0.0);
    if (e == cudaSuccess && E > 0) e = cudaMemcpyAsync(norms->data(), g->d_norms, size_t(E) * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("element norms: ") + cudaGetErrorString(e));
    for (double v : *norms)
        if (!std::isfinite(v)) return fail(AMDG_ERR_NONFINITE, "element indicator is not finite");
    return AMDG_OK;
}

amdg_status grid_coarsen(amdg_grid* g, double eta, const double* d_u2, int64_t* num_elements) {
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    if (g->ctx->adapt_mode == AMDG_ADAPT_DEVICE) {
        PhaseTimer timer(g->ctx, AMDG_PHASE_ADAPT_DEVICE);
        if ((s = grid_device_norms(g, g->d_u, d_u2)) != AMDG_OK || (s = grid_device_coarsen(g, eta, 0.0, nullptr)) != AMDG_OK)
            return s;
        if (num_elements) *num_elements = g->host.num_elements;
        return AMDG_OK;
    }
    if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
    std::vector<double> norms;
    if ((s = grid_norms(g, g->d_u, &norms, d_u2)) != AMDG_OK) return s;
    std::vector<uint64_t> keys;
    {
        PhaseTimer timer(g->ctx, AMDG_PHASE_ADAPT_HOST);
        keys = coarsen_keys(g->host, norms.data(), eta);
    }
    if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
    if (num_elements) *num_elements = g->host.num_elements;
    return AMDG_OK;
}

}  // namespace amdg

namespace {

StageCoef rk3_stage_coef(int stage, double dt) {
    switch (stage) {
        case 0: return StageCoef{1, 0.0, 1.0, dt};
        case 1: return StageCoef{1, 3. / 4., 1. / 4., dt};
        default: return StageCoef{1, 1. / 3., 2. / 3., dt};
    }
}

LinearLaunch linear_launch(const amdg_linear_op* op, amdg_precision prec = AMDG_PREC_FP64) {
    const amdg_grid* g = op->grid;
    LinearLaunch L{};
    L.variant = op->variant[prec == AMDG_PREC_MIXED ? 1 : 0];
    L.dim = g->host.dim;
    L.np = g->host.k + 1;
    L.num_elements = g->host.num_elements;
    L.num_blocks = op->num_blocks;
    L.row_ptr = op->d_row_ptr;
    L.src = op->d_src;
    L.blk = op->d_blk;
    L.blocks64 = op->d_blocks64;
    L.blocks32 = op->d_blocks32;
    L.pairs = reinterpret_cast<const int2*>(op->d_pairs);
    L.blocks64p = op->d_blocks64p;
    L.blocks32p = op->d_blocks32p;
    L.err = op->d_err;
    L.wait_limit = op->wait_limit;
    L.tma_cfg = op->tma_cfg;
    return L;
}

// A bounded copy wait of the bulk-copy variant gave up: report it and clear the flag.
amdg_status check_copy_waits(amdg_linear_op* op) {
    cudaStream_t st = stream_of(op->grid->ctx);
    int h = 0;
    AMDG_CK(cudaMemcpyAsync(&h, op->d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    if (h == 0) return AMDG_OK;
    AMDG_CK(cudaMemsetAsync(op->d_err, 0, sizeof(int), st));
    return fail(AMDG_ERR_TIMEOUT, "linear stage: a bulk copy did not complete within its wait limit; results are invalid");
}

// nsteps SSP-RK3 steps of the state `u` (the grid's own coefficients when null); check:
// read the bulk-copy error flag back at the end (synchronises the stream)
amdg_status rk3_steps_device(amdg_linear_op* op, double dt, int nsteps, amdg_precision prec, double* u = nullptr,
                             bool check = true) {
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(g->ctx);
    if (!u) u = g->d_u;
    LinearLaunch L = linear_launch(op, prec);
    if (prec == AMDG_PREC_MIXED) {
        // the stage vectors live as FP32 (hi, lo) pairs for the whole call:
        // split u once, step without touching the FP64 pipe, merge back once
        float* hi[3] = {op->d_shadow, op->d_shadow + op->capacity, op->d_shadow + 2 * op->capacity};
        float* lo[3] = {op->d_lo, op->d_lo + op->capacity, op->d_lo + 2 * op->capacity};
        if (nsteps == 0) return AMDG_OK;
        AMDG_CK(launch_split(u, hi[0], lo[0], g->dof, st));
        g->ctx->launches++;
        const int in_i[3] = {0, 1, 2}, out_i[3] = {1, 2, 0};
        for (int s = 0; s < nsteps; ++s) {
            for (int stage = 0; stage < 3; ++stage) {
                L.us = nullptr;
                L.un = nullptr;
                L.out = nullptr;
                L.us_shadow = hi[in_i[stage]];
                L.shadow_out = nullptr;
                L.df = df_stage(rk3_stage_coef(stage, dt));
                L.df.us_hi = hi[in_i[stage]];
                L.df.us_lo = lo[in_i[stage]];
                L.df.un_hi = hi[0];
                L.df.un_lo = lo[0];
                L.df.out_hi = hi[out_i[stage]];
                L.df.out_lo = lo[out_i[stage]];
                AMDG_CK(launch_linear(L, true, rk3_stage_coef(stage, dt), st));
                g->ctx->launches++;
            }
        }
        // a copy wait that gave up leaves the state as it was: the merge runs only after the check
        if (L.variant >= 2 && check)
            if (amdg_status s = check_copy_waits(op); s != AMDG_OK) return s;
        AMDG_CK(launch_merge(hi[0], lo[0], u, g->dof, st));
        g->ctx->launches++;
        return AMDG_OK;
    }
    for (int s = 0; s < nsteps; ++s) {
        // u1 = u + dt L(u); u2 = 3/4 u + 1/4 (u1 + dt L(u1)); u = 1/3 u + 2/3 (u2 + dt L(u2))
        double* in[3] = {u, op->d_u1, op->d_u2};
        double* outp[3] = {op->d_u1, op->d_u2, u};
        for (int stage = 0; stage < 3; ++stage) {
            L.us = in[stage];
            L.un = u;
            L.out = outp[stage];
            AMDG_CK(launch_linear(L, false, rk3_stage_coef(stage, dt), st));
            g->ctx->launches++;
        }
    }
    return AMDG_OK;
}

// Pick the kernel variant per precision by timing one fused stage of each on
// the operator's own grid (the grid's state as input, u1 as output).  Small
// grids skip the timing and take the column variant when it applies.
amdg_status autotune_linear(amdg_linear_op* op) {
    amdg_grid* g = op->grid;
    const int dim = g->host.dim, np = g->host.k + 1;
    const bool col = linear_col_supported(dim, np);
    const bool tma = linear_tma_supported(dim, np);
    const bool mma = linear_mma_supported(dim, np);
    for (int p = 0; p < 2; ++p) op->variant[p] = col ? 1 : 0;
    if (!col) return AMDG_OK;
    // small grids time the two CUDA-core variants only (thread per output, column)
    const bool small = g->dof < 200000;
    cudaStream_t st = stream_of(g->ctx);
    cudaEvent_t a, b;
    AMDG_CK(cudaEventCreate(&a));
    AMDG_CK(cudaEventCreate(&b));
    AMDG_CK(launch_split(g->d_u, op->d_shadow, op->d_lo, g->dof, st));
    for (int p = 0; p < 2; ++p) {
        float best = 1e30f;
        for (int v = 0; v < (p == 1 && tma && !small ? 4 : 2); ++v) {
            if (v == 3 && !mma) continue;
            // the bulk-copy variant: time each of its configurations, keep the fastest
            const int ncfg = v == 2 ? kTmaConfigs : 1;
            float best_cfg = 1e30f;
            for (int cfg = 0; cfg < ncfg; ++cfg) {
                if (v == 2 && !linear_tma_supported(dim, np, cfg)) continue;
                LinearLaunch L = linear_launch(op);
                L.variant = v;
                L.tma_cfg = cfg;
                const StageCoef rk{1, 0.0, 1.0, 0.0};
                L.us = g->d_u;
                L.un = g->d_u;
                L.out = op->d_u1;
                if (p == 1) {  // the mixed stage as rk3_steps_device runs it
                    L.us_shadow = op->d_shadow;
                    L.df = df_stage(rk);
                    L.df.us_hi = L.df.un_hi = op->d_shadow;
                    L.df.us_lo = L.df.un_lo = op->d_lo;
                    L.df.out_hi = op->d_shadow + op->capacity;
                    L.df.out_lo = op->d_lo + op->capacity;
                }
                AMDG_CK(launch_linear(L, p == 1, rk, st));  // warm-up
                AMDG_CK(cudaEventRecord(a, st));
                for (int r = 0; r < 3; ++r) AMDG_CK(launch_linear(L, p == 1, rk, st));
                AMDG_CK(cudaEventRecord(b, st));
                AMDG_CK(cudaEventSynchronize(b));
                float ms = 0;
                AMDG_CK(cudaEventElapsedTime(&ms, a, b));
                if (v == 2) op->tma_ms[cfg] = ms / 3;
                if (ms < best_cfg) {
                    best_cfg = ms;
                    if (v == 2) op->tma_cfg = cfg;
                }
            }
            op->variant_ms[p][v] = best_cfg / 3;
            if (best_cfg < best) { best = best_cfg; op->variant[p] = v; }
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return tma ? check_copy_waits(op) : AMDG_OK;
}

// (Re)build the operator's neighbour lists and 1D blocks for the grid's
// current element set; stage vectors grow with the grid.
amdg_status linear_sync(amdg_linear_op* op) {
    amdg_grid* g = op->grid;
    if (op->built_version == g->version) return AMDG_OK;
    Basis1D b{g->host.k, g->host.nmax};
    Oper1D op1d;
    build_oper1d(b, &op1d, false);
    LinearTopology topo;
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    build_linear_topology(g->host, op1d, op->coef.data(), &topo);
    cudaFree(op->d_row_ptr); cudaFree(op->d_src); cudaFree(op->d_blk); cudaFree(op->d_blocks64); cudaFree(op->d_blocks32);
    cudaFree(op->d_pairs); cudaFree(op->d_blocks64p); cudaFree(op->d_blocks32p);
    op->d_pairs = nullptr;
    op->d_blocks64p = nullptr;
    op->d_blocks32p = nullptr;
    op->d_row_ptr = op->d_src = op->d_blk = nullptr;
    op->d_blocks64 = nullptr;
    op->d_blocks32 = nullptr;
    op->pairs = int64_t(topo.src.size());
    op->num_blocks = topo.num_blocks;
    std::vector<float> b32(topo.blocks.begin(), topo.blocks.end());
    // column variant: interleaved (src, blk) pairs and blocks padded to 16-byte multiples
    const int np = g->host.k + 1, bs = (np * np + 3) / 4 * 4;
    std::vector<int32_t> pairs(topo.src.size() * 2);
    for (size_t i = 0; i < topo.src.size(); ++i) { pairs[2 * i] = topo.src[i]; pairs[2 * i + 1] = topo.blk[i]; }
    const size_t nblk = topo.blocks.size() / size_t(np * np);
    std::vector<double> p64(nblk * bs, 0.0);
    for (size_t b = 0; b < nblk; ++b)
        for (int j = 0; j < np * np; ++j) p64[b * bs + j] = topo.blocks[b * np * np + j];
    std::vector<float> p32(p64.begin(), p64.end());
    cudaStream_t st = stream_of(g->ctx);
    amdg_status s;
    if ((s = upload(&op->d_row_ptr, topo.row_ptr, st)) != AMDG_OK || (s = upload(&op->d_src, topo.src, st)) != AMDG_OK ||
        (s = upload(&op->d_blk, topo.blk, st)) != AMDG_OK || (s = upload(&op->d_blocks64, topo.blocks, st)) != AMDG_OK ||
        (s = upload(&op->d_blocks32, b32, st)) != AMDG_OK || (s = upload(&op->d_pairs, pairs, st)) != AMDG_OK ||
        (s = upload(&op->d_blocks64p, p64, st)) != AMDG_OK || (s = upload(&op->d_blocks32p, p32, st)) != AMDG_OK)
        return s;
    if (g->dof > op->capacity) {
        cudaFree(op->d_u1);
        cudaFree(op->d_u2);
        cudaFree(op->d_shadow);
        cudaFree(op->d_lo);
        op->d_u1 = op->d_u2 = nullptr;
        op->d_shadow = op->d_lo = nullptr;
        op->capacity = 0;
        // a multiple of 4 plus 4 spare: the three FP32 arrays start 16-byte
        // aligned and the bulk copies of their last block stay inside
        const int64_t cap = (g->dof + 3) / 4 * 4 + 4;
        if ((s = dev_alloc(&op->d_u1, size_t(cap))) != AMDG_OK || (s = dev_alloc(&op->d_u2, size_t(cap))) != AMDG_OK ||
            (s = dev_alloc(&op->d_shadow, size_t(cap) * 3)) != AMDG_OK ||
            (s = dev_alloc(&op->d_lo, size_t(cap) * 3)) != AMDG_OK)
            return s;
        op->capacity = cap;
    }
    if (!op->d_err) {
        if ((s = dev_alloc(&op->d_err, 1)) != AMDG_OK) return s;
        AMDG_CK(cudaMemsetAsync(op->d_err, 0, sizeof(int), st));
    }
    AMDG_CK(cudaStreamSynchronize(st));
    op->built_version = g->version;
    return autotune_linear(op);
}

}  // namespace

extern "C" {

int amdg_abi_version(void) { return AMDG_ABI_VERSION; }

const char* amdg_status_string(amdg_status s) {
    switch (s) {
        case AMDG_OK: return "ok";
        case AMDG_ERR_ARG: return "invalid argument";
        case AMDG_ERR_CAPACITY: return "capacity exceeded";
        case AMDG_ERR_NONFINITE: return "non-finite value";
        case AMDG_ERR_TIMEOUT: return "device wait timed out";
        case AMDG_ERR_CUDA: return "CUDA error";
        case AMDG_ERR_STATE: return "invalid state";
        case AMDG_ERR_NOMEM: return "out of memory";
    }
    return "unknown status";
}

const char* amdg_last_error(void) { return g_last_error.c_str(); }

amdg_status amdg_context_create(int device, amdg_context** out) {
    AMDG_REQUIRE(out, AMDG_ERR_ARG, "out is null");
    *out = nullptr;
    int n = 0;
    AMDG_CK(cudaGetDeviceCount(&n));
    AMDG_REQUIRE(device >= 0 && device < n, AMDG_ERR_ARG, "device index out of range");
    AMDG_CK(cudaSetDevice(device));
    cudaStream_t st = nullptr;
    AMDG_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    amdg_context* ctx = new (std::nothrow) amdg_context;
    if (!ctx) {
        cudaStreamDestroy(st);
        return fail(AMDG_ERR_NOMEM, "host allocation failed");
    }
    ctx->device = device;
    ctx->stream = st;
    ctx->own_stream = st;
    *out = ctx;
    return AMDG_OK;
}

amdg_status amdg_context_destroy(amdg_context* ctx) {
    if (!ctx) return AMDG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->own_stream) {
        cudaStreamSynchronize(static_cast<cudaStream_t>(ctx->own_stream));
        cudaStreamDestroy(static_cast<cudaStream_t>(ctx->own_stream));
    }
    delete ctx;
    return AMDG_OK;
}

amdg_status amdg_context_set_stream(amdg_context* ctx, void* cuda_stream) {
    AMDG_REQUIRE(ctx, AMDG_ERR_ARG, "ctx is null");
    ctx->stream = cuda_stream ? cuda_stream : ctx->own_stream;
    return AMDG_OK;
}

amdg_status amdg_context_get_stream(amdg_context* ctx, void** cuda_stream) {
    AMDG_REQUIRE(ctx && cuda_stream, AMDG_ERR_ARG, "null argument");
    *cuda_stream = ctx->stream;
    return AMDG_OK;
}

amdg_status amdg_context_synchronize(amdg_context* ctx) {
    AMDG_REQUIRE(ctx, AMDG_ERR_ARG, "ctx is null");
    AMDG_CK(cudaStreamSynchronize(stream_of(ctx)));
    return AMDG_OK;
}

amdg_status amdg_context_launch_count(amdg_context* ctx, int64_t* count) {
    AMDG_REQUIRE(ctx && count, AMDG_ERR_ARG, "null argument");
    *count = ctx->launches;
    return AMDG_OK;
}

amdg_status amdg_debug_fail_device_allocations(int64_t after) {
    AMDG_REQUIRE(after >= -1, AMDG_ERR_ARG, "after must be -1 or more");
    g_fail_after.store(after);
    return AMDG_OK;
}

amdg_status amdg_context_set_adapt_mode(amdg_context* ctx, int mode) {
    AMDG_REQUIRE(ctx && (mode == AMDG_ADAPT_DEVICE || mode == AMDG_ADAPT_HOST), AMDG_ERR_ARG, "bad adapt mode");
    ctx->adapt_mode = mode;
    return AMDG_OK;
}

amdg_status amdg_context_profile(amdg_context* ctx, int enable) {
    AMDG_REQUIRE(ctx, AMDG_ERR_ARG, "null context");
    ctx->profile = enable != 0;
    for (int i = 0; i < AMDG_PHASE_COUNT; ++i) {
        ctx->phase_sec[i] = 0.0;
        ctx->phase_calls[i] = 0;
    }
    return AMDG_OK;
}

amdg_status amdg_context_profile_read(const amdg_context* ctx, double* seconds, int64_t* calls) {
    AMDG_REQUIRE(ctx, AMDG_ERR_ARG, "null context");
    for (int i = 0; i < AMDG_PHASE_COUNT; ++i) {
        if (seconds) seconds[i] = ctx->phase_sec[i];
        if (calls) calls[i] = ctx->phase_calls[i];
    }
    return AMDG_OK;
}

// ---- host-side set-up --------------------------------------------------------

amdg_status amdg_oper1d_build(int nmax, int k, double* u_v, double* u_vx, double* ulft_vjp, double* urgt_vjp) {
    AMDG_REQUIRE(k >= 1 && k <= 3, AMDG_ERR_ARG, "Alpert degree k must be 1..3");
    AMDG_REQUIRE(nmax >= 0 && nmax <= 12, AMDG_ERR_ARG, "nmax must be 0..12");
    Basis1D b{k, nmax};
    Oper1D op;
    build_oper1d(b, &op, u_v != nullptr);
    const size_t n = size_t(op.nb) * op.nb;
    if (u_v) std::memcpy(u_v, op.u_v.data(), n * sizeof(double));
    if (u_vx) std::memcpy(u_vx, op.u_vx.data(), n * sizeof(double));
    if (ulft_vjp) std::memcpy(ulft_vjp, op.ulft_vjp.data(), n * sizeof(double));
    if (urgt_vjp) std::memcpy(urgt_vjp, op.urgt_vjp.data(), n * sizeof(double));
    return AMDG_OK;
}

amdg_status amdg_grid_enumerate(int dim, int nmax, int sparse, int64_t* num_elements, int32_t* level, int32_t* suppt) {
    AMDG_REQUIRE(num_elements, AMDG_ERR_ARG, "num_elements is null");
    AMDG_REQUIRE(dim >= 1 && dim <= kMaxDim, AMDG_ERR_ARG, "dim must be 1..6");
    AMDG_REQUIRE(nmax >= 0 && nmax <= 16 && dim * nmax <= 60, AMDG_ERR_ARG, "nmax out of range");
    HostGrid g;
    build_grid(dim, nmax, sparse, &g);
    *num_elements = g.num_elements;
    if (level) {
        AMDG_REQUIRE(suppt, AMDG_ERR_ARG, "suppt is null");
        for (size_t i = 0; i < g.order.size(); ++i) {
            int lv, j;
            elem_of_order(g.order[i], &lv, &j);
            level[i] = lv;
            suppt[i] = j;
        }
    }
    return AMDG_OK;
}

// ---- grid ------------------------------------------------------------------

amdg_status amdg_grid_create_ex(amdg_context* ctx, int dim, int level_init, int nmax, int k, int sparse, amdg_grid** out) {
    AMDG_REQUIRE(ctx && out, AMDG_ERR_ARG, "null argument");
    *out = nullptr;
    AMDG_REQUIRE(dim >= 1 && dim <= kMaxDim, AMDG_ERR_ARG, "dim must be 1..6");
    AMDG_REQUIRE(k >= 1 && k <= 3, AMDG_ERR_ARG, "Alpert degree k must be 1..3");
    AMDG_REQUIRE(nmax >= 0 && nmax <= 16 && dim * nmax <= 60, AMDG_ERR_ARG, "nmax out of range");
    AMDG_REQUIRE(level_init >= 0 && level_init <= nmax, AMDG_ERR_ARG, "level_init must be 0..nmax");
    amdg_status s = set_device(ctx);
    if (s != AMDG_OK) return s;
    amdg_grid* g = new (std::nothrow) amdg_grid;
    AMDG_REQUIRE(g, AMDG_ERR_NOMEM, "host allocation failed");
    g->ctx = ctx;
    g->device = ctx->device;
    g->host.k = k;
    build_grid(dim, nmax, sparse, &g->host, level_init);
    g->block = ipow(k + 1, dim);
    g->dof = g->host.num_elements * g->block;
    g->capacity = g->host.num_elements;
    g->order_capacity = g->host.num_elements;
    if (g->host.num_elements > (int64_t(1) << 31) - 1) {
        delete g;
        return fail(AMDG_ERR_CAPACITY, "more than 2^31-1 elements");
    }
    cudaStream_t st = stream_of(ctx);
    if ((s = upload(&g->d_order, g->host.order, st)) != AMDG_OK ||
        (s = dev_alloc(&g->d_u, size_t(g->dof))) != AMDG_OK ||
        (s = dev_alloc(&g->d_scratch, size_t(reduce_partials_needed()))) != AMDG_OK) {
        amdg_grid_destroy(g);
        return s;
    }
    g->scratch_bytes = size_t(reduce_partials_needed()) * sizeof(double);
    if ((s = grid_upload_keys(g)) != AMDG_OK) {
        amdg_grid_destroy(g);
        return s;
    }
    cudaError_t e = cudaMemsetAsync(g->d_u, 0, size_t(g->dof) * sizeof(double), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        amdg_grid_destroy(g);
        return fail(AMDG_ERR_CUDA, std::string("grid init: ") + cudaGetErrorString(e));
    }
    *out = g;
    return AMDG_OK;
}

amdg_status amdg_grid_create(amdg_context* ctx, int dim, int nmax, int k, int sparse, amdg_grid** out) {
    return amdg_grid_create_ex(ctx, dim, nmax, nmax, k, sparse, out);
}

amdg_status amdg_grid_destroy(amdg_grid* g) {
    if (!g) return AMDG_OK;
    // cudaFree synchronises with the device; the context may already be gone
    cudaSetDevice(g->device);
    cudaFree(g->d_order);
    cudaFree(g->d_u);
    cudaFree(g->d_scratch);
    cudaFree(g->d_u_spare);
    cudaFree(g->d_map);
    cudaFree(g->d_norms);
    cudaFree(g->d_v);
    cudaFree(g->d_v_spare);
    cudaFree(g->d_pred);
    cudaFree(g->d_pred_spare);
    cudaFree(g->d_pred_v);
    cudaFree(g->d_pred_v_spare);
    cudaFree(g->d_rhs);
    GridDevice& d = g->dev;
    cudaFree(d.key);
    cudaFree(d.key_alt);
    cudaFree(d.hkey);
    cudaFree(d.hval);
    cudaFree(d.newk);
    cudaFree(d.flag);
    cudaFree(d.force);
    cudaFree(d.pos);
    cudaFree(d.missed);
    cudaFree(d.stats);
    cudaFreeHost(d.host_stats);
    cudaFree(d.temp);
    delete g;
    return AMDG_OK;
}

amdg_status amdg_grid_size(const amdg_grid* g, int64_t* num_elements, int64_t* dof) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    if (num_elements) *num_elements = g->host.num_elements;
    if (dof) *dof = g->dof;
    return AMDG_OK;
}

amdg_status amdg_grid_elements(const amdg_grid* g, int32_t* level, int32_t* suppt) {
    AMDG_REQUIRE(g && level && suppt, AMDG_ERR_ARG, "null argument");
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    const size_t n = g->host.order.size();
    for (size_t i = 0; i < n; ++i) {
        int lv, j;
        elem_of_order(g->host.order[i], &lv, &j);
        level[i] = lv;
        suppt[i] = j;
    }
    return AMDG_OK;
}

amdg_status amdg_grid_max_mesh_level(const amdg_grid* g, int32_t* levels) {
    AMDG_REQUIRE(g && levels, AMDG_ERR_ARG, "null argument");
    for (int d = 0; d < g->host.dim; ++d) levels[d] = g->lev_max[d];
    return AMDG_OK;
}

amdg_status amdg_grid_set_coefficients(amdg_grid* g, const double* host, int64_t n) {
    AMDG_REQUIRE(g && host, AMDG_ERR_ARG, "null argument");
    AMDG_REQUIRE(n == g->dof, AMDG_ERR_ARG, "size must equal the grid's dof");
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    AMDG_CK(cudaMemcpyAsync(g->d_u, host, size_t(n) * sizeof(double), cudaMemcpyHostToDevice, st));
    AMDG_CK(cudaStreamSynchronize(st));
    return AMDG_OK;
}

amdg_status amdg_grid_get_coefficients(const amdg_grid* g, double* host, int64_t n) {
    AMDG_REQUIRE(g && host, AMDG_ERR_ARG, "null argument");
    AMDG_REQUIRE(n == g->dof, AMDG_ERR_ARG, "size must equal the grid's dof");
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    AMDG_CK(cudaMemcpyAsync(host, g->d_u, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    return AMDG_OK;
}

amdg_status amdg_grid_coefficients_device(amdg_grid* g, double** device_ptr) {
    AMDG_REQUIRE(g && device_ptr, AMDG_ERR_ARG, "null argument");
    *device_ptr = g->d_u;
    return AMDG_OK;
}

static amdg_status init_separable(amdg_grid* g, int nterms, const Fn1d& f) {
    AMDG_REQUIRE(g && (f.f || f.fb) && nterms > 0, AMDG_ERR_ARG, "bad arguments");
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    std::vector<double> coef;
    if ((s = project_terms(g, nterms, f, &coef)) != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    double* d_coef = nullptr;
    if ((s = upload(&d_coef, coef, st)) != AMDG_OK) return s;
    const int np = g->host.k + 1;
    cudaError_t e = launch_init_separable(g->d_order, d_coef, g->host.dim, np, (1 << g->host.nmax) * np, nterms,
                                          g->host.num_elements, g->d_u, st);
    g->ctx->launches++;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_coef);
    if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("init_separable: ") + cudaGetErrorString(e));
    return AMDG_OK;
}

amdg_status amdg_grid_init_separable(amdg_grid* g, int nterms, amdg_fn1d f, void* user) {
    return init_separable(g, nterms, Fn1d{f, nullptr, user});
}

amdg_status amdg_grid_init_separable_batch(amdg_grid* g, int nterms, amdg_fn1d_batch f, void* user) {
    return init_separable(g, nterms, Fn1d{nullptr, f, user});
}

static amdg_status init_separable_adaptive(amdg_grid* g, int nterms, const Fn1d& f, double eps) {
    AMDG_REQUIRE(g && (f.f || f.fb) && nterms > 0, AMDG_ERR_ARG, "bad arguments");
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    std::vector<double> coef;
    if ((s = project_terms(g, nterms, f, &coef)) != AMDG_OK) return s;
    // refine every leaf whose projected block exceeds eps, fill holes, repeat
    // until nothing changes (DGAdapt::refine_init_separable_scalar_sum)
    // norms depend only on the element, so each is computed once; the element
    // set is refined on the host and the device arrays are rebuilt once at the end
    if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
    HostGrid work = g->host;
    std::unordered_map<uint64_t, double> cache;
    for (;;) {
        HostGrid fresh;
        fresh.dim = work.dim; fresh.nmax = work.nmax; fresh.k = work.k;
        std::vector<uint64_t> todo;
        for (int64_t e = 0; e < work.num_elements; ++e)
            if (!cache.count(work.key[e])) todo.push_back(work.key[e]);
        grid_from_keys(work.dim, work.nmax, work.k, todo, &fresh);
        std::vector<double> fn;
        element_separable_norms(fresh, coef, nterms, &fn);
        for (int64_t e = 0; e < fresh.num_elements; ++e) cache[fresh.key[e]] = fn[e];
        std::vector<double> norms(work.num_elements);
        for (int64_t e = 0; e < work.num_elements; ++e) norms[e] = cache[work.key[e]];
        std::vector<uint64_t> keys = refine_keys(work, norms.data(), eps);
        if (int64_t(keys.size()) == work.num_elements) break;
        grid_from_keys(work.dim, work.nmax, work.k, std::move(keys), &work);
    }
    if (work.num_elements != g->host.num_elements && (s = grid_set_keys(g, work.key)) != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    double* d_coef = nullptr;
    if ((s = upload(&d_coef, coef, st)) != AMDG_OK) return s;
    const int np = g->host.k + 1;
    cudaError_t e = launch_init_separable(g->d_order, d_coef, g->host.dim, np, (1 << g->host.nmax) * np, nterms,
                                          g->host.num_elements, g->d_u, st);
    g->ctx->launches++;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_coef);
    if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("init_separable: ") + cudaGetErrorString(e));
    return AMDG_OK;
}

amdg_status amdg_grid_init_separable_adaptive(amdg_grid* g, int nterms, amdg_fn1d f, void* user, double eps) {
    return init_separable_adaptive(g, nterms, Fn1d{f, nullptr, user}, eps);
}

amdg_status amdg_grid_init_separable_adaptive_batch(amdg_grid* g, int nterms, amdg_fn1d_batch f, void* user,
                                                    double eps) {
    return init_separable_adaptive(g, nterms, Fn1d{nullptr, f, user}, eps);
}

amdg_status amdg_grid_refine(amdg_grid* g, const double* d_indicator, double eps, int64_t* num_elements) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    const double* u2 = g->indicator == AMDG_INDICATOR_U_UT ? g->d_v : nullptr;
    AMDG_REQUIRE(g->indicator != AMDG_INDICATOR_U_UT || u2, AMDG_ERR_STATE,
                 "the u + u_t indicator needs the grid's velocity field");
    if (g->ctx->adapt_mode == AMDG_ADAPT_DEVICE) {
        PhaseTimer timer(g->ctx, AMDG_PHASE_ADAPT_DEVICE);
        if ((s = grid_device_norms(g, d_indicator ? d_indicator : g->d_u, u2)) != AMDG_OK ||
            (s = grid_device_refine(g, eps, nullptr, nullptr, nullptr)) != AMDG_OK)
            return s;
        if (num_elements) *num_elements = g->host.num_elements;
        return AMDG_OK;
    }
    if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
    std::vector<double> norms;
    if ((s = grid_norms(g, d_indicator ? d_indicator : g->d_u, &norms, u2)) != AMDG_OK) return s;
    std::vector<uint64_t> keys;
    {
        PhaseTimer timer(g->ctx, AMDG_PHASE_ADAPT_HOST);
        keys = refine_keys(g->host, norms.data(), eps);
    }
    if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
    if (num_elements) *num_elements = g->host.num_elements;
    return AMDG_OK;
}

amdg_status amdg_grid_coarsen(amdg_grid* g, double eta, int64_t* num_elements) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    const double* u2 = g->indicator == AMDG_INDICATOR_U_UT ? g->d_v : nullptr;
    AMDG_REQUIRE(g->indicator != AMDG_INDICATOR_U_UT || u2, AMDG_ERR_STATE,
                 "the u + u_t indicator needs the grid's velocity field");
    return amdg::grid_coarsen(g, eta, u2, num_elements);
}

amdg_status amdg_grid_set_indicator(amdg_grid* g, int mode) {
    AMDG_REQUIRE(g && (mode == AMDG_INDICATOR_U || mode == AMDG_INDICATOR_U_UT), AMDG_ERR_ARG, "bad arguments");
    g->indicator = mode;
    return AMDG_OK;
}

amdg_status amdg_grid_set_velocity(amdg_grid* g, const double* host, int64_t n) {
    AMDG_REQUIRE(g && host && n == g->dof, AMDG_ERR_ARG, "velocity must have dof entries");
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    if (!g->d_v || g->v_capacity < g->host.num_elements) {
        cudaFree(g->d_v);
        g->d_v = nullptr;
        g->v_capacity = 0;
        const int64_t cap = std::max<int64_t>(g->capacity, g->host.num_elements);
        if ((s = dev_alloc(&g->d_v, size_t(std::max<int64_t>(cap, 1)) * g->block)) != AMDG_OK) return s;
        g->v_capacity = cap;
    }
    cudaStream_t st = stream_of(g->ctx);
    if (n) AMDG_CK(cudaMemcpyAsync(g->d_v, host, size_t(n) * sizeof(double), cudaMemcpyHostToDevice, st));
    AMDG_CK(cudaStreamSynchronize(st));
    return AMDG_OK;
}

amdg_status amdg_grid_get_velocity(const amdg_grid* g, double* host, int64_t n) {
    AMDG_REQUIRE(g && host && n == g->dof, AMDG_ERR_ARG, "velocity must have dof entries");
    AMDG_REQUIRE(g->d_v, AMDG_ERR_STATE, "the grid has no velocity field");
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    if (n) AMDG_CK(cudaMemcpyAsync(host, g->d_v, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    return AMDG_OK;
}

amdg_status amdg_grid_version(const amdg_grid* g, int64_t* version) {
    AMDG_REQUIRE(g && version, AMDG_ERR_ARG, "null argument");
    *version = g->version;
    return AMDG_OK;
}

static amdg_status reduce_grid(const amdg_grid* g, const double* d_coef, int mode, double* out, int nterms = 1) {
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    const int np = g->host.k + 1;
    AMDG_CK(launch_reduce(g->d_u, g->d_order, d_coef, g->host.dim, np, (1 << g->host.nmax) * np, g->host.num_elements,
                          mode, g->d_scratch, st, nterms));
    g->ctx->launches += 2;
    double r = 0.0;
    AMDG_CK(cudaMemcpyAsync(&r, g->d_scratch + kReduceBlocks, sizeof(double), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    if (!std::isfinite(r)) return fail(AMDG_ERR_NONFINITE, "reduction met a non-finite value");
    *out = r;
    return AMDG_OK;
}

amdg_status amdg_grid_l2_norm(const amdg_grid* g, double* out) {
    AMDG_REQUIRE(g && out, AMDG_ERR_ARG, "null argument");
    return reduce_grid(g, nullptr, 0, out);
}

amdg_status amdg_grid_l2_error_separable(const amdg_grid* g, amdg_fn1d f, void* user, double l2_norm_exact, double* out) {
    return amdg_grid_l2_error_separable_sum(g, 1, f, user, l2_norm_exact, out);
}

static amdg_status l2_error_separable_sum(const amdg_grid* g, int nterms, const Fn1d& f, double l2_norm_exact,
                                          double* out) {
    AMDG_REQUIRE(g && (f.f || f.fb) && out && nterms > 0, AMDG_ERR_ARG, "bad arguments");
    std::vector<double> coef;
    amdg_status s = project_terms(g, nterms, f, &coef);
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    double* d_coef = nullptr;
    if ((s = upload(&d_coef, coef, st)) != AMDG_OK) return s;
    double r = 0.0;
    s = reduce_grid(g, d_coef, 1, &r, nterms);
    cudaFree(d_coef);
    if (s != AMDG_OK) return s;
    const double err2 = l2_norm_exact * l2_norm_exact + r;
    *out = std::sqrt(err2 > 0.0 ? err2 : 0.0);
    return AMDG_OK;
}

amdg_status amdg_grid_l2_error_separable_sum(const amdg_grid* g, int nterms, amdg_fn1d f, void* user,
                                             double l2_norm_exact, double* out) {
    return l2_error_separable_sum(g, nterms, Fn1d{f, nullptr, user}, l2_norm_exact, out);
}

amdg_status amdg_grid_l2_error_separable_sum_batch(const amdg_grid* g, int nterms, amdg_fn1d_batch f, void* user,
                                                   double l2_norm_exact, double* out) {
    return l2_error_separable_sum(g, nterms, Fn1d{nullptr, f, user}, l2_norm_exact, out);
}

// ---- linear operator ---------------------------------------------------------

amdg_status amdg_linear_create(amdg_grid* g, const double* coef, amdg_linear_op** out) {
    AMDG_REQUIRE(g && coef && out, AMDG_ERR_ARG, "null argument");
    *out = nullptr;
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    const int dim = g->host.dim;
    for (int d = 0; d < dim; ++d) AMDG_REQUIRE(std::isfinite(coef[d]), AMDG_ERR_ARG, "non-finite coefficient");
    amdg_linear_op* op = new (std::nothrow) amdg_linear_op;
    AMDG_REQUIRE(op, AMDG_ERR_NOMEM, "host allocation failed");
    op->grid = g;
    op->device = g->device;
    op->coef.assign(coef, coef + dim);
    if ((s = linear_sync(op)) != AMDG_OK) {
        amdg_linear_destroy(op);
        return s;
    }
    *out = op;
    return AMDG_OK;
}

amdg_status amdg_linear_destroy(amdg_linear_op* op) {
    if (!op) return AMDG_OK;
    cudaSetDevice(op->device);
    cudaFree(op->d_row_ptr);
    cudaFree(op->d_src);
    cudaFree(op->d_blk);
    cudaFree(op->d_pairs);
    cudaFree(op->d_blocks64p);
    cudaFree(op->d_blocks32p);
    cudaFree(op->d_blocks64);
    cudaFree(op->d_blocks32);
    cudaFree(op->d_u1);
    cudaFree(op->d_u2);
    cudaFree(op->d_err);
    cudaFree(op->d_shadow);
    cudaFree(op->d_lo);
    for (double* p : op->d_io) cudaFree(p);
    for (void* e : op->io_event)
        if (e) cudaEventDestroy(static_cast<cudaEvent_t>(e));
    for (void* c : op->io_stream)
        if (c) cudaStreamDestroy(static_cast<cudaStream_t>(c));
    delete op;
    return AMDG_OK;
}

amdg_status amdg_linear_tuning(const amdg_linear_op* op, int* variants, float* stage_ms) {
    AMDG_REQUIRE(op, AMDG_ERR_ARG, "op is null");
    for (int p = 0; p < 2; ++p) {
        if (variants) variants[p] = op->variant[p];
        for (int v = 0; v < 4; ++v)
            if (stage_ms) stage_ms[p * 4 + v] = op->variant_ms[p][v];
    }
    return AMDG_OK;
}

amdg_status amdg_linear_set_variant(amdg_linear_op* op, amdg_precision prec, int variant) {
    AMDG_REQUIRE(op && (prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED), AMDG_ERR_ARG, "bad arguments");
    const int dim = op->grid->host.dim, np = op->grid->host.k + 1;
    AMDG_REQUIRE(variant == 0 || (variant == 1 && linear_col_supported(dim, np)) ||
                     (variant == 2 && prec == AMDG_PREC_MIXED && linear_tma_supported(dim, np)) ||
                     (variant == 3 && prec == AMDG_PREC_MIXED && linear_mma_supported(dim, np)),
                 AMDG_ERR_ARG, "unsupported kernel variant");
    op->variant[prec == AMDG_PREC_MIXED ? 1 : 0] = variant;
    return AMDG_OK;
}

static_assert(sizeof(amdg_linear_op::tma_ms) / sizeof(float) == kTmaConfigs, "one timing per configuration");

amdg_status amdg_linear_copy_config(const amdg_linear_op* op, int* config, float* stage_ms) {
    AMDG_REQUIRE(op, AMDG_ERR_ARG, "op is null");
    if (config) *config = op->tma_cfg;
    if (stage_ms)
        for (int c = 0; c < kTmaConfigs; ++c) stage_ms[c] = op->tma_ms[c];
    return AMDG_OK;
}

amdg_status amdg_linear_set_copy_config(amdg_linear_op* op, int config) {
    AMDG_REQUIRE(op, AMDG_ERR_ARG, "op is null");
    const int dim = op->grid->host.dim, np = op->grid->host.k + 1;
    AMDG_REQUIRE(linear_tma_supported(dim, np, config), AMDG_ERR_ARG, "unsupported bulk-copy configuration");
    op->tma_cfg = config;
    return AMDG_OK;
}

amdg_status amdg_linear_set_wait_limit(amdg_linear_op* op, uint32_t polls) {
    AMDG_REQUIRE(op, AMDG_ERR_ARG, "null argument");
    op->wait_limit = polls;
    return AMDG_OK;
}

amdg_status amdg_linear_stats(const amdg_linear_op* op, int64_t* pairs, double* flops_per_apply) {
    AMDG_REQUIRE(op, AMDG_ERR_ARG, "op is null");
    const int np = op->grid->host.k + 1;
    if (pairs) *pairs = op->pairs;
    if (flops_per_apply) *flops_per_apply = 2.0 * double(op->pairs) * double(ipow(np, op->grid->host.dim + 1));
    return AMDG_OK;
}

amdg_status amdg_linear_apply(amdg_linear_op* op, const double* d_u, double* d_rhs, amdg_precision prec) {
    AMDG_REQUIRE(op && d_u && d_rhs, AMDG_ERR_ARG, "null argument");
    AMDG_REQUIRE(d_u != d_rhs, AMDG_ERR_ARG, "input and output must differ");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    amdg_status s = set_device(op->grid->ctx);
    if (s != AMDG_OK) return s;
    if ((s = linear_sync(op)) != AMDG_OK) return s;
    LinearLaunch L = linear_launch(op, prec);
    L.us = d_u;
    L.un = nullptr;
    L.out = d_rhs;
    cudaStream_t st = stream_of(op->grid->ctx);
    if (prec == AMDG_PREC_MIXED) {
        AMDG_CK(launch_to_float(d_u, op->d_shadow, op->grid->dof, st));
        op->grid->ctx->launches++;
        L.us_shadow = op->d_shadow;
    }
    AMDG_CK(launch_linear(L, prec == AMDG_PREC_MIXED, StageCoef{0, 0.0, 0.0, 0.0}, st));
    op->grid->ctx->launches++;
    return AMDG_OK;
}

amdg_status amdg_rk3ssp_steps(amdg_linear_op* op, double dt, int nsteps, amdg_precision prec) {
    AMDG_REQUIRE(op && nsteps >= 0 && std::isfinite(dt), AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    amdg_status s = set_device(op->grid->ctx);
    if (s != AMDG_OK) return s;
    if ((s = linear_sync(op)) != AMDG_OK) return s;
    return rk3_steps_device(op, dt, nsteps, prec);
}

amdg_status amdg_rk3ssp_steps_host(amdg_linear_op* op, double dt, int nsteps, double* host_u, amdg_precision prec) {
    AMDG_REQUIRE(op && host_u && nsteps >= 0 && std::isfinite(dt), AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    amdg_grid* g = op->grid;
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    if ((s = linear_sync(op)) != AMDG_OK) return s;
    cudaStream_t st = stream_of(g->ctx);
    const size_t bytes = size_t(g->dof) * sizeof(double);
    AMDG_CK(cudaMemcpyAsync(g->d_u, host_u, bytes, cudaMemcpyHostToDevice, st));
    if ((s = rk3_steps_device(op, dt, nsteps, prec)) != AMDG_OK) return s;
    AMDG_CK(cudaMemcpyAsync(host_u, g->d_u, bytes, cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    return AMDG_OK;
}

amdg_status amdg_rk3ssp_serve_host(amdg_linear_op* op, double dt, int nsteps, amdg_precision prec, int nreq,
                                   const double* const* host_in, double* const* host_out) {
    AMDG_REQUIRE(op && nsteps >= 0 && nreq >= 0 && std::isfinite(dt) && (nreq == 0 || (host_in && host_out)),
                 AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    for (int r = 0; r < nreq; ++r) AMDG_REQUIRE(host_in[r] && host_out[r], AMDG_ERR_ARG, "null request buffer");
    amdg_grid* g = op->grid;
    amdg_status s = set_device(g->ctx);
    if (s != AMDG_OK) return s;
    if ((s = linear_sync(op)) != AMDG_OK) return s;
    const size_t bytes = size_t(g->dof) * sizeof(double);
    constexpr int NB = 3;  // device states: request r is copied in while r - 1 steps and r - 2 is copied out
    if (!op->d_io[0] || op->io_capacity < g->dof) {
        for (int b = 0; b < NB; ++b) {
            cudaFree(op->d_io[b]);
            op->d_io[b] = nullptr;
        }
        op->io_capacity = 0;
        for (int b = 0; b < NB; ++b)
            if ((s = dev_alloc(&op->d_io[b], size_t(g->dof))) != AMDG_OK) return s;
        op->io_capacity = g->dof;
    }
    if (!op->io_stream[0]) {
        for (int i = 0; i < 2; ++i) {
            cudaStream_t c = nullptr;
            AMDG_CK(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
            op->io_stream[i] = c;
        }
        for (int i = 0; i < 3 * NB; ++i) {
            cudaEvent_t e = nullptr;
            AMDG_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            op->io_event[i] = e;
        }
    }
    cudaStream_t st = stream_of(g->ctx);
    cudaStream_t in_st = static_cast<cudaStream_t>(op->io_stream[0]);
    cudaStream_t out_st = static_cast<cudaStream_t>(op->io_stream[1]);
    // per buffer b: copied in, stepped, copied out
    cudaEvent_t in_done[NB], stepped[NB], out_done[NB];
    for (int b = 0; b < NB; ++b) {
        in_done[b] = static_cast<cudaEvent_t>(op->io_event[b]);
        stepped[b] = static_cast<cudaEvent_t>(op->io_event[NB + b]);
        out_done[b] = static_cast<cudaEvent_t>(op->io_event[2 * NB + b]);
    }
    // earlier work on the context stream (the grid's state, the operator's tables) comes first
    AMDG_CK(cudaEventRecord(stepped[0], st));
    AMDG_CK(cudaStreamWaitEvent(in_st, stepped[0], 0));
    auto copy_in = [&](int r) -> amdg_status {
        const int b = r % NB;
        if (r >= NB) AMDG_CK(cudaStreamWaitEvent(in_st, out_done[b], 0));  // buffer b's previous result is out
        AMDG_CK(cudaMemcpyAsync(op->d_io[b], host_in[r], bytes, cudaMemcpyHostToDevice, in_st));
        AMDG_CK(cudaEventRecord(in_done[b], in_st));
        return AMDG_OK;
    };
    // request r + 1 is copied in while request r is stepped and request r - 1 copied out
    if (nreq > 0 && (s = copy_in(0)) != AMDG_OK) return s;
    for (int r = 0; r < nreq; ++r) {
        const int b = r % NB;
        if (r + 1 < nreq && (s = copy_in(r + 1)) != AMDG_OK) return s;
        AMDG_CK(cudaStreamWaitEvent(st, in_done[b], 0));
        if ((s = rk3_steps_device(op, dt, nsteps, prec, op->d_io[b], false)) != AMDG_OK) return s;
        AMDG_CK(cudaEventRecord(stepped[b], st));
        AMDG_CK(cudaStreamWaitEvent(out_st, stepped[b], 0));
        AMDG_CK(cudaMemcpyAsync(host_out[r], op->d_io[b], bytes, cudaMemcpyDeviceToHost, out_st));
        AMDG_CK(cudaEventRecord(out_done[b], out_st));
    }
    AMDG_CK(cudaStreamSynchronize(out_st));
    AMDG_CK(cudaStreamSynchronize(in_st));
    AMDG_CK(cudaStreamSynchronize(st));
    return linear_launch(op, prec).variant >= 2 ? check_copy_waits(op) : AMDG_OK;
}

amdg_status amdg_rk3_stage_update(amdg_context* ctx, int stage, double dt, const double* d_un, double* d_u,
                                  const double* d_rhs, int64_t n) {
    AMDG_REQUIRE(ctx && d_un && d_u && d_rhs && n >= 0, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(stage >= 0 && stage <= 2, AMDG_ERR_ARG, "stage must be 0..2");
    amdg_status s = set_device(ctx);
    if (s != AMDG_OK) return s;
    AMDG_CK(launch_stage_update(d_un, d_u, d_rhs, n, rk3_stage_coef(stage, dt), stream_of(ctx)));
    ctx->launches++;
    return AMDG_OK;
}

}  // extern "C"
