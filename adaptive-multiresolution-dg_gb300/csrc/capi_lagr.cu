// C-ABI of the Lagrange-interpolation path (Burgers flux): set-up of the 1D
// tables and neighbour lists, and the launch sequence of one right-hand-side
// evaluation -- point values by 2^(dim-1) partial sums of dim 1D transforms,
// flux at the points, dim hierarchical-surplus passes, volume and interface
// terms by the same partial sums back to Alpert coefficients, LxF penalty,
// and the SSP-RK3 stage update.
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
#include "kernels_lagr.cuh"
#include "kernels_mlp.cuh"

using namespace amdg;

#define AMDG_CK(...)                                                                              \
    do {                                                                                           \
        cudaError_t amdg_err_ = (__VA_ARGS__);                                                            \
        if (amdg_err_ != cudaSuccess)                                                              \
            return fail(AMDG_ERR_CUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(amdg_err_)); \
    } while (0)

#define AMDG_REQUIRE(cond, code, msg)        \
    do {                                     \
        if (!(cond)) return fail(code, msg); \
    } while (0)

namespace {

template <class T>
amdg_status upload_vec(T** p, const std::vector<T>& host) {
    *p = nullptr;
    if (host.empty()) return AMDG_OK;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), host.size() * sizeof(T));
    if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    AMDG_CK(cudaMemcpy(*p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice));
    return AMDG_OK;
}

amdg_status upload_both(double** d, float** f, const std::vector<double>& host) {
    amdg_status s = upload_vec(d, host);
    if (s != AMDG_OK) return s;
    std::vector<float> h32(host.begin(), host.end());
    return upload_vec(f, h32);
}

amdg_status alloc_bytes(void** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return AMDG_OK;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return AMDG_OK;
}

cudaStream_t stream_of(const amdg_burgers_op* op) { return static_cast<cudaStream_t>(op->grid->ctx->stream); }

template <typename T>
struct Mats {
    const T *a2p, *lv, *lvx, *lflx, *ajump;
};

Mats<double> mats64(const amdg_burgers_op* op) { return {op->d_a2p, op->d_lv, op->d_lvx, op->d_lflx, op->d_ajump}; }
Mats<float> mats32(const amdg_burgers_op* op) { return {op->f_a2p, op->f_lv, op->f_lvx, op->f_lflx, op->f_ajump}; }

int prod(const int* s, int n) {
    int p = 1;
    for (int i = 0; i < n; ++i) p *= s[i];
    return p;
}

template <typename T>
TransformArgs<T> base_args(const amdg_burgers_op* op, int t, const int* from, const int* to, bool flx) {
    const amdg_grid* g = op->grid;
    const int dim = g->host.dim;
    TransformArgs<T> a{};
    a.dim = dim;
    a.t = t;
    a.n_from = from[t];
    a.n_to = to[t];
    a.stride = prod(from + t + 1, dim - t - 1);
    a.in_block = prod(from, dim);
    a.out_block = prod(to, dim);
    a.num_elements = g->host.num_elements;
    a.order = g->d_order;
    a.ptr = flx ? op->d_flx_ptr : op->d_vol_ptr;
    a.nbr = reinterpret_cast<const int2*>(flx ? op->d_flx_nbr : op->d_vol_nbr);
    a.split = flx ? op->d_flx_split : op->d_vol_split;
    a.long_flag = flx ? op->d_flx_long : op->d_vol_long;
    const std::vector<int32_t>& off = flx ? op->flx_long_off : op->vol_long_off;
    a.long_elems = (flx ? op->d_flx_long_elems : op->d_vol_long_elems) + off[t];
    a.num_long = off[t + 1] - off[t];
    return a;
}

// One partial sum: dim successive 1D transforms, the first scaled by coef, the
// last accumulated into out (FastRHS::transform_multiD_partial_sum,
// FastInterpolation::transform_multiD_partial_sum).
template <typename T>
amdg_status partial_sum(amdg_burgers_op* op, const std::vector<int>& dims, const std::vector<int>& lu, int n_in, int n_out,
                        const T* const* mat, const bool* flx, T coef, const T* in, T* out, T* tmp_a, T* tmp_b,
                        cudaStream_t st) {
    const int dim = op->grid->host.dim;
    int from[kMaxDim], to[kMaxDim];
    for (int d = 0; d < dim; ++d) from[d] = n_in;
    const T* cur = in;
    for (int i = 0; i < dim; ++i) {
        const int t = dims[i];
        std::memcpy(to, from, sizeof(int) * dim);
        to[t] = n_out;
        TransformArgs<T> a = base_args<T>(op, t, from, to, flx[t]);
        a.M = mat[t];
        a.ncols = op->n1 * n_out;
        a.lu = lu[i];
        a.coef = (i == 0) ? coef : T(1);
        a.in = cur;
        const bool last = (i == dim - 1);
        T* dst = last ? out : ((cur == tmp_a) ? tmp_b : tmp_a);
        a.out = dst;
        a.accumulate = last ? 1 : 0;
        AMDG_CK(launch_fibre_transform<T>(a, st));
        op->grid->ctx->launches++;
        cur = dst;
        std::memcpy(from, to, sizeof(int) * dim);
    }
    return AMDG_OK;
}

template <typename T>
amdg_status eval_point_values(amdg_burgers_op* op, const Mats<T>& m, const T* u, T* up, cudaStream_t st) {
    const amdg_grid* g = op->grid;
    const int dim = g->host.dim, np = g->host.k + 1;
    AMDG_CK(cudaMemsetAsync(up, 0, size_t(g->host.num_elements) * op->points * sizeof(T), st));
    const T* mats[kMaxDim];
    bool flx[kMaxDim];
    for (int d = 0; d < dim; ++d) { mats[d] = m.a2p; flx[d] = false; }
    T* ta = static_cast<T*>(op->w_a);
    T* tb = static_cast<T*>(op->w_b);
    for (size_t s = 0; s < op->sched_dims.size(); ++s) {
        amdg_status r = partial_sum<T>(op, op->sched_dims[s], op->sched_lu[s], np, 4, mats, flx, T(1), u, up, ta, tb, st);
        if (r != AMDG_OK) return r;
    }
    return AMDG_OK;
}

// flux interpolation coefficients: f(u) at the points, then dim surplus passes (result in op->w_fu)
template <typename T>
amdg_status eval_flux_coefficients(amdg_burgers_op* op, const T* up, cudaStream_t st) {
    const amdg_grid* g = op->grid;
    const int dim = g->host.dim;
    const int64_t n = g->host.num_elements * op->points;
    T* ta = static_cast<T*>(op->w_a);
    T* tb = static_cast<T*>(op->w_b);
    T* fu = static_cast<T*>(op->w_fu);
    AMDG_CK(launch_burgers_flux<T>(up, ta, n, st));
    op->grid->ctx->launches++;
    const T* cur = ta;
    for (int d = 0; d < dim; ++d) {
        SurplusArgs<T> a{};
        a.dim = dim;
        a.d = d;
        a.points = op->points;
        a.stride = 1;
        for (int s = d + 1; s < dim; ++s) a.stride *= 4;
        a.num_elements = g->host.num_elements;
        a.order = g->d_order;
        a.anc = op->d_anc;
        a.anc_point = op->d_anc_point;
        a.anc_rank = op->d_anc_rank;
        for (int i = 0; i < 16; ++i) a.weight[i] = T(op->weight[i]);
        T* dst = (d == dim - 1) ? fu : ((cur == tb) ? ta : tb);
        a.in = cur;
        a.out = dst;
        AMDG_CK(launch_surplus_pass<T>(a, st));
        op->grid->ctx->launches++;
        cur = dst;
    }
    return AMDG_OK;
}

// volume and interface terms from the flux coefficients fu, and the LxF
// penalty from the Alpert coefficients u, into rhs (set, not added)
template <typename T>
amdg_status eval_back_transforms(amdg_burgers_op* op, const Mats<T>& m, const T* fu, const T* u, T* rhs, cudaStream_t st) {
    const amdg_grid* g = op->grid;
    const int dim = g->host.dim, np = g->host.k + 1;
    T* ta = static_cast<T*>(op->w_a);
    T* tb = static_cast<T*>(op->w_b);
    AMDG_CK(cudaMemsetAsync(rhs, 0, size_t(g->dof) * sizeof(T), st));
    for (int d = 0; d < dim; ++d) {
        for (int term = 0; term < 2; ++term) {
            // term 0: volume (u_vx in d, u_v elsewhere, vol sets);
            // term 1: interface (ulft+urgt)_vjp in d on flx sets, coefficient 0.5
            const T* mats[kMaxDim];
            bool flx[kMaxDim];
            for (int t = 0; t < dim; ++t) {
                mats[t] = (t == d) ? (term == 0 ? m.lvx : m.lflx) : m.lv;
                flx[t] = (term == 1 && t == d);
            }
            const T coef = term == 0 ? T(1) : T(0.5);
            for (size_t s = 0; s < op->sched_dims.size(); ++s) {
                amdg_status r = partial_sum<T>(op, op->sched_dims[s], op->sched_lu[s], 4, np, mats, flx, coef, fu, rhs, ta, tb, st);
                if (r != AMDG_OK) return r;
            }
        }
        // LxF penalty -alpha_d/2 ujp_vjp in dimension d (FastRHS::transform_ucoe_alpt_to_rhs, FastMultiplyLU.cpp:46-59)
        int from[kMaxDim];
        for (int t = 0; t < dim; ++t) from[t] = np;
        TransformArgs<T> a = base_args<T>(op, d, from, from, true);
        a.M = m.ajump;
        a.ncols = op->n1 * np;
        a.lu = 1;
        a.coef = T(-op->alpha[d] / 2.0);
        a.in = u;
        a.out = rhs;
        a.accumulate = 1;
        AMDG_CK(launch_fibre_transform<T>(a, st));
        op->grid->ctx->launches++;
    }
    return AMDG_OK;
}

// rhs (FP64, dof entries) of the FP64 state u.  The point values and the
// hierarchical surplus always run in FP64: fine-level surpluses are small
// differences of O(1) point values, which FP32 rounding would swamp.  In mixed
// mode the back transforms (the bulk of the work) and the penalty run in FP32.
amdg_status eval_rhs(amdg_burgers_op* op, const double* u, double* rhs, amdg_precision prec) {
    cudaStream_t st = stream_of(op);
    const int64_t n = op->grid->dof;
    const int64_t npts = op->grid->host.num_elements * op->points;
    double* up = static_cast<double*>(op->w_up);
    amdg_status r = eval_point_values<double>(op, mats64(op), u, up, st);
    if (r != AMDG_OK) return r;
    if ((r = eval_flux_coefficients<double>(op, up, st)) != AMDG_OK) return r;
    const double* fu = static_cast<const double*>(op->w_fu);
    if (prec == AMDG_PREC_FP64) return eval_back_transforms<double>(op, mats64(op), fu, u, rhs, st);
    float* fu32 = static_cast<float*>(op->w_up);  // point values are no longer needed
    float* u32 = static_cast<float*>(op->w_u);
    float* r32 = static_cast<float*>(op->w_rhs);
    AMDG_CK(launch_convert<double, float>(fu, fu32, npts, st));
    AMDG_CK(launch_convert<double, float>(u, u32, n, st));
    op->grid->ctx->launches += 2;
    if ((r = eval_back_transforms<float>(op, mats32(op), fu32, u32, r32, st)) != AMDG_OK) return r;
    AMDG_CK(launch_convert<float, double>(r32, rhs, n, st));
    op->grid->ctx->launches++;
    return AMDG_OK;
}


// Copy a host vector into a grow-only device array of the operator (stream
// ordered: kernels queued before still see the old contents).
template <class T>
amdg_status upload_grow(amdg_burgers_op* op, T** p, const std::vector<T>& host, cudaStream_t st) {
    size_t& cap = op->dev_cap[static_cast<const void*>(p)];
    const size_t bytes = host.size() * sizeof(T);
    if (bytes > cap) {
        cudaFree(*p);
        *p = nullptr;
        cap = 0;
        const size_t want = bytes + bytes / 4 + 256;
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), want);
        if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        cap = want;
    }
    if (bytes) AMDG_CK(cudaMemcpyAsync(*p, host.data(), bytes, cudaMemcpyHostToDevice, st));
    return AMDG_OK;
}

// (Re)build the neighbour lists and surplus ancestors for the grid's current
// element set; device arrays and work buffers only grow.
amdg_status burgers_sync(amdg_burgers_op* op) {
    amdg_grid* g = op->grid;
    if (op->built_version == g->version) return AMDG_OK;
    cudaStream_t st = stream_of(op);
    LagrTables t;
    if (op->anc_order.empty()) {
        // ancestor orders only depend on nmax
        Basis1D b{g->host.k, g->host.nmax};
        t.anc_order.assign(size_t(op->n1) * 4, -1);
        build_lagr_ancestors(b, &t);
        op->anc_order = t.anc_order;
    } else {
        t.anc_order = op->anc_order;
    }
    TransformTopology topo;
    build_transform_topology(g->host, &topo);
    std::vector<int32_t> anc;
    if (!build_surplus_ancestors(g->host, t, &anc)) return fail(AMDG_ERR_STATE, "element set has a hole: a surplus ancestor is missing");
    std::vector<int32_t> vle, fle;
    op->vol_long_off.assign(1, 0);
    op->flx_long_off.assign(1, 0);
    for (int d = 0; d < g->host.dim; ++d) {
        vle.insert(vle.end(), topo.vol_long_elems[d].begin(), topo.vol_long_elems[d].end());
        fle.insert(fle.end(), topo.flx_long_elems[d].begin(), topo.flx_long_elems[d].end());
        op->vol_long_off.push_back(int32_t(vle.size()));
        op->flx_long_off.push_back(int32_t(fle.size()));
    }
    std::vector<int32_t> pg;
    parent_table(g->host, &pg);
    amdg_status s;
    if ((s = upload_grow(op, &op->d_vol_ptr, topo.vol_ptr, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_vol_nbr, topo.vol_nbr, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_flx_ptr, topo.flx_ptr, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_flx_nbr, topo.flx_nbr, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_anc, anc, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_vol_split, topo.vol_split, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_flx_split, topo.flx_split, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_vol_long, topo.vol_long, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_flx_long, topo.flx_long, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_vol_long_elems, vle, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_flx_long_elems, fle, st)) != AMDG_OK ||
        (s = upload_grow(op, &op->d_pg, pg, st)) != AMDG_OK)
        return s;
    const int64_t E = g->host.num_elements;
    if (E > op->capacity) {
        const int64_t cap = E + E / 2 + 16;
        void* bufs[] = {op->w_up, op->w_fu, op->w_a, op->w_b, op->w_rhs, op->w_u, op->d_u1, op->d_rhs64, op->d_pred};
        for (void* p : bufs) cudaFree(p);
        const size_t work = size_t(cap) * op->points * sizeof(double);
        const size_t vec = size_t(cap) * g->block * sizeof(double);
        if ((s = alloc_bytes(&op->w_up, work)) != AMDG_OK || (s = alloc_bytes(&op->w_fu, work)) != AMDG_OK ||
            (s = alloc_bytes(&op->w_a, work)) != AMDG_OK || (s = alloc_bytes(&op->w_b, work)) != AMDG_OK ||
            (s = alloc_bytes(&op->w_rhs, vec)) != AMDG_OK || (s = alloc_bytes(&op->w_u, vec)) != AMDG_OK ||
            (s = alloc_bytes(reinterpret_cast<void**>(&op->d_u1), vec)) != AMDG_OK ||
            (s = alloc_bytes(reinterpret_cast<void**>(&op->d_rhs64), vec)) != AMDG_OK ||
            (s = alloc_bytes(reinterpret_cast<void**>(&op->d_pred), vec)) != AMDG_OK)
            return s;
        op->capacity = cap;
    }
    // the host vectors above are released on return: wait for their copies
    AMDG_CK(cudaStreamSynchronize(st));
    op->built_version = g->version;
    return AMDG_OK;
}

StageCoef stage_coef(int stage, double dt) {
    switch (stage) {
        case 0: return StageCoef{1, 0.0, 1.0, dt};
        case 1: return StageCoef{1, 3. / 4., 1. / 4., dt};
        default: return StageCoef{1, 1. / 3., 2. / 3., dt};
    }
}

}  // namespace

extern "C" {

amdg_status amdg_burgers_create(amdg_grid* g, const double* alpha, amdg_burgers_op** out) {
    AMDG_REQUIRE(g && alpha && out, AMDG_ERR_ARG, "null argument");
    *out = nullptr;
    AMDG_REQUIRE(g->host.k == 2, AMDG_ERR_ARG, "the Lagrange path is built for Alpert degree k = 2");
    AMDG_CK(cudaSetDevice(g->device));
    const int dim = g->host.dim;
    for (int d = 0; d < dim; ++d) AMDG_REQUIRE(std::isfinite(alpha[d]), AMDG_ERR_ARG, "non-finite alpha");
    amdg_burgers_op* op = new (std::nothrow) amdg_burgers_op;
    AMDG_REQUIRE(op, AMDG_ERR_NOMEM, "host allocation failed");
    op->grid = g;
    op->device = g->device;
    op->alpha.assign(alpha, alpha + dim);
    op->points = 1;
    for (int d = 0; d < dim; ++d) op->points *= 4;
    op->n1 = 1 << g->host.nmax;
    Basis1D b{g->host.k, g->host.nmax};
    LagrTables t;
    build_lagr_tables(b, &t);
    std::memcpy(op->weight, t.weight, sizeof(op->weight));
    transform_schedule(dim, &op->sched_dims, &op->sched_lu);
    amdg_status s;
    if ((s = upload_both(&op->d_a2p, &op->f_a2p, t.a2p)) != AMDG_OK || (s = upload_both(&op->d_lv, &op->f_lv, t.lv)) != AMDG_OK ||
        (s = upload_both(&op->d_lvx, &op->f_lvx, t.lvx)) != AMDG_OK ||
        (s = upload_both(&op->d_lflx, &op->f_lflx, t.lflx)) != AMDG_OK ||
        (s = upload_both(&op->d_ajump, &op->f_ajump, t.ajump)) != AMDG_OK ||
        (s = upload_vec(&op->d_anc_point, t.anc_point)) != AMDG_OK || (s = upload_vec(&op->d_anc_rank, t.anc_rank)) != AMDG_OK ||
        (s = burgers_sync(op)) != AMDG_OK) {
        amdg_burgers_destroy(op);
        return s;
    }
    *out = op;
    return AMDG_OK;
}

amdg_status amdg_burgers_destroy(amdg_burgers_op* op) {
    if (!op) return AMDG_OK;
    cudaSetDevice(op->device);
    if (op->graph_exec) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(op->graph_exec));
    void* ptrs[] = {op->d_a2p, op->d_lv, op->d_lvx, op->d_lflx, op->d_ajump, op->f_a2p, op->f_lv, op->f_lvx, op->f_lflx,
                    op->f_ajump, op->d_vol_ptr, op->d_vol_nbr, op->d_flx_ptr, op->d_flx_nbr,
                    op->d_anc, op->d_anc_point, op->d_anc_rank, op->w_up, op->w_fu, op->w_a, op->w_b, op->w_rhs, op->w_u,
                    op->d_u1, op->d_u2, op->d_rhs64, op->d_pred, op->d_vol_split, op->d_flx_split,
                    op->d_vol_long, op->d_flx_long, op->d_vol_long_elems, op->d_flx_long_elems, op->d_pg,
                    op->d_feat, op->d_prob};
    for (void* p : ptrs) cudaFree(p);
    delete op;
    return AMDG_OK;
}

amdg_status amdg_burgers_rhs(amdg_burgers_op* op, const double* d_u, double* d_rhs, amdg_precision prec) {
    AMDG_REQUIRE(op && d_u && d_rhs && d_u != d_rhs, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    return eval_rhs(op, d_u, d_rhs, prec);
}

amdg_status amdg_burgers_point_values(amdg_burgers_op* op, const double* d_u, double* d_up, amdg_precision prec) {
    AMDG_REQUIRE(op && d_u && d_up, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    cudaStream_t st = stream_of(op);
    if (prec == AMDG_PREC_FP64) return eval_point_values<double>(op, mats64(op), d_u, d_up, st);
    const int64_t n = op->grid->dof, np = op->grid->host.num_elements * op->points;
    float* u32 = static_cast<float*>(op->w_u);
    float* up32 = static_cast<float*>(op->w_up);
    AMDG_CK(launch_convert<double, float>(d_u, u32, n, st));
    amdg_status r = eval_point_values<float>(op, mats32(op), u32, up32, st);
    if (r != AMDG_OK) return r;
    AMDG_CK(launch_convert<float, double>(up32, d_up, np, st));
    op->grid->ctx->launches += 2;
    return AMDG_OK;
}

amdg_status amdg_burgers_flux_coefficients(amdg_burgers_op* op, const double* d_u, double* d_fu, amdg_precision prec) {
    AMDG_REQUIRE(op && d_u && d_fu, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    cudaStream_t st = stream_of(op);
    const int64_t np = op->grid->host.num_elements * op->points;
    if (prec == AMDG_PREC_FP64) {
        amdg_status r = eval_point_values<double>(op, mats64(op), d_u, static_cast<double*>(op->w_up), st);
        if (r != AMDG_OK) return r;
        if ((r = eval_flux_coefficients<double>(op, static_cast<double*>(op->w_up), st)) != AMDG_OK) return r;
        AMDG_CK(cudaMemcpyAsync(d_fu, op->w_fu, np * sizeof(double), cudaMemcpyDeviceToDevice, st));
        return AMDG_OK;
    }
    float* u32 = static_cast<float*>(op->w_u);
    AMDG_CK(launch_convert<double, float>(d_u, u32, op->grid->dof, st));
    amdg_status r = eval_point_values<float>(op, mats32(op), u32, static_cast<float*>(op->w_up), st);
    if (r != AMDG_OK) return r;
    if ((r = eval_flux_coefficients<float>(op, static_cast<float*>(op->w_up), st)) != AMDG_OK) return r;
    AMDG_CK(launch_convert<float, double>(static_cast<float*>(op->w_fu), d_fu, np, st));
    op->grid->ctx->launches += 2;
    return AMDG_OK;
}

amdg_status amdg_burgers_rk3_steps(amdg_burgers_op* op, double dt, int nsteps, amdg_precision prec) {
    AMDG_REQUIRE(op && nsteps >= 0 && std::isfinite(dt), AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(op);
    if (nsteps == 0) return AMDG_OK;
    const size_t bytes = size_t(g->dof) * sizeof(double);
    // one step: ucoe is updated in place per stage, ucoe_tn holds u^n (RK3SSP::step_stage)
    auto step = [&]() -> amdg_status {
        AMDG_CK(cudaMemcpyAsync(op->d_u1, g->d_u, bytes, cudaMemcpyDeviceToDevice, st));
        for (int stage = 0; stage < 3; ++stage) {
            if (amdg_status r = eval_rhs(op, op->d_u1, op->d_rhs64, prec); r != AMDG_OK) return r;
            AMDG_CK(launch_stage_update(g->d_u, op->d_u1, op->d_rhs64, g->dof, stage_coef(stage, dt), st));
            g->ctx->launches++;
        }
        AMDG_CK(cudaMemcpyAsync(g->d_u, op->d_u1, bytes, cudaMemcpyDeviceToDevice, st));
        return AMDG_OK;
    };
    const bool graph_valid = op->graph_exec && op->graph_version == g->version && op->graph_prec == int(prec) &&
                             op->graph_dt == dt;
    // the launch sequence of a step is fixed for a grid, precision and dt: it is
    // captured as a CUDA graph once it will be replayed (several steps in this
    // call, or the same configuration as the previous call); a single step on a
    // grid that keeps changing (the adaptive loop) is launched directly
    const bool repeat = op->last_version == g->version && op->last_prec == int(prec) && op->last_dt == dt;
    op->last_version = g->version;
    op->last_prec = int(prec);
    op->last_dt = dt;
    if (!graph_valid && nsteps == 1 && !repeat) return step();
    if (!graph_valid) {
        if (op->graph_exec) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(op->graph_exec));
        op->graph_exec = nullptr;
        const int64_t l0 = g->ctx->launches;
        cudaGraph_t graph = nullptr;
        AMDG_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const amdg_status r = step();
        cudaError_t ec = cudaStreamEndCapture(st, &graph);
        op->graph_launches = g->ctx->launches - l0;
        g->ctx->launches = l0;
        if (r != AMDG_OK) { if (graph) cudaGraphDestroy(graph); return r; }
        if (ec != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return fail(AMDG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
        }
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
        op->graph_exec = exec;
        op->graph_version = g->version;
        op->graph_prec = int(prec);
        op->graph_dt = dt;
    }
    for (int s = 0; s < nsteps; ++s) {
        AMDG_CK(cudaGraphLaunch(static_cast<cudaGraphExec_t>(op->graph_exec), st));
        g->ctx->launches += op->graph_launches;
    }
    return AMDG_OK;
}

static double adaptive_dt(const amdg_grid* g, double cfl, double wave_speed) {
    // dt = cfl / sum_d c_d 2^maxlevel_d  (02_hyperbolic_05_burgers_adapt.cpp:239-247)
    std::vector<int> lv(g->host.dim, 0);
    for (int64_t e = 0; e < g->host.num_elements; ++e)
        for (int d = 0; d < g->host.dim; ++d)
            lv[d] = std::max(lv[d], level_of_order(g->host.order[size_t(e) * g->host.dim + d]));
    double sum_c_dx = 0.0;
    for (int d = 0; d < g->host.dim; ++d) sum_c_dx += wave_speed * std::pow(2.0, lv[d]);
    return cfl / sum_c_dx;
}

// keys of the elements present after a step, to mark coarsened ones
static void mark_removed(const std::vector<uint64_t>& old_keys, const HostGrid& now, int8_t* decisions) {
    for (size_t e = 0; e < old_keys.size(); ++e)
        if (!std::binary_search(now.key.begin(), now.key.end(), old_keys[e])) decisions[e] = 2;
}

amdg_status amdg_burgers_adaptive_step_ex(amdg_burgers_op* op, double cfl, double wave_speed, double eps, double eta,
                                          amdg_precision prec, double* dt_out, int8_t* decisions) {
    AMDG_REQUIRE(op && std::isfinite(cfl) && cfl > 0 && std::isfinite(wave_speed) && wave_speed > 0, AMDG_ERR_ARG,
                 "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(op);
    const double dt = adaptive_dt(g, cfl, wave_speed);
    const std::vector<uint64_t> old_keys = g->host.key;
    // predictor: forward Euler into the prediction buffer (ForwardEuler::step_stage)
    amdg_status s = eval_rhs(op, g->d_u, op->d_rhs64, prec);
    if (s != AMDG_OK) return s;
    AMDG_CK(cudaMemcpyAsync(op->d_pred, g->d_u, size_t(g->dof) * sizeof(double), cudaMemcpyDeviceToDevice, st));
    AMDG_CK(launch_stage_update(g->d_u, op->d_pred, op->d_rhs64, g->dof, stage_coef(0, dt), st));
    g->ctx->launches++;
    // refine on the predicted coefficients; new elements start from zero (DGAdapt::refine, copy_predict_to_ucoe)
    std::vector<double> norms;
    if ((s = grid_norms(g, op->d_pred, &norms)) != AMDG_OK) return s;
    std::vector<uint8_t> refined;
    std::vector<uint64_t> keys = refine_keys(g->host, norms.data(), eps, &refined);
    if (decisions)
        for (size_t e = 0; e < refined.size(); ++e) decisions[e] = refined[e] ? 1 : 0;
    if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
    if ((s = amdg_burgers_rk3_steps(op, dt, 1, prec)) != AMDG_OK) return s;
    if ((s = amdg_grid_coarsen(g, eta, nullptr)) != AMDG_OK) return s;
    if (decisions) mark_removed(old_keys, g->host, decisions);
    if (dt_out) *dt_out = dt;
    return AMDG_OK;
}

amdg_status amdg_burgers_adaptive_step(amdg_burgers_op* op, double cfl, double wave_speed, double eps, double eta,
                                       amdg_precision prec, double* dt_out) {
    return amdg_burgers_adaptive_step_ex(op, cfl, wave_speed, eps, eta, prec, dt_out, nullptr);
}

amdg_status amdg_burgers_features(amdg_burgers_op* op, const double* d_u, float* d_features) {
    AMDG_REQUIRE(op && d_u && d_features, AMDG_ERR_ARG, "null argument");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    const amdg_grid* g = op->grid;
    AMDG_CK(launch_element_features(d_u, op->d_pg, g->host.num_elements, g->host.dim, g->block, d_features, stream_of(op)));
    g->ctx->launches++;
    return AMDG_OK;
}

amdg_status amdg_burgers_adaptive_step_learned(amdg_burgers_op* op, amdg_mlp* mlp, double cfl, double wave_speed,
                                               double eps, double eta, double tau, amdg_precision prec, double* dt_out,
                                               int64_t* stats) {
    AMDG_REQUIRE(op && mlp && std::isfinite(cfl) && cfl > 0 && std::isfinite(wave_speed) && wave_speed > 0, AMDG_ERR_ARG,
                 "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(op);
    const double dt = adaptive_dt(g, cfl, wave_speed);
    const int64_t E = g->host.num_elements;
    const int F = g->block * (1 + 2 * g->host.dim);
    int n_in = 0, n_out = 0;
    mlp_shape(mlp, &n_in, &n_out);
    AMDG_REQUIRE(n_in == F && n_out == 3, AMDG_ERR_ARG,
                 "classifier must take " + std::to_string(F) + " features and give 3 classes");
    // 1. the network's refine/keep/coarsen probabilities from the current coefficients
    amdg_status s = AMDG_OK;
    if (E > op->feat_cap) {
        cudaFree(op->d_feat);
        cudaFree(op->d_prob);
        op->d_feat = op->d_prob = nullptr;
        op->feat_cap = 0;
        const int64_t cap = E + E / 4;
        void *pf = nullptr, *pp = nullptr;
        if ((s = alloc_bytes(&pf, size_t(cap) * F * sizeof(float))) != AMDG_OK) return s;
        op->d_feat = static_cast<float*>(pf);
        if ((s = alloc_bytes(&pp, size_t(cap) * 3 * sizeof(float))) != AMDG_OK) return s;
        op->d_prob = static_cast<float*>(pp);
        op->feat_cap = cap;
    }
    float* d_feat = op->d_feat;
    float* d_prob = op->d_prob;
    AMDG_CK(launch_element_features(g->d_u, op->d_pg, E, g->host.dim, g->block, d_feat, st));
    g->ctx->launches++;
    s = amdg_mlp_predict(mlp, d_feat, E, d_prob);
    if (s != AMDG_OK) return s;
    std::vector<float> prob(size_t(E) * 3);
    AMDG_CK(cudaMemcpyAsync(prob.data(), d_prob, prob.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
    std::vector<double> norms;
    if ((s = grid_norms(g, g->d_u, &norms)) != AMDG_OK) return s;  // synchronises the stream
    // 2. pre-adapt: leaves the network marks "refine" get children; where it is
    //    unsure (max probability < tau) the surplus criterion on the current
    //    coefficients decides instead
    std::vector<uint8_t> force(E, 0);
    int64_t n_net = 0, n_unsure = 0;
    for (int64_t e = 0; e < E; ++e) {
        const float* p = &prob[size_t(e) * 3];
        const int arg = (p[1] > p[0] && p[1] >= p[2]) ? 1 : (p[2] > p[0] ? 2 : 0);
        const float pmax = std::max(p[0], std::max(p[1], p[2]));
        if (pmax < float(tau)) {
            ++n_unsure;
            force[e] = norms[e] > eps ? 1 : 0;
        } else if (arg == 1) {
            force[e] = 1;
            ++n_net;
        }
    }
    std::vector<uint64_t> keys = refine_keys(g->host, norms.data(), eps, nullptr, force.data());
    if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
    // 3. one SSP-RK3 step, no predictor step
    if ((s = amdg_burgers_rk3_steps(op, dt, 1, prec)) != AMDG_OK) return s;
    // 4. the surplus criterion judges the result: leaves still above eps are missed
    //    refinements and get their children now; then the usual coarsening
    if ((s = grid_norms(g, g->d_u, &norms)) != AMDG_OK) return s;
    std::vector<uint8_t> missed;
    keys = refine_keys(g->host, norms.data(), eps, &missed);
    int64_t n_missed = 0;
    for (uint8_t v : missed) n_missed += v;
    if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
    if ((s = amdg_grid_coarsen(g, eta, nullptr)) != AMDG_OK) return s;
    if (dt_out) *dt_out = dt;
    if (stats) {
        stats[0] = n_net;
        stats[1] = n_unsure;
        stats[2] = n_missed;
        stats[3] = g->host.num_elements;
    }
    return AMDG_OK;
}

}  // extern "C"
