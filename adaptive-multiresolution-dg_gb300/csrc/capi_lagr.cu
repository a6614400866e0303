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
#include <type_traits>
#include <vector>

#include "amdg.h"
#include "amdg_internal.hpp"
#include "kernels.cuh"
#include "kernels_lagr.cuh"
#include "kernels_mlp.cuh"
#include "device_alloc.cuh"

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

// device bytes the term slices of one launch may take (sweep buffers and outputs)
constexpr size_t kTermBudget = size_t(3) << 29;

template <class T>
amdg_status upload_vec(T** p, const std::vector<T>& host) {
    *p = nullptr;
    if (host.empty()) return AMDG_OK;
    cudaError_t e = amdg::device_malloc(reinterpret_cast<void**>(p), host.size() * sizeof(T));
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
    cudaError_t e = amdg::device_malloc(p, bytes);
    if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return AMDG_OK;
}

cudaStream_t stream_of(const amdg_burgers_op* op) { return static_cast<cudaStream_t>(op->grid->ctx->stream); }

template <typename T>
struct Mats {
    const T* m[kNumLagrMats];
};

Mats<double> mats64(const amdg_burgers_op* op) {
    return {{op->d_a2p, op->d_lv, op->d_lvx, op->d_lflx, op->d_ajump, op->d_a2pd, op->d_ljv}};
}
Mats<float> mats32(const amdg_burgers_op* op) {
    return {{op->f_a2p, op->f_lv, op->f_lvx, op->f_lflx, op->f_ajump, op->f_a2pd, op->f_ljv}};
}
// double-float tables: only those of the point values
Mats<float2> mats_df(const amdg_burgers_op* op) {
    return {{static_cast<const float2*>(op->df_a2p), nullptr, nullptr, nullptr, nullptr,
             static_cast<const float2*>(op->df_a2pd), nullptr}};
}

// [n1 nf][n1 nt] row-major -> blocked by order pair: [o_from][o_to][nf][nt] (an empty table stays
// empty); false when the size does not match
bool reblock_table(std::vector<double>* m, int n1, int nf, int nt) {
    if (m->empty()) return true;
    const size_t ncols = size_t(n1) * nt;
    if (m->size() != size_t(n1) * nf * ncols) return false;
    std::vector<double> out(m->size());
    size_t w = 0;
    for (int os = 0; os < n1; ++os)
        for (int oe = 0; oe < n1; ++oe)
            for (int p = 0; p < nf; ++p)
                for (int q = 0; q < nt; ++q) out[w++] = (*m)[(size_t(os) * nf + p) * ncols + size_t(oe) * nt + q];
    m->swap(out);
    return true;
}

// a table as double-float pairs (hi = float(v), lo = float(v - hi))
amdg_status upload_df(void** p, const std::vector<double>& host) {
    std::vector<float2> h(host.size());
    for (size_t i = 0; i < host.size(); ++i) {
        const float hi = float(host[i]);
        h[i] = make_float2(hi, float(host[i] - double(hi)));
    }
    float2* d = nullptr;
    amdg_status s = upload_vec(&d, h);
    *p = d;
    return s;
}

int ipow(int b, int e) {
    int p = 1;
    for (int i = 0; i < e; ++i) p *= b;
    return p;
}

// the Burgers operators: flux u^2/2 interpolated by Lagrange (kind 0) or cubic Hermite (kind 3)
// interpolation; both step by SSP-RK3 with the same right-hand-side terms
bool burgers_like(const amdg_burgers_op* op) { return op->kind == 0 || op->kind == 3; }

// partial sums of the schedule with the given matrix and vol/flx choice per
// dimension, reading input `src`, appended to op->terms
void push_psums(amdg_burgers_op* op, const int* mat, const int* flx, double coef, int src) {
    const int dim = op->grid->host.dim;
    for (size_t s = 0; s < op->sched_dims.size(); ++s) {
        PartialSum p{};
        for (int j = 0; j < dim; ++j) {
            const int t = op->sched_dims[s][j];
            p.dims[j] = int8_t(t);
            p.lu[j] = int8_t(op->sched_lu[s][j]);
            p.mat[j] = int8_t(mat[t]);
            p.flx[j] = int8_t(flx[t]);
        }
        p.src = int8_t(src);
        p.kind = 0;
        p.coef = coef;
        op->terms.push_back(p);
    }
}

// a single full transform of the Alpert coefficients along d with the jump matrix (penalty)
void push_penalty(amdg_burgers_op* op, int d, double coef) {
    PartialSum p{};
    p.dims[0] = int8_t(d);
    p.kind = 1;
    p.coef = coef;
    op->terms.push_back(p);
}

// The terms of the path (host side, built once per operator; the wave penalty's
// coefficient follows the finest level, see wave_penalty_coef).
// Burgers:
//  - point values: the 2^(dim-1) partial sums of the schedule with the
//    Alpert-at-Lagrange-point matrix in every dimension (FastLagrIntp::eval_up_Lagr);
//  - right-hand side, in the order the reference adds them: the volume partial
//    sums (u_vx in d, u_v elsewhere, vol sets) for every dimension d, then the
//    interface partial sums (0.5 (ulft+urgt)_vjp in d on the flx sets, u_v
//    elsewhere) for every d (HyperbolicLagrRHS::rhs_vol_scalar /
//    rhs_flx_intp_scalar, FastMultiplyLU.cpp:1125-1189), then the LxF penalty
//    -alpha_d/2 ujp_vjp along every d (HyperbolicAlptRHS::rhs_flx_penalty_scalar,
//    :1269-1276).
// Wave (03_wave_06_var_coeff_adapt.cpp:154-245):
//  - point values: group d < dim is u_{x_d} (the Alpert derivative at the
//    points along d, FastLagrIntp::eval_der_up_Lagr), group dim is u;
//  - right-hand side (sources 0..dim-1: the interpolated K u_{x_d}, source
//    dim: K u): DiffusionRHS::rhs_flx_gradu -{K u_x}[v] with uave_vjp =
//    (ulft+urgt)_vjp/2 along d, rhs_vol -K u_x v_x, rhs_flx_u -1/2 [K u] (v_x^- +
//    v_x^+) (FastMultiplyLU.cpp:1691-1765), each over d; then the IPDG penalty
//    -sigma/dx [u][v] along each d (DiffusionAlpt::assemble_matrix_flx_ujp_vjp,
//    BilinearForm.cpp:920-929).
void build_terms(amdg_burgers_op* op) {
    const int dim = op->grid->host.dim;
    op->terms.clear();
    int mat[kMaxDim], flx[kMaxDim];
    if (op->kind == 2) {  // interpolation init: u_v (Lagrange x Alpert) in every dimension
        op->n_pv_terms = 0;
        for (int t = 0; t < dim; ++t) { mat[t] = kMatLV; flx[t] = 0; }
        push_psums(op, mat, flx, 1.0, 0);
        return;
    }
    if (burgers_like(op)) {
        for (int t = 0; t < dim; ++t) { mat[t] = kMatA2P; flx[t] = 0; }
        push_psums(op, mat, flx, 1.0, 0);
        op->n_pv_terms = int(op->terms.size());
        // the three groups in the order the reference's driver calls them: rhs_vol_scalar (every
        // d), rhs_flx_intp_scalar (every d), rhs_flx_penalty_scalar (every d)
        for (int term = 0; term < 3; ++term) {
            op->grp_first[term] = int(op->terms.size());
            for (int d = 0; d < dim; ++d) {
                if (term == 2) {
                    push_penalty(op, d, -op->alpha[d] / 2.0);
                    continue;
                }
                for (int t = 0; t < dim; ++t) {
                    mat[t] = (t == d) ? (term == 0 ? kMatLVX : kMatLFLX) : kMatLV;
                    flx[t] = (term == 1 && t == d) ? 1 : 0;
                }
                push_psums(op, mat, flx, term == 0 ? 1.0 : 0.5, 0);
            }
            op->grp_count[term] = int(op->terms.size()) - op->grp_first[term];
        }
        return;
    }
    for (int g = 0; g <= dim; ++g) {
        for (int t = 0; t < dim; ++t) { mat[t] = (t == g) ? kMatA2PD : kMatA2P; flx[t] = 0; }
        push_psums(op, mat, flx, 1.0, 0);
    }
    op->n_pv_terms = int(op->terms.size());
    for (int d = 0; d < dim; ++d) {  // -{K u_x}[v]: uave_vjp = lflx / 2 exactly
        for (int t = 0; t < dim; ++t) { mat[t] = (t == d) ? kMatLFLX : kMatLV; flx[t] = (t == d) ? 1 : 0; }
        push_psums(op, mat, flx, -0.5, d);
    }
    for (int d = 0; d < dim; ++d) {  // -K u_x v_x
        for (int t = 0; t < dim; ++t) { mat[t] = (t == d) ? kMatLVX : kMatLV; flx[t] = 0; }
        push_psums(op, mat, flx, -1.0, d);
    }
    for (int d = 0; d < dim; ++d) {  // -1/2 [K u](v_x^- + v_x^+)
        for (int t = 0; t < dim; ++t) { mat[t] = (t == d) ? kMatLJV : kMatLV; flx[t] = (t == d) ? 1 : 0; }
        push_psums(op, mat, flx, -0.5, dim);
    }
    for (int d = 0; d < dim; ++d) push_penalty(op, d, 0.0);  // coefficient set per element set
}

// IPDG coefficient -sigma/dx, dx = 2^-(finest level of the grid) (BilinearForm.cpp:922-923)
double wave_penalty_coef(const amdg_burgers_op* op) {
    int maxl = 0;
    for (int d = 0; d < op->grid->host.dim; ++d) maxl = std::max(maxl, op->grid->lev_max[d]);
    return -op->sigma / (1.0 / std::pow(2.0, maxl));
}

// The nodes of every sweep tree on the device (grown when a tree is added; a step captured as a
// graph refers to the buffer, so growing it drops the graph).
amdg_status upload_nodes(amdg_burgers_op* op, cudaStream_t st) {
    const size_t bytes = op->nodes.size() * sizeof(PartialSum);
    if (bytes > op->nodes_cap) {
        AMDG_CK(cudaStreamSynchronize(st));
        cudaFree(op->d_nodes);
        op->d_nodes = nullptr;
        op->nodes_cap = 0;
        const size_t want = 2 * bytes + 1024;
        if (amdg::device_malloc(reinterpret_cast<void**>(&op->d_nodes), want) != cudaSuccess)
            return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (sweep trees)");
        op->nodes_cap = want;
        op->graph_version = -1;
    }
    if (bytes) AMDG_CK(cudaMemcpyAsync(op->d_nodes, op->nodes.data(), bytes, cudaMemcpyHostToDevice, st));
    AMDG_CK(cudaStreamSynchronize(st));  // op->nodes may change again before the copy would run
    return AMDG_OK;
}

// after a change of term coefficients: the nodes of every tree again (the same structure: only
// the penalty's coefficient changes, and the penalty is never shared)
amdg_status refresh_nodes(amdg_burgers_op* op, cudaStream_t st) {
    op->nodes.clear();
    for (auto& kv : op->trees)
        kv.second = build_sweep_tree(op->terms, kv.first.first, kv.first.second, op->grid->host.dim, &op->nodes);
    return upload_nodes(op, st);
}

// the sweep tree of terms [first, first + count), built and uploaded on first use
amdg_status sweep_tree(amdg_burgers_op* op, int first, int count, SweepTree* out, cudaStream_t st) {
    for (const auto& kv : op->trees)
        if (kv.first.first == first && kv.first.second == count) {
            *out = kv.second;
            return AMDG_OK;
        }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    AMDG_CK(cudaStreamIsCapturing(st, &cap));
    AMDG_REQUIRE(cap == cudaStreamCaptureStatusNone, AMDG_ERR_STATE, "sweep tree built during stream capture");
    op->trees.push_back({{first, count}, build_sweep_tree(op->terms, first, count, op->grid->host.dim, &op->nodes)});
    *out = op->trees.back().second;
    return upload_nodes(op, st);
}

// the trees of every term range the right-hand side launches with the current chunk size, so a
// step captured as a graph finds them all
amdg_status prepare_trees(amdg_burgers_op* op, cudaStream_t st) {
    SweepTree t;
    auto chunks = [&](int first, int total) -> amdg_status {
        for (int c0 = 0; c0 < total; c0 += op->chunk)
            if (amdg_status s = sweep_tree(op, first + c0, std::min(op->chunk, total - c0), &t, st); s != AMDG_OK) return s;
        return AMDG_OK;
    };
    const int nterms = int(op->terms.size()), dim = op->grid->host.dim;
    amdg_status s;
    if (op->kind == 1) {
        const int G = int(op->sched_dims.size());
        for (int f = 0; f <= dim; ++f)
            if ((s = chunks(f * G, G)) != AMDG_OK) return s;
        if ((s = chunks(nterms - dim, dim)) != AMDG_OK) return s;
    } else if ((s = chunks(0, op->n_pv_terms)) != AMDG_OK) {
        return s;
    }
    return chunks(op->n_pv_terms, nterms - op->n_pv_terms);
}

template <typename T>
SweepArgs<T> sweep_args(const amdg_burgers_op* op, const Mats<T>& m) {
    const amdg_grid* g = op->grid;
    SweepArgs<T> a{};
    a.dim = g->host.dim;
    a.np = g->host.k + 1;
    a.n1 = op->n1;
    a.num_elements = g->host.num_elements;
    a.desc = op->d_terms;
    // default kernels (measured on the config-3 runs): warp per (node, element) for the FP32 sweeps
    // (fewer issued instructions), thread per output entry for the FP64 ones (FP64-pipe work per
    // warp kept whole) and the double-float ones (their arithmetic, not the issue overhead, binds)
    a.variant = op->sweep_variant >= 0 ? op->sweep_variant : (std::is_same<T, float>::value ? 2 : 0);
    for (int i = 0; i < kNumLagrMats; ++i) a.mats[i] = m.m[i];
    a.vol_ptr = op->d_vol_ptr;
    a.vol_split = op->d_vol_split;
    a.vol_nbr = reinterpret_cast<const int2*>(op->d_vol_nbr);
    a.flx_ptr = op->d_flx_ptr;
    a.flx_split = op->d_flx_split;
    a.flx_nbr = reinterpret_cast<const int2*>(op->d_flx_nbr);
    a.order = g->d_order;
    return a;
}

// Terms [first, first + count): dim sweeps, the first reading src[term.src],
// the last one into `slots` (count slices of E x n_out^dim, or E x np^dim for
// a right-hand side).
template <typename T>
amdg_status run_terms(amdg_burgers_op* op, const Mats<T>& m, int first, int count, int n_in, int n_out,
                      const T* const* src, int nsrc, const T* pen_in, T* slots, cudaStream_t st) {
    const int dim = op->grid->host.dim;
    const int64_t E = op->grid->host.num_elements;
    T* ping = static_cast<T*>(op->w_s0);
    T* pong = static_cast<T*>(op->w_s1);
    SweepTree tree;
    if (amdg_status s = sweep_tree(op, first, count, &tree, st); s != AMDG_OK) return s;
    SweepArgs<T> a = sweep_args<T>(op, m);
    a.first = 0;
    a.n_in = n_in;
    a.n_out = n_out;
    a.pen_in = pen_in;
    for (int i = 0; i < nsrc && i < kMaxTermSources; ++i) a.src[i] = src[i];
    const T* cur = nullptr;
    for (int j = 0; j < dim; ++j) {
        const bool last = j == dim - 1;
        a.sweep = j;
        a.in = cur;
        a.in_slice = j == 0 ? 0 : E * ipow(n_out, j) * ipow(n_in, dim - j);
        a.out_block = ipow(n_out, j + 1) * ipow(n_in, dim - j - 1);
        a.out = last ? slots : (j % 2 == 0 ? ping : pong);
        a.desc = op->d_nodes + tree.offset[j];
        a.count = tree.count[j];
        AMDG_CK(launch_sweep<T>(a, st));
        op->grid->ctx->launches++;
        cur = a.out;
    }
    return AMDG_OK;
}

// u_h at the interpolation points (FP64 or FP32 arithmetic): into up, or, when
// fp is given, f(u) = u^2/2 at the points into fp
template <typename T>
amdg_status eval_point_values(amdg_burgers_op* op, const Mats<T>& m, const T* u, T* up, T* fp, cudaStream_t st) {
    const int np = op->grid->host.k + 1;
    const int64_t n = op->grid->host.num_elements * op->points;
    const bool herm = op->kind == 3;  // the Hermite flux needs the slopes too: applied after the sum
    T* slots = static_cast<T*>(op->w_slots);
    const T* src[1] = {u};
    for (int c0 = 0; c0 < op->n_pv_terms; c0 += op->chunk) {
        const int cnt = std::min(op->chunk, op->n_pv_terms - c0);
        if (amdg_status r = run_terms<T>(op, m, c0, cnt, np, op->p1, src, 1, nullptr, slots, st); r != AMDG_OK) return r;
        const bool last = c0 + cnt == op->n_pv_terms;
        AMDG_CK(launch_reduce_points<T>(slots, cnt, n, c0 == 0 ? 1 : 0, up, (last && !herm) ? fp : nullptr, st));
        op->grid->ctx->launches++;
    }
    if (herm && fp) {
        AMDG_CK(launch_herm_flux_burgers2d<T>(up, fp, op->grid->host.num_elements, st));
        op->grid->ctx->launches++;
    }
    return AMDG_OK;
}

// u_h at the interpolation points in double-float arithmetic (the mixed mode): the sweeps on the
// FP32 pipe with about 48-bit precision, the slices summed in FP64 into up, or, when fp is
// given, f(u) = u^2/2 at the points into fp
amdg_status eval_point_values_df(amdg_burgers_op* op, const double* u, double* up, double* fp, cudaStream_t st) {
    const int np = op->grid->host.k + 1;
    const int64_t n = op->grid->host.num_elements * op->points;
    float2* udf = static_cast<float2*>(op->w_u);
    AMDG_CK(launch_to_df(u, udf, op->grid->dof, st));
    op->grid->ctx->launches++;
    float2* slots = static_cast<float2*>(op->w_slots);
    const float2* src[1] = {udf};
    for (int c0 = 0; c0 < op->n_pv_terms; c0 += op->chunk) {
        const int cnt = std::min(op->chunk, op->n_pv_terms - c0);
        if (amdg_status r = run_terms<float2>(op, mats_df(op), c0, cnt, np, op->p1, src, 1, nullptr, slots, st);
            r != AMDG_OK)
            return r;
        const bool last = c0 + cnt == op->n_pv_terms;
        AMDG_CK(launch_reduce_points_df(slots, cnt, n, c0 == 0 ? 1 : 0, up, (last && op->kind != 3) ? fp : nullptr, st));
        op->grid->ctx->launches++;
    }
    if (op->kind == 3 && fp) {  // the Hermite flux from the FP64 sums of values and slopes
        AMDG_CK(launch_herm_flux_burgers2d<double>(up, fp, op->grid->host.num_elements, st));
        op->grid->ctx->launches++;
    }
    return AMDG_OK;
}

// interpolation coefficients from values at the points: dim surplus passes
// (w_a / w_b as ping-pong buffers), the last one into `out` (type To)
template <typename T, typename To>
amdg_status eval_surplus(amdg_burgers_op* op, const T* in, To* out, cudaStream_t st) {
    const amdg_grid* g = op->grid;
    const int dim = g->host.dim;
    T* ta = static_cast<T*>(op->w_a);
    T* tb = static_cast<T*>(op->w_b);
    SurplusArgs<T> a{};
    a.dim = dim;
    a.p1 = op->p1;
    a.points = op->points;
    a.num_elements = g->host.num_elements;
    a.order = g->d_order;
    a.anc = op->d_anc;
    a.anc_point = op->d_anc_point;
    a.anc_rank = op->d_anc_rank;
    for (int i = 0; i < kMaxLagrPoints * kMaxLagrPoints; ++i) a.weight[i] = op->weight[i];
    a.herm = op->kind == 3;
    const T* cur = in;
    for (int d = 0; d < dim; ++d) {
        a.d = d;
        a.stride = ipow(op->p1, dim - d - 1);
        if (d == dim - 1) {
            AMDG_CK(launch_surplus_pass<T, To>(a, cur, out, st));
        } else {
            T* dst = (cur == ta) ? tb : ta;
            AMDG_CK(launch_surplus_pass<T, T>(a, cur, dst, st));
            cur = dst;
        }
        op->grid->ctx->launches++;
    }
    return AMDG_OK;
}

// right-hand-side terms [first, first + total) from their sources and the Alpert
// coefficients u (penalty): into rhs, or, when so.fused, straight into the RK
// stage update
template <typename T>
amdg_status eval_term_range(amdg_burgers_op* op, const Mats<T>& m, int first, int total, const T* const* src, int nsrc,
                            const T* u, double* rhs, StageOut so, cudaStream_t st, bool accumulate = false) {
    const int np = op->grid->host.k + 1;
    T* slots = static_cast<T*>(op->w_slots);
    for (int c0 = 0; c0 < total; c0 += op->chunk) {
        const int cnt = std::min(op->chunk, total - c0);
        if (amdg_status r = run_terms<T>(op, m, first + c0, cnt, op->p1, np, src, nsrc, u, slots, st); r != AMDG_OK)
            return r;
        AMDG_CK(launch_reduce_rhs<T>(slots, cnt, op->grid->dof, (c0 == 0 && !accumulate) ? 1 : 0,
                                     c0 + cnt == total ? 1 : 0, rhs, so, st));
        op->grid->ctx->launches++;
    }
    return AMDG_OK;
}

// all right-hand-side terms (those after the point-value terms)
template <typename T>
amdg_status eval_back_transforms(amdg_burgers_op* op, const Mats<T>& m, const T* const* src, int nsrc, const T* u,
                                 double* rhs, StageOut so, cudaStream_t st) {
    return eval_term_range<T>(op, m, op->n_pv_terms, int(op->terms.size()) - op->n_pv_terms, src, nsrc, u, rhs, so, st);
}

// wave: the IPDG term alone, -sigma/dx [u][v] summed over the dimensions, in FP64.  The
// predictor of the adaptive step uses it as its whole right-hand side: EulerODE2nd::
// step_rk_source recomputes rhs as the operator matrix (the IPDG penalty) times u,
// replacing the interpolated terms assembled before it (ODESolver.cpp:402-407,
// BilinearForm.h:23; 03_wave_06_var_coeff_adapt.cpp:215-241).
amdg_status eval_wave_penalty(amdg_burgers_op* op, const double* u, double* rhs, cudaStream_t st) {
    const int dim = op->grid->host.dim;
    const double* src[1] = {u};
    return eval_term_range<double>(op, mats64(op), int(op->terms.size()) - dim, dim, src, 1, u, rhs, StageOut{}, st);
}

// wave: K u_{x_d} (d < dim) and K u at the points, then their interpolation
// coefficients (type To) into fields dim+1 .. 2 dim+1 of w_fields
template <typename To>
amdg_status eval_wave_fields(amdg_burgers_op* op, const double* u, To** fucoe, cudaStream_t st, int f_first = 0,
                             int f_last = -1) {
    amdg_grid* g = op->grid;
    const int dim = g->host.dim, np = g->host.k + 1;
    const int64_t E = g->host.num_elements, n = E * op->points;
    const int G = int(op->sched_dims.size());  // terms per point field
    double* fields = static_cast<double*>(op->w_fields);
    const size_t stride = size_t(op->capacity) * op->points;
    // the mixed mode (FP32 coefficients out) computes the point values in double-float
    constexpr bool df = std::is_same<To, float>::value;
    using Tp = typename std::conditional<df, float2, double>::type;
    Tp* slots = static_cast<Tp*>(op->w_slots);
    const Tp* src[1];
    if constexpr (df) {
        AMDG_CK(launch_to_df(u, static_cast<float2*>(op->w_u), g->dof, st));
        op->grid->ctx->launches++;
        src[0] = static_cast<const float2*>(op->w_u);
    } else {
        src[0] = u;
    }
    const Mats<Tp> m = [&] {
        if constexpr (df) return mats_df(op);
        else return mats64(op);
    }();
    for (int f = f_first; f <= (f_last < 0 ? dim : f_last); ++f) {
        double* kp = fields + size_t(f) * stride;  // K times the point values of field f
        double* acc = static_cast<double*>(op->w_up);
        for (int c0 = 0; c0 < G; c0 += op->chunk) {
            const int cnt = std::min(op->chunk, G - c0);
            if (amdg_status r = run_terms<Tp>(op, m, f * G + c0, cnt, np, op->p1, src, 1, nullptr, slots, st);
                r != AMDG_OK)
                return r;
            auto fold = [&](int first) -> cudaError_t {  // the slices into acc, in FP64
                if constexpr (df) return launch_reduce_points_df(slots, cnt, n, first, acc, nullptr, st);
                else return launch_reduce_points<double>(slots, cnt, n, first, acc, nullptr, st);
            };
            if (c0 + cnt == G) {
                if (c0 > 0) {  // earlier chunks were summed into acc: fold them in as one more slice
                    AMDG_CK(fold(0));
                    AMDG_CK(launch_reduce_points_coef(acc, 1, E, dim, op->p1, g->d_order, op->d_pts, op->amp, kp, st));
                    op->grid->ctx->launches++;
                } else {
                    AMDG_CK(launch_reduce_points_coef(slots, cnt, E, dim, op->p1, g->d_order, op->d_pts, op->amp, kp, st));
                }
            } else {
                AMDG_CK(fold(c0 == 0 ? 1 : 0));
            }
            op->grid->ctx->launches++;
        }
        if (amdg_status r = eval_surplus<double, To>(op, kp, fucoe[f], st); r != AMDG_OK) return r;
    }
    return AMDG_OK;
}

// the coefficient arrays of the wave's point fields (K du/dx_d for d < dim, K u): FP64, or the FP32
// ones of the mixed back transforms, in the second half of w_fields
template <typename To>
void wave_field_coefs(amdg_burgers_op* op, To** fc) {
    const int dim = op->grid->host.dim;
    const size_t stride = size_t(op->capacity) * op->points;
    double* fields = static_cast<double*>(op->w_fields);
    for (int f = 0; f <= dim; ++f) fc[f] = reinterpret_cast<To*>(fields + size_t(dim + 1 + f) * stride);
}

// rhs (FP64, dof entries) of the FP64 state u, or the stage update `so` with it.
// The point values and the hierarchical surplus always run in FP64:
// fine-level surpluses are small differences of O(1) point values, which FP32
// rounding would swamp.  In mixed mode the back transforms (the bulk of the
// work) and the penalty run in FP32, their terms summed in FP64.
amdg_status eval_rhs(amdg_burgers_op* op, const double* u, double* rhs, amdg_precision prec, StageOut so = StageOut{}) {
    PhaseTimer timer(op->grid->ctx, AMDG_PHASE_RHS);
    cudaStream_t st = stream_of(op);
    const int dim = op->grid->host.dim;
    if (op->kind == 1) {
        const size_t stride = size_t(op->capacity) * op->points;
        double* fields = static_cast<double*>(op->w_fields);
        if (prec == AMDG_PREC_FP64) {
            double* fc[kMaxTermSources];
            for (int f = 0; f <= dim; ++f) fc[f] = fields + size_t(dim + 1 + f) * stride;
            if (amdg_status r = eval_wave_fields<double>(op, u, fc, st); r != AMDG_OK) return r;
            return eval_back_transforms<double>(op, mats64(op), fc, dim + 1, u, rhs, so, st);
        }
        float* fc[kMaxTermSources];
        for (int f = 0; f <= dim; ++f) fc[f] = reinterpret_cast<float*>(fields + size_t(dim + 1 + f) * stride);
        if (amdg_status r = eval_wave_fields<float>(op, u, fc, st); r != AMDG_OK) return r;
        float* u32 = static_cast<float*>(op->w_u);
        AMDG_CK(launch_convert<double, float>(u, u32, op->grid->dof, st));
        op->grid->ctx->launches++;
        return eval_back_transforms<float>(op, mats32(op), fc, dim + 1, u32, rhs, so, st);
    }
    double* fp = static_cast<double*>(op->w_a);
    amdg_status r = prec == AMDG_PREC_FP64
                        ? eval_point_values<double>(op, mats64(op), u, static_cast<double*>(op->w_up), fp, st)
                        : eval_point_values_df(op, u, static_cast<double*>(op->w_up), fp, st);
    if (r != AMDG_OK) return r;
    if (prec == AMDG_PREC_FP64) {
        double* fu = static_cast<double*>(op->w_fu);
        if ((r = eval_surplus<double, double>(op, fp, fu, st)) != AMDG_OK) return r;
        const double* src[1] = {fu};
        return eval_back_transforms<double>(op, mats64(op), src, 1, u, rhs, so, st);
    }
    float* fu32 = static_cast<float*>(op->w_fu);
    float* u32 = static_cast<float*>(op->w_u);
    if ((r = eval_surplus<double, float>(op, fp, fu32, st)) != AMDG_OK) return r;
    AMDG_CK(launch_convert<double, float>(u, u32, op->grid->dof, st));
    op->grid->ctx->launches++;
    const float* src[1] = {fu32};
    return eval_back_transforms<float>(op, mats32(op), src, 1, u32, rhs, so, st);
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
        cudaError_t e = amdg::device_malloc(reinterpret_cast<void**>(p), want);
        if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        cap = want;
    }
    if (bytes) AMDG_CK(cudaMemcpyAsync(*p, host.data(), bytes, cudaMemcpyHostToDevice, st));
    return AMDG_OK;
}

// Grow-only device array of the operator with room for `bytes` (contents not kept).
template <typename T>
amdg_status reserve_grow(amdg_burgers_op* op, T** p, size_t bytes) {
    size_t& cap = op->dev_cap[static_cast<const void*>(p)];
    if (bytes <= cap && *p) return AMDG_OK;
    cudaFree(*p);
    *p = nullptr;
    cap = 0;
    const size_t want = bytes + bytes / 4 + 64;
    if (amdg::device_malloc(reinterpret_cast<void**>(p), want) != cudaSuccess) {
        *p = nullptr;
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (neighbour lists)");
    }
    cap = want;
    return AMDG_OK;
}

// The neighbour lists and surplus ancestors built on the device from the grid's keys
// (csrc/adapt_device.cu), into arrays sized by the bounds of the element set's level sums.
amdg_status device_topology(amdg_burgers_op* op, cudaStream_t st) {
    amdg_grid* g = op->grid;
    const int64_t rows = g->host.num_elements * g->host.dim;
    int64_t vb = 0, fb = 0;
    transform_topology_bounds(g, &vb, &fb);
    AMDG_REQUIRE(vb < (int64_t(1) << 31) && fb < (int64_t(1) << 31), AMDG_ERR_CAPACITY, "neighbour lists exceed 2^31 pairs");
    amdg_status s;
    if ((s = reserve_grow(op, &op->d_vol_ptr, size_t(rows + 1) * sizeof(int32_t))) != AMDG_OK ||
        (s = reserve_grow(op, &op->d_flx_ptr, size_t(rows + 1) * sizeof(int32_t))) != AMDG_OK ||
        (s = reserve_grow(op, &op->d_vol_split, size_t(rows + 1) * sizeof(int32_t))) != AMDG_OK ||
        (s = reserve_grow(op, &op->d_flx_split, size_t(rows + 1) * sizeof(int32_t))) != AMDG_OK ||
        (s = reserve_grow(op, &op->d_topo_cnt, size_t(2 * (rows + 1)) * sizeof(int32_t))) != AMDG_OK ||
        (s = reserve_grow(op, &op->d_vol_nbr, size_t(2 * vb) * sizeof(int32_t))) != AMDG_OK ||
        (s = reserve_grow(op, &op->d_flx_nbr, size_t(2 * fb) * sizeof(int32_t))) != AMDG_OK ||
        (s = reserve_grow(op, &op->d_anc, size_t(rows) * op->p1 * sizeof(int32_t))) != AMDG_OK)
        return s;
    if (!op->d_anc_order) {
        std::vector<int32_t> ao = op->anc_order;
        if ((s = upload_vec(&op->d_anc_order, ao)) != AMDG_OK) return s;
    }
    int* err = grid_topology_error_flag(g);
    AMDG_REQUIRE(err, AMDG_ERR_NOMEM, "device adaptivity statistics");
    const size_t vcap = op->dev_cap[static_cast<const void*>(&op->d_vol_nbr)] / (2 * sizeof(int32_t));
    const size_t fcap = op->dev_cap[static_cast<const void*>(&op->d_flx_nbr)] / (2 * sizeof(int32_t));
    DeviceTopoOut out{op->d_vol_ptr, op->d_vol_nbr, op->d_vol_split, op->d_flx_ptr, op->d_flx_nbr, op->d_flx_split,
                      op->d_anc, int64_t(vcap), int64_t(fcap), op->d_anc_order, op->p1, err};
    if ((s = device_transform_topology(g, out, op->d_topo_cnt, st)) != AMDG_OK) return s;
    // a set that came from the host may have holes: report them now (sets the device refine and
    // coarsen produce are hole-free; their build errors surface at the next element-set change)
    if (!g->host_stale) return grid_check_topology(g);
    return AMDG_OK;
}

// (Re)build the neighbour lists and surplus ancestors for the grid's current
// element set; device arrays and work buffers only grow.
amdg_status burgers_sync(amdg_burgers_op* op) {
    amdg_grid* g = op->grid;
    if (op->built_version == g->version) return AMDG_OK;
    PhaseTimer timer(g->ctx, AMDG_PHASE_TOPOLOGY);
    cudaStream_t st = stream_of(op);
    LagrTables t;
    if (op->anc_order.empty()) {
        // ancestor orders only depend on nmax
        Basis1D b{g->host.k, g->host.nmax};
        build_lagr_ancestors(b, op->p1 - 1, &t);
        op->anc_order = t.anc_order;
    } else {
        t.anc_order = op->anc_order;
        t.p1 = op->p1;
    }
    amdg_status s;
    if (g->ctx->adapt_mode == AMDG_ADAPT_DEVICE) {
        if ((s = device_topology(op, st)) != AMDG_OK) return s;
    } else {
        if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
        TransformTopology topo;
        build_transform_topology(g->host, &topo);
        std::vector<int32_t> anc;
        if (!build_surplus_ancestors(g->host, t, &anc))
            return fail(AMDG_ERR_STATE, "element set has a hole: a surplus ancestor is missing");
        if ((s = upload_grow(op, &op->d_vol_ptr, topo.vol_ptr, st)) != AMDG_OK ||
            (s = upload_grow(op, &op->d_vol_nbr, topo.vol_nbr, st)) != AMDG_OK ||
            (s = upload_grow(op, &op->d_flx_ptr, topo.flx_ptr, st)) != AMDG_OK ||
            (s = upload_grow(op, &op->d_flx_nbr, topo.flx_nbr, st)) != AMDG_OK ||
            (s = upload_grow(op, &op->d_anc, anc, st)) != AMDG_OK ||
            (s = upload_grow(op, &op->d_vol_split, topo.vol_split, st)) != AMDG_OK ||
            (s = upload_grow(op, &op->d_flx_split, topo.flx_split, st)) != AMDG_OK)
            return s;
        // the host vectors above are released on return: wait for their copies
        AMDG_CK(cudaStreamSynchronize(st));
    }
    const int64_t E = g->host.num_elements;
    if (E > op->capacity) {
        const int64_t cap = E + E / 2 + 16;
        void* bufs[] = {op->w_up, op->w_fu, op->w_a, op->w_b, op->w_u, op->w_s0, op->w_s1, op->w_slots,
                        op->d_u1, op->d_rhs64, op->d_pred, op->w_fields, op->d_v1, op->d_su, op->d_sv};
        for (void* p : bufs) cudaFree(p);
        op->w_up = op->w_fu = op->w_a = op->w_b = op->w_u = op->w_s0 = op->w_s1 = op->w_slots = op->w_fields = nullptr;
        op->d_u1 = op->d_rhs64 = op->d_pred = op->d_v1 = op->d_su = op->d_sv = nullptr;
        op->capacity = 0;
        const size_t work = size_t(cap) * op->points * sizeof(double);
        const size_t vec = size_t(cap) * g->block * sizeof(double);
        // terms per launch: all of them unless their three slices per term
        // (two sweep buffers and the output) would pass kTermBudget bytes
        const int nterms = int(op->terms.size());
        op->chunk = int(std::max<int64_t>(1, std::min<int64_t>(nterms, int64_t(kTermBudget / (3 * work)))));
        const size_t slices = size_t(op->chunk) * work;
        if ((s = alloc_bytes(&op->w_up, work)) != AMDG_OK || (s = alloc_bytes(&op->w_fu, work)) != AMDG_OK ||
            (s = alloc_bytes(&op->w_a, work)) != AMDG_OK || (s = alloc_bytes(&op->w_b, work)) != AMDG_OK ||
            (s = alloc_bytes(&op->w_u, vec)) != AMDG_OK || (s = alloc_bytes(&op->w_s0, slices)) != AMDG_OK ||
            (s = alloc_bytes(&op->w_s1, slices)) != AMDG_OK || (s = alloc_bytes(&op->w_slots, slices)) != AMDG_OK ||
            (s = alloc_bytes(reinterpret_cast<void**>(&op->d_u1), vec)) != AMDG_OK ||
            (s = alloc_bytes(reinterpret_cast<void**>(&op->d_rhs64), vec)) != AMDG_OK ||
            (s = alloc_bytes(reinterpret_cast<void**>(&op->d_pred), vec)) != AMDG_OK)
            return s;
        if (op->kind == 1 &&
            ((s = alloc_bytes(&op->w_fields, 2 * size_t(g->host.dim + 1) * work)) != AMDG_OK ||
             (s = alloc_bytes(reinterpret_cast<void**>(&op->d_v1), vec)) != AMDG_OK ||
             (s = alloc_bytes(reinterpret_cast<void**>(&op->d_su), vec)) != AMDG_OK ||
             (s = alloc_bytes(reinterpret_cast<void**>(&op->d_sv), vec)) != AMDG_OK))
            return s;
        op->capacity = cap;
    }
    if (op->kind == 1) {  // the IPDG coefficient follows the finest level
        const double c = wave_penalty_coef(op);
        bool changed = false;
        for (PartialSum& p : op->terms)
            if (p.kind == 1 && p.coef != c) { p.coef = c; changed = true; }
        if (changed && (s = refresh_nodes(op, st)) != AMDG_OK) return s;  // only when the finest level changed
    }
    if ((s = prepare_trees(op, st)) != AMDG_OK) return s;
    op->built_version = g->version;
    return AMDG_OK;
}

// Parent / grandparent table of the current element set (uploaded once per
// element set) and classifier buffers for E elements of F features (E = 0:
// the table only).
amdg_status ensure_features(amdg_burgers_op* op, int64_t E, int F) {
    amdg_grid* g = op->grid;
    amdg_status s;
    if (op->pg_version != g->version) {
        if (g->ctx->adapt_mode == AMDG_ADAPT_DEVICE) {
            if ((s = reserve_grow(op, &op->d_pg, size_t(g->host.num_elements) * g->host.dim * 2 * sizeof(int32_t))) !=
                    AMDG_OK ||
                (s = device_parent_table(g, op->d_pg, stream_of(op))) != AMDG_OK)
                return s;
        } else {
            if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
            std::vector<int32_t> pg;
            parent_table(g->host, &pg);
            if ((s = upload_grow(op, &op->d_pg, pg, stream_of(op))) != AMDG_OK) return s;
            AMDG_CK(cudaStreamSynchronize(stream_of(op)));  // pg is released on return
        }
        op->pg_version = g->version;
    }
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

// a Lagrange-path operator of the given kind on g (tables, terms, neighbour lists)
static amdg_status lagr_create(amdg_grid* g, int kind, const double* alpha, double sigma, amdg_burgers_op** out,
                               int lagr_degree = 0) {
    *out = nullptr;
    AMDG_REQUIRE(g->host.k == 2, AMDG_ERR_ARG, "the Lagrange path is built for Alpert degree k = 2");
    AMDG_CK(cudaSetDevice(g->device));
    const int dim = g->host.dim;
    amdg_burgers_op* op = new (std::nothrow) amdg_burgers_op;
    AMDG_REQUIRE(op, AMDG_ERR_NOMEM, "host allocation failed");
    op->kind = kind;
    op->sigma = sigma;
    op->grid = g;
    op->device = g->device;
    if (alpha) op->alpha.assign(alpha, alpha + dim);
    else op->alpha.assign(dim, 0.0);
    // Lagrange degree as the examples set it: 3 for Burgers, 4 for the wave equation; the
    // interpolation init takes the caller's
    const int degree = kind == 1 ? 4 : (kind == 2 ? lagr_degree : 3);  // kind 3: cubic Hermite
    op->p1 = degree + 1;
    op->points = 1;
    for (int d = 0; d < dim; ++d) op->points *= op->p1;
    op->n1 = 1 << g->host.nmax;
    Basis1D b{g->host.k, g->host.nmax};
    LagrTables t;
    if (kind == 3) build_herm_tables(b, &t);
    else build_lagr_tables(b, degree, &t, kind == 1);
    op->anc_order = t.anc_order;
    // the sweeps read the tables blocked by 1D order pair (the rows and columns of one pair contiguous)
    const int np = g->host.k + 1;
    if (!reblock_table(&t.a2p, op->n1, np, op->p1) || !reblock_table(&t.lv, op->n1, op->p1, np) ||
        !reblock_table(&t.lvx, op->n1, op->p1, np) || !reblock_table(&t.lflx, op->n1, op->p1, np) ||
        !reblock_table(&t.ajump, op->n1, np, np) || !reblock_table(&t.a2pd, op->n1, np, op->p1) ||
        !reblock_table(&t.ljv, op->n1, op->p1, np)) {
        delete op;
        return fail(AMDG_ERR_ARG, "Lagrange table of unexpected size");
    }
    std::memcpy(op->weight, t.weight, sizeof(op->weight));
    transform_schedule(dim, &op->sched_dims, &op->sched_lu);
    build_terms(op);
    amdg_status s;
    if ((s = upload_both(&op->d_a2p, &op->f_a2p, t.a2p)) != AMDG_OK || (s = upload_both(&op->d_lv, &op->f_lv, t.lv)) != AMDG_OK ||
        (s = upload_both(&op->d_lvx, &op->f_lvx, t.lvx)) != AMDG_OK ||
        (s = upload_both(&op->d_lflx, &op->f_lflx, t.lflx)) != AMDG_OK ||
        (s = upload_both(&op->d_ajump, &op->f_ajump, t.ajump)) != AMDG_OK ||
        (kind == 1 && ((s = upload_both(&op->d_a2pd, &op->f_a2pd, t.a2pd)) != AMDG_OK ||
                       (s = upload_both(&op->d_ljv, &op->f_ljv, t.ljv)) != AMDG_OK ||
                       (s = upload_vec(&op->d_pts, t.pts)) != AMDG_OK)) ||
        (s = upload_df(&op->df_a2p, t.a2p)) != AMDG_OK || (kind == 1 && (s = upload_df(&op->df_a2pd, t.a2pd)) != AMDG_OK) ||
        (s = upload_vec(&op->d_anc_point, t.anc_point)) != AMDG_OK || (s = upload_vec(&op->d_anc_rank, t.anc_rank)) != AMDG_OK ||
        (s = upload_vec(&op->d_terms, op->terms)) != AMDG_OK || (s = burgers_sync(op)) != AMDG_OK) {
        amdg_burgers_destroy(op);
        return s;
    }
    *out = op;
    return AMDG_OK;
}

amdg_status amdg_burgers_create(amdg_grid* g, const double* alpha, amdg_burgers_op** out) {
    AMDG_REQUIRE(g && alpha && out, AMDG_ERR_ARG, "null argument");
    for (int d = 0; d < g->host.dim; ++d) AMDG_REQUIRE(std::isfinite(alpha[d]), AMDG_ERR_ARG, "non-finite alpha");
    return lagr_create(g, 0, alpha, 0.0, out);
}

amdg_status amdg_burgers_create_herm(amdg_grid* g, const double* alpha, amdg_burgers_op** out) {
    AMDG_REQUIRE(g && alpha && out, AMDG_ERR_ARG, "null argument");
    AMDG_REQUIRE(g->host.dim == 2, AMDG_ERR_ARG, "the Hermite flux interpolation is two-dimensional (nonlinear_Herm_2D_fast)");
    for (int d = 0; d < g->host.dim; ++d) AMDG_REQUIRE(std::isfinite(alpha[d]), AMDG_ERR_ARG, "non-finite alpha");
    return lagr_create(g, 3, alpha, 0.0, out);
}

amdg_status amdg_burgers_destroy(amdg_burgers_op* op) {
    if (!op) return AMDG_OK;
    cudaSetDevice(op->device);
    if (op->graph_exec) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(op->graph_exec));
    void* ptrs[] = {op->d_a2p, op->d_lv, op->d_lvx, op->d_lflx, op->d_ajump, op->f_a2p, op->f_lv, op->f_lvx, op->f_lflx,
                    op->f_ajump, op->d_vol_ptr, op->d_vol_nbr, op->d_flx_ptr, op->d_flx_nbr,
                    op->d_anc, op->d_anc_point, op->d_anc_rank, op->w_up, op->w_fu, op->w_a, op->w_b, op->w_u,
                    op->w_s0, op->w_s1, op->w_slots, op->d_terms,
                    op->d_u1, op->d_u2, op->d_rhs64, op->d_pred, op->d_vol_split, op->d_flx_split,
                    op->d_pg,
                    op->d_feat, op->d_prob, op->d_a2pd, op->d_ljv, op->d_pts, op->f_a2pd, op->f_ljv,
                    op->w_fields, op->d_v1, op->d_su, op->d_sv, op->df_a2p, op->df_a2pd,
                    op->d_anc_order, op->d_topo_cnt, op->d_cls, op->d_nodes};
    for (void* p : ptrs) cudaFree(p);
    cudaFreeHost(op->h_cls);
    delete op;
    return AMDG_OK;
}

amdg_status amdg_burgers_rhs(amdg_burgers_op* op, const double* d_u, double* d_rhs, amdg_precision prec) {
    AMDG_REQUIRE(op && d_u && d_rhs && d_u != d_rhs, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    op->rhs_evaluations++;
    return eval_rhs(op, d_u, d_rhs, prec);
}

amdg_status amdg_burgers_work(amdg_burgers_op* op, double* flops, double* transform_pairs) {
    AMDG_REQUIRE(op, AMDG_ERR_ARG, "null argument");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    const int dim = g->host.dim, np = g->host.k + 1, p1 = op->p1;
    const int64_t E = g->host.num_elements, rows = E * dim;
    // neighbour counts per (dimension, vol/flx, L/full/U) summed over the elements
    std::vector<int32_t> ptr[2], split[2];
    const int32_t* dp[2] = {op->d_vol_ptr, op->d_flx_ptr};
    const int32_t* ds[2] = {op->d_vol_split, op->d_flx_split};
    for (int f = 0; f < 2; ++f) {
        ptr[f].resize(size_t(rows + 1));
        split[f].resize(size_t(std::max<int64_t>(rows, 1)));
        AMDG_CK(cudaMemcpy(ptr[f].data(), dp[f], size_t(rows + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost));
        if (rows) AMDG_CK(cudaMemcpy(split[f].data(), ds[f], size_t(rows) * sizeof(int32_t), cudaMemcpyDeviceToHost));
    }
    double cnt[kMaxDim][2][3] = {};
    for (int64_t r = 0; r < rows; ++r)
        for (int f = 0; f < 2; ++f) {
            const int t = int(r % dim);
            cnt[t][f][0] += ptr[f][r + 1] - split[f][r];  // "L": finer neighbours
            cnt[t][f][1] += ptr[f][r + 1] - ptr[f][r];
            cnt[t][f][2] += split[f][r] - ptr[f][r];      // "U": coarser or equal
        }
    // the sweeps one right-hand side runs: the nodes of the sweep trees of its term ranges
    double fl = 0.0, pairs = 0.0;
    std::vector<std::pair<int, int>> ranges;
    auto chunks = [&](int first, int total) {
        for (int c0 = 0; c0 < total; c0 += op->chunk) ranges.push_back({first + c0, std::min(op->chunk, total - c0)});
    };
    const int nterms = int(op->terms.size());
    if (op->kind == 1) {
        const int G = int(op->sched_dims.size());
        for (int f = 0; f <= dim; ++f) chunks(f * G, G);
    } else {
        chunks(0, op->n_pv_terms);
    }
    chunks(op->n_pv_terms, nterms - op->n_pv_terms);
    for (const auto& r : ranges) {
        SweepTree tree;
        if (amdg_status s = sweep_tree(op, r.first, r.second, &tree, stream_of(op)); s != AMDG_OK) return s;
        const bool pv = r.first < op->n_pv_terms;
        const int n_in = pv ? np : p1, n_out = pv ? p1 : np;
        for (int j = 0; j < dim; ++j)
            for (int k = 0; k < tree.count[j]; ++k) {
                const PartialSum& D = op->nodes[size_t(tree.offset[j] + k)];
                if (D.kind == 1) {  // the penalty: one full transform along dims[0] on the flx sets
                    const double c = cnt[D.dims[0]][1][1];
                    fl += 2.0 * np * ipow(np, dim) * c;
                    pairs += c;
                    continue;
                }
                const double c = cnt[D.dims[j]][D.flx[j]][D.lu[j]];
                fl += 2.0 * n_in * ipow(n_out, j + 1) * ipow(n_in, dim - j - 1) * c;
                pairs += c;
            }
    }
    // hierarchical surplus passes (one field for Burgers, dim + 1 for the wave operator)
    fl += 2.0 * dim * double(E) * op->points * p1 * (op->kind == 1 ? dim + 1 : 1);
    if (flops) *flops = fl;
    if (transform_pairs) *transform_pairs = pairs;
    return AMDG_OK;
}

amdg_status amdg_burgers_set_sweep_variant(amdg_burgers_op* op, int variant) {
    AMDG_REQUIRE(op && variant >= -1 && variant <= 4, AMDG_ERR_ARG, "variant must be -1 .. 4");
    op->sweep_variant = variant;
    op->graph_version = -1;  // a captured step launched the other kernel
    return AMDG_OK;
}

amdg_status amdg_lagr_interpolate(amdg_burgers_op* op, amdg_precision prec) {
    AMDG_REQUIRE(op && burgers_like(op), AMDG_ERR_ARG, "a Burgers operator is required");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(op);
    // point values (FP64, or double-float in mixed mode), the flux u^2/2 at the points, and its
    // surpluses: FP64, or the FP32 coefficients the mixed back transforms read
    double* fp = static_cast<double*>(op->w_a);
    amdg_status r = prec == AMDG_PREC_FP64
                        ? eval_point_values<double>(op, mats64(op), g->d_u, static_cast<double*>(op->w_up), fp, st)
                        : eval_point_values_df(op, g->d_u, static_cast<double*>(op->w_up), fp, st);
    if (r != AMDG_OK) return r;
    r = prec == AMDG_PREC_FP64 ? eval_surplus<double, double>(op, fp, static_cast<double*>(op->w_fu), st)
                               : eval_surplus<double, float>(op, fp, static_cast<float*>(op->w_fu), st);
    if (r != AMDG_OK) return r;
    op->interp_version = g->version;
    op->interp_prec = prec;
    return AMDG_OK;
}

amdg_status amdg_lagr_rhs_add(amdg_burgers_op* op, int group, const double* alpha, amdg_precision prec) {
    AMDG_REQUIRE(op && burgers_like(op), AMDG_ERR_ARG, "a Burgers operator is required");
    AMDG_REQUIRE(group >= AMDG_LAGR_RHS_VOL && group <= AMDG_LAGR_RHS_PENALTY, AMDG_ERR_ARG, "unknown term group");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(op);
    const int dim = g->host.dim;
    if (group != AMDG_LAGR_RHS_PENALTY)
        AMDG_REQUIRE(op->interp_version == g->version && op->interp_prec == int(prec), AMDG_ERR_STATE,
                     "no flux interpolation of this element set and precision: call amdg_lagr_interpolate first");
    if (group == AMDG_LAGR_RHS_PENALTY && alpha) {  // the LxF constants of this call
        bool changed = false;
        for (int d = 0; d < dim; ++d) {
            AMDG_REQUIRE(std::isfinite(alpha[d]), AMDG_ERR_ARG, "non-finite alpha");
            PartialSum& p = op->terms[size_t(op->grp_first[2] + d)];
            if (p.coef != -alpha[d] / 2.0) {
                p.coef = -alpha[d] / 2.0;
                op->alpha[d] = alpha[d];
                changed = true;
            }
        }
        if (changed)
            if (amdg_status s = refresh_nodes(op, st); s != AMDG_OK) return s;
    }
    double* rhs = nullptr;
    if (amdg_status s = grid_rhs(g, &rhs); s != AMDG_OK) return s;
    const int first = op->grp_first[group], count = op->grp_count[group];
    if (prec == AMDG_PREC_FP64) {
        const double* src[1] = {static_cast<const double*>(op->w_fu)};
        return eval_term_range<double>(op, mats64(op), first, count, src, 1, g->d_u, rhs, StageOut{}, st, true);
    }
    float* u32 = static_cast<float*>(op->w_u);
    if (group == AMDG_LAGR_RHS_PENALTY) {
        AMDG_CK(launch_convert<double, float>(g->d_u, u32, g->dof, st));
        g->ctx->launches++;
    }
    const float* src[1] = {static_cast<const float*>(op->w_fu)};
    return eval_term_range<float>(op, mats32(op), first, count, src, 1, u32, rhs, StageOut{}, st, true);
}

amdg_status amdg_burgers_point_values(amdg_burgers_op* op, const double* d_u, double* d_up, amdg_precision prec) {
    AMDG_REQUIRE(op && d_u && d_up, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    cudaStream_t st = stream_of(op);
    if (prec == AMDG_PREC_FP64) return eval_point_values<double>(op, mats64(op), d_u, d_up, nullptr, st);
    const int64_t n = op->grid->dof, np = op->grid->host.num_elements * op->points;
    float* u32 = static_cast<float*>(op->w_u);
    float* up32 = static_cast<float*>(op->w_up);
    AMDG_CK(launch_convert<double, float>(d_u, u32, n, st));
    amdg_status r = eval_point_values<float>(op, mats32(op), u32, up32, nullptr, st);
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
        amdg_status r = eval_point_values<double>(op, mats64(op), d_u, static_cast<double*>(op->w_up),
                                                  static_cast<double*>(op->w_a), st);
        if (r != AMDG_OK) return r;
        return eval_surplus<double, double>(op, static_cast<const double*>(op->w_a), d_fu, st);
    }
    float* u32 = static_cast<float*>(op->w_u);
    AMDG_CK(launch_convert<double, float>(d_u, u32, op->grid->dof, st));
    amdg_status r = eval_point_values<float>(op, mats32(op), u32, static_cast<float*>(op->w_up),
                                             static_cast<float*>(op->w_a), st);
    if (r != AMDG_OK) return r;
    if ((r = eval_surplus<float, float>(op, static_cast<const float*>(op->w_a), static_cast<float*>(op->w_fu), st)) !=
        AMDG_OK)
        return r;
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
    PhaseTimer timer(g->ctx, AMDG_PHASE_RK3);
    cudaStream_t st = stream_of(op);
    if (nsteps == 0) return AMDG_OK;
    const size_t bytes = size_t(g->dof) * sizeof(double);
    // one step: ucoe is updated in place per stage, ucoe_tn holds u^n (RK3SSP::step_stage)
    auto step = [&]() -> amdg_status {
        AMDG_CK(cudaMemcpyAsync(op->d_u1, g->d_u, bytes, cudaMemcpyDeviceToDevice, st));
        for (int stage = 0; stage < 3; ++stage) {
            // the last reduction applies the stage update in place (u1 is the stage input)
            const StageOut so{1, stage_coef(stage, dt), g->d_u, op->d_u1, op->d_u1};
            if (amdg_status r = eval_rhs(op, op->d_u1, op->d_rhs64, prec, so); r != AMDG_OK) return r;
        }
        AMDG_CK(cudaMemcpyAsync(g->d_u, op->d_u1, bytes, cudaMemcpyDeviceToDevice, st));
        return AMDG_OK;
    };
    op->rhs_evaluations += 3 * int64_t(nsteps);
    op->stage_dof_updates += 3 * int64_t(nsteps) * g->dof;
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
    double sum_c_dx = 0.0;
    for (int d = 0; d < g->host.dim; ++d) sum_c_dx += wave_speed * std::pow(2.0, g->lev_max[d]);
    return cfl / sum_c_dx;
}

// keys of the elements present after a step, to mark coarsened ones
static void mark_removed(const std::vector<uint64_t>& old_keys, const HostGrid& now, int8_t* decisions) {
    for (size_t e = 0; e < old_keys.size(); ++e)
        if (!std::binary_search(now.key.begin(), now.key.end(), old_keys[e])) decisions[e] = 2;
}

static amdg_status wave_rk4(amdg_burgers_op* op, double dt, int nsteps, amdg_precision prec);
static amdg_status ensure_velocity(amdg_grid* g);

// one time step of the operator's scheme: SSP-RK3 (Burgers) or RK4ODE2nd (wave)
static amdg_status one_step(amdg_burgers_op* op, double dt, amdg_precision prec) {
    if (burgers_like(op)) return amdg_burgers_rk3_steps(op, dt, 1, prec);
    if (amdg_status s = burgers_sync(op); s != AMDG_OK) return s;
    return wave_rk4(op, dt, 1, prec);
}

// the adaptive time step of either operator: predictor (ForwardEuler on u / EulerODE2nd on
// (u, u_t)), refine on the predicted indicator, one step, coarsen
static amdg_status adaptive_step_any(amdg_burgers_op* op, double cfl, double wave_speed, double eps, double eta,
                                     amdg_precision prec, double* dt_out, int8_t* decisions) {
    AMDG_REQUIRE(op && std::isfinite(cfl) && cfl > 0 && std::isfinite(wave_speed) && wave_speed > 0, AMDG_ERR_ARG,
                 "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    PhaseTimer timer(g->ctx, AMDG_PHASE_ADAPT_STEP);
    cudaStream_t st = stream_of(op);
    const double dt = adaptive_dt(g, cfl, wave_speed);
    const bool on_device = g->ctx->adapt_mode == AMDG_ADAPT_DEVICE;
    amdg_status s;
    std::vector<uint64_t> old_keys;
    if (decisions || !on_device) {
        if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
        old_keys = g->host.key;
    }
    if (burgers_like(op)) {
        op->rhs_evaluations++;
        // forward Euler into the prediction buffer (ForwardEuler::step_stage)
        const StageOut so{1, stage_coef(0, dt), g->d_u, g->d_u, op->d_pred};
        if ((s = eval_rhs(op, g->d_u, op->d_rhs64, prec, so)) != AMDG_OK) return s;
    } else {
        // EulerODE2nd::step_rk_source on copies of (u, v): u + dt v, v + dt (IPDG u)
        if ((s = grid_ensure_velocity(g)) != AMDG_OK) return s;
        if ((s = eval_wave_penalty(op, g->d_u, op->d_rhs64, st)) != AMDG_OK) return s;
        AMDG_CK(launch_rk4_2nd_stage(-1, dt, op->d_rhs64, g->d_u, g->d_v, op->d_pred, op->d_su, nullptr, nullptr, g->dof,
                                     st));
        g->ctx->launches++;
    }
    // refine on the predicted coefficients (and, for the wave, the predicted u_t: the
    // indicator of prob "wave" is ||u|| + ||u_t||); new elements start from zero
    // (DGAdapt::refine, copy_predict_to_ucoe)
    if (on_device) {
        {
            PhaseTimer ta(g->ctx, AMDG_PHASE_ADAPT_DEVICE);
            std::vector<int8_t> refined(decisions ? size_t(g->host.num_elements) : 0);
            if ((s = grid_device_norms(g, op->d_pred, op->kind == 1 ? op->d_su : nullptr)) != AMDG_OK ||
                (s = grid_device_refine(g, eps, nullptr, decisions ? refined.data() : nullptr, nullptr)) != AMDG_OK)
                return s;
            if (decisions) std::copy(refined.begin(), refined.end(), decisions);
        }
        if ((s = one_step(op, dt, prec)) != AMDG_OK) return s;
        if ((s = grid_coarsen(g, eta, op->kind == 1 ? g->d_v : nullptr, nullptr)) != AMDG_OK) return s;
        if (decisions) {
            if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
            mark_removed(old_keys, g->host, decisions);
        }
        if (dt_out) *dt_out = dt;
        return AMDG_OK;
    }
    std::vector<double> norms;
    if ((s = grid_norms(g, op->d_pred, &norms, op->kind == 1 ? op->d_su : nullptr)) != AMDG_OK) return s;
    std::vector<uint8_t> refined;
    std::vector<uint64_t> keys;
    {
        PhaseTimer th(g->ctx, AMDG_PHASE_ADAPT_HOST);
        keys = refine_keys(g->host, norms.data(), eps, &refined);
    }
    if (decisions)
        for (size_t e = 0; e < refined.size(); ++e) decisions[e] = refined[e] ? 1 : 0;
    if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
    if ((s = one_step(op, dt, prec)) != AMDG_OK) return s;
    if ((s = grid_coarsen(g, eta, op->kind == 1 ? g->d_v : nullptr, nullptr)) != AMDG_OK) return s;
    if (decisions) mark_removed(old_keys, g->host, decisions);
    if (dt_out) *dt_out = dt;
    return AMDG_OK;
}

amdg_status amdg_burgers_adaptive_step_ex(amdg_burgers_op* op, double cfl, double wave_speed, double eps, double eta,
                                          amdg_precision prec, double* dt_out, int8_t* decisions) {
    return adaptive_step_any(op, cfl, wave_speed, eps, eta, prec, dt_out, decisions);
}

amdg_status amdg_burgers_adaptive_step(amdg_burgers_op* op, double cfl, double wave_speed, double eps, double eta,
                                       amdg_precision prec, double* dt_out) {
    return adaptive_step_any(op, cfl, wave_speed, eps, eta, prec, dt_out, nullptr);
}

amdg_status amdg_burgers_features(amdg_burgers_op* op, const double* d_u, float* d_features) {
    AMDG_REQUIRE(op && d_u && d_features, AMDG_ERR_ARG, "null argument");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    if (amdg_status s = ensure_features(op, 0, 0); s != AMDG_OK) return s;
    if (op->kind == 1)
        if (amdg_status s = grid_ensure_velocity(g); s != AMDG_OK) return s;
    AMDG_CK(launch_element_features(d_u, op->kind == 1 ? g->d_v : nullptr, op->d_pg, g->host.num_elements, g->host.dim,
                                    g->block, d_features, stream_of(op)));
    g->ctx->launches++;
    return AMDG_OK;
}

// The horizon's time steps on the current grid, no predictor: n - 1 steps of dt (replayed as a CUDA
// graph when n - 1 > 1), the last one of dt_last (n = horizon, or fewer to land on t_left).
static amdg_status horizon_steps(amdg_burgers_op* op, double dt, amdg_precision prec, int horizon, double t_left,
                                 double* t_advanced, int* steps_out) {
    int n = horizon;
    double dt_last = dt;
    if (t_left > 0) {
        const int need = std::max(1, int(std::ceil(t_left / dt - 1e-9)));
        if (need <= n) {
            n = need;
            dt_last = t_left - (n - 1) * dt;
        }
    }
    amdg_status s;
    if (n > 1) {
        if (burgers_like(op)) s = amdg_burgers_rk3_steps(op, dt, n - 1, prec);  // syncs the operator itself
        else if ((s = burgers_sync(op)) == AMDG_OK) s = wave_rk4(op, dt, n - 1, prec);
        if (s != AMDG_OK) return s;
    }
    if ((s = one_step(op, dt_last, prec)) != AMDG_OK) return s;
    if (t_advanced) *t_advanced = (n - 1) * dt + dt_last;
    if (steps_out) *steps_out = n;
    return AMDG_OK;
}

// The learned step with the element-set changes on the device: the classifier's probabilities
// (already in op->d_prob when mlp is given), the criterion's indicators and the missed
// refinements of the previous step decide the refined leaves without leaving the device; the
// coarsening records this step's missed refinements there too.
static amdg_status learned_step_device(amdg_burgers_op* op, amdg_mlp* mlp, double dt, double eps, double eta,
                                       double tau, amdg_precision prec, int horizon, double t_left, double* t_advanced,
                                       int* steps_out, int64_t* stats) {
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(op);
    amdg_status s;
    if (!op->d_cls) {
        void *d = nullptr, *h = nullptr;
        if (amdg::device_malloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess ||
            cudaMallocHost(&h, 2 * sizeof(unsigned long long)) != cudaSuccess) {
            cudaFree(d);
            return fail(AMDG_ERR_NOMEM, "classifier counters");
        }
        op->d_cls = static_cast<unsigned long long*>(d);
        op->h_cls = static_cast<unsigned long long*>(h);
    }
    {
        PhaseTimer ta(g->ctx, AMDG_PHASE_ADAPT_DEVICE);
        uint8_t* d_force = nullptr;
        AMDG_CK(cudaMemsetAsync(op->d_cls, 0, 2 * sizeof(unsigned long long), st));
        if ((s = grid_device_norms(g, g->d_u, op->kind == 1 ? g->d_v : nullptr)) != AMDG_OK ||
            (s = grid_learned_flags(g, mlp ? op->d_prob : nullptr, tau, eps, &d_force, op->d_cls)) != AMDG_OK ||
            (s = grid_mark_missed(g, d_force)) != AMDG_OK)
            return s;
        // read back with the refinement's synchronisation
        AMDG_CK(cudaMemcpyAsync(op->h_cls, op->d_cls, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        if ((s = grid_device_refine(g, eps, d_force, nullptr, nullptr)) != AMDG_OK) return s;
    }
    const int64_t n_net = int64_t(op->h_cls[0]), n_unsure = int64_t(op->h_cls[1]);
    if ((s = horizon_steps(op, dt, prec, horizon, t_left, t_advanced, steps_out)) != AMDG_OK) return s;
    {
        PhaseTimer ta(g->ctx, AMDG_PHASE_ADAPT_DEVICE);
        if ((s = grid_device_norms(g, g->d_u, op->kind == 1 ? g->d_v : nullptr)) != AMDG_OK ||
            (s = grid_device_coarsen(g, eta, eps, nullptr)) != AMDG_OK)
            return s;
    }
    if (stats) {
        stats[0] = n_net;
        stats[1] = n_unsure;
        stats[2] = g->dev.n_missed;
        stats[3] = g->host.num_elements;
    }
    return AMDG_OK;
}

// The learned adaptive step over a horizon of `horizon` time steps on one pre-adapted grid
// (horizon 1: one step).  With t_left > 0 no step goes past t_left: the horizon is cut to
// ceil(t_left / dt) steps and the last one shortened to land on it.  *t_advanced: the time
// stepped; *steps_out: the steps taken.
static amdg_status learned_step_any(amdg_burgers_op* op, amdg_mlp* mlp, double cfl, double wave_speed, double eps,
                                    double eta, double tau, amdg_precision prec, int horizon, double t_left,
                                    double* t_advanced, int* steps_out, int64_t* stats) {
    AMDG_REQUIRE(op && std::isfinite(cfl) && cfl > 0 && std::isfinite(wave_speed) && wave_speed > 0 &&
                     horizon >= 1 && std::isfinite(t_left) && t_left >= 0,
                 AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    PhaseTimer timer(g->ctx, AMDG_PHASE_ADAPT_STEP);
    cudaStream_t st = stream_of(op);
    const int64_t E = g->host.num_elements;
    // the wave classifier also reads u_t (the indicator of prob "wave" adds ||u_t||)
    const int F = g->block * (1 + 2 * g->host.dim) * (op->kind == 1 ? 2 : 1);
    if (mlp) {
        int n_in = 0, n_out = 0;
        mlp_shape(mlp, &n_in, &n_out);
        AMDG_REQUIRE(n_in == F && n_out == 3, AMDG_ERR_ARG,
                     "classifier must take " + std::to_string(F) + " features and give 3 classes");
    }
    // 1. the network's refine/keep/coarsen probabilities from the current coefficients (without
    //    a network every element counts as unsure: the criterion decides everywhere)
    amdg_status s = AMDG_OK;
    std::vector<float> prob(size_t(E) * 3, 0.0f);
    if (mlp) {
        PhaseTimer tc(g->ctx, AMDG_PHASE_CLASSIFIER);
        if ((s = ensure_features(op, E, F)) != AMDG_OK) return s;
        if (op->kind == 1 && (s = grid_ensure_velocity(g)) != AMDG_OK) return s;
        AMDG_CK(launch_element_features(g->d_u, op->kind == 1 ? g->d_v : nullptr, op->d_pg, E, g->host.dim, g->block,
                                        op->d_feat, st));
        g->ctx->launches++;
        if ((s = amdg_mlp_predict(mlp, op->d_feat, E, op->d_prob)) != AMDG_OK) return s;
        if (g->ctx->adapt_mode != AMDG_ADAPT_DEVICE)
            AMDG_CK(cudaMemcpyAsync(prob.data(), op->d_prob, prob.size() * sizeof(float), cudaMemcpyDeviceToHost, st));
    }
    if (op->kind == 1 && (s = grid_ensure_velocity(g)) != AMDG_OK) return s;
    const double* d_ut = op->kind == 1 ? g->d_v : nullptr;  // the wave indicator adds ||u_t||
    // the step size of the element set before the pre-adaptation, as the plain step takes it before
    // its refinement (02_hyperbolic_05_burgers_adapt.cpp:234-243)
    const double dt = adaptive_dt(g, cfl, wave_speed);
    if (g->ctx->adapt_mode == AMDG_ADAPT_DEVICE)
        return learned_step_device(op, mlp, dt, eps, eta, tau, prec, horizon, t_left, t_advanced, steps_out, stats);
    if ((s = grid_ensure_host(g)) != AMDG_OK) return s;
    std::vector<double> norms;
    if ((s = grid_norms(g, g->d_u, &norms, d_ut)) != AMDG_OK) return s;  // synchronises the stream
    // 2. pre-adapt: leaves the network marks "refine" (class 0) get children;
    //    where it is unsure (max probability < tau) the surplus criterion on
    //    the current coefficients decides instead; leaves the criterion found
    //    above eps after the previous step (missed refinements) are refined too
    std::vector<uint8_t> force(E, 0);
    int64_t n_net = 0, n_unsure = 0;
    {
        PhaseTimer th(g->ctx, AMDG_PHASE_ADAPT_HOST);
        for (int64_t e = 0; e < E; ++e) {
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
        for (uint64_t k : op->missed_keys) {
            auto it = std::lower_bound(g->host.key.begin(), g->host.key.end(), k);
            if (it != g->host.key.end() && *it == k) force[it - g->host.key.begin()] = 1;
        }
        std::vector<uint64_t> keys = refine_keys(g->host, norms.data(), eps, nullptr, force.data());
        if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
    }
    // 3. the horizon's time steps on this grid, no predictor
    int n = 0;
    double advanced = 0.0;
    if ((s = horizon_steps(op, dt, prec, horizon, t_left, &advanced, &n)) != AMDG_OK) return s;
    // 4. coarsening (amdg_grid_coarsen), then the surplus criterion judges the
    //    result: leaves still above eps are missed refinements, refined at the
    //    start of the next step
    if ((s = grid_norms(g, g->d_u, &norms, op->kind == 1 ? g->d_v : nullptr)) != AMDG_OK) return s;
    std::vector<std::pair<uint64_t, double>> above;
    {
        PhaseTimer th(g->ctx, AMDG_PHASE_ADAPT_HOST);
        for (int64_t e = 0; e < g->host.num_elements; ++e)
            if (norms[e] > eps) above.emplace_back(g->host.key[e], norms[e]);
        std::vector<uint64_t> keys = coarsen_keys(g->host, norms.data(), eta);
        if (int64_t(keys.size()) != g->host.num_elements && (s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
        std::vector<uint8_t> leaf;
        leaf_flags(g->host, &leaf);
        op->missed_keys.clear();
        for (const auto& kv : above) {
            auto it = std::lower_bound(g->host.key.begin(), g->host.key.end(), kv.first);
            if (it != g->host.key.end() && *it == kv.first && leaf[it - g->host.key.begin()]) op->missed_keys.push_back(kv.first);
        }
    }
    if (t_advanced) *t_advanced = advanced;
    if (steps_out) *steps_out = n;
    if (stats) {
        stats[0] = n_net;
        stats[1] = n_unsure;
        stats[2] = int64_t(op->missed_keys.size());
        stats[3] = g->host.num_elements;
    }
    return AMDG_OK;
}

amdg_status amdg_burgers_adaptive_step_learned(amdg_burgers_op* op, amdg_mlp* mlp, double cfl, double wave_speed,
                                               double eps, double eta, double tau, amdg_precision prec, double* dt_out,
                                               int64_t* stats) {
    return learned_step_any(op, mlp, cfl, wave_speed, eps, eta, tau, prec, 1, 0.0, dt_out, nullptr, stats);
}

amdg_status amdg_burgers_adaptive_steps_learned(amdg_burgers_op* op, amdg_mlp* mlp, double cfl, double wave_speed,
                                                double eps, double eta, double tau, amdg_precision prec, int horizon,
                                                double t_left, double* t_advanced, int* steps, int64_t* stats) {
    return learned_step_any(op, mlp, cfl, wave_speed, eps, eta, tau, prec, horizon, t_left, t_advanced, steps, stats);
}

amdg_status amdg_burgers_counters(const amdg_burgers_op* op, int64_t* stage_dof_updates, int64_t* rhs_evaluations) {
    AMDG_REQUIRE(op, AMDG_ERR_ARG, "null operator");
    if (stage_dof_updates) *stage_dof_updates = op->stage_dof_updates;
    if (rhs_evaluations) *rhs_evaluations = op->rhs_evaluations;
    return AMDG_OK;
}

// ---- wave equation u_tt = div(K grad u) (03_wave_06_var_coeff_adapt.cpp) -----------------

amdg_status amdg_wave_create(amdg_grid* g, double sigma, double amplitude, amdg_wave_op** out) {
    AMDG_REQUIRE(g && out && std::isfinite(sigma) && sigma >= 0 && std::isfinite(amplitude), AMDG_ERR_ARG,
                 "bad arguments");
    *out = nullptr;
    amdg_wave_op* w = new (std::nothrow) amdg_wave_op;
    AMDG_REQUIRE(w, AMDG_ERR_NOMEM, "host allocation failed");
    amdg_status s = lagr_create(g, 1, nullptr, sigma, &w->lagr);
    if (s == AMDG_OK) w->lagr->amp = amplitude;
    if (s != AMDG_OK) {
        delete w;
        return s;
    }
    *out = w;
    return AMDG_OK;
}

amdg_status amdg_wave_destroy(amdg_wave_op* w) {
    if (!w) return AMDG_OK;
    amdg_burgers_destroy(w->lagr);
    delete w;
    return AMDG_OK;
}

amdg_status amdg_wave_set_sigma(amdg_wave_op* w, double sigma) {
    AMDG_REQUIRE(w && std::isfinite(sigma), AMDG_ERR_ARG, "bad arguments");
    amdg_burgers_op* op = w->lagr;
    if (op->sigma == sigma) return AMDG_OK;
    AMDG_CK(cudaSetDevice(op->device));
    op->sigma = sigma;
    op->graph_version = -1;
    if (op->built_version != op->grid->version) return AMDG_OK;  // the next sync sets the coefficient
    const double c = wave_penalty_coef(op);
    for (PartialSum& p : op->terms)
        if (p.kind == 1) p.coef = c;
    return refresh_nodes(op, stream_of(op));
}

amdg_status amdg_wave_interpolate(amdg_wave_op* w, int which, amdg_precision prec) {
    AMDG_REQUIRE(w && (which == AMDG_WAVE_INTERP_GRADU || which == AMDG_WAVE_INTERP_U), AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    amdg_burgers_op* op = w->lagr;
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    const int dim = g->host.dim;
    const int f0 = which == AMDG_WAVE_INTERP_GRADU ? 0 : dim, f1 = which == AMDG_WAVE_INTERP_GRADU ? dim - 1 : dim;
    cudaStream_t st = stream_of(op);
    amdg_status r;
    if (prec == AMDG_PREC_FP64) {
        double* fc[kMaxTermSources];
        wave_field_coefs(op, fc);
        r = eval_wave_fields<double>(op, g->d_u, fc, st, f0, f1);
    } else {
        float* fc[kMaxTermSources];
        wave_field_coefs(op, fc);
        r = eval_wave_fields<float>(op, g->d_u, fc, st, f0, f1);
    }
    if (r != AMDG_OK) return r;
    op->wave_interp_version[which] = g->version;
    op->wave_interp_prec[which] = int(prec);
    return AMDG_OK;
}

amdg_status amdg_wave_rhs_add(amdg_wave_op* w, int group, amdg_precision prec) {
    AMDG_REQUIRE(w && group >= AMDG_WAVE_RHS_FLX_GRADU && group <= AMDG_WAVE_RHS_IPDG, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    amdg_burgers_op* op = w->lagr;
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    amdg_grid* g = op->grid;
    const int dim = g->host.dim;
    if (group != AMDG_WAVE_RHS_IPDG) {
        const int need = group == AMDG_WAVE_RHS_FLX_U ? AMDG_WAVE_INTERP_U : AMDG_WAVE_INTERP_GRADU;
        AMDG_REQUIRE(op->wave_interp_version[need] == g->version && op->wave_interp_prec[need] == int(prec),
                     AMDG_ERR_STATE, "no interpolation of this element set and precision: call amdg_wave_interpolate first");
    }
    // the terms in build_terms order: point values ((dim + 1) fields x G), then per group dim x G
    // right-hand-side terms, then the dim IPDG terms
    const int G = int(op->sched_dims.size());
    const int first = group == AMDG_WAVE_RHS_IPDG ? int(op->terms.size()) - dim : op->n_pv_terms + group * dim * G;
    const int count = group == AMDG_WAVE_RHS_IPDG ? dim : dim * G;
    double* rhs = nullptr;
    if (amdg_status s = grid_rhs(g, &rhs); s != AMDG_OK) return s;
    cudaStream_t st = stream_of(op);
    if (prec == AMDG_PREC_FP64) {
        double* fc[kMaxTermSources];
        wave_field_coefs(op, fc);
        const double* src[kMaxTermSources];
        for (int f = 0; f <= dim; ++f) src[f] = fc[f];
        return eval_term_range<double>(op, mats64(op), first, count, src, dim + 1, g->d_u, rhs, StageOut{}, st, true);
    }
    float* fc[kMaxTermSources];
    wave_field_coefs(op, fc);
    const float* src[kMaxTermSources];
    for (int f = 0; f <= dim; ++f) src[f] = fc[f];
    float* u32 = static_cast<float*>(op->w_u);
    if (group == AMDG_WAVE_RHS_IPDG) {
        AMDG_CK(launch_convert<double, float>(g->d_u, u32, g->dof, st));
        g->ctx->launches++;
    }
    return eval_term_range<float>(op, mats32(op), first, count, src, dim + 1, u32, rhs, StageOut{}, st, true);
}

amdg_status amdg_ode_add_wave_penalty(amdg_ode* o, amdg_wave_op* w) {
    AMDG_REQUIRE(o && w && o->grid == w->lagr->grid, AMDG_ERR_ARG, "the integrator and the operator must share the grid");
    AMDG_REQUIRE(o->grid->version == o->version, AMDG_ERR_STATE, "the element set changed since the integrator was created");
    amdg_burgers_op* op = w->lagr;
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    const int dim = op->grid->host.dim;
    const double* src[1] = {op->grid->d_u};
    return eval_term_range<double>(op, mats64(op), int(op->terms.size()) - dim, dim, src, 1, op->grid->d_u, o->d_rhs,
                                   StageOut{}, stream_of(op), true);
}

amdg_status amdg_wave_set_sweep_variant(amdg_wave_op* w, int variant) {
    AMDG_REQUIRE(w, AMDG_ERR_ARG, "null argument");
    return amdg_burgers_set_sweep_variant(w->lagr, variant);
}

amdg_status amdg_wave_rhs(amdg_wave_op* w, const double* d_u, double* d_rhs, amdg_precision prec) {
    AMDG_REQUIRE(w && d_u && d_rhs && d_u != d_rhs, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    amdg_burgers_op* op = w->lagr;
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    op->rhs_evaluations++;
    return eval_rhs(op, d_u, d_rhs, prec);
}

// nsteps RK4ODE2nd steps of (u, v) (RK4ODE2nd::step_stage, ODESolver.cpp:579-615), the
// right-hand side re-evaluated at every stage
static amdg_status wave_rk4(amdg_burgers_op* op, double dt, int nsteps, amdg_precision prec) {
    amdg_grid* g = op->grid;
    cudaStream_t st = stream_of(op);
    if (amdg_status s = burgers_sync(op); s != AMDG_OK) return s;  // buffers sized for the current grid
    PhaseTimer timer(g->ctx, AMDG_PHASE_RK3);
    if (amdg_status s = grid_ensure_velocity(g); s != AMDG_OK) return s;
    const size_t bytes = size_t(g->dof) * sizeof(double);
    for (int step = 0; step < nsteps; ++step) {
        AMDG_CK(cudaMemcpyAsync(op->d_u1, g->d_u, bytes, cudaMemcpyDeviceToDevice, st));
        AMDG_CK(cudaMemcpyAsync(op->d_v1, g->d_v, bytes, cudaMemcpyDeviceToDevice, st));
        for (int stage = 0; stage < 4; ++stage) {
            if (amdg_status r = eval_rhs(op, op->d_u1, op->d_rhs64, prec); r != AMDG_OK) return r;
            AMDG_CK(launch_rk4_2nd_stage(stage, dt, op->d_rhs64, g->d_u, g->d_v, op->d_u1, op->d_v1, op->d_su, op->d_sv,
                                         g->dof, st));
            g->ctx->launches++;
        }
        op->rhs_evaluations += 4;
        op->stage_dof_updates += 4 * g->dof;
    }
    return AMDG_OK;
}

amdg_status amdg_wave_rk4_steps(amdg_wave_op* w, double dt, int nsteps, amdg_precision prec) {
    AMDG_REQUIRE(w && nsteps >= 0 && std::isfinite(dt), AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(prec == AMDG_PREC_FP64 || prec == AMDG_PREC_MIXED, AMDG_ERR_ARG, "bad precision");
    amdg_burgers_op* op = w->lagr;
    AMDG_CK(cudaSetDevice(op->device));
    if (amdg_status rs = burgers_sync(op); rs != AMDG_OK) return rs;
    return wave_rk4(op, dt, nsteps, prec);
}

amdg_status amdg_wave_adaptive_step(amdg_wave_op* w, double cfl, double wave_speed, double eps, double eta,
                                    amdg_precision prec, double* dt_out) {
    AMDG_REQUIRE(w, AMDG_ERR_ARG, "null operator");
    return adaptive_step_any(w->lagr, cfl, wave_speed, eps, eta, prec, dt_out, nullptr);
}

amdg_status amdg_wave_adaptive_step_ex(amdg_wave_op* w, double cfl, double wave_speed, double eps, double eta,
                                       amdg_precision prec, double* dt_out, int8_t* decisions) {
    AMDG_REQUIRE(w, AMDG_ERR_ARG, "null operator");
    return adaptive_step_any(w->lagr, cfl, wave_speed, eps, eta, prec, dt_out, decisions);
}

amdg_status amdg_wave_features(amdg_wave_op* w, const double* d_u, float* d_features) {
    AMDG_REQUIRE(w, AMDG_ERR_ARG, "null operator");
    return amdg_burgers_features(w->lagr, d_u, d_features);
}

amdg_status amdg_wave_adaptive_step_learned(amdg_wave_op* w, amdg_mlp* mlp, double cfl, double wave_speed, double eps,
                                            double eta, double tau, amdg_precision prec, double* dt_out, int64_t* stats) {
    AMDG_REQUIRE(w, AMDG_ERR_ARG, "null operator");
    return learned_step_any(w->lagr, mlp, cfl, wave_speed, eps, eta, tau, prec, 1, 0.0, dt_out, nullptr, stats);
}

amdg_status amdg_wave_adaptive_steps_learned(amdg_wave_op* w, amdg_mlp* mlp, double cfl, double wave_speed,
                                             double eps, double eta, double tau, amdg_precision prec, int horizon,
                                             double t_left, double* t_advanced, int* steps, int64_t* stats) {
    AMDG_REQUIRE(w, AMDG_ERR_ARG, "null operator");
    return learned_step_any(w->lagr, mlp, cfl, wave_speed, eps, eta, tau, prec, horizon, t_left, t_advanced, steps,
                            stats);
}

amdg_status amdg_wave_counters(const amdg_wave_op* w, int64_t* stage_dof_updates, int64_t* rhs_evaluations) {
    AMDG_REQUIRE(w, AMDG_ERR_ARG, "null operator");
    return amdg_burgers_counters(w->lagr, stage_dof_updates, rhs_evaluations);
}

// The adaptive interpolation of f (DGAdaptIntp::init_adaptive_intp): point values from f on the
// host, surpluses on the device, the indicator and refinement on the host, until the element set
// stops changing; then the Alpert coefficients from the last surpluses by the mass term.
static amdg_status init_adaptive_intp(amdg_burgers_op* op, amdg_fn_points f, void* user, double eps, int* rounds_out) {
    amdg_grid* g = op->grid;
    const int dim = g->host.dim, P1 = op->p1, P = op->points;
    const LagrSpec& S = *lagr_spec(P1 - 1);
    const int n1 = 1 << g->host.nmax;
    std::vector<double> x1(size_t(n1) * P1), m1;
    for (int o = 0; o < n1; ++o)
        for (int p = 0; p < P1; ++p) x1[size_t(o) * P1 + p] = lagr_point(S, o, p);
    lagr_mass_diag(S, g->host.nmax, &m1);
    int stride[kMaxDim];
    for (int d = 0; d < dim; ++d) stride[d] = ipow(P1, dim - 1 - d);
    cudaStream_t st = stream_of(op);
    std::vector<double> x, vals, coe, norms;
    int rounds = 0;
    amdg_status s;
    for (;;) {
        if ((s = burgers_sync(op)) != AMDG_OK) return s;
        const int64_t E = g->host.num_elements, n = E * P;
        x.resize(size_t(n) * dim);
        vals.assign(n, 0.0);
        for (int64_t e = 0; e < E; ++e) {
            const int32_t* oe = &g->host.order[size_t(e) * dim];
            for (int q = 0; q < P; ++q)
                for (int d = 0; d < dim; ++d)
                    x[(size_t(e) * P + q) * dim + d] = x1[size_t(oe[d]) * P1 + (q / stride[d]) % P1];
        }
        f(x.data(), n, dim, vals.data(), user);
        for (double v : vals) AMDG_REQUIRE(std::isfinite(v), AMDG_ERR_NONFINITE, "the function is not finite at a point");
        double* d_up = static_cast<double*>(op->w_up);
        double* d_coe = static_cast<double*>(op->w_fu);
        AMDG_CK(cudaMemcpyAsync(d_up, vals.data(), size_t(n) * sizeof(double), cudaMemcpyHostToDevice, st));
        if ((s = eval_surplus<double, double>(op, d_up, d_coe, st)) != AMDG_OK) return s;
        coe.resize(n);
        AMDG_CK(cudaMemcpyAsync(coe.data(), d_coe, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, st));
        AMDG_CK(cudaStreamSynchronize(st));
        // DGAdaptIntp::indicator_norm_intp_Lag: sum over the points of prod_d M_d * surplus^2
        norms.assign(E, 0.0);
        for (int64_t e = 0; e < E; ++e) {
            const int32_t* oe = &g->host.order[size_t(e) * dim];
            double sum = 0.0;
            for (int q = 0; q < P; ++q) {
                double w = 1.0;
                for (int d = 0; d < dim; ++d) w *= m1[size_t(oe[d]) * P1 + (q / stride[d]) % P1];
                const double c = coe[size_t(e) * P + q];
                sum += w * (c * c);
            }
            norms[e] = std::sqrt(sum);
        }
        std::vector<uint64_t> keys = refine_keys(g->host, norms.data(), eps);
        if (int64_t(keys.size()) == E) break;
        if ((s = grid_set_keys(g, std::move(keys))) != AMDG_OK) return s;
        ++rounds;
    }
    const double* src[1] = {static_cast<const double*>(op->w_fu)};
    if ((s = eval_term_range<double>(op, mats64(op), 0, int(op->terms.size()), src, 1, nullptr, g->d_u, StageOut{}, st)) !=
        AMDG_OK)
        return s;
    AMDG_CK(cudaStreamSynchronize(st));
    if (rounds_out) *rounds_out = rounds;
    return AMDG_OK;
}

amdg_status amdg_grid_init_adaptive_intp(amdg_grid* g, int lagr_degree, amdg_fn_points f, void* user, double eps,
                                         int* rounds) {
    AMDG_REQUIRE(g && f && std::isfinite(eps) && eps >= 0.0, AMDG_ERR_ARG, "bad arguments");
    AMDG_REQUIRE(lagr_degree >= 3 && lagr_degree <= 5, AMDG_ERR_ARG, "Lagrange degree must be 3, 4 or 5");
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    amdg_burgers_op* op = nullptr;
    amdg_status s = lagr_create(g, 2, nullptr, 0.0, &op, lagr_degree);
    if (s != AMDG_OK) return s;
    s = init_adaptive_intp(op, f, user, eps, rounds);
    amdg_burgers_destroy(op);
    return s;
}

}  // extern "C"
