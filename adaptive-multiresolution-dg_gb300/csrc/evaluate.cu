// Point values of the DG solution on tensor meshes and quadrature errors
// against the exact Burgers solution.
//
// DGSolution::val (DGSolution.cpp:613-625) sums, over every element whose
// closed support contains x, the coefficient times the product of 1D Alpert
// values (Element::val, Element.cpp:123-147).  Here the element of each level
// vector that contains x is found by its packed key in an open-addressing
// hash of the element table; the 1D basis values at the mesh coordinates are
// tabulated once on the host per (coordinate, level), with two candidate
// elements where a coordinate sits on a cell boundary.
//
// The error follows DGSolution::get_error_no_separable_scalar
// (DGSolution.cpp:326-335) with Quad::norm_multiD (Quad.cpp:261-318):
// `gauss` Gauss-Legendre points per dimension in every cell of the uniform
// mesh of the finest element level, L1 / L2 / Linf of |u_h - u|, with
// u = a + b v(sum_d x_d - a T + c, b T), T = dim t, v the 1D solution of
// v_t + (v^2/2)_x = 0, v(x,0) = sin(2 pi x) (BurgersExact::exact_1d / norm_1d,
// ExactSolution.cpp:8-71), found by Newton's method from the characteristic
// start value.  One thread per quadrature point, fixed-order block sums.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <set>
#include <string>
#include <vector>

#include "amdg.h"
#include "amdg_internal.hpp"
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

constexpr uint64_t kHashMul = 0x9E3779B97F4A7C15ull;
constexpr int kEvalThreads = 256;
constexpr int kMaxPointsLog2 = 31;  // at most 2^31 mesh points per call

struct EvalArgs {
    int dim, np, B, nmax1, nl, log2cap;
    int64_t n1, total;
    const int32_t* lvec;      // [nl][dim] level vectors present in the grid
    const int8_t* cnt;        // [n1][nmax+1] candidate elements (0, 1, 2) per coordinate and level
    const int32_t* ord;       // [n1][nmax+1][2] their 1D orders
    const double* val;        // [n1][nmax+1][2][np] 1D basis values
    const uint64_t* hkey;     // [cap]
    const int32_t* hval;      // [cap] element index, -1 empty
    const double* u;          // [E][B]
    int nmax;
    // error mode
    const double* x1d;        // [n1]
    const double* w1d;        // [n1] Gauss weights (reference interval)
    double a, b, c, t;
};

__device__ __forceinline__ int64_t hash_find(const EvalArgs& A, uint64_t key) {
    const uint64_t mask = (uint64_t(1) << A.log2cap) - 1;
    uint64_t h = (key * kHashMul) >> (64 - A.log2cap);
    for (uint64_t it = 0; it <= mask; ++it) {
        const int32_t v = __ldg(A.hval + h);
        if (v < 0) return -1;
        if (__ldg(A.hkey + h) == key) return v;
        h = (h + 1) & mask;
    }
    return -1;
}

__device__ double eval_point(const EvalArgs& A, const int64_t* i1) {
    double acc = 0.0;
    for (int lv = 0; lv < A.nl; ++lv) {
        int cnt[kMaxDim], row[kMaxDim];
        int combos = 1;
        for (int d = 0; d < A.dim; ++d) {
            const int l = __ldg(A.lvec + lv * A.dim + d);
            row[d] = int(i1[d] * A.nmax1 + l);
            cnt[d] = __ldg(A.cnt + row[d]);
            combos *= cnt[d];
        }
        for (int cmb = 0; cmb < combos; ++cmb) {
            int sel[kMaxDim];
            int r = cmb;
            uint64_t key = 0;
            for (int d = 0; d < A.dim; ++d) {
                sel[d] = cnt[d] == 2 ? (r & 1) : 0;
                r >>= cnt[d] == 2 ? 1 : 0;
                const uint64_t o = uint64_t(__ldg(A.ord + row[d] * 2 + sel[d]));
                key |= o << (uint64_t(A.nmax) * (A.dim - 1 - d));
            }
            const int64_t e = hash_find(A, key);
            if (e < 0) continue;
            double ve = 0.0;
            for (int idx = 0; idx < A.B; ++idx) {
                int pd[kMaxDim];
                int q = idx;
                for (int d = A.dim - 1; d >= 0; --d) { pd[d] = q % A.np; q /= A.np; }
                double v = __ldg(A.u + e * A.B + idx);
                for (int d = 0; d < A.dim; ++d) v *= __ldg(A.val + (size_t(row[d]) * 2 + sel[d]) * A.np + pd[d]);
                ve += v;
            }
            acc += ve;
        }
    }
    return acc;
}

__device__ __forceinline__ void point_index(const EvalArgs& A, int64_t gid, int64_t* i1) {
    int64_t r = gid;
    for (int d = A.dim - 1; d >= 0; --d) { i1[d] = r % A.n1; r /= A.n1; }
}

__global__ void __launch_bounds__(kEvalThreads) eval_tensor_kernel(EvalArgs A, double* __restrict__ out) {
    for (int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; gid < A.total; gid += int64_t(gridDim.x) * blockDim.x) {
        int64_t i1[kMaxDim];
        point_index(A, gid, i1);
        out[gid] = eval_point(A, i1);
    }
}

// v(x, t): v = sin(2 pi (x - v t)), odd about x = 1/2; NaN when Newton's method
// has not converged after 10 steps
__device__ double burgers_wave(double x, double t) {
    const double pi = 3.14159265358979323846;
    double xp = fmod(x, 1.0);
    if (xp < 0) xp = fmod(xp + 1.0, 1.0);
    if (fabs(xp) < kRoundOff || fabs(1 - xp) < kRoundOff || fabs(xp - 0.5) < kRoundOff) return 0.0;
    double sgn = 1.0;
    if (xp < 0.5) {
        sgn = -1.0;
        xp = fmod(1 - xp, 1.0);
    }
    // start value: the first characteristic x0 + sin(2 pi x0) t, x0 from 1 down to 1/2, left of xp
    const double h = 0.5 / 100;
    double v = 0.0;
    for (int i = 0; i < 100; ++i) {
        const double x0 = 1.0 - i * h;
        if (xp > x0 + sin(2 * pi * x0) * t) {
            v = sin(2 * pi * x0);
            break;
        }
    }
    double err = 1.0;
    int iter = 0;
    while (err > kRoundOff) {
        const double vn = v - (v + sin(2 * pi * (v * t - xp))) / (1 + 2 * pi * t * cos(2 * pi * (v * t - xp)));
        err = fabs(vn - v);
        v = vn;
        if (++iter > 10) return nan("");
    }
    return sgn * v;
}

// per block: sum w |e|, sum w e^2, max |e|, Newton failures
__global__ void __launch_bounds__(kEvalThreads) error_burgers_kernel(EvalArgs A, double* __restrict__ part) {
    __shared__ double s1[kEvalThreads], s2[kEvalThreads], sm[kEvalThreads], sf[kEvalThreads];
    double l1 = 0.0, l2 = 0.0, mx = 0.0, fails = 0.0;
    for (int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; gid < A.total; gid += int64_t(gridDim.x) * blockDim.x) {
        int64_t i1[kMaxDim];
        point_index(A, gid, i1);
        const double uh = eval_point(A, i1);
        double s = 0.0, w = 1.0;
        for (int d = 0; d < A.dim; ++d) {
            s += __ldg(A.x1d + i1[d]);
            w *= __ldg(A.w1d + i1[d]);
        }
        const double T = A.dim * A.t;
        const double v = burgers_wave(s - A.a * T + A.c, A.b * T);
        if (isnan(v)) {
            fails += 1.0;
            continue;
        }
        const double f = fabs(uh - (A.a + A.b * v));
        l1 += w * f;
        l2 += w * f * f;
        mx = fmax(mx, f);
    }
    const int tid = threadIdx.x;
    s1[tid] = l1; s2[tid] = l2; sm[tid] = mx; sf[tid] = fails;
    __syncthreads();
    for (int off = kEvalThreads / 2; off > 0; off >>= 1) {
        if (tid < off) {
            s1[tid] += s1[tid + off];
            s2[tid] += s2[tid + off];
            sm[tid] = fmax(sm[tid], sm[tid + off]);
            sf[tid] += sf[tid + off];
        }
        __syncthreads();
    }
    if (tid == 0) {
        part[blockIdx.x * 4 + 0] = s1[0];
        part[blockIdx.x * 4 + 1] = s2[0];
        part[blockIdx.x * 4 + 2] = sm[0];
        part[blockIdx.x * 4 + 3] = sf[0];
    }
}

// device copies of the per-call tables; freed on destruction
struct EvalTables {
    std::vector<void*> bufs;
    ~EvalTables() {
        for (void* p : bufs) cudaFree(p);
    }
    // an uninitialised device array of n elements
    template <class T>
    amdg_status alloc(size_t n, T** out) {
        void* p = nullptr;
        cudaError_t e = amdg::device_malloc(&p, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        bufs.push_back(p);
        *out = static_cast<T*>(p);
        return AMDG_OK;
    }
    template <class T>
    amdg_status put(const std::vector<T>& h, const T** out) {
        void* p = nullptr;
        const size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
        cudaError_t e = amdg::device_malloc(&p, bytes);
        if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        bufs.push_back(p);
        if (!h.empty()) {
            e = cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
        }
        *out = static_cast<const T*>(p);
        return AMDG_OK;
    }
};

// element hash, level vectors and 1D tables for the coordinates x1d
amdg_status prepare(const amdg_grid* g, const std::vector<double>& x1d, EvalTables* T, EvalArgs* A) {
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    const HostGrid& h = g->host;
    const int dim = h.dim, np = h.k + 1, nmax = h.nmax;
    const int64_t E = h.num_elements;
    A->dim = dim;
    A->np = np;
    A->B = g->block;
    A->nmax = nmax;
    A->nmax1 = nmax + 1;
    A->n1 = int64_t(x1d.size());
    A->u = g->d_u;
    // open-addressing hash of the packed keys, load factor <= 1/2
    int log2cap = 4;
    while ((int64_t(1) << log2cap) < 2 * E) ++log2cap;
    const uint64_t cap = uint64_t(1) << log2cap, mask = cap - 1;
    std::vector<uint64_t> hkey(cap, 0);
    std::vector<int32_t> hval(cap, -1);
    for (int64_t e = 0; e < E; ++e) {
        uint64_t s = (h.key[e] * kHashMul) >> (64 - log2cap);
        while (hval[s] >= 0) s = (s + 1) & mask;
        hkey[s] = h.key[e];
        hval[s] = int32_t(e);
    }
    A->log2cap = log2cap;
    // distinct level vectors
    std::set<std::vector<int32_t>> lv;
    for (int64_t e = 0; e < E; ++e) {
        std::vector<int32_t> v(dim);
        for (int d = 0; d < dim; ++d) v[d] = level_of_order(h.order[size_t(e) * dim + d]);
        lv.insert(v);
    }
    std::vector<int32_t> lvec;
    for (const auto& v : lv) lvec.insert(lvec.end(), v.begin(), v.end());
    A->nl = int(lv.size());
    // 1D tables: for each coordinate and level the elements whose closed support holds it
    Basis1D b{h.k, nmax};
    const int64_t n1 = A->n1;
    std::vector<int8_t> cnt(size_t(n1) * (nmax + 1), 0);
    std::vector<int32_t> ord(size_t(n1) * (nmax + 1) * 2, 0);
    std::vector<double> val(size_t(n1) * (nmax + 1) * 2 * np, 0.0);
    for (int64_t i = 0; i < n1; ++i) {
        const double x = x1d[i];
        if (!(x >= 0.0 && x <= 1.0)) continue;
        for (int n = 0; n <= nmax; ++n) {
            const size_t row = size_t(i) * (nmax + 1) + n;
            int cand[2], nc = 0;
            if (n <= 1) {
                cand[nc++] = n;  // orders 0 and 1 cover [0, 1]
            } else {
                const int64_t cells = int64_t(1) << (n - 1);
                const double w = std::ldexp(1.0, 1 - n);
                int64_t c = int64_t(std::floor(x / w));
                if (c < cells) cand[nc++] = int(cells + c);
                if (c >= 1 && c - 1 < cells && x <= double(c) * w) cand[nc++] = int(cells + c - 1);
            }
            cnt[row] = int8_t(nc);
            for (int q = 0; q < nc; ++q) {
                ord[row * 2 + q] = cand[q];
                for (int p = 0; p < np; ++p) val[(row * 2 + q) * np + p] = b.eval(cand[q] * np + p, 0, x, 0);
            }
        }
    }
    amdg_status s;
    if ((s = T->put(hkey, &A->hkey)) != AMDG_OK || (s = T->put(hval, &A->hval)) != AMDG_OK ||
        (s = T->put(lvec, &A->lvec)) != AMDG_OK || (s = T->put(cnt, &A->cnt)) != AMDG_OK ||
        (s = T->put(ord, &A->ord)) != AMDG_OK || (s = T->put(val, &A->val)) != AMDG_OK)
        return s;
    return AMDG_OK;
}

// out[i] = a_block(ia[i]) . b_block(ib[i]) (ia / ib NULL: the index i itself), one warp per pair
__global__ void __launch_bounds__(kEvalThreads) block_dot_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                               const int32_t* __restrict__ ia,
                                                               const int32_t* __restrict__ ib, int64_t n, int B,
                                                               double* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
    for (int64_t i = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const int64_t ea = ia ? ia[i] : i, eb = ib ? ib[i] : i;
        double s = 0.0;
        for (int q = lane; q < B; q += 32) s = fma(a[ea * B + q], b[eb * B + q], s);
        for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
        if (lane == 0) out[i] = s;
    }
}

unsigned eval_blocks(int64_t total) {
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (total + kEvalThreads - 1) / kEvalThreads;
    return unsigned(std::max<int64_t>(1, std::min<int64_t>(want, int64_t(sms) * 8)));
}

}  // namespace

extern "C" {

amdg_status amdg_grid_eval_tensor(const amdg_grid* g, int n1, const double* x1d, double* d_out) {
    AMDG_REQUIRE(g && x1d && d_out && n1 > 0, AMDG_ERR_ARG, "bad arguments");
    const int dim = g->host.dim;
    AMDG_REQUIRE(double(dim) * std::log2(double(n1)) <= kMaxPointsLog2, AMDG_ERR_CAPACITY,
                 "more than 2^31 mesh points in one call");
    for (int i = 0; i < n1; ++i) AMDG_REQUIRE(std::isfinite(x1d[i]), AMDG_ERR_ARG, "non-finite coordinate");
    AMDG_CK(cudaSetDevice(g->device));
    cudaStream_t st = static_cast<cudaStream_t>(g->ctx->stream);
    AMDG_CK(cudaStreamSynchronize(st));
    EvalTables T;
    EvalArgs A{};
    amdg_status s = prepare(g, std::vector<double>(x1d, x1d + n1), &T, &A);
    if (s != AMDG_OK) return s;
    A.total = 1;
    for (int d = 0; d < dim; ++d) A.total *= n1;
    eval_tensor_kernel<<<eval_blocks(A.total), kEvalThreads, 0, st>>>(A, d_out);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches++;
    AMDG_CK(cudaStreamSynchronize(st));  // the tables are freed on return
    return AMDG_OK;
}

amdg_status amdg_grid_error_burgers(const amdg_grid* g, double a, double b, double c, double t, int gauss_points,
                                    double* err) {
    AMDG_REQUIRE(g && err, AMDG_ERR_ARG, "null argument");
    AMDG_REQUIRE(gauss_points >= 1 && gauss_points <= 10, AMDG_ERR_ARG, "gauss_points must be in 1..10");
    AMDG_REQUIRE(std::isfinite(a) && std::isfinite(b) && std::isfinite(c) && std::isfinite(t) && t >= 0, AMDG_ERR_ARG,
                 "bad exact-solution parameters");
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    const HostGrid& h = g->host;
    int qlev = 0;
    for (int32_t o : h.order) qlev = std::max(qlev, level_of_order(o));
    const int64_t cells = int64_t(1) << qlev;
    const int64_t n1 = cells * gauss_points;
    AMDG_REQUIRE(double(h.dim) * std::log2(double(n1)) <= kMaxPointsLog2, AMDG_ERR_CAPACITY,
                 "more than 2^31 quadrature points");
    AMDG_CK(cudaSetDevice(g->device));
    cudaStream_t st = static_cast<cudaStream_t>(g->ctx->stream);
    AMDG_CK(cudaStreamSynchronize(st));
    std::vector<double> gx(gauss_points), gw(gauss_points);
    gauss_legendre(gauss_points, gx.data(), gw.data());
    const double hcell = 1.0 / double(cells);
    std::vector<double> x1d(n1), w1d(n1);
    for (int64_t ci = 0; ci < cells; ++ci)
        for (int q = 0; q < gauss_points; ++q) {
            const double tl = double(ci) * hcell, tr = double(ci + 1) * hcell;
            x1d[ci * gauss_points + q] = tl + (gx[q] + 1.0) * 0.5 * (tr - tl);
            w1d[ci * gauss_points + q] = gw[q];
        }
    EvalTables T;
    EvalArgs A{};
    amdg_status s = prepare(g, x1d, &T, &A);
    if (s != AMDG_OK) return s;
    if ((s = T.put(x1d, &A.x1d)) != AMDG_OK || (s = T.put(w1d, &A.w1d)) != AMDG_OK) return s;
    A.a = a; A.b = b; A.c = c; A.t = t;
    A.total = 1;
    for (int d = 0; d < h.dim; ++d) A.total *= n1;
    const unsigned nb = eval_blocks(A.total);
    std::vector<double> part(size_t(nb) * 4, 0.0);
    const double* d_part0 = nullptr;
    if ((s = T.put(part, &d_part0)) != AMDG_OK) return s;
    double* d_part = const_cast<double*>(d_part0);
    error_burgers_kernel<<<nb, kEvalThreads, 0, st>>>(A, d_part);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches++;
    AMDG_CK(cudaMemcpyAsync(part.data(), d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    double l1 = 0.0, l2 = 0.0, mx = 0.0, fails = 0.0;
    for (unsigned i = 0; i < nb; ++i) {
        l1 += part[i * 4 + 0];
        l2 += part[i * 4 + 1];
        mx = std::max(mx, part[i * 4 + 2]);
        fails += part[i * 4 + 3];
    }
    AMDG_REQUIRE(fails == 0.0, AMDG_ERR_NONFINITE,
                 "exact solution: Newton's method did not converge at " + std::to_string(int64_t(fails)) +
                     " points (past the shock time?)");
    const double scale = std::pow(hcell / 2.0, h.dim);
    err[0] = l1 * scale;
    err[1] = std::sqrt(l2 * scale);
    err[2] = mx;
    return AMDG_OK;
}

amdg_status amdg_grid_l2_error_split_grid(const amdg_grid* g, const amdg_grid* exact, double* out) {
    AMDG_REQUIRE(g && exact && out, AMDG_ERR_ARG, "null argument");
    if (amdg_status s = grid_ensure_host(g); s != AMDG_OK) return s;
    if (amdg_status s = grid_ensure_host(exact); s != AMDG_OK) return s;
    const HostGrid& h = g->host;
    const HostGrid& he = exact->host;
    AMDG_REQUIRE(h.dim == he.dim && h.nmax == he.nmax && h.k == he.k && g->device == exact->device, AMDG_ERR_ARG,
                 "the grids differ in dimension, finest level, degree or device");
    AMDG_CK(cudaSetDevice(g->device));
    cudaStream_t st = static_cast<cudaStream_t>(g->ctx->stream);
    if (exact->ctx != g->ctx) AMDG_CK(cudaStreamSynchronize(static_cast<cudaStream_t>(exact->ctx->stream)));
    // shared elements by a merge of the two ascending key lists
    std::vector<int32_t> ia, ib;
    for (int64_t i = 0, j = 0; i < h.num_elements && j < he.num_elements;) {
        if (h.key[i] < he.key[j]) ++i;
        else if (he.key[j] < h.key[i]) ++j;
        else {
            ia.push_back(int32_t(i++));
            ib.push_back(int32_t(j++));
        }
    }
    const int64_t E = h.num_elements, Ee = he.num_elements, n = int64_t(ia.size());
    EvalTables T;
    const int32_t *d_ia = nullptr, *d_ib = nullptr;
    double* d_dot = nullptr;  // every entry written by the block products below
    std::vector<double> dots(size_t(E + Ee + n));
    amdg_status s;
    if ((s = T.put(ia, &d_ia)) != AMDG_OK || (s = T.put(ib, &d_ib)) != AMDG_OK || (s = T.alloc(dots.size(), &d_dot)) != AMDG_OK)
        return s;
    const int B = g->block;
    if (Ee > 0) block_dot_kernel<<<eval_blocks(Ee * 32), kEvalThreads, 0, st>>>(exact->d_u, exact->d_u, nullptr, nullptr, Ee, B, d_dot);
    if (E > 0) block_dot_kernel<<<eval_blocks(E * 32), kEvalThreads, 0, st>>>(g->d_u, g->d_u, nullptr, nullptr, E, B, d_dot + Ee);
    if (n > 0) block_dot_kernel<<<eval_blocks(n * 32), kEvalThreads, 0, st>>>(g->d_u, exact->d_u, d_ia, d_ib, n, B, d_dot + Ee + E);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches += 3;
    AMDG_CK(cudaMemcpyAsync(dots.data(), d_dot, dots.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    // the reference's order: |u_exact|^2, then |u|^2, then the shared products
    double err2 = 0.0;
    for (int64_t i = 0; i < Ee + E; ++i) err2 += dots[i];
    for (int64_t i = 0; i < n; ++i) err2 -= 2.0 * dots[Ee + E + i];
    *out = err2 < 0.0 ? err2 : std::sqrt(err2);
    return AMDG_OK;
}

}  // extern "C"
