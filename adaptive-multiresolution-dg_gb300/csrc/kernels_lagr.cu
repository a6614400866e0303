// Device kernels of the Lagrange-interpolation path for nonlinear fluxes.
//
// A right-hand side is a sum of many independent terms, each a partial sum of
// dim 1D transforms (FastMultiplyLU::transform_1D, FastMultiplyLU.cpp:436-512):
// for every element e and every entry of its output block,
//   out[e][idx] = coef * sum_{s in N_t(e), L/U filter} sum_k in[s][idx, dim t <- k] * M[o_t(s)*n_from + k][o_t(e)*n_to + idx_t]
// where N_t(e) is the vol or flx neighbour list of e in dimension t.  Instead
// of one launch per transform, sweep j of every term of a range runs in one
// launch (thread per term, element and output entry) with each term in its own
// slice of the work buffer; the last sweep writes one slice per term and a
// reduction adds the slices in the reference's order (and, for an RK stage,
// applies the stage update), so a whole right-hand side is about a dozen
// launches.
//
// surplus_pass: pass d of the hierarchical surplus
// (LagrInterpolation::eval_fp_to_coe_D_Lag, Interplation.cpp:1222-1434).
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "kernels_lagr.cuh"

namespace amdg {

// ---- double-float arithmetic (float2 = hi + lo, |lo| <= ulp(hi)/2, about 48 bits) -------------
// The error-free transformations two-sum (Knuth) and the FMA-based exact product, combined as in
// the double-double algorithms of Hida, Li and Bailey ("accurate" addition): the point-value
// sweeps of the mixed mode run on the FP32 pipe with near-FP64 accuracy.
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 df_quick_two_sum(float a, float b) {
    const float s = a + b;
    return make_float2(s, b - (s - a));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    float2 s = df_two_sum(a.x, b.x);
    const float2 t = df_two_sum(a.y, b.y);
    s.y += t.x;
    s = df_quick_two_sum(s.x, s.y);
    s.y += t.y;
    return df_quick_two_sum(s.x, s.y);
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return df_quick_two_sum(p, e);
}

// the sweep's arithmetic for T = double, float or float2 (double-float)
__device__ __forceinline__ double madd(double x, double m, double acc) { return fma(x, m, acc); }
__device__ __forceinline__ float madd(float x, float m, float acc) { return fmaf(x, m, acc); }
__device__ __forceinline__ float2 madd(float2 x, float2 m, float2 acc) { return df_add(df_mul(x, m), acc); }
__device__ __forceinline__ double scale(double a, double c) { return a * c; }
__device__ __forceinline__ float scale(float a, float c) { return a * c; }
__device__ __forceinline__ float2 scale(float2 a, float2 c) { return df_mul(a, c); }
template <typename T>
__device__ __forceinline__ T from_double(double v) { return T(v); }
template <>
__device__ __forceinline__ float2 from_double<float2>(double v) {
    const float hi = float(v);
    return make_float2(hi, float(v - double(hi)));
}
__device__ __forceinline__ double to_double(double v) { return v; }
__device__ __forceinline__ double to_double(float v) { return double(v); }
__device__ __forceinline__ double to_double(float2 v) { return double(v.x) + double(v.y); }

// acc + sum over four neighbours j (in order) and k < NF of x[j][k*stride] * m[j][k*ncols],
// all operands loaded before the first multiply-add
template <int NF, typename T>
__device__ __forceinline__ T fibre_quad(const T* const* x, const T* const* m, int stride, int ncols, T acc) {
    T xv[4][NF], mv[4][NF];
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            xv[j][k] = __ldg(x[j] + k * stride);
            mv[j][k] = __ldg(m[j] + size_t(k) * ncols);
        }
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int k = 0; k < NF; ++k) acc = madd(xv[j][k], mv[j][k], acc);
    return acc;
}

// CTAs of 128 threads, at most 64 registers (eight CTAs per multiprocessor).  Measured on the
// 3D adaptive Burgers runs (~1,000 elements): without the register bound the FP64 and
// double-float forms took 80 / 74 registers, three CTAs of 256 fitted, and the FP64 run took 7 %
// longer; 256-thread CTAs under the same bound another 4 % (coarser tails); 64-thread CTAs gained
// nothing more.  A bound of 48 registers spills.
constexpr int kSweepThreads = 128;

// CTA size of the element-wise kernels: 256 threads, halved (down to 64) until the grid has two
// CTAs per multiprocessor -- on the ~1,000-element grids of the adaptive runs a 256-thread grid
// leaves multiprocessors idle
inline int ew_threads(int64_t n) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 152;
    }
    int t = 256;
    while (t > 64 && (n + t - 1) / t < 2 * int64_t(sms)) t /= 2;
    return t;
}
#define AMDG_EW_GRID(n) unsigned(((n) + ew_threads(n) - 1) / ew_threads(n)), ew_threads(n)

// NODE_ROWS: the node is blockIdx.y and the thread's (element, entry) its index in the node's
// E x out_block outputs (32-bit index arithmetic); else one 1D grid over all nodes' outputs
template <typename T, bool NODE_ROWS>
__global__ void __launch_bounds__(kSweepThreads, 1024 / kSweepThreads) sweep_kernel(SweepArgs<T> a) {
    const int64_t per = a.num_elements * a.out_block;
    int slot;
    int64_t r;
    if constexpr (NODE_ROWS) {
        slot = blockIdx.y;
        r = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        if (r >= per) return;
    } else {
        const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
        if (gid >= per * a.count) return;
        slot = int(gid / per);
        r = gid - int64_t(slot) * per;
    }
    const int e = int(r / a.out_block);
    const int idx = int(r - int64_t(e) * a.out_block);
    const PartialSum& D = a.desc[a.first + slot];
    if (D.kind == 1 && a.sweep + 1 < a.dim) return;  // a penalty term is a single (last) sweep
    int t, lu, flx, n_from, n_to, stride = 1, in_block = 1;
    const T* M;
    const T* in;
    T coef;
    if (D.kind == 0) {
        t = D.dims[a.sweep];
        lu = D.lu[a.sweep];
        flx = D.flx[a.sweep];
        M = a.mats[D.mat[a.sweep]];
        n_from = a.n_in;
        n_to = a.n_out;
        coef = from_double<T>(D.coef);
        in = a.sweep == 0 ? a.src[D.src] : a.in + int64_t(D.parent) * a.in_slice;
        // block shape: n_out along the dimensions already transformed, n_in elsewhere
        int done_after = 0;
        for (int j = 0; j < a.sweep; ++j) done_after += D.dims[j] > t ? 1 : 0;
        for (int d = 0; d < a.dim - 1 - t; ++d) stride *= d < done_after ? a.n_out : a.n_in;
        for (int d = 0; d < a.dim; ++d) in_block *= d < a.sweep ? a.n_out : a.n_in;
    } else {
        t = D.dims[0];
        lu = 1;
        flx = 1;
        M = a.mats[kMatAJump];
        n_from = n_to = a.np;
        coef = from_double<T>(D.coef);
        in = a.pen_in;
        for (int d = 0; d < a.dim - 1 - t; ++d) stride *= a.np;
        for (int d = 0; d < a.dim; ++d) in_block *= a.np;
    }
    const int inner = idx % stride;
    const int qt = (idx / stride) % n_to;
    const int outer = idx / (stride * n_to);
    const int64_t et = int64_t(e) * a.dim + t;
    const int32_t* ptr = flx ? a.flx_ptr : a.vol_ptr;
    const int32_t* split = flx ? a.flx_split : a.vol_split;
    const int2* nbr = flx ? a.flx_nbr : a.vol_nbr;
    const int oe = __ldg(a.order + et);
    // "L": neighbours finer than e in dimension t; "U": coarser or equal; neighbours are level-sorted
    const int beg = lu == 0 ? __ldg(split + et) : __ldg(ptr + et);
    const int end = lu == 2 ? __ldg(split + et) : __ldg(ptr + et + 1);
    // the 1D table is blocked by order pair: block (o_s, o_e) holds M[o_s n_from + k][o_e n_to + q]
    // at (k, q), n_from x n_to contiguous
    const int ncols = n_to;
    const T* mcol = M + size_t(oe) * (n_from * n_to) + qt;
    const int in_off = outer * n_from * stride + inner;
    const size_t mstep = size_t(a.n1) * (n_from * n_to);
    T acc = from_double<T>(0.0);
    // four neighbours per pass: their (element, order) pairs and operands are
    // independent loads issued together; the sum keeps the neighbour order
    int i = beg;
    for (; i + 4 <= end; i += 4) {
        int2 nb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) nb[j] = __ldg(nbr + i + j);
        const T* x[4];
        const T* m[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            x[j] = in + int64_t(nb[j].x) * in_block + in_off;
            m[j] = mcol + size_t(nb[j].y) * mstep;
        }
        if (n_from == 4) acc = fibre_quad<4>(x, m, stride, ncols, acc);
        else if (n_from == 3) acc = fibre_quad<3>(x, m, stride, ncols, acc);
        else if (n_from == 5) acc = fibre_quad<5>(x, m, stride, ncols, acc);
        else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                for (int k = 0; k < n_from; ++k) acc = madd(__ldg(x[j] + k * stride), __ldg(m[j] + size_t(k) * ncols), acc);
        }
    }
    for (; i < end; ++i) {
        const int2 nb = __ldg(nbr + i);
        const T* x = in + int64_t(nb.x) * in_block + in_off;
        const T* m = mcol + size_t(nb.y) * mstep;
        for (int k = 0; k < n_from; ++k) acc = madd(__ldg(x + k * stride), __ldg(m + size_t(k) * ncols), acc);
    }
    a.out[int64_t(slot) * per + r] = scale(acc, coef);
}

// Neighbours i and i + 1 of a column: every operand of both loaded, then i's multiply-adds (k
// ascending), then i + 1's -- the order of sweep_kernel.
template <typename T, int NF, int NTO>
__device__ __forceinline__ void col_pair(const T* x0, const T* m0, const T* x1, const T* m1, int stride, int ncols,
                                         T* acc) {
    T xa[NF], xb[NF], ma[NF][NTO], mb[NF][NTO];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        xa[k] = __ldg(x0 + k * stride);
        xb[k] = __ldg(x1 + k * stride);
#pragma unroll
        for (int q = 0; q < NTO; ++q) {
            ma[k][q] = __ldg(m0 + size_t(k) * ncols + q);
            mb[k][q] = __ldg(m1 + size_t(k) * ncols + q);
        }
    }
#pragma unroll
    for (int k = 0; k < NF; ++k)
#pragma unroll
        for (int q = 0; q < NTO; ++q) acc[q] = madd(xa[k], ma[k][q], acc[q]);
#pragma unroll
    for (int k = 0; k < NF; ++k)
#pragma unroll
        for (int q = 0; q < NTO; ++q) acc[q] = madd(xb[k], mb[k][q], acc[q]);
}

// The same sweep with one thread per (node, element, column): a column is one line of the output
// block along the transformed dimension (its NTO entries), so every input value the thread loads
// serves all NTO outputs, and the threads of an element walk the same neighbour list (broadcast
// loads of the pairs and of the 1D matrix rows).  Kind-0 nodes transform NF values per column,
// two neighbours per pass; kind-1 nodes (the penalty, np values) take a plain loop.  Each output is
// summed in the order of sweep_kernel (neighbours in list order, k ascending): identical results.
template <typename T, int NF, int NTO>
__global__ void __launch_bounds__(256) sweep_col_kernel(SweepArgs<T> a) {
    const int cols = a.out_block / NTO;
    const int64_t per = a.num_elements * cols;
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= per * a.count) return;
    const int slot = int(gid / per);
    const int64_t r = gid - int64_t(slot) * per;
    const int64_t e = r / cols;
    const int c = int(r - e * cols);
    const PartialSum& D = a.desc[a.first + slot];
    if (D.kind == 1 && a.sweep + 1 < a.dim) return;  // a penalty term is a single (last) sweep
    int t, lu, flx, n_from, stride = 1, in_block = 1;
    const T* M;
    const T* in;
    if (D.kind == 0) {
        t = D.dims[a.sweep];
        lu = D.lu[a.sweep];
        flx = D.flx[a.sweep];
        M = a.mats[D.mat[a.sweep]];
        n_from = NF;
        in = a.sweep == 0 ? a.src[D.src] : a.in + int64_t(D.parent) * a.in_slice;
        int done_after = 0;
        for (int j = 0; j < a.sweep; ++j) done_after += D.dims[j] > t ? 1 : 0;
        for (int d = 0; d < a.dim - 1 - t; ++d) stride *= d < done_after ? a.n_out : a.n_in;
        for (int d = 0; d < a.dim; ++d) in_block *= d < a.sweep ? a.n_out : a.n_in;
    } else {
        t = D.dims[0];
        lu = 1;
        flx = 1;
        M = a.mats[kMatAJump];
        n_from = a.np;
        in = a.pen_in;
        for (int d = 0; d < a.dim - 1 - t; ++d) stride *= a.np;
        for (int d = 0; d < a.dim; ++d) in_block *= a.np;
    }
    const T coef = from_double<T>(D.coef);
    const int inner = c % stride;
    const int outer = c / stride;
    const int64_t et = e * a.dim + t;
    const int32_t* ptr = flx ? a.flx_ptr : a.vol_ptr;
    const int32_t* split = flx ? a.flx_split : a.vol_split;
    const int2* nbr = flx ? a.flx_nbr : a.vol_nbr;
    const int oe = __ldg(a.order + et);
    const int beg = lu == 0 ? __ldg(split + et) : __ldg(ptr + et);
    const int end = lu == 2 ? __ldg(split + et) : __ldg(ptr + et + 1);
    const int ncols = NTO;  // blocked 1D table: k-rows of a block are NTO apart
    const T* mcol = M + size_t(oe) * (n_from * NTO);
    const int in_off = outer * n_from * stride + inner;
    const size_t mstep = size_t(a.n1) * (n_from * NTO);
    T acc[NTO];
#pragma unroll
    for (int q = 0; q < NTO; ++q) acc[q] = from_double<T>(0.0);
    int i = beg;
    if (D.kind == 0) {
        for (; i + 2 <= end; i += 2) {
            const int2 nb0 = __ldg(nbr + i), nb1 = __ldg(nbr + i + 1);
            col_pair<T, NF, NTO>(in + int64_t(nb0.x) * in_block + in_off, mcol + size_t(nb0.y) * mstep,
                                 in + int64_t(nb1.x) * in_block + in_off, mcol + size_t(nb1.y) * mstep, stride, ncols,
                                 acc);
        }
    }
    for (; i < end; ++i) {
        const int2 nb = __ldg(nbr + i);
        const T* x = in + int64_t(nb.x) * in_block + in_off;
        const T* m = mcol + size_t(nb.y) * mstep;
        for (int k = 0; k < n_from; ++k) {
            const T xv = __ldg(x + k * stride);
            T mv[NTO];
#pragma unroll
            for (int q = 0; q < NTO; ++q) mv[q] = __ldg(m + size_t(k) * ncols + q);
#pragma unroll
            for (int q = 0; q < NTO; ++q) acc[q] = madd(xv, mv[q], acc[q]);
        }
    }
    T* o = a.out + int64_t(slot) * a.num_elements * a.out_block + e * a.out_block + int64_t(outer) * stride * NTO + inner;
#pragma unroll
    for (int q = 0; q < NTO; ++q) o[int64_t(q) * stride] = scale(acc[q], coef);
}

// ---- warp per (node, element) -----------------------------------------------------------------
// The lanes of a warp split as (column c, phase ph): lane = ph * cols + c for cols columns of the
// output block (lines along the transformed dimension, NT outputs each) and P = 32 / cols phases;
// lane (c, ph) walks neighbours beg + ph, beg + ph + P, ... of the element's list, and per neighbour
// loads its column's NF inputs and the NF x NT block of the 1D table for the (neighbour, element)
// order pair (contiguous in the blocked table, so vector loads), then does the NF x NT
// multiply-adds.  The phases' partial sums are added by shuffles (fixed order), and the phase-0
// lanes write.  Every lane of a warp serves the same element, so the neighbour list and the table
// block are broadcast loads and the warp follows one trip count.  Kind-1 nodes (the penalty, np
// inputs per column) take the same path with NF = np.  Sums run in another order than
// sweep_kernel's: results agree to rounding, not bitwise.

// the n entries of a table block (16-byte aligned when n * sizeof(T) is a multiple of 16)
template <typename T, int N>
__device__ __forceinline__ void load_block(const T* p, T (&v)[N]) {
    if constexpr ((N * sizeof(T)) % 16 == 0) {
        constexpr int V = N * sizeof(T) / 16;
        const float4* p4 = reinterpret_cast<const float4*>(p);
        float4 w[V];
#pragma unroll
        for (int i = 0; i < V; ++i) w[i] = __ldg(p4 + i);
        const T* wt = reinterpret_cast<const T*>(w);
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = wt[i];
    } else {
#pragma unroll
        for (int i = 0; i < N; ++i) v[i] = __ldg(p + i);
    }
}

__device__ __forceinline__ double shfl_from(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float shfl_from(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ float2 shfl_from(float2 v, int src) {
    return make_float2(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}
__device__ __forceinline__ double add_t(double a, double b) { return a + b; }
__device__ __forceinline__ float add_t(float a, float b) { return a + b; }
__device__ __forceinline__ float2 add_t(float2 a, float2 b) { return df_add(a, b); }

// one lane's share of a column: neighbours i = first, first + P, ... < end, two per pass
template <typename T, int NF, int NT>
__device__ __forceinline__ void warp_column(const int2* __restrict__ nbr, int first, int end, int P, const T* in,
                                            int64_t in_block, int in_off, int stride, const T* M, size_t mrow, int oe,
                                            T (&acc)[NT]) {
    constexpr int BS = NF * NT;
    int i = first;
    for (; i + P < end; i += 2 * P) {
        const int2 n0 = __ldg(nbr + i), n1 = __ldg(nbr + i + P);
        const T* x0 = in + int64_t(n0.x) * in_block + in_off;
        const T* x1 = in + int64_t(n1.x) * in_block + in_off;
        T xa[NF], xb[NF], ma[BS], mb[BS];
#pragma unroll
        for (int p = 0; p < NF; ++p) {
            xa[p] = __ldg(x0 + p * stride);
            xb[p] = __ldg(x1 + p * stride);
        }
        load_block<T, BS>(M + (size_t(n0.y) * mrow + oe) * BS, ma);
        load_block<T, BS>(M + (size_t(n1.y) * mrow + oe) * BS, mb);
#pragma unroll
        for (int p = 0; p < NF; ++p)
#pragma unroll
            for (int q = 0; q < NT; ++q) acc[q] = madd(xa[p], ma[p * NT + q], acc[q]);
#pragma unroll
        for (int p = 0; p < NF; ++p)
#pragma unroll
            for (int q = 0; q < NT; ++q) acc[q] = madd(xb[p], mb[p * NT + q], acc[q]);
    }
    if (i < end) {
        const int2 n0 = __ldg(nbr + i);
        const T* x0 = in + int64_t(n0.x) * in_block + in_off;
        T xa[NF], ma[BS];
#pragma unroll
        for (int p = 0; p < NF; ++p) xa[p] = __ldg(x0 + p * stride);
        load_block<T, BS>(M + (size_t(n0.y) * mrow + oe) * BS, ma);
#pragma unroll
        for (int p = 0; p < NF; ++p)
#pragma unroll
            for (int q = 0; q < NT; ++q) acc[q] = madd(xa[p], ma[p * NT + q], acc[q]);
    }
}

// node blockIdx.y; warp w of CTA x serves elements x * 8 + w, then every gridDim.x * 8-th after it
// Six CTAs of 256 per multiprocessor (at most 40 registers; 48 without the bound): 7 % faster
// mixed 3D right-hand sides; eight CTAs spill.
template <typename T, int NF, int NT>
__global__ void __launch_bounds__(256, 6) sweep_warp_kernel(SweepArgs<T> a) {
    const int slot = blockIdx.y;
    const PartialSum& D = a.desc[a.first + slot];
    if (D.kind == 1 && a.sweep + 1 < a.dim) return;  // a penalty term is a single (last) sweep
    const int lane = threadIdx.x & 31;
    int t, lu, flx, stride = 1, in_block = 1, nf = NF;
    const T* M;
    const T* in;
    if (D.kind == 0) {
        t = D.dims[a.sweep];
        lu = D.lu[a.sweep];
        flx = D.flx[a.sweep];
        M = a.mats[D.mat[a.sweep]];
        in = a.sweep == 0 ? a.src[D.src] : a.in + int64_t(D.parent) * a.in_slice;
        int done_after = 0;
        for (int j = 0; j < a.sweep; ++j) done_after += D.dims[j] > t ? 1 : 0;
        for (int d = 0; d < a.dim - 1 - t; ++d) stride *= d < done_after ? a.n_out : a.n_in;
        for (int d = 0; d < a.dim; ++d) in_block *= d < a.sweep ? a.n_out : a.n_in;
    } else {
        t = D.dims[0];
        lu = 1;
        flx = 1;
        nf = a.np;
        M = a.mats[kMatAJump];
        in = a.pen_in;
        for (int d = 0; d < a.dim - 1 - t; ++d) stride *= a.np;
        for (int d = 0; d < a.dim; ++d) in_block *= a.np;
    }
    const T coef = from_double<T>(D.coef);
    const int cols = a.out_block / NT;
    const int P = cols >= 32 ? 1 : 32 / cols;
    const int ph = P > 1 ? lane / cols : 0;
    const int32_t* ptr = flx ? a.flx_ptr : a.vol_ptr;
    const int32_t* split = flx ? a.flx_split : a.vol_split;
    const int2* nbr = flx ? a.flx_nbr : a.vol_nbr;
    const int E = int(a.num_elements);
    T* outs = a.out + int64_t(slot) * E * a.out_block;
    const size_t mrow = size_t(a.n1);
    for (int e = blockIdx.x * 8 + (threadIdx.x >> 5); e < E; e += gridDim.x * 8) {
        const int et = e * a.dim + t;
        const int oe = __ldg(a.order + et);
        const int beg = lu == 0 ? __ldg(split + et) : __ldg(ptr + et);
        const int end = lu == 2 ? __ldg(split + et) : __ldg(ptr + et + 1);
        T* oute = outs + int64_t(e) * a.out_block;
        // columns c = lane % cols (phase lane / cols), or c0 + lane when cols > 32
        for (int c0 = 0; c0 < cols; c0 += (P > 1 ? cols : 32)) {
            const int c = P > 1 ? lane % cols : c0 + lane;
            const bool active = P > 1 ? ph < P : c < cols;
            const int inner = c % stride, outer = c / stride;
            T acc[NT];
#pragma unroll
            for (int q = 0; q < NT; ++q) acc[q] = from_double<T>(0.0);
            if (active) {
                if (nf == NF) {
                    warp_column<T, NF, NT>(nbr, beg + ph, end, P, in, in_block, outer * NF * stride + inner, stride, M,
                                           mrow, oe, acc);
                } else if constexpr (NT == 3) {
                    warp_column<T, 3, 3>(nbr, beg + ph, end, P, in, in_block, outer * 3 * stride + inner, stride, M,
                                         mrow, oe, acc);
                }
            }
            // phase sums into the phase-0 lanes: lane l adds lane l + off for off = cols, 2 cols, 4 cols, ...
            if (P > 1) {
                for (int off = cols; off < P * cols; off *= 2) {
                    const int src = lane + off;
#pragma unroll
                    for (int q = 0; q < NT; ++q) {
                        const T v = shfl_from(acc[q], src & 31);
                        if (src < 32 && src < P * cols) acc[q] = add_t(acc[q], v);
                    }
                }
            }
            if (active && ph == 0) {
                T* o = oute + outer * stride * NT + inner;
#pragma unroll
                for (int q = 0; q < NT; ++q) o[q * stride] = scale(acc[q], coef);
            }
        }
    }
}

// epw elements per warp (one CTA of 8 warps per 8 epw elements and node)
template <typename T, int NF, int NT>
static void launch_warp(const SweepArgs<T>& a, int epw, cudaStream_t st) {
    const int64_t per_cta = 8 * epw;
    const int64_t gx = (a.num_elements + per_cta - 1) / per_cta;
    const dim3 grid(unsigned(gx > 0 ? gx : 1), unsigned(a.count));
    sweep_warp_kernel<T, NF, NT><<<grid, 256, 0, st>>>(a);
}

template <typename T>
cudaError_t launch_sweep(const SweepArgs<T>& a, cudaStream_t st) {
    const int64_t total = a.num_elements * a.out_block * a.count;
    if (total == 0) return cudaSuccess;
    // every term of the range writes n_out entries per column (the penalty terms of a right-hand
    // side have n_out = np too)
    const int nto = a.n_out;
    const int64_t cols = total / nto;
    const unsigned blocks = unsigned((cols + 255) / 256);
    // (n_in, n_out) of the transforms the library runs: point values np -> p1, right-hand sides
    // p1 -> np (the penalty np -> np in the same launch), the interpolation init p1 -> np
    if (a.variant >= 2 && a.out_block % nto == 0) {
        const int epw = a.variant == 2 ? 1 : (a.variant == 3 ? 2 : 4);
        switch (a.n_in * 10 + nto) {
            case 33: launch_warp<T, 3, 3>(a, epw, st); return cudaGetLastError();
            case 34: launch_warp<T, 3, 4>(a, epw, st); return cudaGetLastError();
            case 35: launch_warp<T, 3, 5>(a, epw, st); return cudaGetLastError();
            case 36: launch_warp<T, 3, 6>(a, epw, st); return cudaGetLastError();
            case 43: launch_warp<T, 4, 3>(a, epw, st); return cudaGetLastError();
            case 53: launch_warp<T, 5, 3>(a, epw, st); return cudaGetLastError();
            case 63: launch_warp<T, 6, 3>(a, epw, st); return cudaGetLastError();
            default: break;
        }
    }
    const int pair = (a.variant == 1 && a.out_block % nto == 0) ? a.n_in * 10 + nto : 0;
    switch (pair) {
        case 33: sweep_col_kernel<T, 3, 3><<<blocks, 256, 0, st>>>(a); break;
        case 34: sweep_col_kernel<T, 3, 4><<<blocks, 256, 0, st>>>(a); break;
        case 35: sweep_col_kernel<T, 3, 5><<<blocks, 256, 0, st>>>(a); break;
        case 43: sweep_col_kernel<T, 4, 3><<<blocks, 256, 0, st>>>(a); break;
        case 53: sweep_col_kernel<T, 5, 3><<<blocks, 256, 0, st>>>(a); break;
        case 63: sweep_col_kernel<T, 6, 3><<<blocks, 256, 0, st>>>(a); break;
        default:
            // measured: the node-row grid is the faster one for the FP32 sweeps, the flat grid for
            // the FP64 and double-float ones
            if constexpr (!std::is_same<T, float>::value) {
                sweep_kernel<T, false><<<unsigned((total + kSweepThreads - 1) / kSweepThreads), kSweepThreads, 0, st>>>(a);
            } else {
                const dim3 grid(unsigned((a.num_elements * a.out_block + kSweepThreads - 1) / kSweepThreads),
                                unsigned(a.count));
                sweep_kernel<T, true><<<grid, kSweepThreads, 0, st>>>(a);
            }
            break;
    }
    return cudaGetLastError();
}

template cudaError_t launch_sweep<double>(const SweepArgs<double>&, cudaStream_t);
template cudaError_t launch_sweep<float>(const SweepArgs<float>&, cudaStream_t);
template cudaError_t launch_sweep<float2>(const SweepArgs<float2>&, cudaStream_t);

template <typename T>
__global__ void reduce_points_kernel(const T* __restrict__ buf, int count, int64_t n, int first, T* acc, T* fp) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T v = first ? T(0) : acc[i];
    for (int s = 0; s < count; ++s) v += buf[int64_t(s) * n + i];
    if (fp) fp[i] = v * v * T(0.5);  // u^2/2
    else acc[i] = v;
}

// double-float slices summed in FP64 (each slice rounded to double first)
__global__ void reduce_points_df_kernel(const float2* __restrict__ buf, int count, int64_t n, int first, double* acc,
                                        double* fp) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = first ? 0.0 : acc[i];
    for (int s = 0; s < count; ++s) v += to_double(buf[int64_t(s) * n + i]);
    if (fp) fp[i] = v * v * 0.5;  // u^2/2
    else acc[i] = v;
}

cudaError_t launch_reduce_points_df(const float2* buf, int count, int64_t n, int first, double* acc, double* fp,
                                    cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    reduce_points_df_kernel<<<AMDG_EW_GRID(n), 0, st>>>(buf, count, n, first, acc, fp);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_reduce_points(const T* buf, int count, int64_t n, int first, T* acc, T* fp, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    reduce_points_kernel<T><<<AMDG_EW_GRID(n), 0, st>>>(buf, count, n, first, acc, fp);
    return cudaGetLastError();
}

template cudaError_t launch_reduce_points<double>(const double*, int, int64_t, int, double*, double*, cudaStream_t);
template cudaError_t launch_reduce_points<float>(const float*, int, int64_t, int, float*, float*, cudaStream_t);

template <typename T>
__global__ void reduce_rhs_kernel(const T* __restrict__ buf, int count, int64_t n, int first, int last, double* acc,
                                  StageOut so) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = first ? 0.0 : acc[i];
    for (int s = 0; s < count; ++s) v += double(buf[int64_t(s) * n + i]);
    if (last && so.fused) so.out[i] = rk_combine(so.rk.a, so.un[i], so.rk.b, so.us[i], so.rk.dt, v);
    else acc[i] = v;
}

template <typename T>
cudaError_t launch_reduce_rhs(const T* buf, int count, int64_t n, int first, int last, double* acc, StageOut so,
                              cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    reduce_rhs_kernel<T><<<AMDG_EW_GRID(n), 0, st>>>(buf, count, n, first, last, acc, so);
    return cudaGetLastError();
}

template cudaError_t launch_reduce_rhs<double>(const double*, int, int64_t, int, int, double*, StageOut, cudaStream_t);
template cudaError_t launch_reduce_rhs<float>(const float*, int, int64_t, int, int, double*, StageOut, cudaStream_t);

template <typename Ti, typename To>
__global__ void __launch_bounds__(256) surplus_pass_kernel(SurplusArgs<Ti> a, const Ti* __restrict__ in, To* __restrict__ out) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = a.num_elements * a.points;
    if (gid >= total) return;
    const int64_t e = gid / a.points;
    const int p = int(gid - e * a.points);
    Ti c = in[gid];
    const int od = __ldg(a.order + e * a.dim + a.d);
    if (od != 0) {
        const int P1 = a.p1;
        const int pd = (p / a.stride) % P1;
        const int base = p - pd * a.stride;
        const int32_t* anc = a.anc + (e * a.dim + a.d) * P1;
        // Hermite: the level-1 weights scaled to the element's level (a power of two, exact)
        const int lscale = a.herm ? (31 - __clz(od)) : 0;
        for (int ic = 0; ic < P1; ++ic) {
            const int s = __ldg(anc + ic);
            const int q = __ldg(a.anc_point + od * P1 + ic);
            const int r = __ldg(a.anc_rank + od * P1 + ic);
            const double w = a.herm ? ldexp(a.weight[pd * P1 + r], lscale * (pd / 2 - r / 2)) : a.weight[pd * P1 + r];
            c = fma(Ti(w), in[int64_t(s) * a.points + base + q * a.stride], c);
        }
    }
    out[gid] = To(c);
}

template <typename Ti, typename To>
cudaError_t launch_surplus_pass(const SurplusArgs<Ti>& a, const Ti* in, To* out, cudaStream_t st) {
    const int64_t total = a.num_elements * a.points;
    if (total == 0) return cudaSuccess;
    surplus_pass_kernel<Ti, To><<<AMDG_EW_GRID(total), 0, st>>>(a, in, out);
    return cudaGetLastError();
}

template cudaError_t launch_surplus_pass<double, double>(const SurplusArgs<double>&, const double*, double*, cudaStream_t);
template cudaError_t launch_surplus_pass<double, float>(const SurplusArgs<double>&, const double*, float*, cudaStream_t);
template cudaError_t launch_surplus_pass<float, float>(const SurplusArgs<float>&, const float*, float*, cudaStream_t);

template <typename Ti, typename To>
__global__ void convert_kernel(const Ti* __restrict__ in, To* __restrict__ out, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = To(in[i]);
}

template <typename Ti, typename To>
cudaError_t launch_convert(const Ti* in, To* out, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    convert_kernel<Ti, To><<<AMDG_EW_GRID(n), 0, st>>>(in, out, n);
    return cudaGetLastError();
}

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }

// one thread per (element, point pair (q0, q1)): the four dofs of the pair, in the operation
// order of HermInterpolation::eval_fp_Her_2D (Interplation.cpp:2045-2300) with f' = u, f'' = 1
template <typename T>
__global__ void herm_flux_burgers2d_kernel(const T* __restrict__ up, T* __restrict__ fp, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t e = i >> 2;
    const int q0 = int(i & 3) >> 1, q1 = int(i & 1);
    const T* v = up + e * 16;
    T* f = fp + e * 16;
    // entry (p0, p1) at p0 * 4 + p1; p = q (value) or q + 2 (slope)
    const int i00 = q0 * 4 + q1, i10 = (q0 + 2) * 4 + q1, i01 = q0 * 4 + q1 + 2, i11 = (q0 + 2) * 4 + q1 + 2;
    const T u = v[i00], ux = v[i10], uy = v[i01], uxy = v[i11];
    f[i00] = u * u * T(0.5);
    f[i10] = u * ux;
    f[i01] = u * uy;
    f[i11] = add_rn(mul_rn(ux, uy), mul_rn(u, uxy));  // both products rounded, as the reference
}

template <typename T>
cudaError_t launch_herm_flux_burgers2d(const T* up, T* fp, int64_t num_elements, cudaStream_t st) {
    const int64_t n = num_elements * 4;
    if (n == 0) return cudaSuccess;
    herm_flux_burgers2d_kernel<T><<<AMDG_EW_GRID(n), 0, st>>>(up, fp, n);
    return cudaGetLastError();
}

template cudaError_t launch_herm_flux_burgers2d<double>(const double*, double*, int64_t, cudaStream_t);
template cudaError_t launch_herm_flux_burgers2d<float>(const float*, float*, int64_t, cudaStream_t);

template cudaError_t launch_convert<double, float>(const double*, float*, int64_t, cudaStream_t);
template cudaError_t launch_convert<float, double>(const float*, double*, int64_t, cudaStream_t);

template <typename Tin>
__global__ void reduce_points_coef_kernel(const Tin* __restrict__ buf, int count, int64_t E, int dim, int p1,
                                          const int32_t* __restrict__ order, const double* __restrict__ pts, double amp,
                                          double* __restrict__ out) {
    int P = 1;
    for (int d = 0; d < dim; ++d) P *= p1;
    const int64_t n = E * P;
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = 0.0;
    for (int s = 0; s < count; ++s) v += to_double(buf[int64_t(s) * n + i]);
    const int64_t e = i / P;
    int r = int(i - e * P);
    // the coefficient function of the registered wave problem, at this point
    const double pi = 3.14159265358979323846;
    double x[kMaxDim];
    for (int d = dim - 1; d >= 0; --d) {
        x[d] = __ldg(pts + __ldg(order + e * dim + d) * p1 + r % p1);
        r /= p1;
    }
    double prod = 1.0;
    for (int d = 0; d < dim; ++d) prod *= sin(2 * pi * x[d]);
    const double c = 1.0 + amp * prod;
    out[i] = (c * c) * v;
}

template <typename Tin>
cudaError_t launch_reduce_points_coef(const Tin* buf, int count, int64_t E, int dim, int p1, const int32_t* order,
                                      const double* pts, double amp, double* out, cudaStream_t st) {
    int64_t n = E;
    for (int d = 0; d < dim; ++d) n *= p1;
    if (n == 0) return cudaSuccess;
    reduce_points_coef_kernel<Tin><<<AMDG_EW_GRID(n), 0, st>>>(buf, count, E, dim, p1, order, pts, amp,
                                                                               out);
    return cudaGetLastError();
}

template cudaError_t launch_reduce_points_coef<double>(const double*, int, int64_t, int, int, const int32_t*,
                                                       const double*, double, double*, cudaStream_t);
template cudaError_t launch_reduce_points_coef<float2>(const float2*, int, int64_t, int, int, const int32_t*,
                                                       const double*, double, double*, cudaStream_t);

__global__ void to_df_kernel(const double* __restrict__ in, float2* __restrict__ out, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = from_double<float2>(in[i]);
}

cudaError_t launch_to_df(const double* in, float2* out, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    to_df_kernel<<<AMDG_EW_GRID(n), 0, st>>>(in, out, n);
    return cudaGetLastError();
}

// Eigen evaluates each vector expression elementwise with one rounding per operation (no contraction)
__global__ void rk4_2nd_stage_kernel(int stage, double dt, const double* __restrict__ rhs, double* un, double* vn,
                                     double* us, double* vs, double* su, double* sv, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (stage < 0) {  // EulerODE2nd: u = u + dt v, v = v + dt rhs (ODESolver.cpp:409-414)
        const double u0 = un[i], v0 = vn[i];
        us[i] = __dadd_rn(u0, __dmul_rn(dt, v0));
        vs[i] = __dadd_rn(v0, __dmul_rn(dt, rhs[i]));
        return;
    }
    const double ku = __dmul_rn(dt, vs[i]), kv = __dmul_rn(dt, rhs[i]);
    if (stage == 0) {
        su[i] = ku;
        sv[i] = kv;
    } else if (stage < 3) {
        su[i] = __dadd_rn(su[i], __dmul_rn(2.0, ku));
        sv[i] = __dadd_rn(sv[i], __dmul_rn(2.0, kv));
    }
    if (stage < 2) {
        us[i] = __dadd_rn(un[i], ku / 2.);
        vs[i] = __dadd_rn(vn[i], kv / 2.);
    } else if (stage == 2) {
        us[i] = __dadd_rn(un[i], ku);
        vs[i] = __dadd_rn(vn[i], kv);
    } else {
        const double tu = __dadd_rn(su[i], ku), tv = __dadd_rn(sv[i], kv);
        un[i] = __dadd_rn(un[i], __dmul_rn(1. / 6., tu));
        vn[i] = __dadd_rn(vn[i], __dmul_rn(1. / 6., tv));
    }
}

cudaError_t launch_rk4_2nd_stage(int stage, double dt, const double* rhs, double* un, double* vn, double* us, double* vs,
                                 double* su, double* sv, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    rk4_2nd_stage_kernel<<<AMDG_EW_GRID(n), 0, st>>>(stage, dt, rhs, un, vn, us, vs, su, sv, n);
    return cudaGetLastError();
}

}  // namespace amdg
