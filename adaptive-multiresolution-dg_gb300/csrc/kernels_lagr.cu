// Device kernels of the Lagrange-interpolation path for nonlinear fluxes.
//
// fibre_transform: one 1D transform of the fast multi-dimensional algorithm
// (FastMultiplyLU::transform_1D, FastMultiplyLU.cpp:436-512): for every
// element e and every entry of its output block,
//   out[e][idx] (+)= coef * sum_{s in N_t(e), L/U filter} sum_k in[s][idx, dim t <- k] * M[o_t(s)*n_from + k][o_t(e)*n_to + idx_t]
// where N_t(e) is the vol or flx neighbour list of e in dimension t.  The
// per-element block shapes follow the partial-sum schedule
// (series_vec_transform_size, FastMultiplyLU.cpp:596-612).  One thread per
// output entry; the neighbour list is warp-uniform within an element.
//
// surplus_pass: pass d of the hierarchical surplus
// (LagrInterpolation::eval_fp_to_coe_D_Lag, Interplation.cpp:1222-1434).
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels_lagr.cuh"

namespace amdg {

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
        for (int k = 0; k < NF; ++k) acc = fma(xv[j][k], mv[j][k], acc);
    return acc;
}

template <typename T>
__global__ void __launch_bounds__(256) fibre_transform_kernel(TransformArgs<T> a) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = a.num_elements * a.out_block;
    if (gid >= total) return;
    const int64_t e = gid / a.out_block;
    const int idx = int(gid - e * a.out_block);
    const int inner = idx % a.stride;
    const int qt = (idx / a.stride) % a.n_to;
    const int outer = idx / (a.stride * a.n_to);
    const int64_t et = e * a.dim + a.t;
    if (a.long_flag && __ldg(a.long_flag + et)) return;  // done by fibre_transform_long_kernel
    const int oe = __ldg(a.order + e * a.dim + a.t);
    // "L": neighbours finer than e in dimension t; "U": coarser or equal; neighbours are level-sorted
    const int beg = a.lu == 0 ? __ldg(a.split + et) : __ldg(a.ptr + et);
    const int end = a.lu == 2 ? __ldg(a.split + et) : __ldg(a.ptr + et + 1);
    const T* mcol = a.M + size_t(oe) * a.n_to + qt;
    const int in_off = outer * a.n_from * a.stride + inner;
    const size_t mstep = size_t(a.n_from) * a.ncols;
    T acc = T(0);
    // four neighbours per pass: their (element, order) pairs and operands are
    // independent loads issued together; the sum keeps the neighbour order
    int i = beg;
    for (; i + 4 <= end; i += 4) {
        int2 nb[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) nb[j] = __ldg(a.nbr + i + j);
        const T* x[4];
        const T* m[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            x[j] = a.in + int64_t(nb[j].x) * a.in_block + in_off;
            m[j] = mcol + size_t(nb[j].y) * mstep;
        }
        if (a.n_from == 4) acc = fibre_quad<4>(x, m, a.stride, a.ncols, acc);
        else if (a.n_from == 3) acc = fibre_quad<3>(x, m, a.stride, a.ncols, acc);
        else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                for (int k = 0; k < a.n_from; ++k) acc = fma(__ldg(x[j] + k * a.stride), __ldg(m[j] + size_t(k) * a.ncols), acc);
        }
    }
    for (; i < end; ++i) {
        const int2 nb = __ldg(a.nbr + i);
        const T* x = a.in + int64_t(nb.x) * a.in_block + in_off;
        const T* m = mcol + size_t(nb.y) * mstep;
        for (int k = 0; k < a.n_from; ++k) acc = fma(__ldg(x + k * a.stride), __ldg(m + size_t(k) * a.ncols), acc);
    }
    acc *= a.coef;
    if (a.accumulate) a.out[gid] += acc;
    else a.out[gid] = acc;
}

// Long rows (an element at a coarse level of its fibre sees every finer
// element of the fibre): one warp per output entry, lanes stride over the
// neighbours, fixed-order shuffle reduction.  Without the split such rows
// serialise hundreds of dependent neighbour loads in one thread.
template <typename T>
__global__ void __launch_bounds__(256) fibre_transform_long_kernel(TransformArgs<T> a) {
    const int64_t w = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) / 32;
    const int lane = threadIdx.x & 31;
    if (w >= int64_t(a.num_long) * a.out_block) return;
    const int64_t e = __ldg(a.long_elems + w / a.out_block);
    const int idx = int(w % a.out_block);
    const int inner = idx % a.stride;
    const int qt = (idx / a.stride) % a.n_to;
    const int outer = idx / (a.stride * a.n_to);
    const int64_t et = e * a.dim + a.t;
    const int oe = __ldg(a.order + et);
    const int beg = a.lu == 0 ? __ldg(a.split + et) : __ldg(a.ptr + et);
    const int end = a.lu == 2 ? __ldg(a.split + et) : __ldg(a.ptr + et + 1);
    const T* mcol = a.M + size_t(oe) * a.n_to + qt;
    const int in_off = outer * a.n_from * a.stride + inner;
    T acc = T(0);
    for (int i = beg + lane; i < end; i += 32) {
        const int2 nb = __ldg(a.nbr + i);
        const T* x = a.in + int64_t(nb.x) * a.in_block + in_off;
        const T* m = mcol + size_t(nb.y) * a.n_from * a.ncols;
        for (int k = 0; k < a.n_from; ++k) acc = fma(__ldg(x + k * a.stride), __ldg(m + size_t(k) * a.ncols), acc);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
    if (lane == 0) {
        acc *= a.coef;
        const int64_t gid = e * a.out_block + idx;
        if (a.accumulate) a.out[gid] += acc;
        else a.out[gid] = acc;
    }
}

template <typename T>
cudaError_t launch_fibre_transform(const TransformArgs<T>& a, cudaStream_t st) {
    const int64_t total = a.num_elements * a.out_block;
    if (total == 0) return cudaSuccess;
    fibre_transform_kernel<T><<<unsigned((total + 255) / 256), 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !a.long_flag || a.num_long == 0) return e;
    const int64_t warps = int64_t(a.num_long) * a.out_block;
    fibre_transform_long_kernel<T><<<unsigned((warps * 32 + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

template cudaError_t launch_fibre_transform<double>(const TransformArgs<double>&, cudaStream_t);
template cudaError_t launch_fibre_transform<float>(const TransformArgs<float>&, cudaStream_t);

// f(u) = u^2/2 at every interpolation point (FluxFunction::burgers_flux_scalar, Interplation.cpp:5070-5073)
template <typename T>
__global__ void burgers_flux_kernel(const T* __restrict__ up, T* __restrict__ fp, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) {
        const T u = up[i];
        fp[i] = u * u * T(0.5);
    }
}

template <typename T>
cudaError_t launch_burgers_flux(const T* up, T* fp, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    burgers_flux_kernel<T><<<unsigned((n + 255) / 256), 256, 0, st>>>(up, fp, n);
    return cudaGetLastError();
}

template cudaError_t launch_burgers_flux<double>(const double*, double*, int64_t, cudaStream_t);
template cudaError_t launch_burgers_flux<float>(const float*, float*, int64_t, cudaStream_t);

template <typename T>
__global__ void __launch_bounds__(256) surplus_pass_kernel(SurplusArgs<T> a) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = a.num_elements * a.points;
    if (gid >= total) return;
    const int64_t e = gid / a.points;
    const int p = int(gid - e * a.points);
    T c = a.in[gid];
    const int od = __ldg(a.order + e * a.dim + a.d);
    if (od != 0) {
        const int pd = (p / a.stride) % 4;
        const int base = p - pd * a.stride;
        const int32_t* anc = a.anc + (e * a.dim + a.d) * 4;
#pragma unroll
        for (int ic = 0; ic < 4; ++ic) {
            const int s = __ldg(anc + ic);
            const int q = __ldg(a.anc_point + od * 4 + ic);
            const int r = __ldg(a.anc_rank + od * 4 + ic);
            c = fma(a.weight[pd * 4 + r], a.in[int64_t(s) * a.points + base + q * a.stride], c);
        }
    }
    a.out[gid] = c;
}

template <typename T>
cudaError_t launch_surplus_pass(const SurplusArgs<T>& a, cudaStream_t st) {
    const int64_t total = a.num_elements * a.points;
    if (total == 0) return cudaSuccess;
    surplus_pass_kernel<T><<<unsigned((total + 255) / 256), 256, 0, st>>>(a);
    return cudaGetLastError();
}

template cudaError_t launch_surplus_pass<double>(const SurplusArgs<double>&, cudaStream_t);
template cudaError_t launch_surplus_pass<float>(const SurplusArgs<float>&, cudaStream_t);

template <typename Ti, typename To>
__global__ void convert_kernel(const Ti* __restrict__ in, To* __restrict__ out, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = To(in[i]);
}

template <typename Ti, typename To>
cudaError_t launch_convert(const Ti* in, To* out, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    convert_kernel<Ti, To><<<unsigned((n + 255) / 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

template cudaError_t launch_convert<double, float>(const double*, float*, int64_t, cudaStream_t);
template cudaError_t launch_convert<float, double>(const float*, double*, int64_t, cudaStream_t);

}  // namespace amdg
