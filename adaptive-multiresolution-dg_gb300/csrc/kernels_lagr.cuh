// Launch interfaces of the Lagrange-interpolation path kernels (kernels_lagr.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace amdg {

template <typename T>
struct TransformArgs {
    int dim, t;              // dimensions, transform dimension
    int n_from, n_to;        // block size in dimension t before / after
    int stride;              // product of block sizes of the dimensions after t (same in and out)
    int in_block, out_block; // block sizes (entries per element) of in / out
    int ncols;               // columns of M (= 1D elements * n_to)
    int lu;                  // 0 "L" (neighbour level > own), 1 full, 2 "U" (neighbour level <= own)
    int accumulate;          // 0: out = ..., 1: out += ...
    T coef;
    int64_t num_elements;
    const T* M;              // [1D elements * n_from][ncols]
    const int32_t* ptr;      // CSR over (element, dimension)
    const int2* nbr;         // (element, 1D order along t) per neighbour
    const int32_t* split;    // [e*dim+t]: first neighbour finer than e in dimension t
    const int32_t* order;    // [element][dim] 1D orders
    const T* in;
    T* out;
    const uint8_t* long_flag;   // [e*dim+t]: row handled by the warp-per-output kernel (null: none)
    const int32_t* long_elems;  // elements with a long row in dimension t
    int num_long;
};

// rows longer than this many neighbours are split across a warp
constexpr int kLongRow = 24;

template <typename T>
struct SurplusArgs {
    int dim, d, points, stride;  // points = 4^dim, stride of dimension d
    int64_t num_elements;
    const int32_t* order;
    const int32_t* anc;          // [element][dim][4]
    const int32_t* anc_point;    // [1D order][4]
    const int32_t* anc_rank;     // [1D order][4]
    T weight[16];                // [p0][rank]
    const T* in;
    T* out;
};

template <typename T>
cudaError_t launch_fibre_transform(const TransformArgs<T>& a, cudaStream_t st);
template <typename T>
cudaError_t launch_burgers_flux(const T* up, T* fp, int64_t n, cudaStream_t st);
template <typename T>
cudaError_t launch_surplus_pass(const SurplusArgs<T>& a, cudaStream_t st);
template <typename Ti, typename To>
cudaError_t launch_convert(const Ti* in, To* out, int64_t n, cudaStream_t st);

}  // namespace amdg
