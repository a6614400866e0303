// Launch interfaces of the Lagrange-interpolation path kernels (kernels_lagr.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "amdg_internal.hpp"
#include "kernels.cuh"

namespace amdg {

// One sweep over the nodes of a sweep tree (desc[first .. first + count)): thread per (node,
// element, output entry or column).  A kind-0 node of sweep j reads its block shape from the
// dimensions already transformed (n_out there, n_in elsewhere); in sweep 0 it reads its source,
// later its parent's slice of `in`, and it scales by its coef.  Kind-1 nodes (penalty terms,
// only in the last sweep) read pen_in with np entries per dimension.  Output: the node's slice of
// `out`, overwritten (out[slot][e][idx]).
template <typename T>
struct SweepArgs {
    int dim, sweep, n_in, n_out, np, n1;
    int64_t num_elements;
    int first, count;              // nodes [first, first + count) of desc
    const PartialSum* desc;
    const T* mats[kNumLagrMats];   // blocked by order pair: [o_from][o_to][rows per element][cols per element]
    const int32_t *vol_ptr, *vol_split, *flx_ptr, *flx_split;
    const int2 *vol_nbr, *flx_nbr; // (element, 1D order along t)
    const int32_t* order;          // [element][dim]
    const T* src[kMaxTermSources]; // sweep 0: node n reads src[n.src]
    const T* in;                   // later sweeps: node n reads in + n.parent * in_slice
    int64_t in_slice;
    const T* pen_in;               // Alpert coefficients for kind-1 terms
    T* out;
    int out_block;                 // output entries per element (uniform over the range)
    int variant;                   // 0: thread per output entry; 1: thread per column (sweep_col_kernel);
                                   // 2: warp per (node, element), lanes over (column, neighbour phase)
};

template <typename T>
cudaError_t launch_sweep(const SweepArgs<T>& a, cudaStream_t st);

// Point values: acc = (first ? 0 : acc) + sum_s buf[s] over count slices of n
// entries (in order); on the last chunk fp = acc^2/2 (Burgers flux
// FluxFunction::burgers_flux_scalar, Interplation.cpp:5070-5073) instead.
template <typename T>
cudaError_t launch_reduce_points(const T* buf, int count, int64_t n, int first, T* acc, T* fp, cudaStream_t st);

// The same from double-float slices (float2 = hi + lo), summed in FP64.
cudaError_t launch_reduce_points_df(const float2* buf, int count, int64_t n, int first, double* acc, double* fp,
                                    cudaStream_t st);

// Diffusion coefficient at the points: out = K(x) * sum_s buf[s] (in order, in FP64), K = (1 + amp
// prod_d sin(2 pi x_d))^2 at the point's coordinates (pts[order * p1 + p_d] per dimension,
// p1 points per dimension); buf double or double-float (float2).
template <typename Tin>
cudaError_t launch_reduce_points_coef(const Tin* buf, int count, int64_t E, int dim, int p1, const int32_t* order,
                                      const double* pts, double amp, double* out, cudaStream_t st);

// double -> double-float (hi = float(v), lo = float(v - hi))
cudaError_t launch_to_df(const double* in, float2* out, int64_t n, cudaStream_t st);

// One RK4ODE2nd stage (ODESolver.cpp:579-615) given the right-hand side at (us, vs):
// ku = dt vs, kv = dt rhs; stages 0-2 update (us, vs) from (un, vn) and the running sums
// (su, sv); stage 3 writes un + su/6, vn + sv/6 into (un, vn).  EulerODE2nd (stage -1):
// out_u = un + dt vn, out_v = vn + dt rhs into (us, vs).
cudaError_t launch_rk4_2nd_stage(int stage, double dt, const double* rhs, double* un, double* vn, double* us, double* vs,
                                 double* su, double* sv, int64_t n, cudaStream_t st);

// Right-hand side: v = (first ? 0 : acc) + sum_s buf[s] (in order, in FP64);
// not last: acc = v; last: out = rk_combine(rk, un, us, v) when stage is set,
// else acc = v.
struct StageOut {
    int fused;
    StageCoef rk;
    const double* un;
    const double* us;
    double* out;
};
template <typename T>
cudaError_t launch_reduce_rhs(const T* buf, int count, int64_t n, int first, int last, double* acc, StageOut so,
                              cudaStream_t st);

template <typename T>
struct SurplusArgs {
    int dim, d, p1, points, stride;  // p1 points per dimension, points = p1^dim, stride of dimension d
    int64_t num_elements;
    const int32_t* order;
    const int32_t* anc;          // [element][dim][p1]
    const int32_t* anc_point;    // [1D order][p1]
    const int32_t* anc_rank;     // [1D order][p1]
    double weight[kMaxLagrPoints * kMaxLagrPoints];  // [p0][rank]
    int herm;  // Hermite surplus: weight[p0][r] scaled by 2^((level_d - 1)(p0 / 2 - r / 2))
};
// one surplus pass, input and output types may differ (the last pass of the
// mixed mode writes the FP32 coefficients of the back transforms)
template <typename Ti, typename To>
cudaError_t launch_surplus_pass(const SurplusArgs<Ti>& a, const Ti* in, To* out, cudaStream_t st);
template <typename Ti, typename To>
cudaError_t launch_convert(const Ti* in, To* out, int64_t n, cudaStream_t st);
// The Burgers flux f = u^2/2 and its derivatives at the 2D cubic Hermite points (16 per
// element) from u_h and its derivatives there: f, f' u_x, f' u_y, f'' u_x u_y + f' u_xy
template <typename T>
cudaError_t launch_herm_flux_burgers2d(const T* up, T* fp, int64_t num_elements, cudaStream_t st);

}  // namespace amdg
