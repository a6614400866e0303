// Batched independent solves of the linear constant-coefficient operator:
// the element tables of many grids are concatenated and one launch per RK
// stage advances all of them.  Each element carries its solve index; the
// solve's velocity c scales the per-dimension sum of the shared 1D blocks
// (u_vx + upwind flux, one table per flux side), and the solve's dt enters
// the fused SSP-RK3 epilogue.  Column layout as linear_col_kernel; the CTA
// size TH (the tile: TH / np^(dim-1) elements per CTA) is a template
// parameter the batch's autotuner picks (64 to 1024 threads for dim <= 3,
// 256 above), beside the bulk-copy ring kernel of kernels.cu.
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "kernels.cuh"
#include "df_arith.cuh"

namespace amdg {

template <int B, int E>
struct BPow { static constexpr int v = B * BPow<B, E - 1>::v; };
template <int B>
struct BPow<B, 0> { static constexpr int v = 1; };

__device__ __forceinline__ double batch_combine(double a, double un, double b, double us, double dt, double rhs) {
    return __dadd_rn(__dmul_rn(a, un), __dmul_rn(b, __dadd_rn(us, __dmul_rn(dt, rhs))));
}

// the BS entries of a padded 1D block (BS a multiple of 4: 16-byte loads)
template <typename T, int BS>
__device__ __forceinline__ void load_padded_block(const T* p, T (&v)[BS]) {
    constexpr int V = BS * int(sizeof(T)) / 16;
    const float4* p4 = reinterpret_cast<const float4*>(p);
    float4 w[V];
#pragma unroll
    for (int i = 0; i < V; ++i) w[i] = __ldg(p4 + i);
    const T* wt = reinterpret_cast<const T*>(w);
#pragma unroll
    for (int i = 0; i < BS; ++i) v[i] = wt[i];
}

template <int D, int NP, int TH, typename T, typename X>
__global__ void __launch_bounds__(TH) batch_col_kernel(BatchLaunch<T, X> L) {
    constexpr int B = BPow<NP, D>::v;
    constexpr int C = B / NP;
    constexpr int G = TH / C > 0 ? TH / C : 1;  // launch_batch only launches TH >= C
    __shared__ T y[G * B];
    const int tid = threadIdx.x;
    const int g = tid / C, c = tid - (tid / C) * C;
    const int64_t e = int64_t(blockIdx.x) * G + g;
    const bool active = (g < G) && (e < L.num_elements);
    const int solve = active ? __ldg(L.solve_of + e) : 0;
    for (int i = tid; i < G * B; i += blockDim.x) y[i] = T(0);
    __syncthreads();
#pragma unroll
    for (int t = 0; t < D; ++t) {
        int stride = 1;
#pragma unroll
        for (int s = t + 1; s < D; ++s) stride *= NP;
        const int lo = c % stride, hi = c / stride;
        const int base = hi * stride * NP + lo;
        if (active) {
            const T ct = L.coef[solve * D + t];
            const T* table = L.blocks + (ct >= T(0) ? 0 : size_t(L.num_blocks) * NP * NP);
            T acc[NP];
#pragma unroll
            for (int q = 0; q < NP; ++q) acc[q] = T(0);
            const int64_t beg = __ldg(L.row_ptr + e * D + t);
            const int64_t end = __ldg(L.row_ptr + e * D + t + 1);
            if (L.pairs && L.blocks_p) {
                // (src, blk) as one 8-byte load, the 1D block as 16-byte loads of the padded table
                constexpr int BS = (NP * NP + 3) / 4 * 4;
                const T* tab = L.blocks_p + (ct >= T(0) ? 0 : size_t(L.num_blocks) * BS);
                for (int64_t i = beg; i < end; ++i) {
                    const int2 pr = __ldg(L.pairs + i);
                    T mv[BS];
                    load_padded_block<T, BS>(tab + size_t(pr.y) * BS, mv);
                    const X* x = L.xs + int64_t(pr.x) * B + base;
                    T xv[NP];
#pragma unroll
                    for (int p = 0; p < NP; ++p) xv[p] = T(__ldg(x + p * stride));
#pragma unroll
                    for (int p = 0; p < NP; ++p)
#pragma unroll
                        for (int q = 0; q < NP; ++q) acc[q] = fma(mv[p * NP + q], xv[p], acc[q]);
                }
            } else {
                for (int64_t i = beg; i < end; ++i) {
                    const int64_t sidx = __ldg(L.src + i);
                    const T* m = table + __ldg(L.blk + i) * NP * NP;
                    const X* x = L.xs + sidx * B + base;
                    T xv[NP];
#pragma unroll
                    for (int p = 0; p < NP; ++p) xv[p] = T(__ldg(x + p * stride));
#pragma unroll
                    for (int p = 0; p < NP; ++p)
#pragma unroll
                        for (int q = 0; q < NP; ++q) acc[q] = fma(__ldg(m + p * NP + q), xv[p], acc[q]);
                }
            }
            T* yb = y + g * B + base;
#pragma unroll
            for (int q = 0; q < NP; ++q) yb[q * stride] += ct * acc[q];
        }
        __syncthreads();
    }
    const int64_t first = int64_t(blockIdx.x) * G * B;
    const int64_t total = L.num_elements * B;
    for (int i = tid; i < G * B; i += blockDim.x) {
        const int64_t gid = first + i;
        if (gid >= total) break;
        const int sv = __ldg(L.solve_of + gid / B);
        if constexpr (std::is_same<T, float>::value) {
            if (L.df.out_hi) {  // FP32-pair stage state: the double-float update with the solve's step
                DFState df = L.df;
                df.dt = __ldg(L.dt32 + sv);
                df_stage_update(df, gid, float(y[i]));
                continue;
            }
        }
        const double rhs = double(y[i]);
        const double v = L.mode == 0 ? rhs : batch_combine(L.a, L.un[gid], L.b, L.us[gid], L.dt[sv], rhs);
        L.out[gid] = v;
        if (L.shadow_out) L.shadow_out[gid] = float(v);
    }
}

bool batch_tile_supported(int dim, int np, int threads) {
    int c = 1;
    for (int d = 1; d < dim; ++d) c *= np;
    if (threads < c) return false;
    if (dim <= 3) return threads == 64 || threads == 128 || threads == 256 || threads == 512 || threads == 1024;
    return threads == 256;
}

template <int D, int NP, int TH, typename T, typename X>
cudaError_t launch_batch_tile(const BatchLaunch<T, X>& L, cudaStream_t st) {
    constexpr int C = BPow<NP, D>::v / NP;
    if (TH < C) return cudaErrorInvalidValue;
    constexpr int G = TH / C > 0 ? TH / C : 1;
    const int64_t grid = (L.num_elements + G - 1) / G;
    batch_col_kernel<D, NP, TH, T, X><<<unsigned(grid), TH, 0, st>>>(L);
    return cudaGetLastError();
}

template <typename T, typename X>
cudaError_t launch_batch(const BatchLaunch<T, X>& L, cudaStream_t st) {
    if (L.num_elements == 0) return cudaSuccess;
    const int th = L.threads ? L.threads : 256;
    if (!batch_tile_supported(L.dim, L.np, th)) return cudaErrorInvalidValue;
#define AMDG_BCASE3(D, NP)                                                            \
    if (L.dim == D && L.np == NP) {                                                    \
        if (th == 64) return launch_batch_tile<D, NP, 64, T, X>(L, st);                \
        if (th == 128) return launch_batch_tile<D, NP, 128, T, X>(L, st);              \
        if (th == 512) return launch_batch_tile<D, NP, 512, T, X>(L, st);              \
        if (th == 1024) return launch_batch_tile<D, NP, 1024, T, X>(L, st);            \
        return launch_batch_tile<D, NP, 256, T, X>(L, st);                             \
    }
#define AMDG_BCASE1(D, NP) \
    if (L.dim == D && L.np == NP) return launch_batch_tile<D, NP, 256, T, X>(L, st);
    AMDG_BCASE3(1, 2) AMDG_BCASE3(1, 3) AMDG_BCASE3(1, 4)
    AMDG_BCASE3(2, 2) AMDG_BCASE3(2, 3) AMDG_BCASE3(2, 4)
    AMDG_BCASE3(3, 2) AMDG_BCASE3(3, 3) AMDG_BCASE3(3, 4)
    AMDG_BCASE1(4, 2) AMDG_BCASE1(4, 3) AMDG_BCASE1(4, 4)
    AMDG_BCASE1(5, 2) AMDG_BCASE1(5, 3) AMDG_BCASE1(5, 4)
    AMDG_BCASE1(6, 2) AMDG_BCASE1(6, 3)
#undef AMDG_BCASE3
#undef AMDG_BCASE1
    return cudaErrorInvalidValue;
}

template cudaError_t launch_batch<double, double>(const BatchLaunch<double, double>&, cudaStream_t);
template cudaError_t launch_batch<float, float>(const BatchLaunch<float, float>&, cudaStream_t);

}  // namespace amdg
