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

#include <algorithm>
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

// One tile: G elements, (element, column) per thread, into the shared output block y
template <int D, int NP, int TH, typename T, typename X>
__device__ __forceinline__ void col_tile(const BatchLaunch<T, X>& L, int64_t tile, T* y) {
    constexpr int B = BPow<NP, D>::v;
    constexpr int C = B / NP;
    constexpr int G = TH / C > 0 ? TH / C : 1;  // launch_batch only launches TH >= C
    const int tid = threadIdx.x;
    const int g = tid / C, c = tid - (tid / C) * C;
    const int64_t e = tile * G + g;
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
    const int64_t first = tile * G * B;
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

// SCHED 0: one CTA per tile; 1: persistent, a grid of resident CTAs, CTA b takes tiles b, b + grid,
// ...; 2: persistent, tiles taken one at a time from the device counter L.queue (zeroed before
// the launch).  Each tile is computed alike, so the three give identical results.
template <int D, int NP, int TH, typename T, typename X, int SCHED>
__global__ void __launch_bounds__(TH) batch_col_kernel(BatchLaunch<T, X> L) {
    constexpr int B = BPow<NP, D>::v;
    constexpr int C = B / NP;
    constexpr int G = TH / C > 0 ? TH / C : 1;
    __shared__ T y[G * B];
    if constexpr (SCHED == 0) {
        col_tile<D, NP, TH, T, X>(L, blockIdx.x, y);
    } else {
        const int64_t ntiles = (L.num_elements + G - 1) / G;
        __shared__ long long next;
        int64_t tile = SCHED == 1 ? int64_t(blockIdx.x) : 0;
        if constexpr (SCHED == 2) {
            if (threadIdx.x == 0) next = (long long)atomicAdd(L.queue, 1ull);
            __syncthreads();
            tile = next;
        }
        while (tile < ntiles) {
            col_tile<D, NP, TH, T, X>(L, tile, y);
            __syncthreads();  // y and `next` are reused by the next tile
            if constexpr (SCHED == 1) {
                tile += gridDim.x;
            } else {
                if (threadIdx.x == 0) next = (long long)atomicAdd(L.queue, 1ull);
                __syncthreads();
                tile = next;
            }
        }
    }
}

bool batch_tile_supported(int dim, int np, int threads) {
    int c = 1;
    for (int d = 1; d < dim; ++d) c *= np;
    if (threads < c) return false;
    if (dim <= 3) return threads == 64 || threads == 128 || threads == 256 || threads == 512 || threads == 1024;
    return threads == 256;
}

// resident CTAs per multiprocessor of a persistent schedule, queried once per kernel (the first
// query runs when the batch is built, before any stream capture: batch_prepare_persistent)
template <int D, int NP, int TH, typename T, typename X, int SCHED>
int col_per_sm() {
    static int per_sm = 0;
    if (per_sm == 0 &&
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_col_kernel<D, NP, TH, T, X, SCHED>, TH, 0) !=
            cudaSuccess)
        per_sm = 0;
    return per_sm;
}

template <int D, int NP, int TH, typename T, typename X, int SCHED>
cudaError_t launch_col_sched(const BatchLaunch<T, X>& L, cudaStream_t st, bool prepare_only) {
    constexpr int C = BPow<NP, D>::v / NP;
    constexpr int G = TH / C > 0 ? TH / C : 1;
    int64_t grid = (L.num_elements + G - 1) / G;
    if (SCHED != 0) {
        const int per_sm = col_per_sm<D, NP, TH, T, X, SCHED>();
        if (per_sm <= 0) return cudaErrorInvalidConfiguration;
        grid = std::max<int64_t>(1, std::min<int64_t>(grid, int64_t(per_sm) * std::max(L.sms, 1)));
        if (SCHED == 2 && !L.queue && !prepare_only) return cudaErrorInvalidValue;
    }
    if (prepare_only) return cudaSuccess;
    batch_col_kernel<D, NP, TH, T, X, SCHED><<<unsigned(grid), TH, 0, st>>>(L);
    return cudaGetLastError();
}

template <int D, int NP, int TH, typename T, typename X>
cudaError_t launch_batch_tile(const BatchLaunch<T, X>& L, cudaStream_t st, bool prepare_only = false) {
    constexpr int C = BPow<NP, D>::v / NP;
    if (TH < C) return cudaErrorInvalidValue;
    // persistent schedules only for the FP32-pair state
    if constexpr (std::is_same<T, float>::value) {
        if (L.schedule == 1 && L.df.out_hi) return launch_col_sched<D, NP, TH, T, X, 1>(L, st, prepare_only);
        if (L.schedule == 2 && L.df.out_hi) return launch_col_sched<D, NP, TH, T, X, 2>(L, st, prepare_only);
    }
    if (L.schedule != 0) return cudaErrorInvalidValue;
    return launch_col_sched<D, NP, TH, T, X, 0>(L, st, prepare_only);
}

template <typename T, typename X>
cudaError_t dispatch_batch(const BatchLaunch<T, X>& L, cudaStream_t st, bool prepare_only) {
    if (L.num_elements == 0 && !prepare_only) return cudaSuccess;
    const int th = L.threads ? L.threads : 256;
    if (!batch_tile_supported(L.dim, L.np, th)) return cudaErrorInvalidValue;
#define AMDG_BCASE3(D, NP)                                                                      \
    if (L.dim == D && L.np == NP) {                                                              \
        if (th == 64) return launch_batch_tile<D, NP, 64, T, X>(L, st, prepare_only);            \
        if (th == 128) return launch_batch_tile<D, NP, 128, T, X>(L, st, prepare_only);          \
        if (th == 512) return launch_batch_tile<D, NP, 512, T, X>(L, st, prepare_only);          \
        if (th == 1024) return launch_batch_tile<D, NP, 1024, T, X>(L, st, prepare_only);        \
        return launch_batch_tile<D, NP, 256, T, X>(L, st, prepare_only);                         \
    }
#define AMDG_BCASE1(D, NP) \
    if (L.dim == D && L.np == NP) return launch_batch_tile<D, NP, 256, T, X>(L, st, prepare_only);
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

template <typename T, typename X>
cudaError_t launch_batch(const BatchLaunch<T, X>& L, cudaStream_t st) {
    return dispatch_batch(L, st, false);
}

cudaError_t batch_prepare_persistent(int dim, int np) {
    BatchLaunch<float, float> L{};
    float dummy = 0.f;
    L.dim = dim;
    L.np = np;
    L.df.out_hi = &dummy;  // the FP32-pair state form (its persistent schedules)
    for (int th : kBatchTiles) {
        if (!batch_tile_supported(dim, np, th)) continue;
        L.threads = th;
        for (int sched = 1; sched <= 2; ++sched) {
            L.schedule = sched;
            if (cudaError_t e = dispatch_batch(L, nullptr, true); e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

// ---- one warp per element -------------------------------------------------------------------
// Lane i < B holds coefficient i (row-major, last dimension fastest) of the element's output.  For
// dimension t with stride S = np^(dim-1-t), lane i's index along t is p_i = (i / S) % np, and its
// fibre partners are lanes i + (p - p_i) S.  Per neighbour (in list order): the source block's
// B FP32 high parts in one coalesced load, the np^2 block entries in one load (lanes < np^2), then
// acc += M[p][p_i] x[i + (p - p_i) S] for p ascending by warp shuffles -- the summation order of
// batch_col_kernel, so the two agree bitwise.  Neighbours are taken four at a time, their loads
// issued before the arithmetic.  Measured: shuffle throughput (2 np + 2 shuffles per neighbour)
// binds it well above the column kernel on 3D k = 2 batches.
template <int D, int NP>
__device__ __forceinline__ void warp_element(const BatchWarpLaunch& L, int64_t e, int lane) {
    constexpr int B = BPow<NP, D>::v;
    constexpr int BS = (NP * NP + 3) / 4 * 4;
    const int solve = __ldg(L.solve_of + e);
    float acc = 0.0f;
#pragma unroll
    for (int t = 0; t < D; ++t) {
        int stride = 1;
#pragma unroll
        for (int s = t + 1; s < D; ++s) stride *= NP;
        const int pl = lane < B ? (lane / stride) % NP : 0;
        const float ct = __ldg(L.coef + solve * D + t);
        const float* tab = L.blocks + (ct >= 0.0f ? 0 : size_t(L.num_blocks) * BS);
        const int64_t beg = __ldg(L.row_ptr + e * D + t), end = __ldg(L.row_ptr + e * D + t + 1);
        float at = 0.0f;
        for (int64_t c0 = beg; c0 < end; c0 += 32) {
            const int n = int(end - c0 < 32 ? end - c0 : 32);
            const int2 my = lane < n ? __ldg(L.pairs + c0 + lane) : make_int2(0, 0);
            for (int j = 0; j < n; j += 4) {
                float xv[4], mv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int src = __shfl_sync(0xffffffffu, my.x, (j + u) & 31);
                    const int blk = __shfl_sync(0xffffffffu, my.y, (j + u) & 31);
                    const bool live = j + u < n;
                    xv[u] = (live && lane < B) ? __ldg(L.xs + int64_t(src) * B + lane) : 0.0f;
                    mv[u] = (live && lane < NP * NP) ? __ldg(tab + size_t(blk) * BS + lane) : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (j + u >= n) break;  // warp-uniform
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        const int from = lane < B ? lane + (p - pl) * stride : lane;
                        const float xp = __shfl_sync(0xffffffffu, xv[u], from);
                        const float mp = __shfl_sync(0xffffffffu, mv[u], p * NP + pl);
                        at = fmaf(mp, xp, at);
                    }
                }
            }
        }
        acc = fmaf(ct, at, acc);
    }
    if (lane < B) {
        DFState df = L.df;
        df.dt = __ldg(L.dt + solve);
        df_stage_update(df, e * B + lane, acc);
    }
}

// one CTA per W elements
template <int D, int NP, int W>
__global__ void __launch_bounds__(W * 32) batch_warp_kernel(BatchWarpLaunch L) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t e = int64_t(blockIdx.x) * W + warp;
    if (e < L.num_elements) warp_element<D, NP>(L, e, lane);
}

bool batch_warp_supported(int dim, int np, int cfg) {
    if (cfg < 0 || cfg >= kBatchWarpConfigs || np < 2 || np > 4 || dim < 1) return false;
    int b = 1;
    for (int d = 0; d < dim; ++d) b *= np;
    return b <= 32;
}

cudaError_t launch_batch_warp(const BatchWarpLaunch& L, cudaStream_t st) {
    if (!batch_warp_supported(L.dim, L.np, L.cfg)) return cudaErrorInvalidValue;
    if (L.num_elements == 0) return cudaSuccess;
    const unsigned grid = unsigned((L.num_elements + 7) / 8);
#define AMDG_WCASE(D, NP)                                                         \
    if (L.dim == D && L.np == NP) {                                               \
        batch_warp_kernel<D, NP, 8><<<grid, 256, 0, st>>>(L);                     \
        return cudaGetLastError();                                                \
    }
    AMDG_WCASE(1, 2) AMDG_WCASE(1, 3) AMDG_WCASE(1, 4)
    AMDG_WCASE(2, 2) AMDG_WCASE(2, 3) AMDG_WCASE(2, 4)
    AMDG_WCASE(3, 2) AMDG_WCASE(3, 3)
    AMDG_WCASE(4, 2) AMDG_WCASE(5, 2)
#undef AMDG_WCASE
    return cudaErrorInvalidValue;
}

template cudaError_t launch_batch<double, double>(const BatchLaunch<double, double>&, cudaStream_t);
template cudaError_t launch_batch<float, float>(const BatchLaunch<float, float>&, cudaStream_t);

}  // namespace amdg
