// Device kernels of the sparse-grid DG right-hand side (sm_103a).
//
// linear_apply: matrix-free apply of the linear constant-coefficient operator
//   rhs[e][q] = sum_t sum_{(s,b) in N_t(e)} sum_p M_t[b][p][q_t] * u[s][q with q_t <- p]
// i.e. the per-dimension 1D transform of FastMultiplyLU::transform_1D
// (FastMultiplyLU.cpp:436-512) with the "full" schedule, summed over
// dimensions as HyperbolicAlpt assembles it (BilinearForm.cpp:691-710).  One
// thread per output coefficient; every thread of an element walks the same
// neighbour list, so the list and the 1D block are warp-uniform loads and the
// neighbour block reads coalesce through L1.  The SSP-RK3 stage update
// (ODESolver.cpp:285-301) is fused into the epilogue, in FP64 with the
// reference's operation order and no contraction.
#include <cuda_runtime.h>

#include <type_traits>

#include <cstdint>

#include "kernels.cuh"
#include "df_arith.cuh"

namespace amdg {

template <int B, int E>
struct IPow { static constexpr int v = B * IPow<B, E - 1>::v; };
template <int B>
struct IPow<B, 0> { static constexpr int v = 1; };


// X: type of the neighbour values read by the contraction (double, or the
// float shadow of the stage input in mixed mode, so no per-FMA conversion is
// needed: double->float conversion issues on the FP64 pipe, which on this part
// is as slow as an FP64 FMA).  shadow_out, when set, receives float(out).
template <int D, int NP, typename T, typename X>
__global__ void __launch_bounds__(256) linear_apply_kernel(const double* __restrict__ us, const X* __restrict__ xs,
                                                           const double* un, double* out, float* shadow_out,
                                                           const int32_t* __restrict__ row_ptr,
                                                           const int32_t* __restrict__ src, const int32_t* __restrict__ blk,
                                                           const T* __restrict__ blocks, int nblocks, int64_t total,
                                                           StageCoef rk, DFState df) {
    constexpr int B = IPow<NP, D>::v;
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= total) return;
    const int64_t e = gid / B;
    const int q = int(gid - e * B);
    T acc = T(0);
#pragma unroll
    for (int t = 0; t < D; ++t) {
        int stride = 1;
#pragma unroll
        for (int s = t + 1; s < D; ++s) stride *= NP;
        const int qt = (q / stride) % NP;
        const int base = q - qt * stride;
        const int beg = __ldg(row_ptr + e * D + t);
        const int end = __ldg(row_ptr + e * D + t + 1);
        const T* bt = blocks + size_t(t) * nblocks * NP * NP + qt;
        // four neighbours per pass: their indices, block entries and values are independent loads
        // issued together; the multiply-adds keep the neighbour order
        int i = beg;
        for (; i + 4 <= end; i += 4) {
            int sv[4], bv[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                sv[j] = __ldg(src + i + j);
                bv[j] = __ldg(blk + i + j);
            }
            T mv[4][NP], xv[4][NP];
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    mv[j][p] = __ldg(bt + bv[j] * NP * NP + p * NP);
                    xv[j][p] = T(__ldg(xs + int64_t(sv[j]) * B + base + p * stride));
                }
#pragma unroll
            for (int j = 0; j < 4; ++j)
#pragma unroll
                for (int p = 0; p < NP; ++p) acc = fma(mv[j][p], xv[j][p], acc);
        }
        for (; i < end; ++i) {
            const int s = __ldg(src + i);
            const T* m = bt + __ldg(blk + i) * NP * NP;
            const X* x = xs + int64_t(s) * B + base;
#pragma unroll
            for (int p = 0; p < NP; ++p) acc = fma(__ldg(m + p * NP), T(__ldg(x + p * stride)), acc);
        }
    }
    if (df.out_hi) {
        df_stage_update(df, gid, float(acc));
        return;
    }
    const double rhs = double(acc);
    double v;
    if (rk.mode == 0) {
        v = rhs;
    } else {
        v = rk_combine(rk.a, un[gid], rk.b, us[gid], rk.dt, rhs);
    }
    out[gid] = v;
    if (shadow_out) shadow_out[gid] = float(v);
}

// Column variant: a CTA owns G whole elements (G = 256 / C, C = B / NP columns
// of a block along one dimension).  In dimension t thread (g, c) reads the NP
// neighbour values of column c once and produces all NP outputs of that
// column (NP^2 FMAs per NP loads instead of NP FMAs per NP loads), adding
// them into the element's block in shared memory; the dimensions are
// separated by barriers so every output has one writer per dimension.  The
// fused RK epilogue then streams the G blocks out coalesced.
template <typename T, int N>
struct BlockRegs {
    T v[N];
};

// load a padded 1D block (N entries, N a multiple of 4 floats / 2 doubles) with vector loads
template <int N>
__device__ __forceinline__ BlockRegs<float, N> load_block(const float* m) {
    BlockRegs<float, N> r;
#pragma unroll
    for (int j = 0; j < N / 4; ++j) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(m) + j);
        r.v[4 * j] = v.x; r.v[4 * j + 1] = v.y; r.v[4 * j + 2] = v.z; r.v[4 * j + 3] = v.w;
    }
    return r;
}
template <int N>
__device__ __forceinline__ BlockRegs<double, N> load_block(const double* m) {
    BlockRegs<double, N> r;
#pragma unroll
    for (int j = 0; j < N / 2; ++j) {
        const double2 v = __ldg(reinterpret_cast<const double2*>(m) + j);
        r.v[2 * j] = v.x; r.v[2 * j + 1] = v.y;
    }
    return r;
}

template <int D, int NP, typename T, typename X>
__global__ void __launch_bounds__(256) linear_col_kernel(const double* __restrict__ us, const X* __restrict__ xs,
                                                         const double* un, double* out, float* shadow_out,
                                                         const int32_t* __restrict__ row_ptr,
                                                         const int2* __restrict__ pairs,
                                                         const T* __restrict__ blocks, int nblocks, int64_t num_elements,
                                                         StageCoef rk, DFState df) {
    constexpr int B = IPow<NP, D>::v;
    constexpr int C = B / NP;
    constexpr int G = 256 / C;
    constexpr int BS = (NP * NP + 3) / 4 * 4;  // padded block stride (16-byte vector loads)
    __shared__ T y[G * B];
    const int tid = threadIdx.x;
    const int g = tid / C, c = tid - (tid / C) * C;
    const int64_t e = int64_t(blockIdx.x) * G + g;
    const bool active = (g < G) && (e < num_elements);
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
            T acc[NP];
#pragma unroll
            for (int q = 0; q < NP; ++q) acc[q] = T(0);
            const int beg = __ldg(row_ptr + e * D + t);
            const int end = __ldg(row_ptr + e * D + t + 1);
            const T* bt = blocks + size_t(t) * nblocks * BS;
            for (int i = beg; i < end; ++i) {
                const int2 pr = __ldg(pairs + i);  // (neighbour element, block id)
                const BlockRegs<T, BS> m = load_block<BS>(bt + size_t(pr.y) * BS);
                const X* x = xs + int64_t(pr.x) * B + base;
                T xv[NP];
#pragma unroll
                for (int p = 0; p < NP; ++p) xv[p] = T(__ldg(x + p * stride));
#pragma unroll
                for (int p = 0; p < NP; ++p)
#pragma unroll
                    for (int q = 0; q < NP; ++q) acc[q] = fma(m.v[p * NP + q], xv[p], acc[q]);
            }
            T* yb = y + g * B + base;
#pragma unroll
            for (int q = 0; q < NP; ++q) yb[q * stride] += acc[q];
        }
        __syncthreads();
    }
    const int64_t first = int64_t(blockIdx.x) * G * B;
    const int64_t total = num_elements * B;
    for (int i = tid; i < G * B; i += blockDim.x) {
        const int64_t gid = first + i;
        if (gid >= total) break;
        if (df.out_hi) {
            df_stage_update(df, gid, float(y[i]));
            continue;
        }
        const double rhs = double(y[i]);
        const double v = rk.mode == 0 ? rhs : rk_combine(rk.a, un[gid], rk.b, us[gid], rk.dt, rhs);
        out[gid] = v;
        if (shadow_out) shadow_out[gid] = float(v);
    }
}

template <int D, int NP, typename T, typename X>
static cudaError_t launch_col_t(const LinearLaunch& L, const T* blocks, const X* xs, StageCoef rk, cudaStream_t st) {
    constexpr int B = IPow<NP, D>::v;
    constexpr int C = B / NP;
    if constexpr (C > 256) {
        return cudaErrorInvalidValue;
    } else {
        constexpr int G = 256 / C;
        if (L.num_elements == 0) return cudaSuccess;
        const int64_t grid = (L.num_elements + G - 1) / G;
        const T* padded = nullptr;
        if constexpr (sizeof(T) == 4) padded = L.blocks32p; else padded = L.blocks64p;
        linear_col_kernel<D, NP, T, X><<<unsigned(grid), 256, 0, st>>>(L.us, xs, L.un, L.out, L.shadow_out, L.row_ptr,
                                                                      L.pairs, padded, L.num_blocks, L.num_elements, rk,
                                                                      L.df);
        return cudaGetLastError();
    }
}

// ---- column variant fed by bulk asynchronous copies (mixed precision) --------
// One warp (one CTA) per element; lane l owns the columns c = l + 32 j of the
// block along the current dimension.  The element's neighbour blocks (all
// dimensions, in CSR order) stream into a ring of kRing shared-memory slots
// by cp.async.bulk together with their 1D operator blocks, completion
// signalled on one mbarrier per slot; lane 0 refills a slot as soon as the
// warp has read it, so no global load sits on a neighbour's critical path.  The column reads come from
// shared memory and each 1D block is loaded once per lane for all of its
// columns, so a neighbour costs the warp a few dozen instructions besides its
// multiply-adds (the one-thread-per-column variants spend most of their issue
// slots on per-neighbour overhead).  A block of B floats starts 16-byte
// aligned only when its index allows, so the copy takes the aligned superset
// (at most 12 bytes either side, inside the allocation: the FP32 state arrays
// have 16-byte aligned bases and slack) and the reads skip the (e*B mod 4)
// leading floats.  Every wait is bounded (kSpinLimit polls) and agreed on by
// the whole warp; on a timeout the kernel sets *err, waits (bounded) for its
// copies still in flight and returns without writing.
// Configurations (LinearLaunch::tma_cfg, picked by the autotuner): RING slots,
// and whether the 1D operator block rides in the slot as a second bulk copy
// (LDG false) or is read by every lane from the L1-resident table, issued
// before the wait on the slot (LDG true, one bulk copy per neighbour).
constexpr uint32_t kSpinLimit = 1u << 22;
// ... and WARPS elements per CTA (independent warps, each with its own slots and accumulator),
// which lifts the limit of resident CTAs per SM when a warp's share of shared memory is small.
constexpr int kTmaRing[kTmaConfigs] = {3, 3, 6, 2, 4, 1, 1, 1};
constexpr bool kTmaLdg[kTmaConfigs] = {false, true, true, true, true, true, true, true};
constexpr int kTmaWarps[kTmaConfigs] = {1, 1, 1, 1, 1, 1, 2, 4};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for the completion of the phase with parity `parity`
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

template <int D, int NP, int kRing, bool LDG, int WPC>
__global__ void __launch_bounds__(32 * WPC) linear_tma_kernel(const float* __restrict__ xs,
                                                              const int32_t* __restrict__ row_ptr,
                                                              const int2* __restrict__ pairs,
                                                              const float* __restrict__ blocks, int nblocks,
                                                              int64_t num_elements, DFState df, int* err, uint32_t wait_limit) {
    constexpr int B = IPow<NP, D>::v;
    constexpr int C = B / NP;
    constexpr int CPT = (C + 31) / 32;  // columns per lane
    constexpr int BS = (NP * NP + 3) / 4 * 4;
    constexpr int DATA = (B + 3) / 4 * 4 + 4;  // floats: an aligned superset of any block
    constexpr int SLOT = DATA + (LDG ? 0 : BS);  // then (copied) the 1D operator block
    __shared__ __align__(128) float ring_all[WPC * kRing * SLOT];
    __shared__ float y_all[WPC * B];
    __shared__ __align__(8) uint64_t full_all[WPC * kRing];
    __shared__ int lead_all[WPC * kRing];  // floats before the block in its slot
    __shared__ int bidx_all[WPC * kRing];  // LDG: the slot's 1D operator block in the table
    // warp w of the CTA owns element blockIdx.x * WPC + w and its own share of every array
    // (SLOT is a multiple of 4 floats, so every warp's slots stay 16-byte aligned)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* ring = ring_all + warp * kRing * SLOT;
    float* y = y_all + warp * B;
    uint64_t* full = full_all + warp * kRing;
    int* lead = lead_all + warp * kRing;
    int* bidx = bidx_all + warp * kRing;
    const int64_t e = int64_t(blockIdx.x) * WPC + warp;
    if (e >= num_elements) return;
    for (int i = lane; i < B; i += 32) y[i] = 0.f;
    const int beg = __ldg(row_ptr + e * D), n = __ldg(row_ptr + e * D + D) - beg;
    if (lane == 0) {
        for (int b = 0; b < kRing; ++b) mbar_init(&full[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    int issued = 0, idim = 0;  // lane 0: neighbours issued, dimension of the next one
    auto issue = [&]() {       // next neighbour of the element into slot issued % kRing (lane 0)
        const int kk = issued;
        while (kk >= __ldg(row_ptr + e * D + idim + 1) - beg) ++idim;
        const int2 pr = __ldg(pairs + beg + kk);
        const uintptr_t a = reinterpret_cast<uintptr_t>(xs + int64_t(pr.x) * B);
        const uintptr_t a0 = a & ~uintptr_t(15);
        const uint32_t bytes = uint32_t(((a + uintptr_t(B) * 4 + 15) & ~uintptr_t(15)) - a0);
        float* dst = ring + (kk % kRing) * SLOT;
        lead[kk % kRing] = int((a - a0) / 4);
        uint64_t* fb = &full[kk % kRing];
        if constexpr (LDG) {
            bidx[kk % kRing] = idim * nblocks + pr.y;
            mbar_expect_tx(fb, bytes);
            bulk_copy_g2s(dst, reinterpret_cast<const void*>(a0), bytes, fb);
        } else {
            mbar_expect_tx(fb, bytes + uint32_t(BS * sizeof(float)));
            bulk_copy_g2s(dst, reinterpret_cast<const void*>(a0), bytes, fb);
            bulk_copy_g2s(dst + DATA, blocks + (size_t(idim) * nblocks + pr.y) * BS, uint32_t(BS * sizeof(float)), fb);
        }
        ++issued;
    };
    if (lane == 0)
        while (issued < n && issued < kRing) issue();
    __syncwarp();
    bool failed = false;
    int k = 0, slot = 0;
    uint32_t parity = 0;  // bit b: phase parity of slot b's next completion
    for (int t = 0; t < D && !failed; ++t) {
        int stride = 1;
#pragma unroll
        for (int s2 = t + 1; s2 < D; ++s2) stride *= NP;
        int base[CPT];
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const int c = lane + 32 * j;
            base[j] = (c / stride) * stride * NP + c % stride;
        }
        float acc[CPT][NP];
#pragma unroll
        for (int j = 0; j < CPT; ++j)
#pragma unroll
            for (int q = 0; q < NP; ++q) acc[j][q] = 0.f;
        const int kend = __ldg(row_ptr + e * D + t + 1) - beg;
        for (; k < kend; ++k) {
            float m[BS];
            if constexpr (LDG) {  // the operator block's loads are in flight during the wait
                const float4* g4 = reinterpret_cast<const float4*>(blocks + size_t(bidx[slot]) * BS);
#pragma unroll
                for (int jj = 0; jj < BS / 4; ++jj) {
                    const float4 v = __ldg(g4 + jj);
                    m[4 * jj] = v.x; m[4 * jj + 1] = v.y; m[4 * jj + 2] = v.z; m[4 * jj + 3] = v.w;
                }
            }
            const bool ok = mbar_wait_bounded(&full[slot], (parity >> slot) & 1u, wait_limit);
            if (__any_sync(0xffffffffu, !ok)) {
                failed = true;
                break;
            }
            parity ^= 1u << slot;
            const float* x = ring + slot * SLOT + lead[slot];
            if constexpr (!LDG) {
                const float4* m4 = reinterpret_cast<const float4*>(ring + slot * SLOT + DATA);
#pragma unroll
                for (int jj = 0; jj < BS / 4; ++jj) {
                    const float4 v = m4[jj];
                    m[4 * jj] = v.x; m[4 * jj + 1] = v.y; m[4 * jj + 2] = v.z; m[4 * jj + 3] = v.w;
                }
            }
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                if (C % 32 == 0 || lane + 32 * j < C) {
                    float xv[NP];
#pragma unroll
                    for (int p = 0; p < NP; ++p) xv[p] = x[base[j] + p * stride];
#pragma unroll
                    for (int p = 0; p < NP; ++p)
#pragma unroll
                        for (int q = 0; q < NP; ++q) acc[j][q] = fmaf(m[p * NP + q], xv[p], acc[j][q]);
                }
            }
            __syncwarp();  // the warp has read slot `slot`
            if (lane == 0 && issued < n) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue();
            }
            __syncwarp();  // lead[] of the refilled slot is written before any lane reads it
            slot = slot + 1 == kRing ? 0 : slot + 1;
        }
        if (failed) break;
#pragma unroll
        for (int j = 0; j < CPT; ++j)
            if (C % 32 == 0 || lane + 32 * j < C)
#pragma unroll
                for (int q = 0; q < NP; ++q) y[base[j] + q * stride] += acc[j][q];
        __syncwarp();  // next dimension: another column partition
    }
    if (failed) {
        if (lane == 0) {
            atomicExch(err, 1);
            // let the copies still in flight land before the CTA's shared memory is released
            for (int k2 = k; k2 < issued; ++k2) {
                const int s2 = k2 % kRing;
                mbar_wait_bounded(&full[s2], (parity >> s2) & 1u, 1u << 16);
                parity ^= 1u << s2;
            }
        }
        return;
    }
    for (int i = lane; i < B; i += 32) df_stage_update(df, e * B + i, y[i]);
}

// the rings, the accumulators and the mbarriers must fit the static shared-memory limit (48 KB)
constexpr bool tma_fits(int B, int np, int ring, bool ldg, int warps) {
    return B / np <= 256 &&
           size_t(warps) * (size_t(ring * ((B + 3) / 4 * 4 + 4 + (ldg ? 0 : 16)) + B) * sizeof(float) + 512) <=
               48 * 1024;
}

template <int D, int NP, int CFG>
static cudaError_t launch_tma_cfg(const LinearLaunch& L, cudaStream_t st) {
    constexpr int B = IPow<NP, D>::v;
    constexpr int W = kTmaWarps[CFG];
    if constexpr (!tma_fits(B, NP, kTmaRing[CFG], kTmaLdg[CFG], W)) {
        return cudaErrorInvalidValue;
    } else {
        if (L.num_elements == 0) return cudaSuccess;
        const int64_t grid = (L.num_elements + W - 1) / W;
        linear_tma_kernel<D, NP, kTmaRing[CFG], kTmaLdg[CFG], W><<<unsigned(grid), 32 * W, 0, st>>>(
            L.us_shadow, L.row_ptr, L.pairs, L.blocks32p, L.num_blocks, L.num_elements, L.df, L.err, L.wait_limit);
        return cudaGetLastError();
    }
}

// ---- tensor-core variant: the bulk-copy ring feeding 3xTF32 mma.sync ------------
// The same data movement as linear_tma_kernel (one warp per element, its neighbour blocks streamed
// into a ring of shared-memory slots by bulk copies, bounded mbarrier waits), with the per-dimension
// contraction Y[c][q] += sum_{s, p} X_s[c][p] M_s[p][q] on the tensor pipe: the columns c of the
// block are the MMA's M (16-row tiles), the output index q its N (NP of 8 used), and (neighbour, p)
// its K (8 / NP neighbours per k8 step, the rest zero).  Each FP32 operand is split into a TF32
// high part and a TF32 remainder, and the three products lo*hi + hi*lo + hi*hi accumulate in FP32
// (3xTF32, about FP32 accuracy).  Fragment layouts of mma.m16n8k8 (tf32, row.col): lane = 4 g + t;
// A (16 x 8): a0 (g, t), a1 (g + 8, t), a2 (g, t + 4), a3 (g + 8, t + 4); B (8 x 8): b0 (t, g),
// b1 (t + 4, g); D (16 x 8): d0 (g, 2t), d1 (g, 2t + 1), d2 (g + 8, 2t), d3 (g + 8, 2t + 1).
constexpr int kMmaRing = 4;

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// x = hi + lo with hi = tf32(x) and lo = tf32(x - hi) (the difference is exact in FP32)
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
    hi = to_tf32(x);
    lo = to_tf32(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int D, int NP>
__global__ void __launch_bounds__(32) linear_mma_kernel(const float* __restrict__ xs, const int32_t* __restrict__ row_ptr,
                                                        const int2* __restrict__ pairs, const float* __restrict__ blocks,
                                                        int nblocks, int64_t num_elements, DFState df, int* err,
                                                        uint32_t wait_limit) {
    constexpr int B = IPow<NP, D>::v;
    constexpr int C = B / NP;
    constexpr int MT = (C + 15) / 16;          // 16-row tiles of columns
    constexpr int NB = 8 / NP;                 // neighbours per k8 step
    constexpr int BS = (NP * NP + 3) / 4 * 4;
    constexpr int DATA = (B + 3) / 4 * 4 + 4;  // floats: an aligned superset of any block
    static_assert(NB <= kMmaRing, "a k8 step's neighbours must fit the ring");
    __shared__ __align__(128) float ring[kMmaRing * DATA];
    __shared__ float y[B];
    __shared__ __align__(8) uint64_t full[kMmaRing];
    __shared__ int lead[kMmaRing];
    __shared__ int bidx[kMmaRing];
    const int lane = threadIdx.x;
    const int64_t e = blockIdx.x;
    if (e >= num_elements) return;
    for (int i = lane; i < B; i += 32) y[i] = 0.f;
    const int beg = __ldg(row_ptr + e * D), n = __ldg(row_ptr + e * D + D) - beg;
    if (lane == 0) {
        for (int b = 0; b < kMmaRing; ++b) mbar_init(&full[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    int issued = 0, idim = 0;
    auto issue = [&]() {  // next neighbour into slot issued % kMmaRing (lane 0)
        const int kk = issued;
        while (kk >= __ldg(row_ptr + e * D + idim + 1) - beg) ++idim;
        const int2 pr = __ldg(pairs + beg + kk);
        const uintptr_t a = reinterpret_cast<uintptr_t>(xs + int64_t(pr.x) * B);
        const uintptr_t a0 = a & ~uintptr_t(15);
        const uint32_t bytes = uint32_t(((a + uintptr_t(B) * 4 + 15) & ~uintptr_t(15)) - a0);
        const int sl = kk % kMmaRing;
        lead[sl] = int((a - a0) / 4);
        bidx[sl] = idim * nblocks + pr.y;
        mbar_expect_tx(&full[sl], bytes);
        bulk_copy_g2s(ring + sl * DATA, reinterpret_cast<const void*>(a0), bytes, &full[sl]);
        ++issued;
    };
    if (lane == 0)
        while (issued < n && issued < kMmaRing) issue();
    __syncwarp();
    const int g = lane >> 2, t4 = lane & 3;
    // this lane's two k-columns of A (and rows of B): kc = t4 and t4 + 4 -> neighbour j, index p
    const int j0 = t4 / NP, p0 = t4 % NP, j1 = (t4 + 4) / NP, p1 = (t4 + 4) % NP;
    bool failed = false;
    int k = 0, slot = 0;
    uint32_t parity = 0;
    for (int t = 0; t < D && !failed; ++t) {
        int stride = 1;
#pragma unroll
        for (int s2 = t + 1; s2 < D; ++s2) stride *= NP;
        // offsets of the lane's rows g and g + 8 of every tile (columns c; -1 past the last column)
        int rb[MT][2];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int c = 16 * mt + g + 8 * h;
                rb[mt][h] = c < C ? (c / stride) * stride * NP + c % stride : -1;
            }
        float acc[MT][4];
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[mt][r] = 0.f;
        const int kend = __ldg(row_ptr + e * D + t + 1) - beg;
        while (k < kend) {
            const int nv = min(NB, kend - k);
            bool ok = true;
            for (int j = 0; j < nv; ++j) {
                const int sl = (slot + j) % kMmaRing;
                ok = ok && mbar_wait_bounded(&full[sl], (parity >> sl) & 1u, wait_limit);
            }
            if (__any_sync(0xffffffffu, !ok)) {
                failed = true;
                break;
            }
            for (int j = 0; j < nv; ++j) parity ^= 1u << ((slot + j) % kMmaRing);
            const bool u0 = j0 < nv, u1 = j1 < nv;
            const int s0 = (slot + j0) % kMmaRing, s1 = (slot + j1) % kMmaRing;
            // B: this lane's entries M_j[p][q = g] of the step's neighbours (zero outside)
            float bv0 = 0.f, bv1 = 0.f;
            if (g < NP) {
                if (u0) bv0 = __ldg(blocks + size_t(bidx[s0]) * BS + p0 * NP + g);
                if (u1) bv1 = __ldg(blocks + size_t(bidx[s1]) * BS + p1 * NP + g);
            }
            uint32_t bh0, bl0, bh1, bl1;
            split_tf32(bv0, bh0, bl0);
            split_tf32(bv1, bh1, bl1);
            const float* x0 = ring + s0 * DATA + lead[s0] + p0 * stride;
            const float* x1 = ring + s1 * DATA + lead[s1] + p1 * stride;
#pragma unroll
            for (int mt = 0; mt < MT; ++mt) {
                const float a0 = (u0 && rb[mt][0] >= 0) ? x0[rb[mt][0]] : 0.f;
                const float a1 = (u0 && rb[mt][1] >= 0) ? x0[rb[mt][1]] : 0.f;
                const float a2 = (u1 && rb[mt][0] >= 0) ? x1[rb[mt][0]] : 0.f;
                const float a3 = (u1 && rb[mt][1] >= 0) ? x1[rb[mt][1]] : 0.f;
                uint32_t ah0, al0, ah1, al1, ah2, al2, ah3, al3;
                split_tf32(a0, ah0, al0);
                split_tf32(a1, ah1, al1);
                split_tf32(a2, ah2, al2);
                split_tf32(a3, ah3, al3);
                mma_tf32(acc[mt], al0, al1, al2, al3, bh0, bh1);
                mma_tf32(acc[mt], ah0, ah1, ah2, ah3, bl0, bl1);
                mma_tf32(acc[mt], ah0, ah1, ah2, ah3, bh0, bh1);
            }
            __syncwarp();  // the warp has read the step's slots
            if (lane == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                for (int j = 0; j < nv && issued < n; ++j) issue();
            }
            __syncwarp();  // lead[] / bidx[] of the refilled slots are written before any lane reads them
            k += nv;
            slot = (slot + nv) % kMmaRing;
        }
        if (failed) break;
        // D fragment (rows g, g + 8; columns q = 2 t4, 2 t4 + 1) into the element's accumulator
#pragma unroll
        for (int mt = 0; mt < MT; ++mt)
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (rb[mt][h] >= 0) {
                    if (2 * t4 < NP) y[rb[mt][h] + 2 * t4 * stride] += acc[mt][2 * h];
                    if (2 * t4 + 1 < NP) y[rb[mt][h] + (2 * t4 + 1) * stride] += acc[mt][2 * h + 1];
                }
        __syncwarp();
    }
    if (failed) {
        if (lane == 0) {
            atomicExch(err, 1);
            for (int k2 = k; k2 < issued; ++k2) {
                const int s2 = k2 % kMmaRing;
                mbar_wait_bounded(&full[s2], (parity >> s2) & 1u, 1u << 16);
                parity ^= 1u << s2;
            }
        }
        return;
    }
    for (int i = lane; i < B; i += 32) df_stage_update(df, e * B + i, y[i]);
}

constexpr bool mma_fits(int B, int np) {
    return B / np <= 256 && 8 / np >= 1 && size_t(kMmaRing * ((B + 3) / 4 * 4 + 4) + B) * sizeof(float) + 256 <= 48 * 1024;
}

template <int D, int NP>
static cudaError_t launch_mma_t(const LinearLaunch& L, cudaStream_t st) {
    constexpr int B = IPow<NP, D>::v;
    if constexpr (!mma_fits(B, NP)) {
        return cudaErrorInvalidValue;
    } else {
        if (L.num_elements == 0) return cudaSuccess;
        linear_mma_kernel<D, NP><<<unsigned(L.num_elements), 32, 0, st>>>(
            L.us_shadow, L.row_ptr, L.pairs, L.blocks32p, L.num_blocks, L.num_elements, L.df, L.err, L.wait_limit);
        return cudaGetLastError();
    }
}

bool linear_mma_supported(int dim, int np) {
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    return np >= 2 && np <= 4 && mma_fits(B, np);
}

// ---- batched solves on the bulk-copy ring with the FP32-pair stage state ------------------------
// linear_tma_kernel for a batch of independent solves: element e belongs to solve s = solve_of[e],
// whose velocity c_s,t scales dimension t's contraction after the sum over neighbours (the 1D blocks
// u_vx + upwind flux come from the table of the flux side sign(c_s,t)) and whose step dt_s enters
// the double-float stage update.  Same ring, bounded waits and drain as linear_tma_kernel.
template <int D, int NP, int kRing, int WPC>
__global__ void __launch_bounds__(32 * WPC) batch_ring_kernel(BatchRingLaunch L) {
    constexpr int B = IPow<NP, D>::v;
    constexpr int C = B / NP;
    constexpr int CPT = (C + 31) / 32;
    constexpr int BS = (NP * NP + 3) / 4 * 4;
    constexpr int DATA = (B + 3) / 4 * 4 + 4;
    __shared__ __align__(128) float ring_all[WPC * kRing * DATA];
    __shared__ float y_all[WPC * B];
    __shared__ __align__(8) uint64_t full_all[WPC * kRing];
    __shared__ int lead_all[WPC * kRing];
    __shared__ int bidx_all[WPC * kRing];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float* ring = ring_all + warp * kRing * DATA;
    float* y = y_all + warp * B;
    uint64_t* full = full_all + warp * kRing;
    int* lead = lead_all + warp * kRing;
    int* bidx = bidx_all + warp * kRing;
    const int64_t e = int64_t(blockIdx.x) * WPC + warp;
    if (e >= L.num_elements) return;
    const int solve = __ldg(L.solve_of + e);
    for (int i = lane; i < B; i += 32) y[i] = 0.f;
    const int64_t beg = __ldg(L.row_ptr + e * D);
    const int n = int(__ldg(L.row_ptr + e * D + D) - beg);
    if (lane == 0) {
        for (int b = 0; b < kRing; ++b) mbar_init(&full[b], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    int issued = 0, idim = 0;
    auto issue = [&]() {  // next neighbour into slot issued % kRing (lane 0)
        const int kk = issued;
        while (kk >= int(__ldg(L.row_ptr + e * D + idim + 1) - beg)) ++idim;
        const int2 pr = __ldg(L.pairs + beg + kk);
        const uintptr_t a = reinterpret_cast<uintptr_t>(L.xs + int64_t(pr.x) * B);
        const uintptr_t a0 = a & ~uintptr_t(15);
        const uint32_t bytes = uint32_t(((a + uintptr_t(B) * 4 + 15) & ~uintptr_t(15)) - a0);
        const int sl = kk % kRing;
        lead[sl] = int((a - a0) / 4);
        const int side = __ldg(L.coef + solve * D + idim) >= 0.f ? 0 : 1;
        bidx[sl] = side * L.num_blocks + pr.y;
        mbar_expect_tx(&full[sl], bytes);
        bulk_copy_g2s(ring + sl * DATA, reinterpret_cast<const void*>(a0), bytes, &full[sl]);
        ++issued;
    };
    if (lane == 0)
        while (issued < n && issued < kRing) issue();
    __syncwarp();
    bool failed = false;
    int k = 0, slot = 0;
    uint32_t parity = 0;
    for (int t = 0; t < D && !failed; ++t) {
        int stride = 1;
#pragma unroll
        for (int s2 = t + 1; s2 < D; ++s2) stride *= NP;
        int base[CPT];
#pragma unroll
        for (int j = 0; j < CPT; ++j) {
            const int c = lane + 32 * j;
            base[j] = (c / stride) * stride * NP + c % stride;
        }
        float acc[CPT][NP];
#pragma unroll
        for (int j = 0; j < CPT; ++j)
#pragma unroll
            for (int q = 0; q < NP; ++q) acc[j][q] = 0.f;
        const int kend = int(__ldg(L.row_ptr + e * D + t + 1) - beg);
        for (; k < kend; ++k) {
            float m[BS];
            {
                const float4* g4 = reinterpret_cast<const float4*>(L.blocks + size_t(bidx[slot]) * BS);
#pragma unroll
                for (int jj = 0; jj < BS / 4; ++jj) {
                    const float4 v = __ldg(g4 + jj);
                    m[4 * jj] = v.x; m[4 * jj + 1] = v.y; m[4 * jj + 2] = v.z; m[4 * jj + 3] = v.w;
                }
            }
            const bool ok = mbar_wait_bounded(&full[slot], (parity >> slot) & 1u, L.wait_limit);
            if (__any_sync(0xffffffffu, !ok)) {
                failed = true;
                break;
            }
            parity ^= 1u << slot;
            const float* x = ring + slot * DATA + lead[slot];
#pragma unroll
            for (int j = 0; j < CPT; ++j) {
                if (C % 32 == 0 || lane + 32 * j < C) {
                    float xv[NP];
#pragma unroll
                    for (int p = 0; p < NP; ++p) xv[p] = x[base[j] + p * stride];
#pragma unroll
                    for (int p = 0; p < NP; ++p)
#pragma unroll
                        for (int q = 0; q < NP; ++q) acc[j][q] = fmaf(m[p * NP + q], xv[p], acc[j][q]);
                }
            }
            __syncwarp();
            if (lane == 0 && issued < n) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                issue();
            }
            __syncwarp();
            slot = slot + 1 == kRing ? 0 : slot + 1;
        }
        if (failed) break;
        const float ct = __ldg(L.coef + solve * D + t);
#pragma unroll
        for (int j = 0; j < CPT; ++j)
            if (C % 32 == 0 || lane + 32 * j < C)
#pragma unroll
                for (int q = 0; q < NP; ++q) y[base[j] + q * stride] += ct * acc[j][q];
        __syncwarp();
    }
    if (failed) {
        if (lane == 0) {
            atomicExch(L.err, 1);
            for (int k2 = k; k2 < issued; ++k2) {
                const int s2 = k2 % kRing;
                mbar_wait_bounded(&full[s2], (parity >> s2) & 1u, 1u << 16);
                parity ^= 1u << s2;
            }
        }
        return;
    }
    DFState df = L.df;
    df.dt = __ldg(L.dt + solve);
    for (int i = lane; i < B; i += 32) df_stage_update(df, e * B + i, y[i]);
}

constexpr bool batch_ring_fits(int B, int np, int ring, int warps) {
    return B / np <= 256 && size_t(warps) * (size_t(ring * ((B + 3) / 4 * 4 + 4)) + B) * sizeof(float) + 512 <= 48 * 1024;
}

template <int D, int NP, int R, int W>
static cudaError_t launch_batch_ring_cfg(const BatchRingLaunch& L, cudaStream_t st) {
    constexpr int B = IPow<NP, D>::v;
    if constexpr (!batch_ring_fits(B, NP, R, W)) {
        return cudaErrorInvalidValue;
    } else {
        if (L.num_elements == 0) return cudaSuccess;
        batch_ring_kernel<D, NP, R, W><<<unsigned((L.num_elements + W - 1) / W), 32 * W, 0, st>>>(L);
        return cudaGetLastError();
    }
}

template <int D, int NP>
static cudaError_t launch_batch_ring_t(const BatchRingLaunch& L, cudaStream_t st) {
    switch (L.cfg) {
        case 0: return launch_batch_ring_cfg<D, NP, 1, 1>(L, st);
        case 1: return launch_batch_ring_cfg<D, NP, 1, 2>(L, st);
        case 2: return launch_batch_ring_cfg<D, NP, 1, 4>(L, st);
        case 3: return launch_batch_ring_cfg<D, NP, 2, 1>(L, st);
        case 4: return launch_batch_ring_cfg<D, NP, 2, 2>(L, st);
        case 5: return launch_batch_ring_cfg<D, NP, 2, 4>(L, st);
        default: return cudaErrorInvalidValue;
    }
}

constexpr int kBatchRingShape[kBatchRingConfigs][2] = {{1, 1}, {1, 2}, {1, 4}, {2, 1}, {2, 2}, {2, 4}};

bool batch_ring_supported(int dim, int np, int cfg) {
    if (cfg < 0 || cfg >= kBatchRingConfigs || np < 2 || np > 4 || dim < 1 || dim > 6) return false;
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    return batch_ring_fits(B, np, kBatchRingShape[cfg][0], kBatchRingShape[cfg][1]);
}

cudaError_t launch_batch_ring(const BatchRingLaunch& L, cudaStream_t st) {
    if (!batch_ring_supported(L.dim, L.np, L.cfg)) return cudaErrorInvalidValue;
#define AMDG_RCASE(D, NP) \
    if (L.dim == D && L.np == NP) return launch_batch_ring_t<D, NP>(L, st);
    AMDG_RCASE(1, 2) AMDG_RCASE(1, 3) AMDG_RCASE(1, 4)
    AMDG_RCASE(2, 2) AMDG_RCASE(2, 3) AMDG_RCASE(2, 4)
    AMDG_RCASE(3, 2) AMDG_RCASE(3, 3) AMDG_RCASE(3, 4)
    AMDG_RCASE(4, 2) AMDG_RCASE(4, 3) AMDG_RCASE(4, 4)
    AMDG_RCASE(5, 2) AMDG_RCASE(5, 3) AMDG_RCASE(5, 4)
    AMDG_RCASE(6, 2) AMDG_RCASE(6, 3)
#undef AMDG_RCASE
    return cudaErrorInvalidValue;
}

template <int D, int NP>
static cudaError_t launch_tma_t(const LinearLaunch& L, cudaStream_t st) {
    switch (L.tma_cfg) {
        case 1: return launch_tma_cfg<D, NP, 1>(L, st);
        case 2: return launch_tma_cfg<D, NP, 2>(L, st);
        case 3: return launch_tma_cfg<D, NP, 3>(L, st);
        case 4: return launch_tma_cfg<D, NP, 4>(L, st);
        case 5: return launch_tma_cfg<D, NP, 5>(L, st);
        case 6: return launch_tma_cfg<D, NP, 6>(L, st);
        case 7: return launch_tma_cfg<D, NP, 7>(L, st);
        default: return launch_tma_cfg<D, NP, 0>(L, st);
    }
}

bool linear_tma_supported(int dim, int np, int cfg) {
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    if (cfg < 0 || cfg >= kTmaConfigs) return false;
    return tma_fits(B, np, kTmaRing[cfg], kTmaLdg[cfg], kTmaWarps[cfg]);
}

bool linear_col_supported(int dim, int np) {
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    return B / np <= 256;
}

template <int D, int NP, typename T, typename X>
static cudaError_t launch_linear_t(const LinearLaunch& L, const T* blocks, const X* xs, StageCoef rk, cudaStream_t st) {
    constexpr int B = IPow<NP, D>::v;
    const int64_t total = L.num_elements * B;
    if (total == 0) return cudaSuccess;
    // small grids: smaller CTAs until there are two per multiprocessor (a grid of a few thousand
    // coefficients otherwise runs on a few SMs, bound by their FP64 pipes)
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            sms = 152;
    }
    int threads = 256;
    while (threads > 32 && (total + threads - 1) / threads < 2 * int64_t(sms)) threads /= 2;
    const int64_t grid = (total + threads - 1) / threads;
    linear_apply_kernel<D, NP, T, X><<<unsigned(grid), threads, 0, st>>>(L.us, xs, L.un, L.out, L.shadow_out, L.row_ptr,
                                                                        L.src, L.blk, blocks, L.num_blocks, total, rk, L.df);
    return cudaGetLastError();
}

template <typename T, typename X>
static cudaError_t dispatch_linear(const LinearLaunch& L, const T* blocks, const X* xs, StageCoef rk, cudaStream_t st) {
    // variant 2 runs on the FP32-pair stage state only (float shadow input, FP32-pair output)
    // variant 3 (tensor cores) likewise
    bool tma = false, mma = false;
    if constexpr (std::is_same<T, float>::value && std::is_same<X, float>::value) {
        const bool df_state = L.df.out_hi && L.err && L.us_shadow;
        tma = L.variant == 2 && df_state;
        mma = L.variant == 3 && df_state;
    }
#define AMDG_CASE(D, NP)                                                                \
    if (L.dim == D && L.np == NP) {                                                       \
        if constexpr (std::is_same<T, float>::value && std::is_same<X, float>::value) {   \
            if (tma) return launch_tma_t<D, NP>(L, st);                                   \
            if (mma) return launch_mma_t<D, NP>(L, st);                                   \
        }                                                                                 \
        return L.variant >= 1 ? launch_col_t<D, NP, T, X>(L, blocks, xs, rk, st)          \
                              : launch_linear_t<D, NP, T, X>(L, blocks, xs, rk, st);      \
    }
    AMDG_CASE(1, 2) AMDG_CASE(1, 3) AMDG_CASE(1, 4)
    AMDG_CASE(2, 2) AMDG_CASE(2, 3) AMDG_CASE(2, 4)
    AMDG_CASE(3, 2) AMDG_CASE(3, 3) AMDG_CASE(3, 4)
    AMDG_CASE(4, 2) AMDG_CASE(4, 3) AMDG_CASE(4, 4)
    AMDG_CASE(5, 2) AMDG_CASE(5, 3) AMDG_CASE(5, 4)
    AMDG_CASE(6, 2) AMDG_CASE(6, 3) AMDG_CASE(6, 4)
#undef AMDG_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_linear(const LinearLaunch& L, bool mixed, StageCoef rk, cudaStream_t st) {
    if (!mixed) return dispatch_linear<double, double>(L, L.blocks64, L.us, rk, st);
    if (L.us_shadow) return dispatch_linear<float, float>(L, L.blocks32, L.us_shadow, rk, st);
    return dispatch_linear<float, double>(L, L.blocks32, L.us, rk, st);
}

__global__ void split_kernel(const double* __restrict__ in, float* __restrict__ hi, float* __restrict__ lo, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = in[i];
    const float h = __double2float_rn(d);
    hi[i] = h;
    lo[i] = __double2float_rn(d - double(h));
}

cudaError_t launch_split(const double* in, float* hi, float* lo, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    split_kernel<<<unsigned((n + 255) / 256), 256, 0, st>>>(in, hi, lo, n);
    return cudaGetLastError();
}

__global__ void merge_kernel(const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ out, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = double(hi[i]) + double(lo[i]);
}

cudaError_t launch_merge(const float* hi, const float* lo, double* out, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    merge_kernel<<<unsigned((n + 255) / 256), 256, 0, st>>>(hi, lo, out, n);
    return cudaGetLastError();
}

DFState df_stage(StageCoef rk) {
    DFState d{};
    d.ah = float(rk.a);
    d.al = float(rk.a - double(d.ah));
    d.bh = float(rk.b);
    d.bl = float(rk.b - double(d.bh));
    d.dt = float(rk.dt);
    return d;
}

__global__ void to_float_kernel(const double* __restrict__ in, float* __restrict__ out, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) out[i] = float(in[i]);
}

cudaError_t launch_to_float(const double* in, float* out, int64_t n, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    to_float_kernel<<<unsigned((n + 255) / 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

// ---- stage update for an externally computed rhs --------------------------
__global__ void stage_update_kernel(const double* un, double* u, const double* __restrict__ rhs,
                                    int64_t n, StageCoef rk) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) u[i] = rk_combine(rk.a, un[i], rk.b, u[i], rk.dt, rhs[i]);
}

cudaError_t launch_stage_update(const double* un, double* u, const double* rhs, int64_t n, StageCoef rk, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const int threads = 256;
    stage_update_kernel<<<unsigned((n + threads - 1) / threads), threads, 0, st>>>(un, u, rhs, n, rk);
    return cudaGetLastError();
}

// ---- separable initialisation ----------------------------------------------
// u[e][q] = sum_term prod_d coef1d[term][d][o_d*(k+1) + q_d]
// (DGSolution::init_elem_separable, DGSolution.cpp:170-184; same product order)
__global__ void init_separable_kernel(const int32_t* __restrict__ order, const double* __restrict__ coef1d, int dim, int np,
                                      int nb1, int nterms, int B, int64_t total, double* __restrict__ u) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= total) return;
    const int64_t e = gid / B;
    const int q = int(gid - e * B);
    int dig[8];
    int rem = q;
    for (int d = dim - 1; d >= 0; --d) { dig[d] = rem % np; rem /= np; }
    double sum = 0.0;
    for (int t = 0; t < nterms; ++t) {
        double v = 1.0;
        for (int d = 0; d < dim; ++d) v = __dmul_rn(v, coef1d[(size_t(t) * dim + d) * nb1 + order[e * dim + d] * np + dig[d]]);
        sum = __dadd_rn(sum, v);
    }
    u[gid] = sum;
}

cudaError_t launch_init_separable(const int32_t* order, const double* coef1d, int dim, int np, int nb1, int nterms,
                                  int64_t num_elements, double* u, cudaStream_t st) {
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    const int64_t total = num_elements * B;
    if (total == 0) return cudaSuccess;
    init_separable_kernel<<<unsigned((total + 255) / 256), 256, 0, st>>>(order, coef1d, dim, np, nb1, nterms, B, total, u);
    return cudaGetLastError();
}

// ---- FP64 reductions (deterministic two-pass) -------------------------------
// mode 0: sum u^2;  mode 1: sum (u^2 - 2 u prod_d c_exact) (split L2 error,
// DGSolution.cpp:217-256)
constexpr int kReduceThreads = 256;

__global__ void reduce_pass1(const double* __restrict__ u, const int32_t* __restrict__ order,
                             const double* __restrict__ coef1d, int dim, int np, int nb1, int B, int64_t total, int mode,
                             int nterms, double* __restrict__ partial) {
    __shared__ double sh[kReduceThreads];
    double s = 0.0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += int64_t(gridDim.x) * blockDim.x) {
        const double v = u[i];
        double term = v * v;
        if (mode == 1) {
            const int64_t e = i / B;
            int rem = int(i - e * B);
            int dig[8];
            for (int d = dim - 1; d >= 0; --d) { dig[d] = rem % np; rem /= np; }
            double c = 0.0;
            for (int t = 0; t < nterms; ++t) {
                double p = 1.0;
                for (int d = 0; d < dim; ++d) p *= coef1d[(size_t(t) * dim + d) * nb1 + order[e * dim + d] * np + dig[d]];
                c += p;
            }
            term -= 2.0 * v * c;
        }
        s += term;
    }
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void reduce_pass2(const double* __restrict__ partial, int n, double* __restrict__ result) {
    __shared__ double sh[kReduceThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += partial[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) result[0] = sh[0];
}

int reduce_partials_needed() { return kReduceBlocks + 1; }

cudaError_t launch_reduce(const double* u, const int32_t* order, const double* coef1d, int dim, int np, int nb1,
                          int64_t num_elements, int mode, double* scratch, cudaStream_t st, int nterms) {
    int B = 1;
    for (int d = 0; d < dim; ++d) B *= np;
    const int64_t total = num_elements * B;
    reduce_pass1<<<kReduceBlocks, kReduceThreads, 0, st>>>(u, order, coef1d, dim, np, nb1, B, total, mode, nterms, scratch);
    cudaError_t err = cudaGetLastError();
    if (err != cudaSuccess) return err;
    reduce_pass2<<<1, kReduceThreads, 0, st>>>(scratch, kReduceBlocks, scratch + kReduceBlocks);
    return cudaGetLastError();
}

}  // namespace amdg

namespace amdg {

// ---- adaptivity -----------------------------------------------------------------
// Indicator of every element: sqrt of the sum of squares of its block, summed in
// block order (DGAdapt::indicator_norm, DGAdapt.cpp:1018-1030; VecMultiD::norm).
__global__ void element_norm_kernel(const double* __restrict__ u, int B, int64_t E, double* __restrict__ out) {
    const int64_t e = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= E) return;
    const double* x = u + e * B;
    double s = 0.0;
    for (int q = 0; q < B; ++q) s = __dadd_rn(s, __dmul_rn(x[q], x[q]));
    out[e] = sqrt(s);
}

cudaError_t launch_element_norms(const double* u, int B, int64_t E, double* out, cudaStream_t st) {
    if (E == 0) return cudaSuccess;
    element_norm_kernel<<<unsigned((E + 127) / 128), 128, 0, st>>>(u, B, E, out);
    return cudaGetLastError();
}

// new[e] = old[map[e]] block-wise, zero where map[e] < 0 (elements created by refinement)
__global__ void remap_kernel(const double* __restrict__ old_u, const int32_t* __restrict__ map, int B, int64_t total,
                             double* __restrict__ new_u) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int64_t e = i / B;
    const int q = int(i - e * B);
    const int32_t src = map[e];
    new_u[i] = src >= 0 ? old_u[int64_t(src) * B + q] : 0.0;
}

cudaError_t launch_remap(const double* old_u, const int32_t* map, int B, int64_t E_new, double* new_u, cudaStream_t st) {
    const int64_t total = E_new * B;
    if (total == 0) return cudaSuccess;
    remap_kernel<<<unsigned((total + 255) / 256), 256, 0, st>>>(old_u, map, B, total, new_u);
    return cudaGetLastError();
}

}  // namespace amdg
