// Launch interfaces of the device kernels (kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace amdg {

// Stage update coefficients: mode 0 writes rhs; mode 1 writes a*un + b*(us + dt*rhs).
struct StageCoef {
    int mode;
    double a, b, dt;
};

#ifdef __CUDACC__
// a*un + b*(us + dt*rhs), each operation rounded (no FMA), as Eigen evaluates it
__device__ __forceinline__ double rk_combine(double a, double un, double b, double us, double dt, double rhs) {
    return __dadd_rn(__dmul_rn(a, un), __dmul_rn(b, __dadd_rn(us, __dmul_rn(dt, rhs))));
}
#endif

// Mixed-mode stage state as FP32 (hi, lo) pairs: the stage vectors stay at
// ~48-bit precision without touching the FP64 pipe (a double->float
// conversion or an FP64 add costs an FP64-pipe slot, 1/64 of the FP32 rate on
// this part).  hi doubles as the FP32 value read by the operator apply.
struct DFState {
    const float *us_hi, *us_lo, *un_hi, *un_lo;
    float *out_hi, *out_lo;  // out_hi == nullptr: FP64 epilogue
    float ah, al, bh, bl;    // stage coefficients a, b as (hi, lo)
    float dt;
};

struct LinearLaunch {
    int dim, np;
    int variant;             // 0: thread per output coefficient; 1: column variant (linear_col_supported);
                             // 2: column variant fed by bulk asynchronous copies (linear_tma_supported;
                             //    FP32-pair stage state only, else as 1); 3: the bulk-copy ring with the
                             //    contraction as 3xTF32 on the tensor pipe (linear_mma_supported; same state)
    int64_t num_elements;
    int num_blocks;
    const double* us;        // input coefficients of the stage
    const float* us_shadow;  // float copy of us (mixed mode), or null to convert on the fly
    float* shadow_out;       // receives float(out) when not null
    const double* un;        // coefficients at t_n (mode 1)
    double* out;             // rhs (mode 0) or updated coefficients (mode 1)
    const int32_t* row_ptr;  // CSR over (element, dimension)
    const int32_t* src;
    const int32_t* blk;
    const double* blocks64;
    const float* blocks32;
    const int2* pairs;        // column variant: (src, blk) interleaved
    const double* blocks64p;  // column variant: blocks padded to a multiple of 4 entries
    const float* blocks32p;
    DFState df;              // zero-initialised: FP64 epilogue
    int* err;                // variants 2, 3: set to 1 when a copy wait gives up (device flag)
    uint32_t wait_limit;     // variants 2, 3: polls of a copy wait before it gives up (0: at once)
    int tma_cfg;             // variant 2: ring depth / operator-block source (kernels.cu, kTmaRing, kTmaLdg)
};

// Batched solves: concatenated element tables, per-element solve index.
template <typename T, typename X>
struct BatchLaunch {
    int dim, np, mode;       // mode 0: rhs; 1: RK stage a*un + b*(us + dt[solve]*rhs)
    int threads;             // CTA size (the tile: threads / (np^(dim-1)) elements per CTA); 0 = 256
    double a, b;
    int64_t num_elements;
    int num_blocks;
    const double* us;
    const X* xs;             // neighbour values (us, or its float shadow)
    const double* un;
    double* out;
    float* shadow_out;
    const int64_t* row_ptr;  // CSR over (element, dimension)
    const int64_t* src;
    const int32_t* blk;
    const T* blocks;         // [2][num_blocks][np][np]: u_vx + ulft_vjp, u_vx + urgt_vjp
    const T* coef;           // [solve][dim] velocities
    const double* dt;        // [solve] step sizes
    const int32_t* solve_of; // [element]
    // T = float only: with df.out_hi set the stage vectors are FP32 (hi, lo) pairs (df, the step of
    // solve s is dt32[s]) and us / un / out / shadow_out are unused
    DFState df;
    const float* dt32;
    // when both are set: (src, blk) as int32 pairs and the table padded to (np^2 + 3) / 4 * 4
    // entries per block (vector loads)
    const int2* pairs;
    const T* blocks_p;
    // FP32-pair state only: 0 one CTA per tile; 1 persistent (grid of resident CTAs, static tile
    // order); 2 persistent, tiles taken from the counter `queue` (zero before the launch)
    int schedule;
    unsigned long long* queue;
    int sms;  // multiprocessors of the device (persistent grids)
};
template <typename T, typename X>
cudaError_t launch_batch(const BatchLaunch<T, X>& L, cudaStream_t st);
// CTA sizes launch_batch offers (those of at least (k+1)^(dim-1) threads fit at least one element)
constexpr int kBatchTileCount = 5;
constexpr int kBatchTiles[kBatchTileCount] = {64, 128, 256, 512, 1024};
bool batch_tile_supported(int dim, int np, int threads);
// the occupancy queries of the persistent schedules, run before any stream capture
cudaError_t batch_prepare_persistent(int dim, int np);

// Batched solves on the bulk-copy ring (kernels.cu, batch_ring_kernel): the stage input's FP32
// high parts (xs) stream into shared memory by bulk copies, the stage vectors are FP32 (hi, lo)
// pairs (df; df.dt unused: dt[solve] per element), one warp per element.  Configurations cfg:
// (ring slots, elements per CTA) = (1, 1), (1, 2), (1, 4), (2, 1), (2, 2), (2, 4).
constexpr int kBatchRingConfigs = 6;
struct BatchRingLaunch {
    int dim, np, cfg;
    int64_t num_elements;
    int num_blocks;
    const int64_t* row_ptr;  // CSR over (element, dimension)
    const int2* pairs;       // (src, blk)
    const float* blocks;     // [2][num_blocks][(np^2 + 3) / 4 * 4]: the two flux sides, padded
    const float* coef;       // [solve][dim]
    const float* dt;         // [solve]
    const int32_t* solve_of; // [element]
    const float* xs;         // stage input, high parts (16-byte aligned base, 16 bytes of slack)
    DFState df;
    int* err;
    uint32_t wait_limit;
};
bool batch_ring_supported(int dim, int np, int cfg);
cudaError_t launch_batch_ring(const BatchRingLaunch& L, cudaStream_t st);

// Batched solves, one warp per element (kernels_batch.cu, batch_warp_kernel): lane i holds
// coefficient i of the element block (blocks of at most 32 coefficients), each neighbour block is
// one coalesced load of its FP32 high parts, the 1D block one load of its np^2 entries, and the
// contraction along a dimension gathers the np values of a lane's fibre by warp shuffles; one CTA
// of 8 warps per 8 elements.  FP32 (hi, lo) stage state as BatchRingLaunch.
constexpr int kBatchWarpConfigs = 1;
struct BatchWarpLaunch {
    int dim, np, cfg;
    int64_t num_elements;
    int num_blocks;
    const int64_t* row_ptr;
    const int2* pairs;
    const float* blocks;     // padded as BatchRingLaunch
    const float* coef;
    const float* dt;
    const int32_t* solve_of;
    const float* xs;
    DFState df;
};
bool batch_warp_supported(int dim, int np, int cfg);
cudaError_t launch_batch_warp(const BatchWarpLaunch& L, cudaStream_t st);

constexpr int kReduceBlocks = 1216;  // 8 CTAs per SM on 152 SMs

cudaError_t launch_linear(const LinearLaunch& L, bool mixed, StageCoef rk, cudaStream_t st);
// Variant 2 needs the FP32 stage state with 16-byte aligned array bases and
// at least 16 bytes readable past the last coefficient.
constexpr int kTmaConfigs = 8;
bool linear_tma_supported(int dim, int np, int cfg = 0);
bool linear_col_supported(int dim, int np);
bool linear_mma_supported(int dim, int np);
// FP64 vector <-> FP32 (hi, lo) pairs
cudaError_t launch_split(const double* in, float* hi, float* lo, int64_t n, cudaStream_t st);
cudaError_t launch_merge(const float* hi, const float* lo, double* out, int64_t n, cudaStream_t st);
DFState df_stage(StageCoef rk);
cudaError_t launch_to_float(const double* in, float* out, int64_t n, cudaStream_t st);
cudaError_t launch_stage_update(const double* un, double* u, const double* rhs, int64_t n, StageCoef rk, cudaStream_t st);
cudaError_t launch_init_separable(const int32_t* order, const double* coef1d, int dim, int np, int nb1, int nterms,
                                  int64_t num_elements, double* u, cudaStream_t st);
// scratch: kReduceBlocks + 1 doubles; result in scratch[kReduceBlocks]
cudaError_t launch_reduce(const double* u, const int32_t* order, const double* coef1d, int dim, int np, int nb1,
                          int64_t num_elements, int mode, double* scratch, cudaStream_t st, int nterms = 1);
int reduce_partials_needed();
cudaError_t launch_element_norms(const double* u, int B, int64_t E, double* out, cudaStream_t st);
cudaError_t launch_remap(const double* old_u, const int32_t* map, int B, int64_t E_new, double* new_u, cudaStream_t st);

}  // namespace amdg
