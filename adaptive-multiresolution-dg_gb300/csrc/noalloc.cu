// SSP-RK3 steps of the linear operator for callers that cannot allocate
// device memory.
//
// The stage vectors u1 and u2 live in one file-scope device array of fixed
// size instead of in memory allocated by amdg_linear_create.  Callers that
// cannot call cudaMalloc -- host callbacks launched with cudaLaunchHostFunc
// (which may not call CUDA at all), processes whose device memory is fully
// handed to another allocator, loops that must not allocate -- can step a
// small grid with this entry point.
//
// Limits and sharing:
//   * at most kNoAllocMaxDof coefficients (2 x 262,144 doubles = 4 MiB of
//     scratch, held by every device that loads the library until exit);
//   * every call shares the one array; it keeps the last call's contents.
//     Nothing needs clearing: each stage fully writes its stage vector before
//     any thread reads it;
//   * calls whose work overlaps on the GPU (different streams, different host
//     threads) race on the array and give wrong results; issue them in order.
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "amdg.h"
#include "amdg_internal.hpp"
#include "kernels.cuh"

namespace {

constexpr int64_t kNoAllocMaxDof = 262144;
constexpr int kMaxDevices = 64;

// u1 = [0, kNoAllocMaxDof), u2 = [kNoAllocMaxDof, 2*kNoAllocMaxDof)
static __device__ __align__(256) double g_rk3_scratch[2 * kNoAllocMaxDof];

std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of g_rk3_scratch on `device` (which must be current); the
// host-side symbol itself is not a device address.
amdg_status scratch_address(int device, double** out) {
    if (device < 0 || device >= kMaxDevices) return amdg::fail(AMDG_ERR_ARG, "device index beyond the set-up table");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_rk3_scratch);
        if (e != cudaSuccess)
            return amdg::fail(AMDG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_addr[device] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[device];
    return AMDG_OK;
}

}  // namespace

extern "C" amdg_status amdg_rk3ssp_steps_noalloc(amdg_linear_op* op, double* d_u, double dt, int nsteps,
                                                amdg_precision prec) {
    using namespace amdg;
    if (!op || !d_u || nsteps < 0 || !std::isfinite(dt)) return fail(AMDG_ERR_ARG, "bad arguments");
    if (prec != AMDG_PREC_FP64 && prec != AMDG_PREC_MIXED) return fail(AMDG_ERR_ARG, "bad precision");
    const amdg_grid* g = op->grid;
    if (op->built_version != g->version)
        return fail(AMDG_ERR_STATE, "the grid changed since the operator was last used; call amdg_rk3ssp_steps or "
                                    "amdg_linear_apply once (they rebuild the operator) before this entry point");
    if (g->dof > kNoAllocMaxDof)
        return fail(AMDG_ERR_CAPACITY, "grid has " + std::to_string(g->dof) +
                                           " coefficients; the allocation-free RK3 step holds at most " +
                                           std::to_string(kNoAllocMaxDof));
    cudaError_t e = cudaSetDevice(g->device);
    if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    double* scratch = nullptr;
    amdg_status s = scratch_address(g->device, &scratch);
    if (s != AMDG_OK) return s;
    double* u1 = scratch;
    double* u2 = scratch + kNoAllocMaxDof;
    cudaStream_t st = static_cast<cudaStream_t>(g->ctx->stream);
    LinearLaunch L{};
    // the operator's kernel variant; this call has no FP32 (hi, lo) stage state, so in mixed mode
    // the column variant reads the FP64 stage vectors and converts each value as it loads it
    // (the bulk-copy variant needs the FP32 state and is not taken)
    L.variant = op->variant[prec == AMDG_PREC_MIXED ? 1 : 0];
    L.dim = g->host.dim;
    L.np = g->host.k + 1;
    L.num_elements = g->host.num_elements;
    L.num_blocks = op->num_blocks;
    L.row_ptr = op->d_row_ptr;
    L.src = op->d_src;
    L.blk = op->d_blk;
    L.blocks64 = op->d_blocks64;
    L.blocks32 = op->d_blocks32;
    L.pairs = reinterpret_cast<const int2*>(op->d_pairs);
    L.blocks64p = op->d_blocks64p;
    L.blocks32p = op->d_blocks32p;
    const StageCoef coef[3] = {{1, 0.0, 1.0, dt}, {1, 3. / 4., 1. / 4., dt}, {1, 1. / 3., 2. / 3., dt}};
    for (int step = 0; step < nsteps; ++step) {
        const double* in[3] = {d_u, u1, u2};
        double* out[3] = {u1, u2, d_u};
        for (int stage = 0; stage < 3; ++stage) {
            L.us = in[stage];
            L.un = d_u;
            L.out = out[stage];
            e = launch_linear(L, prec == AMDG_PREC_MIXED, coef[stage], st);
            if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("linear stage: ") + cudaGetErrorString(e));
            g->ctx->launches++;
        }
    }
    return AMDG_OK;
}
