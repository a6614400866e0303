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

struct LinearLaunch {
    int dim, np;
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
};

constexpr int kReduceBlocks = 1216;  // 8 CTAs per SM on 152 SMs

cudaError_t launch_linear(const LinearLaunch& L, bool mixed, StageCoef rk, cudaStream_t st);
cudaError_t launch_to_float(const double* in, float* out, int64_t n, cudaStream_t st);
cudaError_t launch_stage_update(const double* un, double* u, const double* rhs, int64_t n, StageCoef rk, cudaStream_t st);
cudaError_t launch_init_separable(const int32_t* order, const double* coef1d, int dim, int np, int nb1, int nterms,
                                  int64_t num_elements, double* u, cudaStream_t st);
// scratch: kReduceBlocks + 1 doubles; result in scratch[kReduceBlocks]
cudaError_t launch_reduce(const double* u, const int32_t* order, const double* coef1d, int dim, int np, int nb1,
                          int64_t num_elements, int mode, double* scratch, cudaStream_t st);
int reduce_partials_needed();
cudaError_t launch_element_norms(const double* u, int B, int64_t E, double* out, cudaStream_t st);
cudaError_t launch_remap(const double* old_u, const int32_t* map, int B, int64_t E_new, double* new_u, cudaStream_t st);

}  // namespace amdg
