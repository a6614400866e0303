// The reference's explicit time integrators as device objects (ODESolver.h:17-205):
// an amdg_ode holds the solution at t_n (ODESolver::init) and the solver's own
// right-hand-side vector, and advances the grid's coefficients one stage at a
// time from the grid's Element::rhs (add_rhs_to_eigenvec).  With them and the
// grid's rhs / prediction vectors, a reference driver's stage loop
// (example/07_vlasov_maxwell_adapt.cpp:278-320, 02_hyperbolic_05_burgers_adapt.cpp:
// 223-476) runs call for call on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>

#include "amdg_internal.hpp"
#include "kernels.cuh"
#include "kernels_lagr.cuh"
#include "device_alloc.cuh"

using namespace amdg;

#define AMDG_CK(...)                                                                                    \
    do {                                                                                                \
        cudaError_t amdg_err_ = (__VA_ARGS__);                                                          \
        if (amdg_err_ != cudaSuccess)                                                                   \
            return fail(AMDG_ERR_CUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(amdg_err_)); \
    } while (0)
#define AMDG_REQUIRE(cond, code, msg) \
    do {                              \
        if (!(cond)) return fail(code, msg); \
    } while (0)

namespace {

cudaStream_t stream_of(const amdg_grid* g) { return static_cast<cudaStream_t>(g->ctx->stream); }

// y += a x, evaluated as Eigen does it (one rounding for the product, one for the sum)
__global__ void axpy_kernel(double a, const double* __restrict__ x, double* __restrict__ y, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __dadd_rn(y[i], __dmul_rn(a, x[i]));
}
// y += x (Eigen's vector +=)
__global__ void add_kernel(const double* __restrict__ x, double* __restrict__ y, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __dadd_rn(y[i], x[i]);
}

amdg_status alloc_vec(double** p, int64_t n) {
    *p = nullptr;
    if (amdg::device_malloc(reinterpret_cast<void**>(p), size_t(std::max<int64_t>(n, 1)) * sizeof(double)) != cudaSuccess) {
        *p = nullptr;
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (time integrator vectors)");
    }
    return AMDG_OK;
}

}  // namespace

namespace amdg {

amdg_status grid_ensure_velocity(amdg_grid* g) {
    if (g->d_v) return AMDG_OK;
    const int64_t cap = std::max<int64_t>(g->capacity, 1);
    if (amdg::device_malloc(&g->d_v, size_t(cap) * g->block * sizeof(double)) != cudaSuccess) {
        g->d_v = nullptr;
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (velocity field)");
    }
    AMDG_CK(cudaMemsetAsync(g->d_v, 0, size_t(cap) * g->block * sizeof(double), stream_of(g)));
    g->v_capacity = cap;
    return AMDG_OK;
}

amdg_status grid_rhs(amdg_grid* g, double** d_rhs) {
    const int64_t E = g->host.num_elements;
    cudaStream_t st = stream_of(g);
    if (E > g->rhs_capacity || !g->d_rhs) {
        cudaFree(g->d_rhs);
        g->d_rhs = nullptr;
        g->rhs_capacity = 0;
        const int64_t cap = E + E / 4 + 16;
        if (alloc_vec(&g->d_rhs, cap * g->block) != AMDG_OK) return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (rhs)");
        g->rhs_capacity = cap;
        g->rhs_version = -1;
    }
    if (g->rhs_version != g->version) {  // a new element set starts with a zero right-hand side
        AMDG_CK(cudaMemsetAsync(g->d_rhs, 0, size_t(g->dof) * sizeof(double), st));
        g->rhs_version = g->version;
    }
    *d_rhs = g->d_rhs;
    return AMDG_OK;
}

}  // namespace amdg

extern "C" {

amdg_status amdg_grid_set_rhs_zero(amdg_grid* g) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    AMDG_CK(cudaSetDevice(g->device));
    double* r = nullptr;
    if (amdg_status s = grid_rhs(g, &r); s != AMDG_OK) return s;
    AMDG_CK(cudaMemsetAsync(r, 0, size_t(g->dof) * sizeof(double), stream_of(g)));
    return AMDG_OK;
}

amdg_status amdg_grid_rhs_device(amdg_grid* g, double** device_ptr) {
    AMDG_REQUIRE(g && device_ptr, AMDG_ERR_ARG, "null argument");
    AMDG_CK(cudaSetDevice(g->device));
    return grid_rhs(g, device_ptr);
}

amdg_status amdg_grid_get_rhs(amdg_grid* g, double* host, int64_t n) {
    AMDG_REQUIRE(g && host && n == g->dof, AMDG_ERR_ARG, "host buffer must have dof entries");
    AMDG_CK(cudaSetDevice(g->device));
    double* r = nullptr;
    if (amdg_status s = grid_rhs(g, &r); s != AMDG_OK) return s;
    cudaStream_t st = stream_of(g);
    if (n) AMDG_CK(cudaMemcpyAsync(host, r, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    return AMDG_OK;
}

amdg_status amdg_grid_copy_ucoe_to_predict(amdg_grid* g) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    AMDG_CK(cudaSetDevice(g->device));
    const int64_t E = g->host.num_elements;
    if (!g->d_pred || E > g->pred_capacity) {
        cudaFree(g->d_pred);
        g->d_pred = nullptr;
        g->pred_capacity = 0;
        const int64_t cap = E + E / 4 + 16;
        if (amdg_status s = alloc_vec(&g->d_pred, cap * g->block); s != AMDG_OK) return s;
        g->pred_capacity = cap;
    }
    if (g->dof)
        AMDG_CK(cudaMemcpyAsync(g->d_pred, g->d_u, size_t(g->dof) * sizeof(double), cudaMemcpyDeviceToDevice, stream_of(g)));
    return AMDG_OK;
}

amdg_status amdg_grid_copy_predict_to_ucoe(amdg_grid* g) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    AMDG_REQUIRE(g->d_pred, AMDG_ERR_STATE, "no prediction: call amdg_grid_copy_ucoe_to_predict first");
    AMDG_CK(cudaSetDevice(g->device));
    if (g->dof)
        AMDG_CK(cudaMemcpyAsync(g->d_u, g->d_pred, size_t(g->dof) * sizeof(double), cudaMemcpyDeviceToDevice, stream_of(g)));
    return AMDG_OK;
}

amdg_status amdg_grid_copy_ucoe_ut_to_predict(amdg_grid* g) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    AMDG_CK(cudaSetDevice(g->device));
    if (amdg_status s = grid_ensure_velocity(g); s != AMDG_OK) return s;
    const int64_t E = g->host.num_elements;
    if (!g->d_pred_v || E > g->pred_v_capacity) {
        cudaFree(g->d_pred_v);
        g->d_pred_v = nullptr;
        g->pred_v_capacity = 0;
        const int64_t cap = E + E / 4 + 16;
        if (amdg_status s = alloc_vec(&g->d_pred_v, cap * g->block); s != AMDG_OK) return s;
        g->pred_v_capacity = cap;
    }
    if (g->dof)
        AMDG_CK(cudaMemcpyAsync(g->d_pred_v, g->d_v, size_t(g->dof) * sizeof(double), cudaMemcpyDeviceToDevice,
                                stream_of(g)));
    return AMDG_OK;
}

amdg_status amdg_grid_copy_predict_to_ucoe_ut(amdg_grid* g) {
    AMDG_REQUIRE(g, AMDG_ERR_ARG, "grid is null");
    AMDG_REQUIRE(g->d_pred_v, AMDG_ERR_STATE, "no prediction: call amdg_grid_copy_ucoe_ut_to_predict first");
    AMDG_CK(cudaSetDevice(g->device));
    if (amdg_status s = grid_ensure_velocity(g); s != AMDG_OK) return s;
    if (g->dof)
        AMDG_CK(cudaMemcpyAsync(g->d_v, g->d_pred_v, size_t(g->dof) * sizeof(double), cudaMemcpyDeviceToDevice,
                                stream_of(g)));
    return AMDG_OK;
}

amdg_status amdg_vector_axpy(amdg_context* ctx, double a, const double* d_x, double* d_y, int64_t n) {
    AMDG_REQUIRE(ctx && n >= 0 && (n == 0 || (d_x && d_y)), AMDG_ERR_ARG, "bad arguments");
    if (n == 0) return AMDG_OK;
    AMDG_CK(cudaSetDevice(ctx->device));
    axpy_kernel<<<unsigned((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(ctx->stream)>>>(a, d_x, d_y, n);
    AMDG_CK(cudaGetLastError());
    ctx->launches++;
    return AMDG_OK;
}

amdg_status amdg_ode_create(amdg_grid* g, int scheme, double dt, amdg_ode** out) {
    AMDG_REQUIRE(g && out, AMDG_ERR_ARG, "null argument");
    *out = nullptr;
    AMDG_REQUIRE(scheme >= AMDG_ODE_FORWARD_EULER && scheme <= AMDG_ODE_RK4ODE2ND, AMDG_ERR_ARG, "unknown scheme");
    AMDG_REQUIRE(std::isfinite(dt), AMDG_ERR_ARG, "dt must be finite");
    AMDG_CK(cudaSetDevice(g->device));
    amdg_ode* o = new (std::nothrow) amdg_ode;
    AMDG_REQUIRE(o, AMDG_ERR_NOMEM, "host allocation failed");
    o->grid = g;
    o->device = g->device;
    o->scheme = scheme;
    o->dt = dt;
    o->n = g->dof;
    o->version = g->version;
    const bool second = scheme == AMDG_ODE_EULER_ODE2ND || scheme == AMDG_ODE_RK4ODE2ND;
    amdg_status s;
    if ((s = alloc_vec(&o->d_un, o->n)) != AMDG_OK || (s = alloc_vec(&o->d_rhs, o->n)) != AMDG_OK ||
        (second && ((s = grid_ensure_velocity(g)) != AMDG_OK || (s = alloc_vec(&o->d_vn, o->n)) != AMDG_OK ||
                    (s = alloc_vec(&o->d_su, o->n)) != AMDG_OK || (s = alloc_vec(&o->d_sv, o->n)) != AMDG_OK))) {
        amdg_ode_destroy(o);
        return s;
    }
    cudaStream_t st = stream_of(g);
    // ODESolver::init: the coefficients (and u_t) at t_n; the solver's right-hand side starts at zero
    const size_t bytes = size_t(o->n) * sizeof(double);
    cudaError_t e = o->n ? cudaMemcpyAsync(o->d_un, g->d_u, bytes, cudaMemcpyDeviceToDevice, st) : cudaSuccess;
    if (e == cudaSuccess && o->n) e = cudaMemsetAsync(o->d_rhs, 0, bytes, st);
    if (e == cudaSuccess && o->n && second) e = cudaMemcpyAsync(o->d_vn, g->d_v, bytes, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        amdg_ode_destroy(o);
        return fail(AMDG_ERR_CUDA, std::string("amdg_ode_create: ") + cudaGetErrorString(e));
    }
    *out = o;
    return AMDG_OK;
}

amdg_status amdg_ode_destroy(amdg_ode* o) {
    if (!o) return AMDG_OK;
    cudaSetDevice(o->device);
    cudaFree(o->d_un);
    cudaFree(o->d_rhs);
    cudaFree(o->d_vn);
    cudaFree(o->d_su);
    cudaFree(o->d_sv);
    delete o;
    return AMDG_OK;
}

amdg_status amdg_ode_set_rhs_zero(amdg_ode* o) {
    AMDG_REQUIRE(o, AMDG_ERR_ARG, "null argument");
    AMDG_CK(cudaSetDevice(o->device));
    if (o->n) AMDG_CK(cudaMemsetAsync(o->d_rhs, 0, size_t(o->n) * sizeof(double), stream_of(o->grid)));
    return AMDG_OK;
}

amdg_status amdg_ode_add_rhs_to_eigenvec(amdg_ode* o) {
    AMDG_REQUIRE(o, AMDG_ERR_ARG, "null argument");
    amdg_grid* g = o->grid;
    AMDG_REQUIRE(g->version == o->version, AMDG_ERR_STATE, "the element set changed since the integrator was created");
    AMDG_CK(cudaSetDevice(o->device));
    double* r = nullptr;
    if (amdg_status s = grid_rhs(g, &r); s != AMDG_OK) return s;
    if (o->n == 0) return AMDG_OK;
    add_kernel<<<unsigned((o->n + 255) / 256), 256, 0, stream_of(g)>>>(r, o->d_rhs, o->n);
    AMDG_CK(cudaGetLastError());
    g->ctx->launches++;
    return AMDG_OK;
}

amdg_status amdg_ode_step_stage(amdg_ode* o, int stage) {
    AMDG_REQUIRE(o, AMDG_ERR_ARG, "null argument");
    amdg_grid* g = o->grid;
    AMDG_REQUIRE(g->version == o->version, AMDG_ERR_STATE, "the element set changed since the integrator was created");
    const int nstage = o->scheme == AMDG_ODE_RK3SSP ? 3 : (o->scheme == AMDG_ODE_RK4ODE2ND ? 4 : 1);
    AMDG_REQUIRE(stage >= 0 && stage < nstage, AMDG_ERR_ARG, "stage out of range");
    AMDG_CK(cudaSetDevice(o->device));
    if (o->scheme == AMDG_ODE_EULER_ODE2ND || o->scheme == AMDG_ODE_RK4ODE2ND) {
        // the stage state goes into the grid's (u, u_t); the RK4ODE2nd step's end (stage 3) is
        // computed into the t_n copies, then copied to the grid
        AMDG_REQUIRE(g->d_v, AMDG_ERR_STATE, "the grid has no velocity field");
        cudaStream_t st = stream_of(g);
        const int kstage = o->scheme == AMDG_ODE_EULER_ODE2ND ? -1 : stage;
        AMDG_CK(launch_rk4_2nd_stage(kstage, o->dt, o->d_rhs, o->d_un, o->d_vn, g->d_u, g->d_v, o->d_su, o->d_sv, o->n,
                                     st));
        g->ctx->launches++;
        if (kstage == 3 && o->n) {
            const size_t bytes = size_t(o->n) * sizeof(double);
            AMDG_CK(cudaMemcpyAsync(g->d_u, o->d_un, bytes, cudaMemcpyDeviceToDevice, st));
            AMDG_CK(cudaMemcpyAsync(g->d_v, o->d_vn, bytes, cudaMemcpyDeviceToDevice, st));
        }
        return AMDG_OK;
    }
    // ForwardEuler::step_stage (ODESolver.cpp:209-213) and RK3SSP::step_stage (:285-301):
    // u = un + dt rhs; u = 3/4 un + 1/4 (u + dt rhs); u = 1/3 un + 2/3 (u + dt rhs)
    StageCoef rk{1, 0.0, 1.0, o->dt};
    if (stage == 1) rk = StageCoef{1, 3. / 4., 1. / 4., o->dt};
    if (stage == 2) rk = StageCoef{1, 1. / 3., 2. / 3., o->dt};
    AMDG_CK(launch_stage_update(o->d_un, g->d_u, o->d_rhs, o->n, rk, stream_of(g)));
    g->ctx->launches++;
    return AMDG_OK;
}

amdg_status amdg_ode_final(amdg_ode* o) {
    // ODESolver::final copies back to the elements (the state already is the grid's) and zeroes
    // the solver's rhs
    return amdg_ode_set_rhs_zero(o);
}

}  // extern "C"
