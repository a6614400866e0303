// C-ABI of the learned refine/keep/coarsen classifier: parameters, inference,
// loss gradient (for checking against an independent CPU implementation) and
// Adam training on device-resident samples, all with the kernels of
// kernels_mlp.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "amdg.h"
#include "amdg_internal.hpp"
#include "kernels_mlp.cuh"
#include "device_alloc.cuh"

using namespace amdg;

#define AMDG_CK(...)                                                                                    \
    do {                                                                                                \
        cudaError_t amdg_err_ = (__VA_ARGS__);                                                          \
        if (amdg_err_ != cudaSuccess)                                                                   \
            return fail(AMDG_ERR_CUDA, std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(amdg_err_)); \
    } while (0)

#define AMDG_REQUIRE(cond, code, msg)        \
    do {                                     \
        if (!(cond)) return fail(code, msg); \
    } while (0)

struct amdg_mlp {
    amdg_context* ctx = nullptr;
    int device = 0;
    std::vector<int> dims;            // n_in, hidden..., n_out
    std::vector<int64_t> w_off, b_off;
    int64_t nparams = 0;
    float *d_params = nullptr, *d_grad = nullptr, *d_m = nullptr, *d_v = nullptr;
    int adam_step = 0;
    int64_t ws_n = 0;                 // workspace capacity in samples
    float *d_act = nullptr, *d_delta = nullptr, *d_loss = nullptr, *d_probs = nullptr;
    std::vector<int64_t> act_off;     // offsets of layer outputs in d_act (per sample count ws_n)
};

namespace {

cudaStream_t stream_of(const amdg_mlp* m) { return static_cast<cudaStream_t>(m->ctx->stream); }

int layers(const amdg_mlp* m) { return int(m->dims.size()) - 1; }

amdg_status ensure_ws(amdg_mlp* m, int64_t n) {
    if (n <= m->ws_n) return AMDG_OK;
    cudaFree(m->d_act); cudaFree(m->d_delta); cudaFree(m->d_loss); cudaFree(m->d_probs);
    m->d_act = m->d_delta = m->d_loss = m->d_probs = nullptr;
    int64_t tot = 0, widest = 0;
    m->act_off.assign(m->dims.size(), 0);
    for (size_t l = 1; l < m->dims.size(); ++l) {
        m->act_off[l] = tot;
        tot += int64_t(m->dims[l]) * n;
    }
    for (int d : m->dims) widest = std::max<int64_t>(widest, d);
    const int k = m->dims.back();
    cudaError_t e = amdg::device_malloc(&m->d_act, size_t(tot) * sizeof(float));
    if (e == cudaSuccess) e = amdg::device_malloc(&m->d_delta, size_t(2 * widest * n) * sizeof(float));
    if (e == cudaSuccess) e = amdg::device_malloc(&m->d_loss, size_t(n) * sizeof(float));
    if (e == cudaSuccess) e = amdg::device_malloc(&m->d_probs, size_t(n) * k * sizeof(float));
    if (e != cudaSuccess) return fail(AMDG_ERR_NOMEM, std::string("mlp workspace: ") + cudaGetErrorString(e));
    m->ws_n = n;
    return AMDG_OK;
}

// forward pass over n samples; activations of layer l (1..L) at d_act + act_off[l]
amdg_status forward(amdg_mlp* m, const float* x, int64_t n, cudaStream_t st) {
    const int L = layers(m);
    const float* in = x;
    for (int l = 0; l < L; ++l) {
        float* out = m->d_act + m->act_off[l + 1];
        AMDG_CK(launch_dense_forward(in, m->d_params + m->w_off[l], m->d_params + m->b_off[l], out, n, m->dims[l],
                                     m->dims[l + 1], l + 1 < L, st));
        m->ctx->launches++;
        in = out;
    }
    return AMDG_OK;
}

// gradient of the mean cross entropy over n samples into d_grad; per-sample losses in d_loss
amdg_status backward(amdg_mlp* m, const float* x, const int32_t* labels, int64_t n, cudaStream_t st) {
    const int L = layers(m);
    const int k = m->dims.back();
    int64_t widest = 0;
    for (int d : m->dims) widest = std::max<int64_t>(widest, d);
    float* da = m->d_delta;
    float* db = m->d_delta + widest * n;
    AMDG_CK(launch_softmax_xent(m->d_act + m->act_off[L], labels, n, k, m->d_probs, da, m->d_loss, st));
    m->ctx->launches++;
    for (int l = L - 1; l >= 0; --l) {
        const float* xin = l == 0 ? x : m->d_act + m->act_off[l];
        AMDG_CK(launch_dense_backward(da, xin, m->d_params + m->w_off[l], l > 0 ? db : nullptr, m->d_grad + m->w_off[l],
                                      m->d_grad + m->b_off[l], n, m->dims[l], m->dims[l + 1], true, st));
        m->ctx->launches += l > 0 ? 2 : 1;
        std::swap(da, db);
    }
    return AMDG_OK;
}

__global__ void gather_rows(const float* __restrict__ x, const int32_t* __restrict__ lab, const int64_t* __restrict__ idx,
                            int64_t n, int f, float* __restrict__ xo, int32_t* __restrict__ lo) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= n * f) return;
    const int64_t r = gid / f;
    const int c = int(gid - r * f);
    const int64_t src = idx[r];
    xo[gid] = x[src * f + c];
    if (c == 0) lo[r] = lab[src];
}

}  // namespace

void amdg::mlp_shape(const amdg_mlp* m, int* n_in, int* n_out) {
    *n_in = m->dims.front();
    *n_out = m->dims.back();
}

extern "C" {

amdg_status amdg_mlp_create(amdg_context* ctx, int n_in, int hidden, int n_hidden_layers, int n_out, uint64_t seed,
                            amdg_mlp** out) {
    AMDG_REQUIRE(ctx && out && n_in > 0 && hidden > 0 && n_hidden_layers >= 0 && n_out > 1, AMDG_ERR_ARG, "bad arguments");
    *out = nullptr;
    AMDG_CK(cudaSetDevice(ctx->device));
    amdg_mlp* m = new (std::nothrow) amdg_mlp;
    AMDG_REQUIRE(m, AMDG_ERR_NOMEM, "host allocation failed");
    m->ctx = ctx;
    m->device = ctx->device;
    m->dims.push_back(n_in);
    for (int i = 0; i < n_hidden_layers; ++i) m->dims.push_back(hidden);
    m->dims.push_back(n_out);
    int64_t off = 0;
    for (int l = 0; l < layers(m); ++l) {
        m->w_off.push_back(off);
        off += int64_t(m->dims[l]) * m->dims[l + 1];
        m->b_off.push_back(off);
        off += m->dims[l + 1];
    }
    m->nparams = off;
    // He-normal weights from a seeded generator, zero biases
    std::vector<float> p(off, 0.f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < layers(m); ++l) {
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / m->dims[l]));
        for (int64_t i = 0; i < int64_t(m->dims[l]) * m->dims[l + 1]; ++i) p[m->w_off[l] + i] = float(nd(rng));
    }
    cudaError_t e = amdg::device_malloc(&m->d_params, size_t(off) * sizeof(float));
    if (e == cudaSuccess) e = amdg::device_malloc(&m->d_grad, size_t(off) * sizeof(float));
    if (e == cudaSuccess) e = amdg::device_malloc(&m->d_m, size_t(off) * sizeof(float));
    if (e == cudaSuccess) e = amdg::device_malloc(&m->d_v, size_t(off) * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(m->d_params, p.data(), size_t(off) * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->d_m, 0, size_t(off) * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->d_v, 0, size_t(off) * sizeof(float));
    if (e != cudaSuccess) {
        amdg_mlp_destroy(m);
        return fail(AMDG_ERR_NOMEM, std::string("mlp create: ") + cudaGetErrorString(e));
    }
    *out = m;
    return AMDG_OK;
}

amdg_status amdg_mlp_destroy(amdg_mlp* m) {
    if (!m) return AMDG_OK;
    cudaSetDevice(m->device);
    void* ptrs[] = {m->d_params, m->d_grad, m->d_m, m->d_v, m->d_act, m->d_delta, m->d_loss, m->d_probs};
    for (void* p : ptrs) cudaFree(p);
    delete m;
    return AMDG_OK;
}

amdg_status amdg_mlp_num_params(const amdg_mlp* m, int64_t* n) {
    AMDG_REQUIRE(m && n, AMDG_ERR_ARG, "null argument");
    *n = m->nparams;
    return AMDG_OK;
}

amdg_status amdg_mlp_get_params(const amdg_mlp* m, float* host, int64_t n) {
    AMDG_REQUIRE(m && host && n == m->nparams, AMDG_ERR_ARG, "bad arguments");
    AMDG_CK(cudaSetDevice(m->device));
    AMDG_CK(cudaMemcpy(host, m->d_params, size_t(n) * sizeof(float), cudaMemcpyDeviceToHost));
    return AMDG_OK;
}

amdg_status amdg_mlp_set_params(amdg_mlp* m, const float* host, int64_t n) {
    AMDG_REQUIRE(m && host && n == m->nparams, AMDG_ERR_ARG, "bad arguments");
    AMDG_CK(cudaSetDevice(m->device));
    AMDG_CK(cudaMemcpy(m->d_params, host, size_t(n) * sizeof(float), cudaMemcpyHostToDevice));
    m->adam_step = 0;
    AMDG_CK(cudaMemset(m->d_m, 0, size_t(n) * sizeof(float)));
    AMDG_CK(cudaMemset(m->d_v, 0, size_t(n) * sizeof(float)));
    return AMDG_OK;
}

amdg_status amdg_mlp_predict(amdg_mlp* m, const float* d_x, int64_t n, float* d_probs) {
    AMDG_REQUIRE(m && d_x && d_probs && n >= 0, AMDG_ERR_ARG, "bad arguments");
    AMDG_CK(cudaSetDevice(m->device));
    amdg_status s = ensure_ws(m, n);
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(m);
    if ((s = forward(m, d_x, n, st)) != AMDG_OK) return s;
    AMDG_CK(launch_softmax_xent(m->d_act + m->act_off[layers(m)], nullptr, n, m->dims.back(), d_probs, nullptr, nullptr, st));
    m->ctx->launches++;
    return AMDG_OK;
}

amdg_status amdg_mlp_loss_grad(amdg_mlp* m, const float* d_x, const int32_t* d_labels, int64_t n, double* loss,
                               float* host_grad) {
    AMDG_REQUIRE(m && d_x && d_labels && n > 0, AMDG_ERR_ARG, "bad arguments");
    AMDG_CK(cudaSetDevice(m->device));
    amdg_status s = ensure_ws(m, n);
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(m);
    if ((s = forward(m, d_x, n, st)) != AMDG_OK) return s;
    if ((s = backward(m, d_x, d_labels, n, st)) != AMDG_OK) return s;
    std::vector<float> l(n);
    AMDG_CK(cudaMemcpyAsync(l.data(), m->d_loss, size_t(n) * sizeof(float), cudaMemcpyDeviceToHost, st));
    if (host_grad) AMDG_CK(cudaMemcpyAsync(host_grad, m->d_grad, size_t(m->nparams) * sizeof(float), cudaMemcpyDeviceToHost, st));
    AMDG_CK(cudaStreamSynchronize(st));
    double sum = 0;
    for (float v : l) sum += v;
    if (loss) *loss = sum / double(n);
    return AMDG_OK;
}

amdg_status amdg_mlp_train(amdg_mlp* m, const float* d_x, const int32_t* d_labels, int64_t n, int epochs, int batch,
                           float lr, uint64_t seed, double* final_loss) {
    AMDG_REQUIRE(m && d_x && d_labels && n > 0 && epochs >= 0 && batch > 0 && lr > 0, AMDG_ERR_ARG, "bad arguments");
    AMDG_CK(cudaSetDevice(m->device));
    const int f = m->dims[0];
    amdg_status s = ensure_ws(m, std::min<int64_t>(batch, n));
    if (s != AMDG_OK) return s;
    cudaStream_t st = stream_of(m);
    float* xs = nullptr;
    int32_t* ls = nullptr;
    int64_t* d_idx = nullptr;
    if (amdg::device_malloc(&xs, size_t(n) * f * sizeof(float)) != cudaSuccess ||
        amdg::device_malloc(&ls, size_t(n) * sizeof(int32_t)) != cudaSuccess ||
        amdg::device_malloc(&d_idx, size_t(n) * sizeof(int64_t)) != cudaSuccess) {
        cudaFree(xs);
        cudaFree(ls);
        cudaFree(d_idx);
        return fail(AMDG_ERR_NOMEM, "cudaMalloc failed (training minibatches)");
    }
    std::vector<int64_t> idx(n);
    std::mt19937_64 rng(seed);
    double last = 0.0;
    for (int ep = 0; ep < epochs && s == AMDG_OK; ++ep) {
        for (int64_t i = 0; i < n; ++i) idx[i] = i;
        std::shuffle(idx.begin(), idx.end(), rng);
        cudaMemcpyAsync(d_idx, idx.data(), size_t(n) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
        gather_rows<<<unsigned((n * f + 255) / 256), 256, 0, st>>>(d_x, d_labels, d_idx, n, f, xs, ls);
        m->ctx->launches++;
        double ep_loss = 0.0;
        std::vector<float> lb;
        for (int64_t b0 = 0; b0 < n && s == AMDG_OK; b0 += batch) {
            const int64_t nb = std::min<int64_t>(batch, n - b0);
            if ((s = forward(m, xs + b0 * f, nb, st)) != AMDG_OK) break;
            if ((s = backward(m, xs + b0 * f, ls + b0, nb, st)) != AMDG_OK) break;
            ++m->adam_step;
            cudaError_t e = launch_adam(m->d_params, m->d_grad, m->d_m, m->d_v, m->nparams, lr, 0.9f, 0.999f, 1e-8f,
                                        m->adam_step, st);
            m->ctx->launches++;
            if (e != cudaSuccess) { s = fail(AMDG_ERR_CUDA, cudaGetErrorString(e)); break; }
            if (ep == epochs - 1) {
                lb.resize(nb);
                cudaMemcpyAsync(lb.data(), m->d_loss, size_t(nb) * sizeof(float), cudaMemcpyDeviceToHost, st);
                cudaStreamSynchronize(st);
                for (float v : lb) ep_loss += v;
            }
        }
        last = ep_loss / double(n);
    }
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(xs);
    cudaFree(ls);
    cudaFree(d_idx);
    if (s != AMDG_OK) return s;
    if (e != cudaSuccess) return fail(AMDG_ERR_CUDA, std::string("mlp train: ") + cudaGetErrorString(e));
    if (final_loss) *final_loss = last;
    return AMDG_OK;
}

}  // extern "C"
