// Per-element refine/keep/coarsen classifier: a small fully connected network
// (ReLU hidden layers, softmax output) with hand-written forward, backward
// and Adam kernels, and the feature gather from the DG coefficients.  Sizes
// are small (tens of thousands of samples, 64-wide layers), so every kernel
// is a plain one-thread-per-output loop with deterministic reductions.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels_mlp.cuh"

namespace amdg {

// y[n][j] = act(b[j] + sum_i W[j][i] x[n][i])
__global__ void dense_forward_kernel(const float* __restrict__ x, const float* __restrict__ W, const float* __restrict__ b,
                                     float* __restrict__ y, int64_t n, int in, int out, int relu) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= n * out) return;
    const int64_t s = gid / out;
    const int j = int(gid - s * out);
    const float* xs = x + s * in;
    const float* w = W + int64_t(j) * in;
    float acc = b[j];
    for (int i = 0; i < in; ++i) acc = fmaf(w[i], xs[i], acc);
    y[gid] = (relu && acc < 0.f) ? 0.f : acc;
}

// softmax of logits; when labels are given also the per-sample cross entropy and
// dlogits = (p - onehot) / n
__global__ void softmax_xent_kernel(const float* __restrict__ logits, const int32_t* __restrict__ labels, int64_t n, int k,
                                    float* __restrict__ probs, float* __restrict__ dlogits, float* __restrict__ loss) {
    const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const float* z = logits + s * k;
    float m = z[0];
    for (int j = 1; j < k; ++j) m = fmaxf(m, z[j]);
    float sum = 0.f;
    for (int j = 0; j < k; ++j) sum += expf(z[j] - m);
    for (int j = 0; j < k; ++j) {
        const float p = expf(z[j] - m) / sum;
        if (probs) probs[s * k + j] = p;
        if (labels) dlogits[s * k + j] = (p - (labels[s] == j ? 1.f : 0.f)) / float(n);
    }
    if (labels) loss[s] = -(z[labels[s]] - m - logf(sum));
}

// dx[n][i] = (sum_j W[j][i] dy[n][j]) * (x[n][i] > 0 when relu_mask)
__global__ void dense_backward_input_kernel(const float* __restrict__ dy, const float* __restrict__ W,
                                            const float* __restrict__ xact, float* __restrict__ dx, int64_t n, int in,
                                            int out, int relu_mask) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= n * in) return;
    const int64_t s = gid / in;
    const int i = int(gid - s * in);
    float acc = 0.f;
    for (int j = 0; j < out; ++j) acc = fmaf(W[int64_t(j) * in + i], dy[s * out + j], acc);
    if (relu_mask && !(xact[gid] > 0.f)) acc = 0.f;
    dx[gid] = acc;
}

// dW[j][i] = sum_n dy[n][j] x[n][i]; db[j] = sum_n dy[n][j]  (thread per weight, samples in order)
__global__ void dense_backward_weight_kernel(const float* __restrict__ dy, const float* __restrict__ x, float* __restrict__ dW,
                                             float* __restrict__ db, int64_t n, int in, int out) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (gid >= int64_t(out) * (in + 1)) return;
    const int j = int(gid / (in + 1));
    const int i = int(gid - int64_t(j) * (in + 1));
    float acc = 0.f;
    if (i < in) {
        for (int64_t s = 0; s < n; ++s) acc = fmaf(dy[s * out + j], x[s * in + i], acc);
        dW[int64_t(j) * in + i] = acc;
    } else {
        for (int64_t s = 0; s < n; ++s) acc += dy[s * out + j];
        db[j] = acc;
    }
}

__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                            int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// features of element e: magnitudes of its block, then for every dimension
// the blocks of its parent and grandparent in that dimension (zero when absent)
__global__ void element_features_kernel(const double* __restrict__ u, const double* __restrict__ u2,
                                        const int32_t* __restrict__ anc, int64_t E, int dim, int B,
                                        float* __restrict__ feat) {
    const int64_t gid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int F1 = B * (1 + 2 * dim), F = u2 ? 2 * F1 : F1;
    if (gid >= E * F) return;
    const int64_t e = gid / F;
    int f = int(gid - e * F);
    const double* field = u;
    if (f >= F1) {  // second field's block of the row
        f -= F1;
        field = u2;
    }
    const int slot = f / B, q = f - slot * B;
    int64_t src = e;
    if (slot > 0) {
        const int d = (slot - 1) / 2, gen = (slot - 1) % 2;  // gen 0: parent, 1: grandparent
        src = anc[(e * dim + d) * 2 + gen];
    }
    float v = 0.f;
    if (src >= 0) {
        const double c = fabs(field[src * B + q]);
        v = float(log10(c + 1e-20) / 20.0 + 1.0);
    }
    feat[gid] = v;
}

static unsigned blocks_for(int64_t n) { return unsigned((n + 255) / 256); }

cudaError_t launch_dense_forward(const float* x, const float* W, const float* b, float* y, int64_t n, int in, int out,
                                 bool relu, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dense_forward_kernel<<<blocks_for(n * out), 256, 0, st>>>(x, W, b, y, n, in, out, relu ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_softmax_xent(const float* logits, const int32_t* labels, int64_t n, int k, float* probs, float* dlogits,
                                float* loss, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    softmax_xent_kernel<<<blocks_for(n), 256, 0, st>>>(logits, labels, n, k, probs, dlogits, loss);
    return cudaGetLastError();
}

cudaError_t launch_dense_backward(const float* dy, const float* x, const float* W, float* dx, float* dW, float* db,
                                  int64_t n, int in, int out, bool relu_mask_input, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    dense_backward_weight_kernel<<<blocks_for(int64_t(out) * (in + 1)), 256, 0, st>>>(dy, x, dW, db, n, in, out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !dx) return e;
    dense_backward_input_kernel<<<blocks_for(n * in), 256, 0, st>>>(dy, W, x, dx, n, in, out, relu_mask_input ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                        int step, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    float c1 = 1.f, c2 = 1.f;
    for (int i = 0; i < step; ++i) { c1 *= b1; c2 *= b2; }
    adam_kernel<<<blocks_for(n), 256, 0, st>>>(p, g, m, v, n, lr, b1, b2, eps, 1.f - c1, 1.f - c2);
    return cudaGetLastError();
}

cudaError_t launch_element_features(const double* u, const double* u2, const int32_t* anc, int64_t E, int dim, int B,
                                    float* feat, cudaStream_t st) {
    const int64_t total = E * int64_t(B) * (1 + 2 * dim) * (u2 ? 2 : 1);
    if (total == 0) return cudaSuccess;
    element_features_kernel<<<blocks_for(total), 256, 0, st>>>(u, u2, anc, E, dim, B, feat);
    return cudaGetLastError();
}

}  // namespace amdg
