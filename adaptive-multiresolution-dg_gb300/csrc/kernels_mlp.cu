// Per-element refine/keep/coarsen classifier: a small fully connected network
// (ReLU hidden layers, softmax output) with hand-written forward, backward
// and Adam kernels, and the feature gather from the DG coefficients.  The
// dense layers (forward, input and weight gradients) run as one shared-memory
// tiled product kernel; every reduction has a fixed order (deterministic).
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels_mlp.cuh"

namespace amdg {

#define AMDG_CK_CUDA(x)                          \
    do {                                         \
        const cudaError_t e_ = (x);              \
        if (e_ != cudaSuccess) return e_;        \
    } while (0)

// ---- dense layers as one tiled product kernel ------------------------------------------------
// C[m][n] = (bias ? bias[n] : 0) + sum_k A(m, k) B(k, n), A and B given by element strides, so
// the forward pass (x W^T), the input gradient (dy W) and the weight gradient (dy^T x) are the same
// kernel.  A CTA of 256 threads owns a 32 x 64 tile of C and walks k in chunks of 32 staged in
// shared memory; each thread keeps a 2 x 4 register tile.  Every output sums k in ascending order
// from its bias (one rounding per multiply-add), the order of a plain loop over k.
constexpr int kTM = 32, kTN = 64, kTK = 32;

struct DenseArgs {
    const float* A;
    int64_t sam, sak;  // A(m, k) = A[m * sam + k * sak]
    const float* B;
    int64_t sbk, sbn;  // B(k, n) = B[k * sbk + n * sbn]
    float* C;          // C[m * N + n]
    const float* bias; // [N] or null
    const float* mask; // C[m][n] = 0 where mask[m * N + n] <= 0 (null: no mask)
    int relu;
    int64_t M;
    int N, K;
};

__global__ void __launch_bounds__(256) dense_tile_kernel(DenseArgs a) {
    __shared__ float As[kTK][kTM + 1];
    __shared__ __align__(16) float Bs[kTK][kTN];
    const int tid = threadIdx.x;
    const int ty = tid / 16, tx = tid % 16;  // rows 2 ty, 2 ty + 1; columns 4 tx .. 4 tx + 3
    const int64_t m0 = int64_t(blockIdx.x) * kTM;
    const int n0 = blockIdx.y * kTN;
    float acc[2][4];
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int n = n0 + 4 * tx + c;
            acc[r][c] = (a.bias && n < a.N) ? a.bias[n] : 0.f;
        }
    for (int k0 = 0; k0 < a.K; k0 += kTK) {
        for (int i = tid; i < kTK * kTM; i += 256) {  // A tile, k-major in shared memory
            const int kk = i / kTM, mm = i % kTM;
            const int64_t m = m0 + mm;
            const int k = k0 + kk;
            As[kk][mm] = (m < a.M && k < a.K) ? a.A[m * a.sam + int64_t(k) * a.sak] : 0.f;
        }
        for (int i = tid; i < kTK * kTN; i += 256) {
            const int kk = i / kTN, nn = i % kTN;
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < a.N && k < a.K) ? a.B[int64_t(k) * a.sbk + int64_t(n) * a.sbn] : 0.f;
        }
        __syncthreads();
        const int kn = min(kTK, a.K - k0);
        for (int kk = 0; kk < kn; ++kk) {
            const float x0 = As[kk][2 * ty], x1 = As[kk][2 * ty + 1];
            const float4 w = *reinterpret_cast<const float4*>(&Bs[kk][4 * tx]);
            acc[0][0] = fmaf(x0, w.x, acc[0][0]);
            acc[0][1] = fmaf(x0, w.y, acc[0][1]);
            acc[0][2] = fmaf(x0, w.z, acc[0][2]);
            acc[0][3] = fmaf(x0, w.w, acc[0][3]);
            acc[1][0] = fmaf(x1, w.x, acc[1][0]);
            acc[1][1] = fmaf(x1, w.y, acc[1][1]);
            acc[1][2] = fmaf(x1, w.z, acc[1][2]);
            acc[1][3] = fmaf(x1, w.w, acc[1][3]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        const int64_t m = m0 + 2 * ty + r;
        if (m >= a.M) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int n = n0 + 4 * tx + c;
            if (n >= a.N) continue;
            float v = acc[r][c];
            if (a.relu && v < 0.f) v = 0.f;
            if (a.mask && !(a.mask[m * a.N + n] > 0.f)) v = 0.f;
            a.C[m * a.N + n] = v;
        }
    }
}

static cudaError_t launch_dense_tile(const DenseArgs& a, cudaStream_t st) {
    if (a.M == 0 || a.N == 0) return cudaSuccess;
    const dim3 grid(unsigned((a.M + kTM - 1) / kTM), unsigned((a.N + kTN - 1) / kTN));
    dense_tile_kernel<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

// db[j] = sum_n dy[n][j] (samples in order)
__global__ void bias_grad_kernel(const float* __restrict__ dy, float* __restrict__ db, int64_t n, int out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= out) return;
    float acc = 0.f;
    for (int64_t s = 0; s < n; ++s) acc += dy[s * out + j];
    db[j] = acc;
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
    // y = x W^T + b: A(s, i) = x[s in + i], B(i, j) = W[j in + i]
    DenseArgs a{x, in, 1, W, 1, in, y, b, nullptr, relu ? 1 : 0, n, out, in};
    return launch_dense_tile(a, st);
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
    // dW = dy^T x: A(j, s) = dy[s out + j], B(s, i) = x[s in + i]
    DenseArgs gw{dy, 1, out, x, in, 1, dW, nullptr, nullptr, 0, out, in, int(n)};
    AMDG_CK_CUDA(launch_dense_tile(gw, st));
    bias_grad_kernel<<<unsigned((out + 127) / 128), 128, 0, st>>>(dy, db, n, out);
    AMDG_CK_CUDA(cudaGetLastError());
    if (!dx) return cudaSuccess;
    // dx = (dy W) * (x > 0): A(s, j) = dy[s out + j], B(j, i) = W[j in + i]
    DenseArgs gi{dy, out, 1, W, in, 1, dx, nullptr, relu_mask_input ? x : nullptr, 0, n, in, out};
    return launch_dense_tile(gi, st);
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
