// Launch interfaces of the refine/coarsen classifier kernels (kernels_mlp.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace amdg {

cudaError_t launch_dense_forward(const float* x, const float* W, const float* b, float* y, int64_t n, int in, int out,
                                 bool relu, cudaStream_t st);
cudaError_t launch_softmax_xent(const float* logits, const int32_t* labels, int64_t n, int k, float* probs, float* dlogits,
                                float* loss, cudaStream_t st);
// weight gradient always; input gradient (masked by x > 0) when dx is not null
cudaError_t launch_dense_backward(const float* dy, const float* x, const float* W, float* dx, float* dW, float* db,
                                  int64_t n, int in, int out, bool relu_mask_input, cudaStream_t st);
cudaError_t launch_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                        int step, cudaStream_t st);
// anc: [e][d][2] parent / grandparent element in dimension d, -1 when absent.  Row e holds the
// B (1 + 2 dim) features of u, followed by those of u2 when u2 is given.
cudaError_t launch_element_features(const double* u, const double* u2, const int32_t* anc, int64_t E, int dim, int B,
                                    float* feat, cudaStream_t st);

}  // namespace amdg
