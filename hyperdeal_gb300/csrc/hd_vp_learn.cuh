// hd_vp_learn.cuh -- learned initial guess for the Vlasov-Poisson CG.
//
// A two-layer linear network y ~ s * W2 (W1 (x~ / s)), s = ||x~||,
// x~ = x - mean(x), with a rank-r bottleneck (W1: r x n, W2: n x r, FP32),
// is trained online with Adam on the (x, y) pairs that the solver itself
// produces (a ring of the last H pairs); the caller passes density and
// potential differences between consecutive solves.  Training and inference
// run in this project's own kernels (hd_vp_learn.cu).  The caller weighs the
// resulting guess against the previous potential by the initial CG residual;
// the better one starts CG, which still converges to the same tolerance.
#pragma once

#include <cuda_runtime.h>

namespace hd {

struct VpModel;

VpModel* vp_model_create(long long n, int rank, int history);
void vp_model_destroy(VpModel* m);
bool vp_model_ready(const VpModel* m);
// y_out = model(x) (FP64 in / out; mean-free)
cudaError_t vp_model_predict(VpModel* m, const double* x, double* y_out, cudaStream_t s);
// store the pair; with `train`, run the configured number of Adam steps
cudaError_t vp_model_observe(VpModel* m, const double* x, const double* y, cudaStream_t s, bool train = true);
long long vp_model_steps(const VpModel* m);

// loss = 1/(2B) sum_b ||W2 W1 x_b - y_b||^2 (skipped when loss is null) and its gradients (device pointers, column-major
// X, Y: n x B; W1: r x n row-major; W2: n x r row-major)
cudaError_t vp_model_loss_grad(long long n, int r, int B, const float* W1, const float* W2, const float* X,
                               const float* Y, float* dW1, float* dW2, float* loss, float* work, cudaStream_t s);
size_t vp_model_work_floats(long long n, int r, int B);

}  // namespace hd
