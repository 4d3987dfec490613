// hd_vp_learn.cu -- training and inference kernels of the learned CG initial
// guess (see hd_vp_learn.cuh).  All products are small (n x r x B with
// n = x-DoFs, r <= 64, B <= 128), so plain SIMT kernels with one output
// element per thread and a fixed summation order are used (deterministic).
#include <cuda_runtime.h>

#include <cmath>
#include <new>

#include "hd_vp_learn.cuh"

namespace hd {

namespace {

// C[m][c] = alpha * sum_k A[m*as0 + k*as1] * B[k*bs0 + c*bs1] (+ beta C)
__global__ void small_gemm(int M, int Nc, int K, float alpha, const float* __restrict__ A, long long as0,
                           long long as1, const float* __restrict__ B, long long bs0, long long bs1, float beta,
                           float* __restrict__ C) {
  const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (idx >= (long long)M * Nc) return;
  const int m = int(idx / Nc), c = int(idx % Nc);
  float s = 0.f;
  for (int k = 0; k < K; ++k) s = fmaf(A[m * as0 + k * as1], B[k * bs0 + c * bs1], s);
  C[idx] = beta == 0.f ? alpha * s : fmaf(alpha, s, beta * C[idx]);
}

// the same product for few outputs and a long reduction (K = x-DoFs): one
// block per output element, threads stride over k, fixed-order block sum
__global__ void longk_gemm(int Nc, int K, float alpha, const float* __restrict__ A, long long as0, long long as1,
                           const float* __restrict__ B, long long bs0, long long bs1, float* __restrict__ C) {
  __shared__ float sh[32];
  const int m = blockIdx.x / Nc, c = blockIdx.x % Nc;
  float s = 0.f;
  for (int k = threadIdx.x; k < K; k += blockDim.x) s = fmaf(A[m * as0 + k * as1], B[k * bs0 + c * bs1], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int k = 0; k < (int)(blockDim.x / 32); ++k) t += sh[k];
    C[blockIdx.x] = alpha * t;
  }
}

void gemm(int M, int Nc, int K, float alpha, const float* A, long long as0, long long as1, const float* B,
          long long bs0, long long bs1, float beta, float* C, cudaStream_t s) {
  const long long total = (long long)M * Nc;
  if (beta == 0.f && K >= 1024 && total <= 8192) {
    longk_gemm<<<unsigned(total), 256, 0, s>>>(Nc, K, alpha, A, as0, as1, B, bs0, bs1, C);
    return;
  }
  small_gemm<<<unsigned((total + 255) / 256), 256, 0, s>>>(M, Nc, K, alpha, A, as0, as1, B, bs0, bs1, beta, C);
}

__global__ void sub_kernel(long long n, const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ c) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] - b[i];
}

__global__ void sumsq_kernel(long long n, const float* __restrict__ e, float scale, float* __restrict__ out) {
  __shared__ float sh[32];
  float s = 0.f;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s = fmaf(e[i], e[i], s);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int k = 0; k < (int)(blockDim.x / 32); ++k) t += sh[k];
    *out = scale * t;
  }
}

__global__ void adam_kernel(long long n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// mean and norm of rho - mean (one block; x-space vectors are small)
__device__ void mean_norm(long long n, const double* __restrict__ x, double* mean_out, double* norm_out) {
  __shared__ double sh[32];
  __shared__ double res;
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x / 32); ++k) t += sh[k];
    res = t / double(n);
  }
  __syncthreads();
  const double mean = res;
  double q = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) q += (x[i] - mean) * (x[i] - mean);
  for (int o = 16; o > 0; o >>= 1) q += __shfl_down_sync(0xffffffffu, q, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x / 32] = q;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x / 32); ++k) t += sh[k];
    res = sqrt(t);
  }
  __syncthreads();
  *mean_out = mean;
  *norm_out = res;
}

// store the normalised pair (rho~/s, (phi - mean phi)/s) as row `row` of X and Y
__global__ void store_pair(long long n, const double* __restrict__ rho, const double* __restrict__ phi, float* X,
                           float* Y, int row) {
  double mr, sr, mp, sp;
  mean_norm(n, rho, &mr, &sr);
  mean_norm(n, phi, &mp, &sp);
  const double inv = sr > 0.0 ? 1.0 / sr : 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) {
    X[row * n + i] = float((rho[i] - mr) * inv);
    Y[row * n + i] = float((phi[i] - mp) * inv);
  }
}

// x = rho~/s (float), and s into scale[0]
__global__ void predict_prep(long long n, const double* __restrict__ rho, float* __restrict__ x, double* scale) {
  double mr, sr;
  mean_norm(n, rho, &mr, &sr);
  const double inv = sr > 0.0 ? 1.0 / sr : 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) x[i] = float((rho[i] - mr) * inv);
  if (threadIdx.x == 0) *scale = sr;
}

// phi = s * (y - mean y): the guess stays orthogonal to the constants, the
// null space of the periodic problem, so CG from it converges to the same
// mean-free potential as CG from zero (one block; x-space vectors are small)
__global__ void predict_finish(long long n, const float* __restrict__ y, const double* __restrict__ scale,
                               double* __restrict__ phi) {
  __shared__ double sh[32];
  __shared__ double mean;
  double s = 0.0;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) s += double(y[i]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x / 32] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x / 32); ++k) t += sh[k];
    mean = t / double(n);
  }
  __syncthreads();
  const double sc = *scale, m = mean;
  for (long long i = threadIdx.x; i < n; i += blockDim.x) phi[i] = (double(y[i]) - m) * sc;
}

__global__ void init_weights(long long n, float* w, float amp, unsigned seed) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned h = unsigned(i) * 2654435761u ^ seed;
  h ^= h >> 16;
  h *= 2246822519u;
  h ^= h >> 13;
  h *= 3266489917u;
  h ^= h >> 16;
  w[i] = amp * (float(h & 0xffffff) / float(0x1000000) * 2.f - 1.f);
}

}  // namespace

size_t vp_model_work_floats(long long n, int r, int B) { return size_t(B) * (2 * r + 2 * n) + 1; }

// work: Ht (B x r) | dHt (B x r) | Pt/Et (B x n) | spare (B x n)
cudaError_t vp_model_loss_grad(long long n, int r, int B, const float* W1, const float* W2, const float* X,
                               const float* Y, float* dW1, float* dW2, float* loss, float* work, cudaStream_t s) {
  float* Ht = work;
  float* dHt = Ht + size_t(B) * r;
  float* Et = dHt + size_t(B) * r;
  const float invB = 1.f / float(B);
  // Ht[b][k] = sum_j X[b][j] W1[k][j]
  gemm(B, r, int(n), 1.f, X, n, 1, W1, 1, n, 0.f, Ht, s);
  // Et = Ht W2^T - Y
  gemm(B, int(n), r, 1.f, Ht, r, 1, W2, 1, r, 0.f, Et, s);
  sub_kernel<<<unsigned((size_t(B) * n + 255) / 256), 256, 0, s>>>(size_t(B) * n, Et, Y, Et);
  if (loss) sumsq_kernel<<<1, 1024, 0, s>>>(size_t(B) * n, Et, 0.5f * invB, loss);
  // dW2[i][k] = 1/B sum_b E[b][i] H[b][k]
  gemm(int(n), r, B, invB, Et, 1, n, Ht, r, 1, 0.f, dW2, s);
  // dHt[b][k] = sum_i E[b][i] W2[i][k]
  gemm(B, r, int(n), 1.f, Et, n, 1, W2, r, 1, 0.f, dHt, s);
  // dW1[k][j] = 1/B sum_b dH[b][k] X[b][j]
  gemm(r, int(n), B, invB, dHt, 1, r, X, n, 1, 0.f, dW1, s);
  return cudaGetLastError();
}

struct VpModel {
  long long n;
  int r, H, count, head, iters_per_obs;
  long long steps;
  float lr;
  float *W, *G, *M, *V;  // W = [W1 | W2], gradients, Adam moments (2 r n each)
  float *X, *Y;          // history rows (H x n)
  float *work, *loss, *xs, *hs, *ys;
  double* scale;
};

VpModel* vp_model_create(long long n, int rank, int history) {
  VpModel* m = new (std::nothrow) VpModel;
  if (!m) return nullptr;
  m->n = n;
  m->r = rank;
  m->H = history;
  m->count = m->head = 0;
  m->iters_per_obs = 4;
  m->steps = 0;
  m->lr = 2e-3f;
  const size_t nw = size_t(2) * rank * n;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](float** p, size_t cnt) {
    *p = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(p, sizeof(float) * cnt);
  };
  alloc(&m->W, nw);
  alloc(&m->G, nw);
  alloc(&m->M, nw);
  alloc(&m->V, nw);
  alloc(&m->X, size_t(history) * n);
  alloc(&m->Y, size_t(history) * n);
  alloc(&m->work, vp_model_work_floats(n, rank, history));
  alloc(&m->loss, 1);
  alloc(&m->xs, size_t(n));
  alloc(&m->hs, size_t(rank));
  alloc(&m->ys, size_t(n));
  m->scale = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&m->scale, sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(m->M, 0, sizeof(float) * nw);
  if (e == cudaSuccess) e = cudaMemset(m->V, 0, sizeof(float) * nw);
  if (e == cudaSuccess) e = cudaMemset(m->W + size_t(rank) * n, 0, sizeof(float) * size_t(rank) * n);  // W2 = 0
  if (e == cudaSuccess) {
    init_weights<<<unsigned((size_t(rank) * n + 255) / 256), 256>>>(size_t(rank) * n, m->W,
                                                                   float(std::sqrt(3.0 / double(n))), 12345u);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    vp_model_destroy(m);
    return nullptr;
  }
  return m;
}

void vp_model_destroy(VpModel* m) {
  if (!m) return;
  cudaFree(m->W);
  cudaFree(m->G);
  cudaFree(m->M);
  cudaFree(m->V);
  cudaFree(m->X);
  cudaFree(m->Y);
  cudaFree(m->work);
  cudaFree(m->loss);
  cudaFree(m->xs);
  cudaFree(m->hs);
  cudaFree(m->ys);
  cudaFree(m->scale);
  delete m;
}

bool vp_model_ready(const VpModel* m) { return m && m->count >= 2; }
long long vp_model_steps(const VpModel* m) { return m ? m->steps : 0; }

cudaError_t vp_model_predict(VpModel* m, const double* rho, double* phi_out, cudaStream_t s) {
  const long long n = m->n;
  predict_prep<<<1, 1024, 0, s>>>(n, rho, m->xs, m->scale);
  // h = W1 x ; y = W2 h
  gemm(m->r, 1, int(n), 1.f, m->W, n, 1, m->xs, 1, 1, 0.f, m->hs, s);
  gemm(int(n), 1, m->r, 1.f, m->W + size_t(m->r) * n, m->r, 1, m->hs, 1, 1, 0.f, m->ys, s);
  predict_finish<<<1, 1024, 0, s>>>(n, m->ys, m->scale, phi_out);
  return cudaGetLastError();
}

cudaError_t vp_model_observe(VpModel* m, const double* rho, const double* phi, cudaStream_t s, bool train) {
  const long long n = m->n;
  store_pair<<<1, 1024, 0, s>>>(n, rho, phi, m->X, m->Y, m->head);
  m->head = (m->head + 1) % m->H;
  if (m->count < m->H) ++m->count;
  if (!train) return cudaGetLastError();
  const int B = m->count;
  const size_t nw = size_t(2) * m->r * n;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int it = 0; it < m->iters_per_obs; ++it) {
    cudaError_t e = vp_model_loss_grad(n, m->r, B, m->W, m->W + size_t(m->r) * n, m->X, m->Y, m->G,
                                       m->G + size_t(m->r) * n, nullptr, m->work, s);
    if (e != cudaSuccess) return e;
    ++m->steps;
    const float c1 = 1.f - std::pow(b1, float(m->steps)), c2 = 1.f - std::pow(b2, float(m->steps));
    adam_kernel<<<unsigned((nw + 255) / 256), 256, 0, s>>>(nw, m->W, m->G, m->M, m->V, m->lr, b1, b2, eps, c1, c2);
  }
  return cudaGetLastError();
}

}  // namespace hd
