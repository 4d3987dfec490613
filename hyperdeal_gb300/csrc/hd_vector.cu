// hd_vector.cu -- vector kernels around the advection operator:
// nodal interpolation, L2 norm / error, and the low-storage Runge-Kutta
// stage update for the unfused path.
//
// Reference: include/hyper.deal/numerics/vector_tools.h:81-223 (interpolate,
// norm_and_error), include/hyper.deal/base/time_integrators.templates.h:111-135
// (stage update).
#include <cuda_runtime.h>

#include "hd_ecl.cuh"
#include "hd_vector.cuh"

namespace hd {

// geometry of a nodal DG vector (cell gid, node -> coordinates)
__device__ __forceinline__ void node_coords(const VecGeom& g, long long i, double* x, double* jxw) {
  const long long gid = i / g.NC;
  int node = int(i - gid * g.NC);
  long long gx = gid % g.ncx, gv = gid / g.ncx;
  double j = 1.0;
  for (int d = 0; d < g.D; ++d) {
    int c;
    if (d < g.dim_x) { c = int(gx % g.cells[d]); gx /= g.cells[d]; }
    else { c = int(gv % g.cells[d]); gv /= g.cells[d]; }
    const int id = node % g.N;
    node /= g.N;
    x[d] = g.lo[d] + (c + g.gl[id]) * g.h[d];
    j *= g.h[d] * g.glw[id];
  }
  *jxw = j;
}

template <typename T>
__global__ void interpolate_kernel(VecGeom g, DevFunction f, double t, T* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double x[kMaxDim], jxw;
    node_coords(g, i, x, &jxw);
    dst[i] = T(eval_function(f, x, g.D, t));
  }
}

// per-block partial sums of (v^2 JxW, (v - f)^2 JxW) in fixed order
template <typename T>
__global__ void norm_error_kernel(VecGeom g, DevFunction f, double t, const T* __restrict__ src, long long n,
                                  double* __restrict__ partials) {
  double s0 = 0.0, s1 = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double x[kMaxDim], jxw;
    node_coords(g, i, x, &jxw);
    const double v = double(src[i]);
    const double e = v - eval_function(f, x, g.D, t);
    s0 += v * v * jxw;
    s1 += e * e * jxw;
  }
  __shared__ double r0[32], r1[32];
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) { r0[w] = s0; r1[w] = s1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < (int)(blockDim.x / 32); ++k) { a += r0[k]; b += r1[k]; }
    partials[2 * blockIdx.x] = a;
    partials[2 * blockIdx.x + 1] = b;
  }
}

__global__ void reduce_partials_kernel(const double* __restrict__ partials, int nblocks, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nblocks; ++k) { a += partials[2 * k]; b += partials[2 * k + 1]; }
    out[0] = sqrt(a);
    out[1] = sqrt(b);
  }
}

// sol = sol + bi K ; if ai != 0: next_T = sol_old + ai K
template <typename T>
__global__ void lsrk_update_kernel(long long n, T bi, T ai, const T* __restrict__ K, T* __restrict__ sol,
                                   T* __restrict__ next_T) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const T k = K[i], s0 = sol[i];
    sol[i] = s0 + bi * k;
    if (next_T) next_T[i] = s0 + ai * k;
  }
}

static unsigned grid_for(long long n, int threads, int max_blocks) {
  long long b = (n + threads - 1) / threads;
  if (b > max_blocks) b = max_blocks;
  if (b < 1) b = 1;
  return unsigned(b);
}

cudaError_t launch_interpolate(const VecGeom& g, const DevFunction& f, double t, void* dst, int is_f32,
                               cudaStream_t s) {
  const long long n = g.n_dofs;
  const unsigned grid = grid_for(n, 256, 152 * 32);
  if (is_f32) interpolate_kernel<float><<<grid, 256, 0, s>>>(g, f, t, (float*)dst, n);
  else interpolate_kernel<double><<<grid, 256, 0, s>>>(g, f, t, (double*)dst, n);
  return cudaGetLastError();
}

cudaError_t launch_norm_error(const VecGeom& g, const DevFunction& f, double t, const void* src, int is_f32,
                              double* partials, double* out, cudaStream_t s) {
  const long long n = g.n_dofs;
  const unsigned grid = kNormBlocks;
  if (is_f32) norm_error_kernel<float><<<grid, 256, 0, s>>>(g, f, t, (const float*)src, n, partials);
  else norm_error_kernel<double><<<grid, 256, 0, s>>>(g, f, t, (const double*)src, n, partials);
  reduce_partials_kernel<<<1, 32, 0, s>>>(partials, int(grid), out);
  return cudaGetLastError();
}

cudaError_t launch_lsrk_update(int is_f32, long long n, double bi, double ai, const void* K, void* sol,
                               void* next_T, cudaStream_t s) {
  const unsigned grid = grid_for(n, 256, 152 * 16);
  if (is_f32)
    lsrk_update_kernel<float><<<grid, 256, 0, s>>>(n, float(bi), float(ai), (const float*)K, (float*)sol,
                                                    (float*)next_T);
  else
    lsrk_update_kernel<double><<<grid, 256, 0, s>>>(n, bi, ai, (const double*)K, (double*)sol,
                                                     (double*)next_T);
  return cudaGetLastError();
}

}  // namespace hd
