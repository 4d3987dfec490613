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

// The analytic functions are products of one-dimensional factors, so their
// values at the nodes are products of table entries: table[off_d + c*N + i]
// holds factor d at x_d = lo_d + (c + gl_i) h_d (kind 2); the amplitude is
// applied once per node.  One table kernel per call, then one block per cell.
__global__ void function_table_kernel(VecGeom g, DevFunction f, double t, double* __restrict__ table, int total,
                                      int at_gauss) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= total) return;
  int d = 0, off = 0;
  while (d < g.D - 1 && e >= off + g.cells[d] * g.N) {
    off += g.cells[d] * g.N;
    ++d;
  }
  const int c = (e - off) / g.N, i = (e - off) % g.N;
  const double x = g.lo[d] + (c + (at_gauss ? g.gq[i] : g.gl[i])) * g.h[d];
  const double arg = f.omega[d] * (x - f.speed[d] * t) + f.phase[d];
  table[e] = f.cosine[d] ? cos(arg) : sin(arg);
}

// cell coordinates of cell gid and the table offsets of its factors
__device__ __forceinline__ void cell_offsets(const VecGeom& g, long long gid, int* toff) {
  long long gx = gid % g.ncx, gv = gid / g.ncx;
  int off = 0;
  for (int d = 0; d < g.D; ++d) {
    int c;
    if (d < g.dim_x) { c = int(gx % g.cells[d]); gx /= g.cells[d]; }
    else { c = int(gv % g.cells[d]); gv /= g.cells[d]; }
    toff[d] = off + c * g.N;
    off += g.cells[d] * g.N;
  }
}

__device__ __forceinline__ double node_value(const VecGeom& g, const DevFunction& f, const double* table,
                                             const int* toff, int node, double* jxw) {
  double v = f.kind == 0 ? 0.0 : f.amp, j = 1.0;
  for (int d = 0; d < g.D; ++d) {
    const int id = node % g.N;
    node /= g.N;
    if (f.kind == 2) v *= table[toff[d] + id];
    j *= g.h[d] * g.glw[id];
  }
  *jxw = j;
  return v;
}

template <typename T>
__global__ void interpolate_kernel(VecGeom g, DevFunction f, const double* __restrict__ table, T* __restrict__ dst,
                                   long long n_cells) {
  for (long long gid = blockIdx.x; gid < n_cells; gid += gridDim.x) {
    int toff[kMaxDim];
    cell_offsets(g, g.gid0 + gid, toff);
    T* out = dst + gid * g.NC;
    for (int node = threadIdx.x; node < g.NC; node += blockDim.x) {
      double jxw;
      out[node] = T(node_value(g, f, table, toff, node, &jxw));
    }
  }
}

// per-block partial sums of (v^2 JxW, (v - f)^2 JxW); block b handles cells b, b + gridDim, ...
template <typename T>
__global__ void norm_error_kernel(VecGeom g, DevFunction f, const double* __restrict__ table,
                                  const T* __restrict__ src, long long n_cells, double* __restrict__ partials) {
  double s0 = 0.0, s1 = 0.0;
  for (long long gid = blockIdx.x; gid < n_cells; gid += gridDim.x) {
    int toff[kMaxDim];
    cell_offsets(g, g.gid0 + gid, toff);
    const T* in = src + gid * g.NC;
    for (int node = threadIdx.x; node < g.NC; node += blockDim.x) {
      double jxw;
      const double ex = node_value(g, f, table, toff, node, &jxw);
      const double v = double(in[node]);
      const double e = v - ex;
      s0 += v * v * jxw;
      s1 += e * e * jxw;
    }
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

// Gauss quadrature (vector_tools.h:144-223 with quadrature 0 = Gauss): per
// cell the Gauss-point values (S in every direction, in shared memory), then
// the same sums with the Gauss weights and the function at the Gauss points
template <typename T>
__global__ void norm_error_gauss_kernel(VecGeom g, DevFunction f, const double* __restrict__ table,
                                        const T* __restrict__ src, long long n_cells, double* __restrict__ partials) {
  extern __shared__ double sv[];
  double s0 = 0.0, s1 = 0.0;
  const int N = g.N, NC = g.NC, NL = g.NC / g.N;
  for (long long gid = blockIdx.x; gid < n_cells; gid += gridDim.x) {
    const T* in = src + gid * NC;
    for (int node = threadIdx.x; node < NC; node += blockDim.x) sv[node] = double(in[node]);
    __syncthreads();
    int se = 1;
    for (int e = 0; e < g.D; ++e) {
      for (int line = threadIdx.x; line < NL; line += blockDim.x) {
        int base = 0, stride = 1, l = line;
        for (int f2 = 0; f2 < g.D; ++f2) {
          if (f2 != e) {
            base += (l % N) * stride;
            l /= N;
          }
          stride *= N;
        }
        double u[kMaxN];
        for (int q = 0; q < N; ++q) u[q] = sv[base + q * se];
        for (int i = 0; i < N; ++i) {
          double acc = 0.0;
          for (int q = 0; q < N; ++q) acc += g.S[i * N + q] * u[q];
          sv[base + i * se] = acc;
        }
      }
      se *= N;
      __syncthreads();
    }
    int toff[kMaxDim];
    cell_offsets(g, g.gid0 + gid, toff);
    for (int node = threadIdx.x; node < NC; node += blockDim.x) {
      double ex = f.kind == 0 ? 0.0 : f.amp, jxw = 1.0;
      int t = node;
      for (int d = 0; d < g.D; ++d) {
        const int id = t % N;
        t /= N;
        if (f.kind == 2) ex *= table[toff[d] + id];
        jxw *= g.h[d] * g.gw[id];
      }
      const double v = sv[node];
      const double e = v - ex;
      s0 += v * v * jxw;
      s1 += e * e * jxw;
    }
    __syncthreads();
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

static int table_size(const VecGeom& g) {
  int total = 0;
  for (int d = 0; d < g.D; ++d) total += g.cells[d] * g.N;
  return total;
}

static cudaError_t fill_table(const VecGeom& g, const DevFunction& f, double t, double* table, cudaStream_t s,
                              int at_gauss = 0) {
  if (f.kind != 2) return cudaSuccess;
  const int total = table_size(g);
  function_table_kernel<<<(total + 127) / 128, 128, 0, s>>>(g, f, t, table, total, at_gauss);
  return cudaGetLastError();
}

static int node_threads(const VecGeom& g) { return g.NC >= 256 ? 256 : ((g.NC + 31) / 32) * 32; }

cudaError_t launch_interpolate(const VecGeom& g, const DevFunction& f, double t, void* dst, int is_f32,
                               double* table, cudaStream_t s) {
  cudaError_t e = fill_table(g, f, t, table, s);
  if (e != cudaSuccess) return e;
  const long long n_cells = g.n_dofs / g.NC;
  const unsigned grid = unsigned(n_cells < 152 * 64 ? n_cells : 152 * 64);
  if (is_f32) interpolate_kernel<float><<<grid, node_threads(g), 0, s>>>(g, f, table, (float*)dst, n_cells);
  else interpolate_kernel<double><<<grid, node_threads(g), 0, s>>>(g, f, table, (double*)dst, n_cells);
  return cudaGetLastError();
}

cudaError_t launch_norm_error(const VecGeom& g, const DevFunction& f, double t, const void* src, int is_f32,
                              double* table, double* partials, double* out, cudaStream_t s) {
  cudaError_t e = fill_table(g, f, t, table, s, g.gauss);
  if (e != cudaSuccess) return e;
  const long long n_cells = g.n_dofs / g.NC;
  const unsigned grid = kNormBlocks;
  if (g.gauss) {
    const size_t smem = sizeof(double) * g.NC;
    if (smem > 48 * 1024) {
      e = cudaFuncSetAttribute(is_f32 ? (const void*)norm_error_gauss_kernel<float>
                                      : (const void*)norm_error_gauss_kernel<double>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
    }
    if (is_f32)
      norm_error_gauss_kernel<float><<<grid, node_threads(g), smem, s>>>(g, f, table, (const float*)src, n_cells,
                                                                         partials);
    else
      norm_error_gauss_kernel<double><<<grid, node_threads(g), smem, s>>>(g, f, table, (const double*)src, n_cells,
                                                                          partials);
  } else if (is_f32)
    norm_error_kernel<float><<<grid, node_threads(g), 0, s>>>(g, f, table, (const float*)src, n_cells, partials);
  else
    norm_error_kernel<double><<<grid, node_threads(g), 0, s>>>(g, f, table, (const double*)src, n_cells, partials);
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

// The face pack of a partitioned operator (hd_adv_pack_faces): one face slab
// per cell of a layer, gathered into the contiguous buffer the receiving part
// keeps as its ghost region.  16-byte words when every address and size
// allows, 4-byte words otherwise; consecutive threads copy consecutive words.
template <typename W>
__global__ void pack_faces_kernel(const char* __restrict__ src, long long stride, long long words_per_face,
                                  long long n_faces, char* __restrict__ dst) {
  const long long total = words_per_face * n_faces;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long f = i / words_per_face, j = i - f * words_per_face;
    reinterpret_cast<W*>(dst)[i] = __ldcs(reinterpret_cast<const W*>(src + f * stride) + j);
  }
}

cudaError_t launch_pack_faces(const void* src, long long stride_bytes, long long face_bytes, long long n_faces,
                              void* dst, cudaStream_t s) {
  if (n_faces <= 0 || face_bytes <= 0) return cudaSuccess;
  const bool w16 = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0 &&
                   stride_bytes % 16 == 0 && face_bytes % 16 == 0;
  const long long words = n_faces * (face_bytes / (w16 ? 16 : 4));
  const long long want = (words + 255) / 256;
  const unsigned grid = unsigned(want < 152 * 16 ? want : 152 * 16);
  if (w16)
    pack_faces_kernel<float4><<<grid, 256, 0, s>>>((const char*)src, stride_bytes, face_bytes / 16, n_faces,
                                                   (char*)dst);
  else
    pack_faces_kernel<float><<<grid, 256, 0, s>>>((const char*)src, stride_bytes, face_bytes / 4, n_faces,
                                                  (char*)dst);
  return cudaGetLastError();
}

}  // namespace hd
