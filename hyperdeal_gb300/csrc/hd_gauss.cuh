// hd_gauss.cuh -- the ECL advection operator with Gauss quadrature
// (n_points = degree + 1, non-collocation), the reference's second branch
// (advection_operation.h:294-316 basis change, :426-449 face values,
// :536-559 inverse mass through inverse_shape_values).
//
// The DoFs are Gauss-Lobatto nodal values.  With S[q][j] = L_j(xi_q) (the
// Gauss-Lobatto Lagrange basis at the Gauss points) a cell's values at the
// Gauss points are v = (S x ... x S) u.  In the Gauss-point Lagrange basis the
// Gauss-quadrature mass matrix is diagonal, so the operator is: transform,
// apply one-dimensional line operators along every direction (dense M_d
// from the reference's volume and face formulas, a dense inflow vector c_d
// times the upwind face value), then transform back with S^{-1}: exactly
// the reference's M^{-1} r with M = S^T W S.  The upwind neighbour's face
// value at a face point is its Gauss-Lobatto end-node value in the normal
// direction (the basis interpolates there), transformed by S in the
// tangential directions.
#pragma once

#include <cuda_runtime.h>

#include "hd_ecl.cuh"

namespace hd {

// data of the Gauss path beside EclParams (op[d].M holds M_d in the Gauss
// basis; op[d].in_node/nb_node/step/active as in the collocation path)
template <typename T>
struct GaussExtra {
  T S[kMaxN * kMaxN];         // Gauss-Lobatto nodal -> Gauss-point values
  T Si[kMaxN * kMaxN];        // its inverse
  T cv[kMaxDim][kMaxN];       // inflow coefficient vector of direction d
  T le[kMaxDim][kMaxN];       // own face value at the inflow face: le[d] . v_line
  double gq[kMaxN];           // Gauss points on [0,1] (boundary data coordinates)
};

// 4 tiles: staged nodal input (2, cp.async double buffer), Gauss values, accumulator, face slabs
template <int D, int N, typename T>
struct GaussShape {
  using S = EclShape<D, N, T>;
  static constexpr int NC = S::NC, TPC = S::TPC, CPB = S::CPB, THREADS = S::THREADS;
  static constexpr bool SUPPORTED = size_t(5) * CPB * NC * sizeof(T) + 48 <= 220 * 1024;
};

// elements of one (unpadded) cell tile buffer of this path, rounded to 16 bytes
template <int D, int N, typename T>
__host__ __device__ constexpr long long gauss_buffer_elems(int cpb) {
  const long long bytes = (long long)cpb * EclShape<D, N, T>::NC * sizeof(T);
  return ((bytes + 15) / 16) * 16 / (long long)sizeof(T);
}

// apply the N x N matrix A (row-major, A[i*N + q]) along direction e to every
// line of the cell tile x (in place); threads tl of TPC share the lines
template <int D, int N, typename T>
__device__ __forceinline__ void gauss_pass(T* x, const T* A, int e, int tl, int TPC, int nlines) {
  const int se = ipow(N, e);
  for (int line = tl; line < nlines; line += TPC) {
    // base node of the line: the digits of `line` fill the other directions
    int base = 0, stride = 1, l = line;
#pragma unroll
    for (int f = 0; f < D; ++f) {
      if (f != e) {
        base += (l % N) * stride;
        l /= N;
      }
      stride *= N;
    }
    T u[N], r[N];
#pragma unroll
    for (int q = 0; q < N; ++q) u[q] = x[base + q * se];
#pragma unroll
    for (int i = 0; i < N; ++i) {
      T s = T(0);
#pragma unroll
      for (int q = 0; q < N; ++q) s = fma(A[i * N + q], u[q], s);
      r[i] = s;
    }
#pragma unroll
    for (int i = 0; i < N; ++i) x[base + i * se] = r[i];
  }
}

// MODE is a run-time argument here (this path is not the bandwidth-critical
// one; one kernel per (D, N, T) keeps the build small)
template <int D, int N, typename T>
__device__ __forceinline__ void gauss_block(const EclParams<T>& P, const GaussExtra<T>& G, int MODE, long long cell0,
                                            int lc, int tl, const T* su_all, T* sv_all, T* so_all, T* sf_all) {
  constexpr int NC = EclShape<D, N, T>::NC, TPC = EclShape<D, N, T>::TPC;
  constexpr int NL = NC / N;  // lines per direction
  const long long gid = cell0 + lc;
  const bool valid = gid < P.n_cells;
  const T* su = su_all + lc * NC;
  T* sv = sv_all + lc * NC;
  T* so = so_all + lc * NC;
  T* sf = sf_all + lc * NC;
  int cc[D];
  cell_coords<D>(P, valid ? gid : 0, cc);
  // 1. Gauss-point values v, accumulator 0
  for (int i = tl; i < NC; i += TPC) {
    sv[i] = su[i];
    so[i] = T(0);
  }
  __syncthreads();
#pragma unroll
  for (int e = 0; e < D; ++e) {
    gauss_pass<D, N, T>(sv, G.S, e, tl, TPC, NL);
    __syncthreads();
  }
  // 2. directions one after the other: the upwind face slab (in sf at the
  // nodes with digit d = 0), then the lines along d
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const LineOp<T>& L = P.op[d];
    const int sd = ipow(N, d);
    const bool act = valid && L.active;
    const long long nb = act ? neighbour(P, gid, cc, d) : -1;
    // (every barrier below is reached by all threads; the per-cell
    // conditions only guard the work between them)
    if (nb >= 0) {
      const T* src = P.tin + nb * NC;
      for (int t = tl; t < NL; t += TPC) {
        // t enumerates the tangential digits; node with digit d = nb_node
        int base = 0, stride = 1, l = t;
#pragma unroll
        for (int f = 0; f < D; ++f) {
          if (f != d) {
            base += (l % N) * stride;
            l /= N;
          }
          stride *= N;
        }
        sf[base] = __ldg(src + base + L.nb_node * sd);
      }
    }
    __syncthreads();
    // tangential transforms of the slab (lines along e inside the d = 0 hyperplane)
#pragma unroll
    for (int e = 0; e < D; ++e) {
      if (e == d) continue;
      if (nb >= 0) {
        const int se = ipow(N, e);
        for (int line = tl; line < NL / N; line += TPC) {
          int base = 0, stride = 1, l = line;
#pragma unroll
          for (int f = 0; f < D; ++f) {
            if (f != e && f != d) {
              base += (l % N) * stride;
              l /= N;
            }
            stride *= N;
          }
          T u[N], r[N];
#pragma unroll
          for (int q = 0; q < N; ++q) u[q] = sf[base + q * se];
#pragma unroll
          for (int i = 0; i < N; ++i) {
            T s = T(0);
#pragma unroll
            for (int q = 0; q < N; ++q) s = fma(G.S[i * N + q], u[q], s);
            r[i] = s;
          }
#pragma unroll
          for (int i = 0; i < N; ++i) sf[base + i * se] = r[i];
        }
      }
      __syncthreads();
    }
    // lines along d: acc += M_d v + cv_d * u+
    for (int t = tl; t < NL; t += TPC) {
      int base = 0, stride = 1, l = t;
#pragma unroll
      for (int f = 0; f < D; ++f) {
        if (f != d) {
          base += (l % N) * stride;
          l /= N;
        }
        stride *= N;
      }
      if (!act) continue;
      T v[N];
#pragma unroll
      for (int q = 0; q < N; ++q) v[q] = sv[base + q * sd];
      T up;
      if (nb >= 0) {
        up = sf[base];
      } else {
        // boundary face: u+ = -u- + 2 g(x) at the face point (tangential Gauss coordinates)
        T um = T(0);
#pragma unroll
        for (int q = 0; q < N; ++q) um = fma(G.le[d][q], v[q], um);
        up = -um;
        if (P.bc_inhom) {
          double x[kMaxDim];
          int node = base;
#pragma unroll
          for (int f = 0; f < D; ++f) {
            const int id = node % N;
            node /= N;
            x[f] = (f == d) ? node_coord(P.lo[f], cc[f], L.step > 0 ? 1.0 : 0.0, P.h[f])
                            : node_coord(P.lo[f], cc[f], G.gq[id], P.h[f]);
          }
          up = T(dirichlet_exterior(double(um), eval_function(P.bc, x, D, P.time)));
        }
      }
#pragma unroll
      for (int i = 0; i < N; ++i) {
        T s = so[base + i * sd];
#pragma unroll
        for (int q = 0; q < N; ++q) s = fma(L.M[i * N + q], v[q], s);
        s = fma(G.cv[d][i], up, s);
        so[base + i * sd] = s;
      }
    }
    __syncthreads();
  }
  // 3. back to Gauss-Lobatto nodal values
#pragma unroll
  for (int e = 0; e < D; ++e) {
    gauss_pass<D, N, T>(so, G.Si, e, tl, TPC, NL);
    __syncthreads();
  }
  // 4. result
  if (valid) {
    const long long g0 = gid * NC;
    for (int i = tl; i < NC; i += TPC) {
      const T k = so[i];
      if (MODE == kApply) {
        P.uout[g0 + i] = k;
      } else {
        const T u = (MODE == kStageFirst) ? su[i] : P.uin[g0 + i];
        P.uout[g0 + i] = fma(P.fb, k, u);
        if (MODE != kStageLast) P.tout[g0 + i] = fma(P.fa, k, u);
      }
    }
  }
}

template <int D, int N, typename T>
__global__ void __launch_bounds__(EclShape<D, N, T>::THREADS)
    gauss_kernel(const __grid_constant__ EclParams<T> P, const __grid_constant__ GaussExtra<T> G, int mode) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cpb = P.cpb;
  const long long bufe = gauss_buffer_elems<D, N, T>(cpb);
  T* const s_in0 = reinterpret_cast<T*>(smem_raw);
  T* const s_in1 = s_in0 + bufe;
  T* const s_v = s_in0 + 2 * bufe;
  T* const s_o = s_in0 + 3 * bufe;
  T* const s_f = s_in0 + 4 * bufe;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int lc = tid / TPC, tl = tid % TPC;
  const long long nblk = (P.n_cells + cpb - 1) / cpb;
  auto stage = [&](T* dst, long long blk) {
    const long long c0 = blk * cpb;
    const long long ncell = (P.n_cells - c0) < cpb ? (P.n_cells - c0) : cpb;
    stage_async(dst, P.tin + c0 * NC, ncell * NC, tid, nthr);
  };
  long long b = blockIdx.x;
  if (b < nblk) stage(s_in0, b);
  cp_async_commit();
  bool odd = false;
  for (; b < nblk; b += gridDim.x) {
    T* const cur = odd ? s_in1 : s_in0;
    T* const nxt = odd ? s_in0 : s_in1;
    const long long nb = b + gridDim.x;
    if (nb < nblk) stage(nxt, nb);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    gauss_block<D, N, T>(P, G, mode, b * cpb, lc, tl, cur, s_v, s_o, s_f);
    __syncthreads();
    odd = !odd;
  }
  cp_async_wait<0>();
}

template <int D, int N, typename T>
cudaError_t launch_gauss(const EclParams<T>& P0, const GaussExtra<T>& G, int mode, cudaStream_t stream) {
  using GS = GaussShape<D, N, T>;
  using S = EclShape<D, N, T>;
  if constexpr (!GS::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    EclParams<T> P = P0;
    if (P.cpb < 1 || P.cpb > S::CPB) P.cpb = ecl_default_cpb<D, N, T>();
    const int threads = S::TPC * P.cpb;
    const size_t smem = size_t(5 * gauss_buffer_elems<D, N, T>(P.cpb)) * sizeof(T);
    if (mode < kApply || mode > kStageLast) return cudaErrorInvalidValue;
    static bool attr_done = false;
    static int sms = 0;
    auto kern = gauss_kernel<D, N, T>;
    if (!attr_done) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(5 * gauss_buffer_elems<D, N, T>(S::CPB) * sizeof(T)));
      if (e != cudaSuccess) return e;
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      attr_done = true;
    }
    int per_sm = P.ctas_per_sm;
    if (per_sm < 1) {
      cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) per_sm = 1;
    }
    const long long nblk = (P.n_cells + P.cpb - 1) / P.cpb;
    const long long want = (long long)sms * per_sm;
    kern<<<unsigned(nblk < want ? nblk : want), threads, smem, stream>>>(P, G, mode);
    return cudaGetLastError();
  }
}

struct GaussLaunchers {
  cudaError_t (*f64)(const EclParams<double>&, const GaussExtra<double>&, int, cudaStream_t);
  cudaError_t (*f32)(const EclParams<float>&, const GaussExtra<float>&, int, cudaStream_t);
  bool ok_f64, ok_f32;
};

template <int D, int N>
GaussLaunchers make_gauss_launchers() {
  return GaussLaunchers{&launch_gauss<D, N, double>, &launch_gauss<D, N, float>, GaussShape<D, N, double>::SUPPORTED,
                        GaussShape<D, N, float>::SUPPORTED};
}

GaussLaunchers gauss_launchers(int D, int N);

}  // namespace hd
