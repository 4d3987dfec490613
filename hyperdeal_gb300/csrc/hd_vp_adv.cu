// hd_vp_adv.cu -- ECL advection with the Vlasov-Poisson phase-space velocity.
//
// Along every line of a cell the velocity component of that line's direction
// is constant: for an x-direction d it is the line's v-coordinate v_d (the
// line moves in x only), for a v-direction it is grad(phi)_d at the line's
// x-node (the line moves in v only).  The operator on a line is therefore
// (a/h) [G u + upwind face terms], with the upwind side chosen per line by
// the sign of a -- the reference's flux 0.5((u-+u+)a.n + |a.n|(u- - u+))
// evaluated at the line's face points (advection_operation.h:325-526 with
// the velocities of velocity_field_view.h:103-209 of the VP example).
#include <cuda_runtime.h>

#include "hd_ecl.cuh"
#include "hd_vp.cuh"

namespace hd {

template <typename T>
struct VpLine {
  T G[kMaxN * kMaxN];  // G[i*N + q]
  T winv0, winvk;      // 1/w_0, 1/w_{N-1}
};

template <int D, int N, typename T>
__global__ void __launch_bounds__(EclShape<D, N, T>::THREADS)
    vp_adv_kernel(const __grid_constant__ VpAdvParams<T> P, const __grid_constant__ VpLine<T> Lk) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC, CPB = S::CPB, DX = D / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_u = reinterpret_cast<T*>(smem_raw);
  T* s_o = s_u + CPB * NC;
  const VpGeom& g = P.g;

  const int tid = threadIdx.x;
  const int lc = tid / TPC, tl = tid % TPC;
  const long long cell0 = (long long)blockIdx.x * CPB;
  const long long gid = cell0 + lc;
  const bool valid = gid < g.n_cells;
  const long long ncell_here = (g.n_cells - cell0) < CPB ? (g.n_cells - cell0) : CPB;
  {
    const T* src = P.src + cell0 * NC;
    const long long nval = ncell_here * NC;
    for (long long i = tid; i < nval; i += S::THREADS) s_u[i] = __ldg(src + i);
  }
  __syncthreads();

  int cc[D];
  long long nbL[D], nbR[D];
  long long gx = 0;
  {
    const long long gg = valid ? gid : 0;
    gx = gg % g.ncx;
    long long a = gx, b = gg / g.ncx;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if (d < DX) { cc[d] = int(a % g.cells[d]); a /= g.cells[d]; }
      else { cc[d] = int(b % g.cells[d]); b /= g.cells[d]; }
      const long long cs = g.cstride[d];
      nbL[d] = cc[d] > 0 ? gg - cs : gg + (long long)(g.cells[d] - 1) * cs;
      nbR[d] = cc[d] + 1 < g.cells[d] ? gg + cs : gg - (long long)(g.cells[d] - 1) * cs;
    }
  }
  T* su = s_u + lc * NC;
  T* so = s_o + lc * NC;

  // velocity / h of the line along d through node `bnode` (any node of the line)
  auto line_scale = [&](int d, int bnode) -> T {
    if (d < DX) {
      const int e = DX + d;
      const int ie = (bnode / ipow(N, e)) % N;
      return __ldg(P.xs + (d * g.cells[e] + cc[e]) * N + ie);
    }
    return __ldg(P.es + (gx * g.NCx + (bnode % ipow(N, DX))) * DX + (d - DX));
  };

  // phases of two directions; each line: out += (a/h) [G u + upwind face terms]
#pragma unroll
  for (int ph = 0; ph < S::NPH; ++ph) {
    const int dA = 2 * ph;
    const int dB = (2 * ph + 1 < D) ? 2 * ph + 1 : -1;
    const int strideA = ipow(N, dA);
    const int strideB = strideA * N;
    const int nitems = dB >= 0 ? ipow(N, D - 2) : ipow(N, D - 1);
    const bool last = (ph == S::NPH - 1);
    for (int item = tl; item < nitems; item += TPC) {
      const int base = item_base<D, N>(item, dA, dB);
      if (dB >= 0) {
        T uu[N][N], acc[N][N];
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
          for (int b = 0; b < N; ++b) {
            const int node = base + a * strideA + b * strideB;
            uu[a][b] = su[node];
            acc[a][b] = ph == 0 ? T(0) : so[node];
          }
        if (valid) {
          // direction A: lines indexed by b
#pragma unroll
          for (int b = 0; b < N; ++b) {
            const int bn = base + b * strideB;
            const T sc = line_scale(dA, bn);
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = T(0);
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(Lk.G[i * N + q], uu[q][b], s);
              acc[i][b] = fma(sc, s, acc[i][b]);
            }
            const bool pos = sc > T(0);
            const T up = __ldg(P.src + (pos ? nbL[dA] * NC + bn + (N - 1) * strideA : nbR[dA] * NC + bn));
            if (sc != T(0)) {
              if (pos) {
                acc[N - 1][b] = fma(-sc * Lk.winvk, uu[N - 1][b], acc[N - 1][b]);
                acc[0][b] = fma(sc * Lk.winv0, up, acc[0][b]);
              } else {
                acc[0][b] = fma(sc * Lk.winv0, uu[0][b], acc[0][b]);
                acc[N - 1][b] = fma(-sc * Lk.winvk, up, acc[N - 1][b]);
              }
            }
          }
          // direction B: lines indexed by a
#pragma unroll
          for (int a = 0; a < N; ++a) {
            const int bn = base + a * strideA;
            const T sc = line_scale(dB, bn);
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = T(0);
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(Lk.G[i * N + q], uu[a][q], s);
              acc[a][i] = fma(sc, s, acc[a][i]);
            }
            const bool pos = sc > T(0);
            const T up = __ldg(P.src + (pos ? nbL[dB] * NC + bn + (N - 1) * strideB : nbR[dB] * NC + bn));
            if (sc != T(0)) {
              if (pos) {
                acc[a][N - 1] = fma(-sc * Lk.winvk, uu[a][N - 1], acc[a][N - 1]);
                acc[a][0] = fma(sc * Lk.winv0, up, acc[a][0]);
              } else {
                acc[a][0] = fma(sc * Lk.winv0, uu[a][0], acc[a][0]);
                acc[a][N - 1] = fma(-sc * Lk.winvk, up, acc[a][N - 1]);
              }
            }
          }
        }
        if (!last) {
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = 0; b < N; ++b) so[base + a * strideA + b * strideB] = acc[a][b];
        } else if (valid) {
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = 0; b < N; ++b) P.dst[gid * NC + base + a * strideA + b * strideB] = acc[a][b];
        }
      } else {
        T uu[N], acc[N];
#pragma unroll
        for (int a = 0; a < N; ++a) {
          uu[a] = su[base + a * strideA];
          acc[a] = ph == 0 ? T(0) : so[base + a * strideA];
        }
        if (valid) {
          const T sc = line_scale(dA, base);
#pragma unroll
          for (int i = 0; i < N; ++i) {
            T s = T(0);
#pragma unroll
            for (int q = 0; q < N; ++q) s = fma(Lk.G[i * N + q], uu[q], s);
            acc[i] = fma(sc, s, acc[i]);
          }
          const bool pos = sc > T(0);
          const T up = __ldg(P.src + (pos ? nbL[dA] * NC + base + (N - 1) * strideA : nbR[dA] * NC + base));
          if (sc != T(0)) {
            if (pos) {
              acc[N - 1] = fma(-sc * Lk.winvk, uu[N - 1], acc[N - 1]);
              acc[0] = fma(sc * Lk.winv0, up, acc[0]);
            } else {
              acc[0] = fma(sc * Lk.winv0, uu[0], acc[0]);
              acc[N - 1] = fma(-sc * Lk.winvk, up, acc[N - 1]);
            }
          }
        }
        if (!last) {
#pragma unroll
          for (int a = 0; a < N; ++a) so[base + a * strideA] = acc[a];
        } else if (valid) {
#pragma unroll
          for (int a = 0; a < N; ++a) P.dst[gid * NC + base + a * strideA] = acc[a];
        }
      }
    }
    if (!last) __syncthreads();
  }
}

template <int D, int N, typename T>
static cudaError_t launch_vp_dn(const VpAdvParams<T>& P, cudaStream_t s) {
  using S = EclShape<D, N, T>;
  if constexpr (!S::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    constexpr size_t kSmem = size_t(2) * S::CPB * S::NC * sizeof(T);  // cell tile + accumulator tile
    VpLine<T> Lk;
    for (int i = 0; i < N * N; ++i) Lk.G[i] = T(P.g.G[i]);
    Lk.winv0 = T(1.0 / P.g.glw[0]);
    Lk.winvk = T(1.0 / P.g.glw[N - 1]);
    static bool attr = false;
    if (!attr) {
      cudaError_t e = cudaFuncSetAttribute(vp_adv_kernel<D, N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           int(kSmem));
      if (e != cudaSuccess) return e;
      attr = true;
    }
    const unsigned grid = unsigned((P.g.n_cells + S::CPB - 1) / S::CPB);
    vp_adv_kernel<D, N, T><<<grid, S::THREADS, kSmem, s>>>(P, Lk);
    return cudaGetLastError();
  }
}

template <typename T>
static cudaError_t launch_vp_any(const VpAdvParams<T>& P, cudaStream_t s) {
#define HD_VP_CASE(DD, NN) \
  if (P.g.D == DD && P.g.N == NN) return launch_vp_dn<DD, NN, T>(P, s);
  HD_VP_CASE(2, 2) HD_VP_CASE(2, 3) HD_VP_CASE(2, 4) HD_VP_CASE(2, 5) HD_VP_CASE(2, 6)
  HD_VP_CASE(4, 2) HD_VP_CASE(4, 3) HD_VP_CASE(4, 4) HD_VP_CASE(4, 5) HD_VP_CASE(4, 6)
  HD_VP_CASE(6, 2) HD_VP_CASE(6, 3) HD_VP_CASE(6, 4)
#undef HD_VP_CASE
  return cudaErrorNotSupported;
}

cudaError_t launch_vp_advection(const VpAdvParams<float>& P, cudaStream_t s) { return launch_vp_any(P, s); }
cudaError_t launch_vp_advection(const VpAdvParams<double>& P, cudaStream_t s) { return launch_vp_any(P, s); }

}  // namespace hd
