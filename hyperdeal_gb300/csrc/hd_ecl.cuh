// hd_ecl.cuh -- element-centric (ECL) upwind-DG advection kernels for sm_103a.
//
// One CTA owns CPB whole cells.  Each cell's (k+1)^D nodal values are staged
// in shared memory with coalesced 16-byte loads; the D one-dimensional line
// operators are applied two directions at a time ("plane phases") with the
// plane's N x N values held in registers, and the upwind neighbour's face
// trace is read straight from global memory (L2) -- there is no face loop and
// no atomics.  The inverse (diagonal) mass, the upwind flux and the downwind
// self-term are folded into the per-direction line operator M_d and the
// inflow coefficient c_d that the host derives from the reference's formulas,
// so one phase does  acc_line += M_d u_line  and  acc[in_node] += c_d u+.
// The last phase writes the result once: either K = A(u) (apply) or, fused
// with the low-storage Runge-Kutta stage, U' = U + b K and T' = U + a K.
//
// Reference operator: include/hyper.deal/operators/advection/
// advection_operation.h:218-566 (volume :325-404, faces :406-526, inverse
// mass :528-563); stage update: base/time_integrators.templates.h:111-135.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace hd {

constexpr int kMaxDim = 6;
constexpr int kMaxN = 6;  // nodes per direction (degree <= 5)

__host__ __device__ constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// analytic function  amp * prod_d trig(omega_d (x_d - speed_d t) + phase_d)
struct DevFunction {
  int kind;
  double amp;
  double omega[kMaxDim], speed[kMaxDim], phase[kMaxDim];
  int cosine[kMaxDim];
};

// one-dimensional line operator of one direction (see hd_capi.cu: derived
// from the reference's volume + face + inverse-mass formulas)
template <typename T>
struct LineOp {
  T M[kMaxN * kMaxN];  // out_i += M[i*N + q] * u_q
  T cin;               // out_{in_node} += cin * u+
  T c0, cl;            // the same coefficient split by target: node 0 / node N-1 (the other is 0)
  int in_node;         // node of the line that receives the inflow term
  int nb_node;         // node of the upwind neighbour's line giving u+
  int step;            // -1: upwind neighbour on the left, +1: on the right
  int active;          // 0: nothing to do in this direction
};

template <typename T>
struct EclParams {
  const T* tin;   // operator input (also read at neighbours)
  const T* uin;   // RK solution (own cell only); may equal tin
  T* uout;        // apply: result K; stage: new solution
  T* tout;        // stage: next stage input (unused for the last stage)
  T fb, fa;       // stage factors b_s dt, a_s dt
  long long n_cells;
  int D, dim_x;
  int cells[kMaxDim];
  long long cstride[kMaxDim];
  int periodic[kMaxDim];
  LineOp<T> op[kMaxDim];
  int bc_inhom;
  DevFunction bc;
  double time;
  double lo[kMaxDim], h[kMaxDim];
  double gl[kMaxN];  // Gauss-Lobatto nodes on [0,1]
};

enum EclMode { kApply = 0, kStageFirst = 1, kStageMid = 2, kStageLast = 3 };

__device__ __forceinline__ double eval_function(const DevFunction& f, const double* x, int D, double t) {
  if (f.kind == 0) return 0.0;
  if (f.kind == 1) return f.amp;
  double r = f.amp;
  for (int d = 0; d < D; ++d) {
    const double arg = f.omega[d] * (x[d] - f.speed[d] * t) + f.phase[d];
    r *= f.cosine[d] ? cos(arg) : sin(arg);
  }
  return r;
}

// threads per cell and cells per CTA
template <int D, int N, typename T>
struct EclShape {
  static constexpr int NC = ipow(N, D);                       // nodes per cell
  static constexpr int NPLANE = D >= 2 ? ipow(N, D - 2) : 1;  // planes per phase
  static constexpr int TB = (N <= 4 ? 256 : 128);             // target CTA size
  static constexpr int TPC = NPLANE < TB ? NPLANE : TB;       // threads per cell
  static constexpr int CPB = TB / TPC > 0 ? TB / TPC : 1;     // cells per CTA
  static constexpr int THREADS = TPC * CPB;
  static constexpr size_t SMEM = size_t(2) * CPB * NC * sizeof(T);
  static constexpr int NPH = (D + 1) / 2;                     // phases
  static constexpr bool SUPPORTED = SMEM <= 200 * 1024;
};

// shared-memory index of node i (identity layout)
template <int D, int N, typename T>
__device__ __forceinline__ int sidx(int i) { return i; }

// node index of the plane/line base for work item `item` in phase with
// directions (dA, dB) (dB = -1 for a single-direction phase): the digits of
// `item` enumerate the remaining directions in increasing order
template <int D, int N>
__device__ __forceinline__ int item_base(int item, int dA, int dB) {
  int base = 0, stride = 1;
#pragma unroll
  for (int e = 0; e < D; ++e) {
    if (e != dA && e != dB) {
      base += (item % N) * stride;
      item /= N;
    }
    stride *= N;
  }
  return base;
}

// upwind neighbour of cell `gid` with coordinates cc along d (-1: domain boundary)
template <typename T>
__device__ __forceinline__ long long neighbour(const EclParams<T>& P, long long gid, const int* cc, int d) {
  const int step = P.op[d].step;
  const int c = cc[d] + step;
  if (c >= 0 && c < P.cells[d]) return gid + step * P.cstride[d];
  if (!P.periodic[d]) return -1;
  return gid + step * P.cstride[d] - (long long)step * P.cells[d] * P.cstride[d];
}

// exterior value on a boundary (inflow) face: u+ = -u- (+ 2 g(x, t))
template <int D, int N, typename T>
__device__ __forceinline__ T boundary_value(const EclParams<T>& P, const int* cc, int d, int node, T um) {
  if (!P.bc_inhom) return -um;
  double x[kMaxDim];
  int t = node;
#pragma unroll
  for (int e = 0; e < D; ++e) {
    const int ie = t % N;
    t /= N;
    x[e] = (e == d) ? P.lo[e] + (cc[e] + (P.op[d].step > 0 ? 1 : 0)) * P.h[e]
                    : P.lo[e] + (cc[e] + P.gl[ie]) * P.h[e];
  }
  return T(-double(um) + 2.0 * eval_function(P.bc, x, D, P.time));
}

template <int D, int N, typename T, int MODE>
__global__ void __launch_bounds__(EclShape<D, N, T>::THREADS)
    ecl_kernel(const __grid_constant__ EclParams<T> P) {
  using S = EclShape<D, N, T>;
  constexpr int NC = S::NC, TPC = S::TPC, CPB = S::CPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_u = reinterpret_cast<T*>(smem_raw);
  T* s_o = s_u + CPB * NC;

  const int tid = threadIdx.x;
  const int lc = tid / TPC, tl = tid % TPC;
  const long long cell0 = (long long)blockIdx.x * CPB;
  const long long gid = cell0 + lc;
  const bool valid = gid < P.n_cells;
  const long long ncell_here = (P.n_cells - cell0) < CPB ? (P.n_cells - cell0) : CPB;

  // ---- stage the CTA's contiguous block of cells in shared memory
  {
    const T* src = P.tin + cell0 * NC;
    const long long nval = ncell_here * NC;
    if constexpr ((NC * sizeof(T)) % 16 == 0) {
      constexpr int VPV = 16 / sizeof(T);
      const long long nvec = nval / VPV;
      const int4* s4 = reinterpret_cast<const int4*>(src);
      for (long long v = tid; v < nvec; v += S::THREADS) {
        const int4 x = __ldg(s4 + v);
        const T* xv = reinterpret_cast<const T*>(&x);
#pragma unroll
        for (int j = 0; j < VPV; ++j) {
          const long long i = v * VPV + j;
          s_u[(i / NC) * NC + sidx<D, N, T>(int(i % NC))] = xv[j];
        }
      }
    } else {
      for (long long i = tid; i < nval; i += S::THREADS)
        s_u[(i / NC) * NC + sidx<D, N, T>(int(i % NC))] = __ldg(src + i);
    }
  }
  __syncthreads();

  // ---- cell coordinates
  int cc[D];
  {
    long long g = valid ? gid : 0;
    long long gx = g % (P.cstride[P.dim_x]), gv = g / (P.cstride[P.dim_x]);
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if (d < P.dim_x) { cc[d] = int(gx % P.cells[d]); gx /= P.cells[d]; }
      else { cc[d] = int(gv % P.cells[d]); gv /= P.cells[d]; }
    }
  }
  T* su = s_u + lc * NC;
  T* so = s_o + lc * NC;

#pragma unroll
  for (int ph = 0; ph < S::NPH; ++ph) {
    const int dA = 2 * ph;
    const int dB = (2 * ph + 1 < D) ? 2 * ph + 1 : -1;
    const int strideA = ipow(N, dA);
    const int strideB = strideA * N;
    const int nitems = dB >= 0 ? ipow(N, D - 2) : ipow(N, D - 1);
    const bool last = (ph == S::NPH - 1);
    const long long nbA = valid && P.op[dA].active ? neighbour(P, gid, cc, dA) : -1;
    const long long nbB = (dB >= 0 && valid && P.op[dB].active) ? neighbour(P, gid, cc, dB) : -1;

    for (int item = tl; item < nitems; item += TPC) {
      const int base = item_base<D, N>(item, dA, dB);
      if (dB >= 0) {
        T uu[N][N], acc[N][N];  // [a][b]: node base + a*strideA + b*strideB
#pragma unroll
        for (int a = 0; a < N; ++a)
#pragma unroll
          for (int b = 0; b < N; ++b) {
            const int node = base + a * strideA + b * strideB;
            uu[a][b] = su[sidx<D, N, T>(node)];
            acc[a][b] = ph == 0 ? T(0) : so[sidx<D, N, T>(node)];
          }
        if (valid && P.op[dA].active) {
          const LineOp<T>& L = P.op[dA];
#pragma unroll
          for (int b = 0; b < N; ++b) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = acc[i][b];
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(L.M[i * N + q], uu[q][b], s);
              acc[i][b] = s;
            }
            const bool first = L.in_node == 0;
            const T um = first ? uu[0][b] : uu[N - 1][b];
            const T up = nbA >= 0 ? __ldg(P.tin + nbA * NC + base + L.nb_node * strideA + b * strideB)
                                  : boundary_value<D, N, T>(P, cc, dA, base + L.in_node * strideA + b * strideB, um);
            acc[0][b] = fma(L.c0, up, acc[0][b]);
            acc[N - 1][b] = fma(L.cl, up, acc[N - 1][b]);
          }
        }
        if (valid && P.op[dB].active) {
          const LineOp<T>& L = P.op[dB];
#pragma unroll
          for (int a = 0; a < N; ++a) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              T s = acc[a][i];
#pragma unroll
              for (int q = 0; q < N; ++q) s = fma(L.M[i * N + q], uu[a][q], s);
              acc[a][i] = s;
            }
            const bool first = L.in_node == 0;
            const T um = first ? uu[a][0] : uu[a][N - 1];
            const T up = nbB >= 0 ? __ldg(P.tin + nbB * NC + base + a * strideA + L.nb_node * strideB)
                                  : boundary_value<D, N, T>(P, cc, dB, base + a * strideA + L.in_node * strideB, um);
            acc[a][0] = fma(L.c0, up, acc[a][0]);
            acc[a][N - 1] = fma(L.cl, up, acc[a][N - 1]);
          }
        }
        if (!last) {
#pragma unroll
          for (int a = 0; a < N; ++a)
#pragma unroll
            for (int b = 0; b < N; ++b) so[sidx<D, N, T>(base + a * strideA + b * strideB)] = acc[a][b];
        } else if (valid) {
          const long long g0 = gid * NC;
#pragma unroll
          for (int b = 0; b < N; ++b)
#pragma unroll
            for (int a = 0; a < N; ++a) {
              const long long gi = g0 + base + a * strideA + b * strideB;
              const T k = acc[a][b];
              if constexpr (MODE == kApply) {
                P.uout[gi] = k;
              } else {
                const T u = (MODE == kStageFirst) ? uu[a][b] : P.uin[gi];
                P.uout[gi] = fma(P.fb, k, u);
                if constexpr (MODE != kStageLast) P.tout[gi] = fma(P.fa, k, u);
              }
            }
        }
      } else {
        // single-direction phase (odd D): lines along dA
        T uu[N], acc[N];
#pragma unroll
        for (int a = 0; a < N; ++a) {
          const int node = base + a * strideA;
          uu[a] = su[sidx<D, N, T>(node)];
          acc[a] = ph == 0 ? T(0) : so[sidx<D, N, T>(node)];
        }
        if (valid && P.op[dA].active) {
          const LineOp<T>& L = P.op[dA];
#pragma unroll
          for (int i = 0; i < N; ++i) {
            T s = acc[i];
#pragma unroll
            for (int q = 0; q < N; ++q) s = fma(L.M[i * N + q], uu[q], s);
            acc[i] = s;
          }
          const T um = L.in_node == 0 ? uu[0] : uu[N - 1];
          const T up = nbA >= 0 ? __ldg(P.tin + nbA * NC + base + L.nb_node * strideA)
                                : boundary_value<D, N, T>(P, cc, dA, base + L.in_node * strideA, um);
          acc[0] = fma(L.c0, up, acc[0]);
          acc[N - 1] = fma(L.cl, up, acc[N - 1]);
        }
        if (!last) {
#pragma unroll
          for (int a = 0; a < N; ++a) so[sidx<D, N, T>(base + a * strideA)] = acc[a];
        } else if (valid) {
          const long long g0 = gid * NC;
#pragma unroll
          for (int a = 0; a < N; ++a) {
            const long long gi = g0 + base + a * strideA;
            const T k = acc[a];
            if constexpr (MODE == kApply) {
              P.uout[gi] = k;
            } else {
              const T u = (MODE == kStageFirst) ? uu[a] : P.uin[gi];
              P.uout[gi] = fma(P.fb, k, u);
              if constexpr (MODE != kStageLast) P.tout[gi] = fma(P.fa, k, u);
            }
          }
        }
      }
    }
    if (!last) __syncthreads();
  }
}

// host launcher for one (D, N, T)
template <int D, int N, typename T>
cudaError_t launch_ecl(const EclParams<T>& P, int mode, cudaStream_t stream) {
  using S = EclShape<D, N, T>;
  if constexpr (!S::SUPPORTED) {
    return cudaErrorNotSupported;
  } else {
    static bool attr_done[4] = {false, false, false, false};
    const unsigned grid = unsigned((P.n_cells + S::CPB - 1) / S::CPB);
    auto go = [&](auto kern) -> cudaError_t {
      if (!attr_done[mode]) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(S::SMEM));
        if (e != cudaSuccess) return e;
        attr_done[mode] = true;
      }
      kern<<<grid, S::THREADS, S::SMEM, stream>>>(P);
      return cudaGetLastError();
    };
    switch (mode) {
      case kApply: return go(ecl_kernel<D, N, T, kApply>);
      case kStageFirst: return go(ecl_kernel<D, N, T, kStageFirst>);
      case kStageMid: return go(ecl_kernel<D, N, T, kStageMid>);
      case kStageLast: return go(ecl_kernel<D, N, T, kStageLast>);
      default: return cudaErrorInvalidValue;
    }
  }
}

// launcher table entry
struct EclLaunchers {
  cudaError_t (*f64)(const EclParams<double>&, int, cudaStream_t);
  cudaError_t (*f32)(const EclParams<float>&, int, cudaStream_t);
  size_t smem_f64, smem_f32;
  int threads_f64, threads_f32, cells_per_cta_f64, cells_per_cta_f32;
  bool ok_f64, ok_f32;
};

template <int D, int N>
EclLaunchers make_launchers() {
  using S64 = EclShape<D, N, double>;
  using S32 = EclShape<D, N, float>;
  return EclLaunchers{&launch_ecl<D, N, double>, &launch_ecl<D, N, float>, S64::SMEM, S32::SMEM,
                      S64::THREADS, S32::THREADS, S64::CPB, S32::CPB, S64::SUPPORTED, S32::SUPPORTED};
}

// message of the last failure for hd_last_error() (hd_capi.cu)
void set_last_error(const char* msg);

// pipelined 6D degree-3 FP32 kernel (hd_ecl6.cu): eligible for fully periodic
// 3x+3v meshes; err receives a device error code on a bounded-wait time-out
bool ecl6_eligible(const EclParams<float>& P);
cudaError_t launch_ecl6(const EclParams<float>& P, int* err, int mode, cudaStream_t stream);

// defined in hd_ecl_d{2..6}.cu
EclLaunchers ecl_launchers_d2(int N);
EclLaunchers ecl_launchers_d3(int N);
EclLaunchers ecl_launchers_d4(int N);
EclLaunchers ecl_launchers_d5(int N);
EclLaunchers ecl_launchers_d6(int N);

}  // namespace hd
