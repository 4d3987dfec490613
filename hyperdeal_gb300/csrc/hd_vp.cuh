// hd_vp.cuh -- Vlasov-Poisson pieces on the GPU (Gauss-Lobatto collocation or
// Gauss quadrature, dim_x == dim_v, periodic x- and v-meshes):
//   * velocity moment rho(x) = int f dv (FP64 accumulation),
//   * Poisson right-hand side, SIPG Laplacian and conjugate gradients (FP64,
//     one cooperative launch per solve),
//   * the field grad(phi) at the x-quadrature points,
//   * the ECL advection operator with the phase-space velocity (v, grad phi),
//   * diagnostics (field energy, mass, L2 norm, kinetic energy, momentum).
// Reference: examples/vlasov_poisson/include/application.h:516-602,
// poisson.h:100-255, derivative_container.h:158-251,
// velocity_field_view.h:103-209, diagnostics.h:28-141,
// include/hyper.deal/numerics/vector_tools.h:230-315.
#pragma once

#include <cuda_runtime.h>

#include "hd_ecl.cuh"

namespace hd {

// v-cells per direction at most (the x-line velocity table holds a block of
// this many cells per direction)
constexpr int kVpMaxCellsV = 64;

struct VpGeom {
  int D, dx, N, NCx, NC;
  long long ncx, ncv, n_cells, nx_dofs;
  int cells[kMaxDim];
  DivU64 dcell[kMaxDim], dncx;  // invariant divisors of cells[d] and ncx
  long long cstride[kMaxDim + 1];
  double lo[kMaxDim], h[kMaxDim];
  double gl[kMaxN], glw[kMaxN];
  double Dm[kMaxN * kMaxN];  // Dm[q*N + j] = l_j'(x_q) on [0,1]
  double K1[kMaxN * kMaxN];  // 1D stiffness on [0,1]: sum_q Dm[q][i] w_q Dm[q][j]
  double G[kMaxN * kMaxN];   // advection line matrix on [0,1]: G[i*N + q] = Dm[q][i] w_q / w_i
  double pen;                // max(k,1) (k+1)
  // Gauss quadrature (non-collocation, k + 1 points): the DoFs stay
  // Gauss-Lobatto nodal values; integrals, the field and the advection
  // operator work at the Gauss points gq (the reference's second quadrature
  // branch, advection_operation.h:294-316, :426-449, :536-559)
  int gauss;
  double gq[kMaxN], gw[kMaxN];   // Gauss points and weights on [0,1]
  double S[kMaxN * kMaxN];       // S[q*N + j] = l_j(gq_q): nodal values -> Gauss-point values
  double Si[kMaxN * kMaxN];      // S^{-1}
  double GS[kMaxN * kMaxN];      // GS[q*N + j] = l_j'(gq_q): nodal values -> derivative at the Gauss points
  double M1[kMaxN * kMaxN];      // 1D mass on [0,1]: sum_q gw_q S[q][i] S[q][j]
  // advection along a line in the Gauss-point basis, velocity a, extent h:
  // r += (a/h) (Ap v + cp u_up) for a > 0 (u_up: the left neighbour's trace),
  // r += (a/h) (Am v + cm u_up) for a < 0 (the right neighbour's), the
  // inverse Gauss weights folded in
  double Ap[kMaxN * kMaxN], Am[kMaxN * kMaxN];
  double cp[kMaxN], cm[kMaxN];
};

// coordinates of cell gid (gid = gid_x + ncx gid_v, each part lexicographic);
// returns gid_x
template <int D>
__device__ __forceinline__ long long vp_cell_coords(const VpGeom& g, long long gid, int* cc) {
  const unsigned long long ug = (unsigned long long)gid;
  unsigned long long b = divu64(ug, g.dncx);
  const unsigned long long gx = ug - b * g.dncx.d;
  unsigned long long a = gx;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const bool x = d < D / 2;
    const unsigned long long r = x ? a : b;
    const unsigned long long q = divu64(r, g.dcell[d]);
    cc[d] = int(r - q * g.dcell[d].d);
    if (x) a = q;
    else b = q;
  }
  return (long long)gx;
}

// x <- A applied along direction e of an nd-dimensional tensor x with N^nd
// entries (A row-major N x N, A[i*N + j]), in place; the block's threads
// share the lines, one line per thread (Gauss-point transforms)
template <typename T>
__device__ inline void vp_line_pass(T* x, const double* A, int N, int nd, int e, int tid, int nthr) {
  int total = 1;
  for (int f = 0; f < nd; ++f) total *= N;
  int se = 1;
  for (int f = 0; f < e; ++f) se *= N;
  const int lines = total / N;
  for (int line = tid; line < lines; line += nthr) {
    const int lo = line % se, hi = line / se;
    const int base = lo + hi * se * N;
    T u[kMaxN];
    for (int j = 0; j < N; ++j) u[j] = x[base + j * se];
    for (int i = 0; i < N; ++i) {
      T acc = T(0);
      for (int j = 0; j < N; ++j) acc = fma(T(A[i * N + j]), u[j], acc);
      x[base + i * se] = acc;
    }
  }
}

// advection with the phase-space velocity: dst = A(src).  The velocities
// enter divided by the cell extent of the line's direction, precomputed in
// FP64 and rounded to T once (no FP64 arithmetic in the kernel):
//   x-direction d: xs[(d * kVpMaxCellsV + c) * N + i] = v_d(c, i) / h_{x_d}, the
//                  v-coordinate of node i (quadrature point with Gauss) of
//                  v-cell c of v-direction d (a block per direction, so that
//                  v-meshes with different cell counts per direction index alike),
//   v-direction d: es[(gid_x * NCx + i_x) * dx + d] = d_d phi(x-node) / h_{v_d}.
//
// mode kApply: dst = A(src); stage modes (fused LSRK stage, as hd_ecl.cuh):
// uout = uin + fb A(src), tout = uin + fa A(src) (kStageFirst: uin = src;
// kStageLast: no tout).
template <typename T>
struct VpAdvParams {
  const T* src;
  T* dst;        // apply: the result; stage modes: uout
  const T* uin;
  T* tout;
  T fb, fa;
  const T* xs;
  const T* es;
  VpGeom g;
};

// (with P.g.gauss the Gauss-quadrature kernel, FP64 or FP32 storage, native arithmetic)
cudaError_t launch_vp_advection(const VpAdvParams<float>& P, int mode, cudaStream_t s);
// x2: FP32x2 arithmetic (hd_df.cuh) for FP64 storage; 1x1v and 2x2v shapes
cudaError_t launch_vp_advection(const VpAdvParams<double>& P, int mode, cudaStream_t s, bool x2 = false);
// the TMA-pipelined kernel (hd_vp_pipe.cuh): FP32, 2x+2v, degree 3, collocation,
// 16 cells along x0; state = {device error flag, unit ticket} (2 device ints)
bool vp_pipe_eligible(const VpGeom& g);
cudaError_t launch_vp_pipelined(const VpAdvParams<float>& P, int mode, cudaStream_t s, int* state,
                                unsigned wait_limit = 0, int skip_issue = -1);

}  // namespace hd
