// hd_vp.cu -- Vlasov-Poisson right-hand side on the GPU and its C ABI
// (hd_vp_* in include/hyperdeal_gb300.h).
//
// One evaluation (examples/vlasov_poisson/include/application.h:516-602):
//   1. rho(x) = int f dv at the x-nodes (FP64 accumulation, fixed order)
//   2. rhs = -M (rho - mean rho), mean removed (singular periodic problem)
//   3. SIPG Poisson solve by conjugate gradients in FP64 from an initial
//      guess (zero, the previous potential, or the learned model), one
//      cooperative launch per solve
//   4. E = grad(phi) at the x-nodes
//   5. dst = ECL advection of src with the phase-space velocity (v, E)
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/hyperdeal_gb300.h"
#include "hd_ecl.cuh"
#include "hd_rules.h"
#include "hd_vp.cuh"
#include "hd_vp_learn.cuh"

namespace cgrp = cooperative_groups;

namespace hd {

namespace {

constexpr int kMomChunk = 16;   // v-cells whose values a thread of the moment kernel loads together
constexpr int kMomBlockChunks = 4;  // chunks summed by one block (64 v-cells)
constexpr int kCgThreads = 64;  // small blocks: the x-space system is small, spread it over many SMs
constexpr int kLsMax = 16;      // basis columns of the least-squares learned guess (upper bound)
constexpr int kLsRed = kLsMax + 1;
constexpr double kLsCut = 1e-12;  // a pair joins the basis if its new direction is above this fraction

// device-side solver statistics (read by hd_vp_cg_stats; no host synchronisation per solve)
struct VpStats {
  long long total_iters, solves, learned_picked;
  double last_res;
  int last_iters, pad;
};

// ---------------------------------------------------------------- moments
// sum of f over the kMomChunk v-cells gv0.. at one node of x-cell gxc (the
// values are loaded independently before they are summed)
template <typename T>
__device__ __forceinline__ double moment_chunk_sum(const VpGeom& g, const T* __restrict__ f, long long gxc,
                                                   long long gv0, int node) {
  T vals[kMomChunk];
#pragma unroll
  for (int k = 0; k < kMomChunk; ++k) {
    const long long gv = gv0 + k;
    const long long gvc = gv < g.ncv ? gv : g.ncv - 1;  // valid address even if loaded unconditionally
    vals[k] = gv < g.ncv ? __ldg(f + (gxc + g.ncx * gvc) * g.NC + node) : T(0);
  }
  if constexpr (sizeof(T) == 4) {
    // FP32 storage: compensated pairwise sum on the FP32 pipe (the FP64 pipe
    // is the scarce resource here): every pairwise add is Knuth's TwoSum,
    // whose rounding error is kept in a second float and summed alongside,
    // so the chunk sum hi + lo carries about twice FP32's precision before
    // it is widened to FP64 (Ogita, Rump, Oishi, SIAM J. Sci. Comput. 2005)
    float hi[kMomChunk], lo[kMomChunk];
#pragma unroll
    for (int k = 0; k < kMomChunk; ++k) {
      hi[k] = vals[k];
      lo[k] = 0.f;
    }
#pragma unroll
    for (int w = kMomChunk / 2; w > 0; w /= 2)
#pragma unroll
      for (int k = 0; k < w; ++k) {
        float sum, err;
        two_sum(hi[k], hi[k + w], sum, err);
        hi[k] = sum;
        lo[k] = __fadd_rn(__fadd_rn(lo[k], lo[k + w]), err);
      }
    return x2_to_double(f32x2{hi[0], lo[0]});
  } else {
    // FP64 storage: summed pairwise in FP64
    T h[kMomChunk];
#pragma unroll
    for (int k = 0; k < kMomChunk; ++k) h[k] = vals[k];
#pragma unroll
    for (int w = kMomChunk / 2; w > 0; w /= 2)
#pragma unroll
      for (int k = 0; k < w; ++k) h[k] += h[k + w];
    return double(h[0]);
  }
}

// partial[block][gx*NCx + ix] = sum over the block's kMomBlockChunks chunks of
// v-cells and the v-nodes of f * JxW_v (the chunk sums of a node added in
// FP64, in order)
template <typename T>
__global__ void moment_partials(VpGeom g, const T* __restrict__ f, const double* __restrict__ wv,
                                double* __restrict__ partial) {
  extern __shared__ double sh[];
  const long long gxc = blockIdx.x;  // x-cell
  const int chunk = blockIdx.y;
  const int NCv = g.NC / g.NCx;
  for (int node = threadIdx.x; node < g.NC; node += blockDim.x) {
    double node_sum = 0.0;
    for (int cb = 0; cb < kMomBlockChunks; ++cb) {
      const long long gv0 = ((long long)chunk * kMomBlockChunks + cb) * kMomChunk;
      if (gv0 >= g.ncv) break;
      node_sum += moment_chunk_sum(g, f, gxc, gv0, node);
    }
    sh[node] = node_sum * wv[node / g.NCx];
  }
  __syncthreads();
  for (int ix = threadIdx.x; ix < g.NCx; ix += blockDim.x) {
    double s = 0.0;
    for (int iv = 0; iv < NCv; ++iv) s += sh[ix + g.NCx * iv];
    partial[(long long)chunk * g.nx_dofs + gxc * g.NCx + ix] = s;
  }
}

// block-wide sum in a fixed order (all threads receive the result)
__device__ double block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int k = 0; k < (int)(blockDim.x / 32); ++k) s += sh[k];
  return s;
}

// JxW of x-quadrature point ix (Gauss-Lobatto nodes, or Gauss points with g.gauss)
__host__ __device__ double x_qw(const VpGeom& g, int ix) {
  double j = 1.0;
  for (int d = 0; d < g.dx; ++d) {
    j *= g.h[d] * (g.gauss ? g.gw[ix % g.N] : g.glw[ix % g.N]);
    ix /= g.N;
  }
  return j;
}

// Gauss quadrature: sum_j M[i][j] (u_j - shift) over the x-cell of row i, M
// the x-cell mass matrix (M1 h_d in every direction, M1 = S^T W S)
__device__ double x_mass_row(const VpGeom& g, const double* u, long long i, double shift) {
  const long long c0 = (i / g.NCx) * g.NCx;
  const int il = int(i - c0);
  double s = 0.0;
  for (int j = 0; j < g.NCx; ++j) {
    double w = 1.0;
    int a = il, b = j;
    for (int d = 0; d < g.dx; ++d) {
      w *= g.h[d] * g.M1[(a % g.N) * g.N + (b % g.N)];
      a /= g.N;
      b /= g.N;
    }
    s = fma(w, u[c0 + j] - shift, s);
  }
  return s;
}

__host__ __device__ double x_jxw(const VpGeom& g, int ix) {
  double j = 1.0;
  for (int d = 0; d < g.dx; ++d) {
    j *= g.h[d] * g.glw[ix % g.N];
    ix /= g.N;
  }
  return j;
}

// ---------------------------------------------------------------- SIPG row
// (A u)_i for x-DoF i: cell stiffness + for both faces of every direction the
// SIPG terms sigma [u][v] - {d_n u}[v] - [u]{d_n v} at the Gauss-Lobatto face
// points (poisson.h:131-255).  u(k) returns entry k.  Constants are in the
// kernel, so the reference's removal of the input mean does not change the
// result.  Used once, to assemble the matrix (ELL format, see below).
template <class U>
__device__ double sipg_row(const VpGeom& g, U u, long long i) {
  const int N = g.N;
  const long long gx = i / g.NCx;
  const int ix = int(i - gx * g.NCx);
  int id[3], cc[3];
  {
    int t = ix;
    long long c = gx;
    for (int d = 0; d < g.dx; ++d) {
      id[d] = t % N;
      t /= N;
      cc[d] = int(c % g.cells[d]);
      c /= g.cells[d];
    }
  }
  double val = 0.0;
  int s = 1;
  for (int d = 0; d < g.dx; ++d) {
    const int base = ix - id[d] * s;
    const long long cs = g.cstride[d];
    const long long gL = cc[d] > 0 ? gx - cs : gx + (long long)(g.cells[d] - 1) * cs;
    const long long gR = cc[d] + 1 < g.cells[d] ? gx + cs : gx - (long long)(g.cells[d] - 1) * cs;
    double L[kMaxN], Lf[kMaxN], R[kMaxN];
    for (int j = 0; j < N; ++j) {
      L[j] = u(gx * g.NCx + base + j * s);
      Lf[j] = u(gL * g.NCx + base + j * s);
      R[j] = u(gR * g.NCx + base + j * s);
    }
    double wface = 1.0;
    for (int e = 0; e < g.dx; ++e)
      if (e != d) wface *= g.h[e] * g.glw[id[e]];
    const double h = g.h[d];
    double vol = 0.0;
    for (int j = 0; j < N; ++j) vol += g.K1[id[d] * N + j] * L[j];
    val += wface / h * vol;
    const double sigma = (1.0 / h + 1.0 / h) * g.pen;
    double dLk = 0.0, dR0 = 0.0, dLfk = 0.0, dL0 = 0.0;
    for (int j = 0; j < N; ++j) {
      dLk += g.Dm[(N - 1) * N + j] * L[j];
      dR0 += g.Dm[j] * R[j];
      dLfk += g.Dm[(N - 1) * N + j] * Lf[j];
      dL0 += g.Dm[j] * L[j];
    }
    {  // right face: this cell is the minus side
      const double jump = L[N - 1] - R[0], avg = 0.5 * (dLk + dR0) / h;
      const double vt = (sigma * jump - avg) * wface, nt = -0.5 * jump * wface;
      val += (id[d] == N - 1 ? vt : 0.0) + g.Dm[(N - 1) * N + id[d]] / h * nt;
    }
    {  // left face: this cell is the plus side
      const double jump = Lf[N - 1] - L[0], avg = 0.5 * (dLfk + dL0) / h;
      const double vt = (sigma * jump - avg) * wface, nt = -0.5 * jump * wface;
      val += (id[d] == 0 ? -vt : 0.0) + g.Dm[id[d]] / h * nt;
    }
    s *= N;
  }
  return val;
}

// The SIPG matrix in ELL form: row i has at most W = 3 N dim_x entries (the
// own-cell line and both neighbours' lines through i along every direction);
// col/val are stored [k][i] so that consecutive rows read consecutive words.
// Each coefficient is the row's linear form applied to a unit vector.
__global__ void assemble_sipg_ell(VpGeom g, int W, int* __restrict__ col, double* __restrict__ val) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long n = g.nx_dofs;
  if (i >= n) return;
  const int N = g.N;
  const long long gx = i / g.NCx;
  const int ix = int(i - gx * g.NCx);
  long long cand[3 * 3 * kMaxN];
  int m = 0;
  int s = 1;
  long long c = gx;
  for (int d = 0; d < g.dx; ++d) {
    const int idd = (ix / s) % N, cd = int(c % g.cells[d]);
    c /= g.cells[d];
    const int base = ix - idd * s;
    const long long cs = g.cstride[d];
    const long long gL = cd > 0 ? gx - cs : gx + (long long)(g.cells[d] - 1) * cs;
    const long long gR = cd + 1 < g.cells[d] ? gx + cs : gx - (long long)(g.cells[d] - 1) * cs;
    const long long cells3[3] = {gx, gL, gR};
    for (int q = 0; q < 3; ++q)
      for (int j = 0; j < N; ++j) {
        const long long k = cells3[q] * g.NCx + base + j * s;
        bool dup = false;
        for (int e = 0; e < m; ++e) dup |= cand[e] == k;
        if (!dup) cand[m++] = k;
      }
    s *= N;
  }
  for (int e = 0; e < W; ++e) {
    long long k = i;
    double a = 0.0;
    if (e < m) {
      k = cand[e];
      a = sipg_row(g, [k](long long t) { return t == k ? 1.0 : 0.0; }, i);
    }
    col[(long long)e * n + i] = int(k);
    val[(long long)e * n + i] = a;
  }
}

// (A u)_i from the ELL matrix; the matrix is read through the read-only path
// (it stays in L1 across the CG iterations), u through L2 (other blocks write it)
__device__ __forceinline__ double spmv_row(int W, long long n, const int* __restrict__ col,
                                           const double* __restrict__ val, const double* u, long long i) {
  double s = 0.0;
  int e = 0;
  for (; e + 8 <= W; e += 8) {
    double a[8], b[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      a[q] = __ldg(val + (long long)(e + q) * n + i);
      b[q] = __ldcg(u + __ldg(col + (long long)(e + q) * n + i));
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) s = fma(a[q], b[q], s);
  }
  for (; e < W; ++e) s = fma(__ldg(val + (long long)e * n + i), __ldcg(u + __ldg(col + (long long)e * n + i)), s);
  return s;
}

struct PoissonArgs {
  VpGeom g;
  int W;
  const int* col;
  const double* val;
  const double* partial;  // moment partials (nchunks x nx)
  int nchunks;
  int phases;             // bit 0: rho and rhs from the partials; bit 1: CG and the field; bit 2: the field only
  double* rho;
  double* rhs;
  double* x;              // potential: initial guess in, solution out
  double* r;
  double* p;
  double* Ap;
  double* red;            // [2][3 gridDim] partial sums
  double* z;              // preconditioned residual (the residual itself without a preconditioner)
  const double* binv;     // cell-block Jacobi: inverse of every x-cell's diagonal block (NCx x NCx), or null
  double rel_tol;
  int rhs_relative;       // 1: stop at ||r|| <= rel_tol ||rhs||; 0: at rel_tol ||r_0||
  int max_iter;
  double* E;              // E[i*dx + d] = d_d phi at the x-node
  void* es;               // E / h_v in the storage precision
  int es_f32;
  VpStats* stats;
  // least-squares learned guess (lsQ null: off).  The network phi = Z (Q^T rhs)
  // has the layers W1 = Q^T (k x n) and W2 = Z (n x k): Q is an orthonormal
  // basis of the right-hand sides A x_j of the recent solves and Z holds the
  // same combinations of their potentials x_j, so that W2 W1 maps every
  // recent rhs to its potential -- the minimum-norm least-squares fit of the
  // recent (rhs, phi) pairs.  The ring lsX / lsB keeps the last ls_kkeep pairs
  // (x, A x = rhs - r); when the basis holds ls_kmax columns it is rebuilt
  // from the ring.
  double* lsQ;
  double* lsZ;
  double* lsX;
  double* lsB;
  int* lsCount;   // basis columns (device; read at the start, written at the end)
  double* redk;   // [2][kLsRed gridDim] partial sums of grid_sum_k
  int ls_kmax, ls_kkeep, ls_head, ls_nraw;  // ring slot of this solve; ring entries including it
};

// fixed-order grid-wide sums of two values; consecutive calls alternate
// between the two halves of `red`, so a half is rewritten only after every
// block has read it.  Every warp adds the block partials lane-parallel in the
// same fixed order, so all threads of the grid obtain identical values.
__device__ double2 grid_sum2(cgrp::grid_group& grid, double v0, double v1, double* red, int& slot, double* sh) {
  const double b0 = block_sum(v0, sh);
  const double b1 = block_sum(v1, sh);
  double* half = red + slot * 2 * gridDim.x;
  if (threadIdx.x == 0) {
    half[2 * blockIdx.x] = b0;
    half[2 * blockIdx.x + 1] = b1;
  }
  grid.sync();
  const int lane = threadIdx.x & 31;
  double s0 = 0.0, s1 = 0.0;
  for (int k = lane; k < (int)gridDim.x; k += 32) {
    s0 += __ldcg(half + 2 * k);
    s1 += __ldcg(half + 2 * k + 1);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  slot ^= 1;
  return make_double2(__shfl_sync(0xffffffffu, s0, 0), __shfl_sync(0xffffffffu, s1, 0));
}

// the same for three values (the preconditioned CG's (r,z), (Az,z) and (r,r))
__device__ double3 grid_sum3(cgrp::grid_group& grid, double v0, double v1, double v2, double* red, int& slot,
                             double* sh) {
  const double b0 = block_sum(v0, sh);
  const double b1 = block_sum(v1, sh);
  const double b2 = block_sum(v2, sh);
  double* part = red + slot * 3 * gridDim.x;
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = b0;
    part[3 * blockIdx.x + 1] = b1;
    part[3 * blockIdx.x + 2] = b2;
  }
  grid.sync();
  const int lane = threadIdx.x & 31;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0;
  for (int k = lane; k < (int)gridDim.x; k += 32) {
    s0 += __ldcg(part + 3 * k);
    s1 += __ldcg(part + 3 * k + 1);
    s2 += __ldcg(part + 3 * k + 2);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  slot ^= 1;
  return make_double3(__shfl_sync(0xffffffffu, s0, 0), __shfl_sync(0xffffffffu, s1, 0),
                      __shfl_sync(0xffffffffu, s2, 0));
}

// fixed-order grid-wide sums of v[0..k) (k <= kLsRed), in place; every
// thread of the grid obtains identical values.  The halves of `red`
// (2 x kLsRed x gridDim) alternate as in grid_sum2; the grid barrier also
// frees `shk` (warps x kLsRed) for the next call.
__device__ void grid_sum_k(cgrp::grid_group& grid, double* v, int k, double* red, int& slot, double* shk) {
  const int w = threadIdx.x / 32, l = threadIdx.x % 32, nw = blockDim.x / 32;
#pragma unroll
  for (int j = 0; j < kLsRed; ++j) {
    if (j < k) {
      double t = v[j];
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      if (l == 0) shk[w * kLsRed + j] = t;
    }
  }
  __syncthreads();
  double* part = red + (size_t)slot * kLsRed * gridDim.x;
  if ((int)threadIdx.x < k) {
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t += shk[q * kLsRed + threadIdx.x];
    part[(size_t)blockIdx.x * kLsRed + threadIdx.x] = t;
  }
  grid.sync();
#pragma unroll
  for (int j = 0; j < kLsRed; ++j) {
    if (j < k) {
      double t = 0.0;
      for (int b = l; b < (int)gridDim.x; b += 32) t += __ldcg(part + (size_t)b * kLsRed + j);
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      v[j] = __shfl_sync(0xffffffffu, t, 0);
    }
  }
  slot ^= 1;
}

// Appends the pair of ring slot `src` to the basis of k columns: q = A x and
// z = x are orthogonalised against Q (classical Gram-Schmidt, twice), with
// the same operations on z, into column k; the column is kept (returns k + 1)
// when ||q|| is above kLsCut of ||A x||, i.e. when the pair adds a direction
// that is not round-off.  Each pass reduces its coefficients together with
// the squared length of its input; the final length follows from the second
// pass, ||q2||^2 = ||q1||^2 - sum a2_j^2 (Q orthonormal, a2 small).  Two
// grid-wide sums per pair; row-local otherwise.
template <typename Args>
__device__ int ls_append(cgrp::grid_group& grid, const Args& A, int src, int k, long long t0, long long stride,
                         int& slotk, double* shk) {
  const long long n = A.g.nx_dofs;
  const double* xs = A.lsX + (size_t)src * n;
  const double* bs = A.lsB + (size_t)src * n;
  double* q = A.lsQ + (size_t)k * n;
  double* z = A.lsZ + (size_t)k * n;
  for (long long i = t0; i < n; i += stride) {
    q[i] = bs[i];
    z[i] = xs[i];
  }
  double n0 = 0.0, len2 = 0.0;
  for (int pass = 0; pass < 2; ++pass) {
    double a[kLsRed];
    double nn = 0.0;
#pragma unroll
    for (int j = 0; j < kLsRed; ++j) a[j] = 0.0;
    for (long long i = t0; i < n; i += stride) {
      const double qi = q[i];
#pragma unroll
      for (int j = 0; j < kLsMax; ++j)
        if (j < k) a[j] = fma(A.lsQ[(size_t)j * n + i], qi, a[j]);
      nn = fma(qi, qi, nn);
    }
#pragma unroll
    for (int j = 0; j < kLsRed; ++j)
      if (j == k) a[j] = nn;
    grid_sum_k(grid, a, k + 1, A.redk, slotk, shk);
    double sq = 0.0, aa = 0.0;
#pragma unroll
    for (int j = 0; j < kLsRed; ++j) {
      if (j == k) sq = a[j];
      if (j < k) aa = fma(a[j], a[j], aa);
    }
    if (pass == 0) n0 = sqrt(sq);
    else len2 = sq - aa;
    for (long long i = t0; i < n; i += stride) {
      double qi = q[i], zi = z[i];
#pragma unroll
      for (int j = 0; j < kLsMax; ++j)
        if (j < k) {
          qi = fma(-a[j], A.lsQ[(size_t)j * n + i], qi);
          zi = fma(-a[j], A.lsZ[(size_t)j * n + i], zi);
        }
      q[i] = qi;
      z[i] = zi;
    }
  }
  const double len = len2 > 0.0 ? sqrt(len2) : 0.0;
  if (!(len > kLsCut * n0) || !(len > 0.0)) return k;
  const double inv = 1.0 / len;
  for (long long i = t0; i < n; i += stride) {
    q[i] *= inv;
    z[i] *= inv;
  }
  return k + 1;
}

// z_i = sum_j B^{-1}_c[i][j] r_j over the rows j of row i's x-cell c
__device__ __forceinline__ double block_jacobi_row(const VpGeom& g, const double* __restrict__ binv,
                                                   const double* r, long long i) {
  const long long c = i / g.NCx;
  const int il = int(i - c * g.NCx);
  const double* B = binv + (c * g.NCx + il) * g.NCx;
  const double* rc = r + c * g.NCx;
  double z = 0.0;
  for (int j = 0; j < g.NCx; ++j) z = fma(__ldg(B + j), __ldcg(rc + j), z);
  return z;
}

// the field E = grad(phi) at the x-nodes (derivative_container.h:158-251),
// and E / h_v in the storage precision, for this thread's rows
__device__ void poisson_field(const PoissonArgs& A, long long t0, long long stride) {
  const VpGeom& g = A.g;
  const long long n = g.nx_dofs;
  const int N = g.N;
  for (long long i = t0; i < n; i += stride) {
    const long long gx = i / g.NCx;
    const int ix = int(i - gx * g.NCx);
    int s = 1;
    for (int d = 0; d < g.dx; ++d) {
      const int idd = (ix / s) % N;
      const int base = ix - idd * s;
      double a = 0.0;
      if (g.gauss) {
        // at Gauss point ix: the derivative along d, the values (S) along the others
        for (int j = 0; j < g.NCx; ++j) {
          double w = 1.0;
          int qa = ix, jb = j;
          for (int e2 = 0; e2 < g.dx; ++e2) {
            const int q = qa % N, jj = jb % N;
            w *= e2 == d ? g.GS[q * N + jj] : g.S[q * N + jj];
            qa /= N;
            jb /= N;
          }
          a = fma(w, A.x[gx * g.NCx + j], a);
        }
      } else {
        for (int j = 0; j < N; ++j) a += g.Dm[idd * N + j] * A.x[gx * g.NCx + base + j * s];
      }
      const double e = a / g.h[d];
      A.E[i * g.dx + d] = e;
      const double es = e / g.h[g.dx + d];
      if (A.es_f32) static_cast<float*>(A.es)[i * g.dx + d] = float(es);
      else static_cast<double*>(A.es)[i * g.dx + d] = es;
      s *= N;
    }
  }
}

// One cooperative launch per solve (or two around the learned guess):
// rho and the right-hand side (application.h:531-568: rho~ = rho - mean,
// rhs = -M rho~, rhs -= mean), conjugate gradients on the SIPG system, and
// the field E = grad(phi) at the x-nodes (derivative_container.h:158-251).
// CG is the Chronopoulos-Gear form (one fused reduction of (r,z), (Az,z)
// and (r,r) per iteration: two grid barriers instead of three); in exact
// arithmetic it produces the iterates of plain CG, preconditioned by
// z = B^{-1} r with B the block diagonal of the x-cells (cell-block Jacobi)
// or unpreconditioned (z = r).  The reference preconditions its CG as well,
// with geometric multigrid (examples/vlasov_poisson/include/poisson.h:612-742).
// The preconditioner needs the residual of the row's cell only; when the
// block size is a multiple of the cell's DoFs every block holds whole cells
// (rows are handed out in block-sized chunks), so a block barrier suffices,
// otherwise a grid barrier separates the residual update from z.
__global__ void __launch_bounds__(kCgThreads) poisson_kernel(PoissonArgs A) {
  cgrp::grid_group grid = cgrp::this_grid();
  __shared__ double sh[32];
  __shared__ double shk[(kCgThreads / 32) * kLsRed];
  const VpGeom& g = A.g;
  const long long n = g.nx_dofs;
  const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x, stride = (long long)gridDim.x * blockDim.x;
  int slot = 0;
  if (A.phases & 1) {
    double ls = 0.0;
    for (long long i = t0; i < n; i += stride) {
      // eight independent partial sums (fixed order) keep eight loads in flight
      double s8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      int c = 0;
      for (; c + 8 <= A.nchunks; c += 8)
#pragma unroll
        for (int q = 0; q < 8; ++q) s8[q] += A.partial[(long long)(c + q) * n + i];
      for (; c < A.nchunks; ++c) s8[0] += A.partial[(long long)c * n + i];
      const double s = ((s8[0] + s8[1]) + (s8[2] + s8[3])) + ((s8[4] + s8[5]) + (s8[6] + s8[7]));
      A.rho[i] = s;
      ls += s;
    }
    const double mean = grid_sum2(grid, ls, 0.0, A.red, slot, sh).x / double(n);
    double l2 = 0.0;
    for (long long i = t0; i < n; i += stride) {
      // rhs = -M (rho - mean): the diagonal Gauss-Lobatto mass, or the Gauss one
      const double v = g.gauss ? -x_mass_row(g, A.rho, i, mean) : -(A.rho[i] - mean) * x_jxw(g, int(i % g.NCx));
      A.rhs[i] = v;
      l2 += v;
    }
    const double mean2 = grid_sum2(grid, l2, 0.0, A.red, slot, sh).x / double(n);
    for (long long i = t0; i < n; i += stride) A.rhs[i] -= mean2;
  }
  if (A.phases & 4) {
    // direct solve: x was written by the dense product (an earlier launch)
    poisson_field(A, t0, stride);
    if (t0 == 0) {
      A.stats->last_iters = 0;
      A.stats->solves += 1;
      A.stats->last_res = 0.0;
    }
    return;
  }
  if (!(A.phases & 2)) return;
  // least-squares learned guess: x = Z (Q^T rhs), or 0 before the first pair
  const bool ls = A.lsQ != nullptr;
  int lsk = 0, slotk = 0;
  if (ls) {
    lsk = *A.lsCount;
    double c[kLsRed];
#pragma unroll
    for (int j = 0; j < kLsRed; ++j) c[j] = 0.0;
    for (long long i = t0; i < n; i += stride) {
      const double b = A.rhs[i];
#pragma unroll
      for (int j = 0; j < kLsMax; ++j)
        if (j < lsk) c[j] = fma(A.lsQ[(size_t)j * n + i], b, c[j]);
    }
    if (lsk > 0) grid_sum_k(grid, c, lsk, A.redk, slotk, shk);
    for (long long i = t0; i < n; i += stride) {
      double x = 0.0;
#pragma unroll
      for (int j = 0; j < kLsMax; ++j)
        if (j < lsk) x = fma(c[j], A.lsZ[(size_t)j * n + i], x);
      A.x[i] = x;
    }
    grid.sync();  // the guess complete before A x reads it
  }
  double* const r = A.r;
  double* const p = A.p;
  double* const w = A.Ap;    // A z
  double* const sv = A.Ap + n;  // A p
  const bool pre = A.binv != nullptr;
  double* const z = pre ? A.z : r;
  const bool block_local = (blockDim.x % g.NCx) == 0;
  // z = B^{-1} r for this thread's rows, after every residual entry of their cells is written
  auto precondition = [&]() {
    if (!pre) return;
    if (block_local) __syncthreads();
    else grid.sync();
    for (long long i = t0; i < n; i += stride) z[i] = block_jacobi_row(g, A.binv, r, i);
  };
  double lbb = 0.0, lr0 = 0.0;
  for (long long i = t0; i < n; i += stride) {
    const double ri = A.rhs[i] - spmv_row(A.W, n, A.col, A.val, A.x, i);
    r[i] = ri;
    lbb += A.rhs[i] * A.rhs[i];
    lr0 += ri * ri;
  }
  double bb = -1.0;  // ||rhs||^2 once summed
  if (ls && lsk > 0) {
    // the selection: the guess starts CG only if its residual is below ||rhs|| (that of 0)
    const double2 jb = grid_sum2(grid, lbb, lr0, A.red, slot, sh);
    bb = jb.x;
    const bool keep = jb.y < jb.x;
    if (!keep)
      for (long long i = t0; i < n; i += stride) {
        A.x[i] = 0.0;
        r[i] = A.rhs[i];
      }
    if (keep && t0 == 0) A.stats->learned_picked += 1;
  }
  precondition();
  grid.sync();  // z complete before A z
  double lrz = 0.0, lwz = 0.0, lrr = 0.0;
  for (long long i = t0; i < n; i += stride) {
    const double wi = spmv_row(A.W, n, A.col, A.val, z, i);
    w[i] = wi;
    lrz += r[i] * z[i];
    lwz += wi * z[i];
    lrr += r[i] * r[i];
  }
  double3 t = grid_sum3(grid, lrz, lwz, lrr, A.red, slot, sh);
  if (bb < 0.0) bb = grid_sum2(grid, lbb, 0.0, A.red, slot, sh).x;
  double gamma = t.x, delta = t.y, rnorm = sqrt(t.z);
  const double r0 = rnorm;
  const double stop = A.rhs_relative ? A.rel_tol * sqrt(bb) : fmax(A.rel_tol * r0, 1e-14 * sqrt(bb));
  int it = 0;
  double alpha = delta > 0.0 ? gamma / delta : 0.0, beta = 0.0;
  while (rnorm > stop && it < A.max_iter && alpha > 0.0) {
    for (long long i = t0; i < n; i += stride) {
      const double pi = z[i] + (it ? beta * p[i] : 0.0);
      const double si = w[i] + (it ? beta * sv[i] : 0.0);
      p[i] = pi;
      sv[i] = si;
      A.x[i] += alpha * pi;
      r[i] -= alpha * si;
    }
    ++it;
    precondition();
    grid.sync();  // z complete before A z
    lrz = 0.0;
    lwz = 0.0;
    lrr = 0.0;
    for (long long i = t0; i < n; i += stride) {
      const double wi = spmv_row(A.W, n, A.col, A.val, z, i);
      w[i] = wi;
      lrz += r[i] * z[i];
      lwz += wi * z[i];
      lrr += r[i] * r[i];
    }
    t = grid_sum3(grid, lrz, lwz, lrr, A.red, slot, sh);
    const double gn = t.x;
    delta = t.y;
    rnorm = sqrt(t.z);
    beta = gn / gamma;
    const double den = delta - beta * gn / alpha;
    alpha = den > 0.0 ? gn / den : 0.0;
    gamma = gn;
  }
  if (pre) {
    // the block preconditioner does not keep the iterates orthogonal to the
    // constants (the null space of the periodic problem); the residual never
    // sees that component, so it is removed once at the end: phi mean-free
    grid.sync();
    double lx = 0.0;
    for (long long i = t0; i < n; i += stride) lx += A.x[i];
    const double mean_x = grid_sum2(grid, lx, 0.0, A.red, slot, sh).x / double(n);
    for (long long i = t0; i < n; i += stride) A.x[i] -= mean_x;
  }
  if (ls) {
    // this solve's pair (x, A x = rhs - r) into the ring, then into the basis
    // (or the basis rebuilt from the ring when it is full)
    double* xh = A.lsX + (size_t)A.ls_head * n;
    double* bh = A.lsB + (size_t)A.ls_head * n;
    for (long long i = t0; i < n; i += stride) {
      xh[i] = A.x[i];
      bh[i] = A.rhs[i] - r[i];
    }
    if (lsk >= A.ls_kmax) {
      lsk = 0;
      for (int e = 0; e < A.ls_nraw; ++e) {
        const int src = (A.ls_head - A.ls_nraw + 1 + e + 2 * A.ls_kkeep) % A.ls_kkeep;
        lsk = ls_append(grid, A, src, lsk, t0, stride, slotk, shk);
      }
    } else {
      lsk = ls_append(grid, A, A.ls_head, lsk, t0, stride, slotk, shk);
    }
    if (t0 == 0) *A.lsCount = lsk;
  }
  grid.sync();  // x complete before the field reads it
  poisson_field(A, t0, stride);
  if (t0 == 0) {
    A.stats->last_iters = it;
    A.stats->total_iters += it;
    A.stats->solves += 1;
    A.stats->last_res = r0 > 0.0 ? rnorm / r0 : 0.0;
  }
}

// ---------------------------------------------------------------- direct solve
// The x-space SIPG matrix A (fixed for the whole run) is singular only in the
// constants; the right-hand sides are mean-free, and on them the inverse of
// A + beta 1 1^T acts as the pseudo-inverse.  It is formed once, densely, by
// Gauss-Jordan elimination in place without pivoting (the matrix is symmetric
// positive definite): step k scales the pivot row by 1/a_kk and subtracts
// a_ik times it from every other row, keeping -a_ik/a_kk in column k.

// M = beta everywhere, then += A from the ELL form (each thread its own row)
__global__ void dense_from_ell(long long n, int W, const int* __restrict__ col, const double* __restrict__ val,
                               double* __restrict__ M) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < W; ++k) {
    const double v = val[(size_t)k * n + i];
    if (v != 0.0) M[i * n + col[(size_t)k * n + i]] += v;
  }
}

__global__ void fill_kernel(long long n, double v, double* __restrict__ x) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

// step k, part 1: the pivot row divided by the pivot (its diagonal entry
// 1/a_kk) and the pivot column, before the step overwrites them
__global__ void gj_pivot(long long n, int k, const double* __restrict__ M, double* __restrict__ rowk,
                         double* __restrict__ colk) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double piv = M[(long long)k * n + k];
  rowk[i] = i == k ? 1.0 / piv : M[(long long)k * n + i] / piv;
  colk[i] = M[i * n + k];
}

// step k, part 2: every entry (row blockIdx.y)
__global__ void gj_update(long long n, int k, double* __restrict__ M, const double* __restrict__ rowk,
                          const double* __restrict__ colk) {
  const long long i = blockIdx.y;
  const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (j >= n) return;
  double* const e = M + i * n + j;
  if (i == k) *e = rowk[j];
  else if (j == k) *e = -colk[i] * rowk[k];
  else *e = fma(-colk[i], rowk[j], *e);
}

// x = M b: one warp per row, the lanes over the columns, a fixed-order reduction
__global__ void dense_gemv(long long n, const double* __restrict__ M, const double* __restrict__ b,
                           double* __restrict__ x) {
  const long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;  // (whole warps)
  const double* r = M + row * n;
  // eight independent partial sums: eight 256-byte row loads of the warp in flight
  double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  long long j = lane;
  for (; j + 7 * 32 < n; j += 8 * 32) {
    double m[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) m[u] = __ldcs(r + j + 32 * u);  // streamed: read once per solve
#pragma unroll
    for (int u = 0; u < 8; ++u) acc[u] = fma(m[u], __ldg(b + j + 32 * u), acc[u]);
  }
  double tail = 0.0;
  for (; j < n; j += 32) tail = fma(__ldcs(r + j), __ldg(b + j), tail);
  double s = (((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]))) + tail;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) x[row] = s;
}

// per-block partial sums of ||rhs - A u||^2 for two candidate vectors u0, u1
__global__ void residual_partials(long long n, int W, const int* __restrict__ col, const double* __restrict__ val,
                                  const double* __restrict__ rhs, const double* __restrict__ u0,
                                  const double* __restrict__ u1, double* __restrict__ partial) {
  __shared__ double sh[32];
  double a = 0.0, b = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double r0 = rhs[i] - spmv_row(W, n, col, val, u0, i), r1 = rhs[i] - spmv_row(W, n, col, val, u1, i);
    a += r0 * r0;
    b += r1 * r1;
  }
  a = block_sum(a, sh);
  b = block_sum(b, sh);
  if (threadIdx.x == 0) {
    partial[2 * blockIdx.x] = a;
    partial[2 * blockIdx.x + 1] = b;
  }
}

// the selection: the candidate with the smaller initial residual starts CG
// (u1 is copied over u0 when it wins, and counted)
__global__ void choose_guess(long long n, int nblocks, const double* __restrict__ partial, double* __restrict__ u0,
                             const double* __restrict__ u1, VpStats* stats) {
  __shared__ int pick;
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < nblocks; ++k) {
      a += partial[2 * k];
      b += partial[2 * k + 1];
    }
    pick = b < a ? 1 : 0;
    stats->learned_picked += pick;
  }
  __syncthreads();
  if (pick)
    for (long long i = threadIdx.x; i < n; i += blockDim.x) u0[i] = u1[i];
}

// c = a - b
__global__ void diff_kernel(long long n, const double* __restrict__ a, const double* __restrict__ b,
                            double* __restrict__ c) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) c[i] = a[i] - b[i];
}

// y += x
__global__ void add_kernel(long long n, const double* __restrict__ x, double* __restrict__ y) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}

// ---------------------------------------------------------------- diagnostics
// block partials of mass, f^2, |v|^2 f, v_d f (3 + dv values) over cells
template <typename T>
__global__ void phase_diag_kernel(VpGeom g, const T* __restrict__ f, double* __restrict__ partial) {
  __shared__ double sh[32];
  const int dv = g.D - g.dx;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (long long gid = blockIdx.x; gid < g.n_cells; gid += gridDim.x) {
    int cc[kMaxDim];
    long long a = gid % g.ncx, b = gid / g.ncx;
    for (int d = 0; d < g.D; ++d) {
      if (d < g.dx) { cc[d] = int(a % g.cells[d]); a /= g.cells[d]; }
      else { cc[d] = int(b % g.cells[d]); b /= g.cells[d]; }
    }
    for (int node = threadIdx.x; node < g.NC; node += blockDim.x) {
      const double fv = double(f[gid * g.NC + node]);
      double jxw = 1.0, vv = 0.0, vel[3] = {0, 0, 0};
      int t = node;
      for (int d = 0; d < g.D; ++d) {
        const int id = t % g.N;
        t /= g.N;
        jxw *= g.h[d] * g.glw[id];
        if (d >= g.dx) {
          vel[d - g.dx] = g.lo[d] + (cc[d] + g.gl[id]) * g.h[d];
          vv += vel[d - g.dx] * vel[d - g.dx];
        }
      }
      acc[0] += fv * jxw;
      acc[1] += fv * fv * jxw;
      acc[2] += vv * fv * jxw;
      for (int d = 0; d < dv; ++d) acc[3 + d] += vel[d] * fv * jxw;
    }
  }
  for (int k = 0; k < 3 + dv; ++k) {
    const double s = block_sum(acc[k], sh);
    if (threadIdx.x == 0) partial[blockIdx.x * 6 + k] = s;
  }
}

// the same partials with Gauss quadrature: one block per cell (grid-stride),
// the cell's values taken to the Gauss points (S along every direction) in
// shared memory (NC doubles) before they are integrated
template <typename T>
__global__ void phase_diag_gauss_kernel(VpGeom g, const T* __restrict__ f, double* __restrict__ partial) {
  extern __shared__ double vq[];
  __shared__ double sh[32];
  const int dv = g.D - g.dx;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (long long gid = blockIdx.x; gid < g.n_cells; gid += gridDim.x) {
    int cc[kMaxDim];
    long long a = gid % g.ncx, b = gid / g.ncx;
    for (int d = 0; d < g.D; ++d) {
      if (d < g.dx) { cc[d] = int(a % g.cells[d]); a /= g.cells[d]; }
      else { cc[d] = int(b % g.cells[d]); b /= g.cells[d]; }
    }
    for (int i = threadIdx.x; i < g.NC; i += blockDim.x) vq[i] = double(f[gid * g.NC + i]);
    __syncthreads();
    for (int e = 0; e < g.D; ++e) {
      vp_line_pass(vq, g.S, g.N, g.D, e, threadIdx.x, blockDim.x);
      __syncthreads();
    }
    for (int q = threadIdx.x; q < g.NC; q += blockDim.x) {
      const double fv = vq[q];
      double jxw = 1.0, vv = 0.0, vel[3] = {0, 0, 0};
      int t = q;
      for (int d = 0; d < g.D; ++d) {
        const int id = t % g.N;
        t /= g.N;
        jxw *= g.h[d] * g.gw[id];
        if (d >= g.dx) {
          vel[d - g.dx] = g.lo[d] + (cc[d] + g.gq[id]) * g.h[d];
          vv += vel[d - g.dx] * vel[d - g.dx];
        }
      }
      acc[0] += fv * jxw;
      acc[1] += fv * fv * jxw;
      acc[2] += vv * fv * jxw;
      for (int d = 0; d < dv; ++d) acc[3 + d] += vel[d] * fv * jxw;
    }
    __syncthreads();  // vq is rewritten by the next cell
  }
  for (int k = 0; k < 3 + dv; ++k) {
    const double s = block_sum(acc[k], sh);
    if (threadIdx.x == 0) partial[blockIdx.x * 6 + k] = s;
  }
}

__global__ void energy_kernel(VpGeom g, const double* __restrict__ E, double* __restrict__ out) {
  __shared__ double sh[32];
  for (int d = 0; d < g.dx; ++d) {
    double s = 0.0;
    for (long long i = threadIdx.x; i < g.nx_dofs; i += blockDim.x) {
      const double e = E[i * g.dx + d];
      s += e * e * x_qw(g, int(i % g.NCx));
    }
    const double t = block_sum(s, sh);
    if (threadIdx.x == 0) out[d] = t;
  }
}

__global__ void diag_finish(int nblocks, int nq, const double* __restrict__ partial, double* __restrict__ out) {
  __shared__ double sh[32];
  for (int k = 0; k < nq; ++k) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partial[b * 6 + k];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[k] = k == 1 ? sqrt(s) : s;
  }
}

// kind 3: (1 + amp prod_{cosine[d]==1} cos(omega_d x_d + phase_d)) prod_{cosine[d]==2} exp(-x_d^2/2)/sqrt(2 pi),
// the perturbed Maxwellian of examples/vlasov_poisson/cases/hyperrectangle.h:45-58; kinds 0-2 as the operator's
__device__ double vp_eval_function(const DevFunction& f, const double* x, int D, double t) {
  if (f.kind != 3) return eval_function(f, x, D, t);
  double pert = f.amp, r = 1.0;
  for (int d = 0; d < D; ++d)
    if (f.cosine[d] == 1) pert *= cos(f.omega[d] * x[d] + f.phase[d]);
  r += pert;
  for (int d = 0; d < D; ++d)
    if (f.cosine[d] == 2) r = r * exp(-0.5 * x[d] * x[d]) / sqrt(2.0 * 3.14159265358979323846);
  return r;
}

// function values: interpolation of an analytic function at the nodes (kind 0-3)
template <typename T>
__global__ void vp_interpolate_kernel(VpGeom g, DevFunction f, double t, T* __restrict__ dst) {
  for (long long gid = blockIdx.x; gid < g.n_cells; gid += gridDim.x) {
    int cc[kMaxDim];
    long long a = gid % g.ncx, b = gid / g.ncx;
    for (int d = 0; d < g.D; ++d) {
      if (d < g.dx) { cc[d] = int(a % g.cells[d]); a /= g.cells[d]; }
      else { cc[d] = int(b % g.cells[d]); b /= g.cells[d]; }
    }
    for (int node = threadIdx.x; node < g.NC; node += blockDim.x) {
      double x[kMaxDim];
      int tt = node;
      for (int d = 0; d < g.D; ++d) {
        x[d] = g.lo[d] + (cc[d] + g.gl[tt % g.N]) * g.h[d];
        tt /= g.N;
      }
      dst[gid * g.NC + node] = T(vp_eval_function(f, x, g.D, t));
    }
  }
}

}  // namespace

}  // namespace hd

// ------------------------------------------------------------------ handle
struct hd_vp {
  hd_vp_desc desc;
  hd::VpGeom g;
  int dtype;
  int arith;          // HD_ARITH_NATIVE / HD_ARITH_FP32X2 of the FP64 advection
  int kernel;         // HD_KERNEL_AUTO / HD_KERNEL_GENERIC of the FP32 advection
  int* d_pipe;        // pipelined advection: device error flag and unit ticket
  unsigned pipe_wait; // its bounded waits' try_wait rounds (0: the default)
  int pipe_skip;      // its test hook (hd_vp_set_wait_test; -1: off)
  double* d_wv;       // v-node weights (NCv)
  double* d_partial;  // moment partials (nchunks * nx)
  int nchunks;
  double* d_rho;
  double* d_rhs;
  double* d_phi;
  double* d_E;
  void* d_xs;         // x-line velocities / h_x in the storage precision
  void* d_es;         // E / h_v in the storage precision
  double* d_cg;       // r, p, A z, A p, z (5 * nx) + reductions (2 halves * 3 values * cg_grid)
  double* d_binv;     // cell-block Jacobi preconditioner: ncx blocks of NCx x NCx (null: none)
  double* d_ainv;     // direct solve: the pseudo-inverse of the SIPG matrix, nx x nx (null: CG)
  int ell_w;          // SIPG matrix in ELL form (ell_w entries per row, [k][row])
  int* d_ell_col;
  double* d_ell_val;
  hd::VpStats* d_stats;
  double* d_diag;     // phase-space partials (blocks * 6) + outputs
  double* d_guess;    // learned prediction (nx)
  double* d_rho_prev; // rho and phi of the previous solve (the learned model
  double* d_phi_prev; //   maps rho - rho_prev to phi - phi_prev)
  double* d_dx;       // rho - rho_prev
  double* d_dy;       // phi - phi_prev
  bool have_prev;
  long long observed;  // pairs given to the learned model
  double* d_pick;     // residual partials of the guess selection
  int cg_grid;
  int guess;
  hd::VpModel* model;  // learned initial guess, Adam-trained (HD_VP_FIT_ADAM)
  // learned initial guess, least-squares fit (HD_VP_FIT_LEAST_SQUARES):
  // basis Q, Z (ls_kmax x nx each), ring of pairs X, B (ls_kkeep x nx each),
  // column count (device int), sums of the fit (2 x 17 x cg_grid)
  double* d_ls;
  int* d_ls_count;
  double* d_redk;
  int ls_kmax, ls_kkeep, ls_head, ls_nraw;
};

namespace {

int vfail(int code, const char* msg) {
  hd::set_last_error(msg);
  return code;
}

int vcuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return HD_OK;
  char buf[256];
  std::snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  hd::set_last_error(buf);
  return HD_ERR_CUDA;
}

// 1D tables on [0,1] from the Gauss-Lobatto rule (same construction as the operator's)
// inverse of a small dense matrix (Gauss-Jordan, partial pivoting); false if singular
bool invert_small(int n, const double* A, double* Ai) {
  double a[hd::kMaxN][2 * hd::kMaxN];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 2 * n; ++j) a[i][j] = j < n ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(a[i][k]) > std::fabs(a[piv][k])) piv = i;
    if (!(std::fabs(a[piv][k]) > 0.0)) return false;
    if (piv != k)
      for (int j = 0; j < 2 * n; ++j) std::swap(a[k][j], a[piv][j]);
    const double dk = 1.0 / a[k][k];
    for (int j = 0; j < 2 * n; ++j) a[k][j] *= dk;
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      const double f = a[i][k];
      if (f != 0.0)
        for (int j = 0; j < 2 * n; ++j) a[i][j] -= f * a[k][j];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Ai[i * n + j] = a[i][n + j];
  return true;
}

void vp_tables(int n, double* x, double* w, double* D) {
  const int m = n - 1;
  auto legendre = [](int nn, double z, double* p, double* dp) {
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= nn; ++k) {
      const double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = pk;
    }
    *p = p1;
    *dp = nn * (p0 - z * p1) / (1.0 - z * z);
  };
  x[0] = 0.0;
  x[n - 1] = 1.0;
  for (int i = 1; i < m; ++i) {
    double z = -std::cos(M_PI * i / m);
    for (int it = 0; it < 100; ++it) {
      double p, dp;
      legendre(m, z, &p, &dp);
      const double dz = dp / ((2.0 * z * dp - m * (m + 1.0) * p) / (1.0 - z * z));
      z -= dz;
      if (std::fabs(dz) < 1e-17) break;
    }
    x[i] = 0.5 * (1.0 + z);
  }
  for (int i = 0; i < n; ++i) {
    double p = 1.0, dp;
    if (i == 0) p = (m % 2) ? -1.0 : 1.0;
    else if (i < n - 1) legendre(m, 2.0 * x[i] - 1.0, &p, &dp);
    w[i] = 1.0 / (m * (m + 1.0) * p * p);
  }
  for (int i = 0; i < n / 2; ++i) {
    const double xs = 0.5 * (x[i] + (1.0 - x[n - 1 - i])), ws = 0.5 * (w[i] + w[n - 1 - i]);
    x[i] = xs;
    x[n - 1 - i] = 1.0 - xs;
    w[i] = ws;
    w[n - 1 - i] = ws;
  }
  if (n % 2) x[n / 2] = 0.5;
  for (int q = 0; q < n; ++q)
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int l = 0; l < n; ++l) {
        if (l == j) continue;
        double t = 1.0 / (x[j] - x[l]);
        for (int mm = 0; mm < n; ++mm)
          if (mm != j && mm != l) t *= (x[q] - x[mm]) / (x[j] - x[mm]);
        s += t;
      }
      D[q * n + j] = s;
    }
}

void vp_free(hd_vp* v) {
  if (!v) return;
  cudaFree(v->d_wv);
  cudaFree(v->d_partial);
  cudaFree(v->d_rho);
  cudaFree(v->d_rhs);
  cudaFree(v->d_phi);
  cudaFree(v->d_E);
  cudaFree(v->d_xs);
  cudaFree(v->d_es);
  cudaFree(v->d_cg);
  cudaFree(v->d_ell_col);
  cudaFree(v->d_ell_val);
  cudaFree(v->d_stats);
  cudaFree(v->d_diag);
  cudaFree(v->d_guess);
  cudaFree(v->d_rho_prev);
  cudaFree(v->d_phi_prev);
  cudaFree(v->d_dx);
  cudaFree(v->d_dy);
  cudaFree(v->d_pick);
  cudaFree(v->d_binv);
  cudaFree(v->d_ainv);
  cudaFree(v->d_pipe);
  cudaFree(v->d_ls);
  cudaFree(v->d_ls_count);
  cudaFree(v->d_redk);
  hd::vp_model_destroy(v->model);
  delete v;
}

// The SIPG matrix with Gauss quadrature, assembled on the host into the ELL
// arrays (row i: W = NCx (1 + 2 dim_x) entries, [k][i]).  With values and
// gradients taken to the Gauss points through S and GS, the bilinear form of
// poisson.h:131-255 is a sum of tensor products: the cell term
// sum_d K_d (x) prod_{e != d} M_e and, for every face normal to d, the
// one-dimensional face matrix F_d on the two cells' lines times the
// tangential masses -- K = GS^T W GS / h, M = S^T W S h, and
// F = sigma j j^T - j m^T - m j^T with j = (e_{N-1}, -e_0) the jump and
// m = (l'(1), l'(0)) / (2h) the mean normal derivative of the two cells'
// nodal bases.  All x-cells have the same extents, so the blocks are the same
// for every cell; columns that coincide (1 or 2 cells along a direction,
// periodic) are summed.
void assemble_sipg_gauss(const hd::VpGeom& g, int W, std::vector<int>& col, std::vector<double>& val) {
  const int N = g.N, m = g.NCx, dx = g.dx;
  const long long nx = g.nx_dofs;
  std::vector<double> K(N * N), M(N * N);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double k = 0.0, mm = 0.0;
      for (int q = 0; q < N; ++q) {
        k += g.gw[q] * g.GS[q * N + i] * g.GS[q * N + j];
        mm += g.gw[q] * g.S[q * N + i] * g.S[q * N + j];
      }
      K[i * N + j] = k;
      M[i * N + j] = mm;
    }
  // blocks: own (row cell c), plus[d] (column cell c + e_d), minus[d] (c - e_d)
  std::vector<double> own(size_t(m) * m, 0.0), plus(size_t(dx) * m * m, 0.0), minus(size_t(dx) * m * m, 0.0);
  for (int d = 0; d < dx; ++d) {
    const double h = g.h[d], sigma = (1.0 / h + 1.0 / h) * g.pen;
    double jv[2 * hd::kMaxN], mv[2 * hd::kMaxN], F[4 * hd::kMaxN * hd::kMaxN];
    for (int i = 0; i < N; ++i) {
      jv[i] = i == N - 1 ? 1.0 : 0.0;
      jv[N + i] = i == 0 ? -1.0 : 0.0;
      mv[i] = 0.5 * g.Dm[(N - 1) * N + i] / h;
      mv[N + i] = 0.5 * g.Dm[i] / h;
    }
    for (int a = 0; a < 2 * N; ++a)
      for (int b = 0; b < 2 * N; ++b) F[a * 2 * N + b] = sigma * jv[a] * jv[b] - jv[a] * mv[b] - mv[a] * jv[b];
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) {
        double t = 1.0;  // tangential mass
        int a = i, b = j, id = 0, jd = 0;
        for (int e = 0; e < dx; ++e) {
          if (e == d) { id = a % N; jd = b % N; }
          else t *= M[(a % N) * N + (b % N)] * g.h[e];
          a /= N;
          b /= N;
        }
        own[size_t(i) * m + j] += (K[id * N + jd] / h + F[(N + id) * 2 * N + N + jd] + F[id * 2 * N + jd]) * t;
        plus[(size_t(d) * m + i) * m + j] = F[id * 2 * N + N + jd] * t;
        minus[(size_t(d) * m + i) * m + j] = F[(N + id) * 2 * N + jd] * t;
      }
  }
  col.assign(size_t(W) * nx, 0);
  val.assign(size_t(W) * nx, 0.0);
  std::vector<long long> cols;
  std::vector<double> vals;
  for (long long gx = 0; gx < g.ncx; ++gx) {
    int cc[3] = {0, 0, 0};
    long long t = gx;
    for (int d = 0; d < dx; ++d) { cc[d] = int(t % g.cells[d]); t /= g.cells[d]; }
    for (int i = 0; i < m; ++i) {
      const long long row = gx * m + i;
      cols.clear();
      vals.clear();
      auto add = [&](long long cell, const double* blk) {
        for (int j = 0; j < m; ++j) {
          const long long c2 = cell * m + j;
          const double a = blk[size_t(i) * m + j];
          size_t k = 0;
          while (k < cols.size() && cols[k] != c2) ++k;
          if (k == cols.size()) { cols.push_back(c2); vals.push_back(a); }
          else vals[k] += a;
        }
      };
      add(gx, own.data());
      for (int d = 0; d < dx; ++d) {
        const long long cs = g.cstride[d];
        const long long gp = cc[d] + 1 < g.cells[d] ? gx + cs : gx - (long long)(g.cells[d] - 1) * cs;
        const long long gm = cc[d] > 0 ? gx - cs : gx + (long long)(g.cells[d] - 1) * cs;
        add(gp, plus.data() + size_t(d) * m * m);
        add(gm, minus.data() + size_t(d) * m * m);
      }
      for (int k = 0; k < W; ++k) {
        col[size_t(k) * nx + row] = int(k < (int)cols.size() ? cols[k] : row);
        val[size_t(k) * nx + row] = k < (int)cols.size() ? vals[k] : 0.0;
      }
    }
  }
}

// Cell-block Jacobi preconditioner: the diagonal block of every x-cell (the
// entries of its rows whose columns lie in the same cell) read back from the
// assembled ELL matrix, inverted on the host (Gauss-Jordan with partial
// pivoting; the SIPG blocks are symmetric positive definite) and uploaded.
int build_block_jacobi(hd_vp* v) {
  const hd::VpGeom& g = v->g;
  const long long nx = g.nx_dofs;
  const int W = v->ell_w, m = g.NCx;
  std::vector<int> col(size_t(W) * nx);
  std::vector<double> val(size_t(W) * nx);
  cudaError_t e = cudaMemcpy(col.data(), v->d_ell_col, sizeof(int) * col.size(), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(val.data(), v->d_ell_val, sizeof(double) * val.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return vcuda(e, "hd_vp_create: matrix read-back");
  std::vector<double> inv(size_t(g.ncx) * m * m);
  std::vector<double> a(size_t(m) * 2 * m);
  for (long long c = 0; c < g.ncx; ++c) {
    std::fill(a.begin(), a.end(), 0.0);
    for (int i = 0; i < m; ++i) {
      const long long row = c * m + i;
      for (int k = 0; k < W; ++k) {
        const long long j = col[size_t(k) * nx + row];
        if (j / m == c) a[size_t(i) * 2 * m + (j - c * m)] += val[size_t(k) * nx + row];
      }
      a[size_t(i) * 2 * m + m + i] = 1.0;
    }
    for (int k = 0; k < m; ++k) {
      int piv = k;
      for (int i = k + 1; i < m; ++i)
        if (std::fabs(a[size_t(i) * 2 * m + k]) > std::fabs(a[size_t(piv) * 2 * m + k])) piv = i;
      if (!(std::fabs(a[size_t(piv) * 2 * m + k]) > 0.0))
        return vfail(HD_ERR_INVALID, "hd_vp_create: singular diagonal block of the Poisson matrix");
      if (piv != k)
        for (int j = 0; j < 2 * m; ++j) std::swap(a[size_t(k) * 2 * m + j], a[size_t(piv) * 2 * m + j]);
      const double d = 1.0 / a[size_t(k) * 2 * m + k];
      for (int j = 0; j < 2 * m; ++j) a[size_t(k) * 2 * m + j] *= d;
      for (int i = 0; i < m; ++i) {
        if (i == k) continue;
        const double f = a[size_t(i) * 2 * m + k];
        if (f != 0.0)
          for (int j = 0; j < 2 * m; ++j) a[size_t(i) * 2 * m + j] -= f * a[size_t(k) * 2 * m + j];
      }
    }
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) inv[(size_t(c) * m + i) * m + j] = a[size_t(i) * 2 * m + m + j];
  }
  e = cudaMalloc(&v->d_binv, sizeof(double) * inv.size());
  if (e == cudaSuccess) e = cudaMemcpy(v->d_binv, inv.data(), sizeof(double) * inv.size(), cudaMemcpyHostToDevice);
  return vcuda(e, "hd_vp_create: preconditioner");
}

// Direct solve: A + beta 1 1^T (beta = the mean diagonal entry over nx, so
// that the constants get an eigenvalue of the size of A's diagonal) formed
// densely on the device and inverted in place by Gauss-Jordan elimination
// (2 nx launches, once per operator).
constexpr long long kDirectMaxDofs = 8192;
int build_direct(hd_vp* v) {
  const long long nx = v->g.nx_dofs;
  if (nx > kDirectMaxDofs) return vfail(HD_ERR_UNSUPPORTED, "hd_vp_create: direct Poisson solve up to 8192 x-DoFs");
  const int W = v->ell_w;
  std::vector<int> col(size_t(W) * nx);
  std::vector<double> val(size_t(W) * nx);
  cudaError_t e = cudaMemcpy(col.data(), v->d_ell_col, sizeof(int) * col.size(), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(val.data(), v->d_ell_val, sizeof(double) * val.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return vcuda(e, "hd_vp_create: matrix read-back");
  double tr = 0.0;
  for (long long i = 0; i < nx; ++i)
    for (int k = 0; k < W; ++k)
      if (col[size_t(k) * nx + i] == i) tr += val[size_t(k) * nx + i];
  if (!(tr > 0.0)) return vfail(HD_ERR_INVALID, "hd_vp_create: Poisson matrix without a positive diagonal");
  const double beta = tr / double(nx) / double(nx);
  double* buf = nullptr;
  e = cudaMalloc(&v->d_ainv, sizeof(double) * size_t(nx) * nx);
  if (e == cudaSuccess) e = cudaMalloc(&buf, sizeof(double) * 2 * nx);
  if (e != cudaSuccess) {
    cudaFree(buf);
    return vcuda(e, "hd_vp_create: direct solve storage");
  }
  const long long nn = nx * nx;
  hd::fill_kernel<<<unsigned((nn + 255) / 256), 256>>>(nn, beta, v->d_ainv);
  hd::dense_from_ell<<<unsigned((nx + 255) / 256), 256>>>(nx, W, v->d_ell_col, v->d_ell_val, v->d_ainv);
  const dim3 ug(unsigned((nx + 255) / 256), unsigned(nx));
  for (int k = 0; k < nx; ++k) {
    hd::gj_pivot<<<unsigned((nx + 255) / 256), 256>>>(nx, k, v->d_ainv, buf, buf + nx);
    hd::gj_update<<<ug, 256>>>(nx, k, v->d_ainv, buf, buf + nx);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  cudaFree(buf);
  return vcuda(e, "hd_vp_create: direct solve (Gauss-Jordan)");
}

hd::PoissonArgs poisson_args(hd_vp* v, int phases) {
  hd::PoissonArgs A;
  const long long nx = v->g.nx_dofs;
  A.g = v->g;
  A.W = v->ell_w;
  A.col = v->d_ell_col;
  A.val = v->d_ell_val;
  A.partial = v->d_partial;
  A.nchunks = v->nchunks;
  A.phases = phases;
  A.rho = v->d_rho;
  A.rhs = v->d_rhs;
  A.x = v->d_phi;
  A.r = v->d_cg;
  A.p = v->d_cg + nx;
  A.Ap = v->d_cg + 2 * nx;
  A.z = v->d_cg + 4 * nx;
  A.red = v->d_cg + 5 * nx;
  A.binv = v->d_binv;
  A.rel_tol = v->desc.cg_tol;
  A.rhs_relative = v->desc.cg_rhs_relative;
  A.max_iter = v->desc.cg_max_iter;
  A.E = v->d_E;
  A.es = v->d_es;
  A.es_f32 = v->dtype == HD_F32;
  A.stats = v->d_stats;
  A.lsQ = A.lsZ = A.lsX = A.lsB = nullptr;
  A.lsCount = nullptr;
  A.redk = v->d_redk;
  A.ls_kmax = v->ls_kmax;
  A.ls_kkeep = v->ls_kkeep;
  A.ls_head = v->ls_head;
  A.ls_nraw = v->ls_nraw;
  if (v->guess == HD_VP_GUESS_LEARNED && v->d_ls) {
    const size_t kx = size_t(v->ls_kmax) * nx, kr = size_t(v->ls_kkeep) * nx;
    A.lsQ = v->d_ls;
    A.lsZ = v->d_ls + kx;
    A.lsX = v->d_ls + 2 * kx;
    A.lsB = v->d_ls + 2 * kx + kr;
    A.lsCount = v->d_ls_count;
  }
  return A;
}

// the least-squares learned guess's buffers (once) and an empty fit
int ls_reset(hd_vp* v) {
  const long long nx = v->g.nx_dofs;
  if (!v->d_ls) {
    const size_t n = size_t(2) * (v->ls_kmax + v->ls_kkeep) * nx;
    int rc = vcuda(cudaMalloc((void**)&v->d_ls, sizeof(double) * n), "learned guess: cudaMalloc");
    if (!rc) rc = vcuda(cudaMalloc((void**)&v->d_ls_count, sizeof(int)), "learned guess: cudaMalloc");
    if (!rc) rc = vcuda(cudaMalloc((void**)&v->d_redk, sizeof(double) * 2 * hd::kLsRed * v->cg_grid),
                        "learned guess: cudaMalloc");
    if (rc) return rc;
  }
  v->ls_head = v->ls_kkeep - 1;
  v->ls_nraw = 0;
  return vcuda(cudaMemset(v->d_ls_count, 0, sizeof(int)), "learned guess: reset");
}

// the learned guess of the descriptor's fit, starting without pairs
int learned_create(hd_vp* v) {
  if (v->desc.learn_fit == HD_VP_FIT_LEAST_SQUARES) return ls_reset(v);
  if (!v->model) {
    v->model = hd::vp_model_create(v->g.nx_dofs, v->desc.learn_rank > 0 ? v->desc.learn_rank : 32,
                                   v->desc.learn_history > 0 ? v->desc.learn_history : 64);
    if (!v->model) return vfail(HD_ERR_ALLOC, "learned-guess model");
  }
  return HD_OK;
}

int launch_poisson(hd_vp* v, int phases, cudaStream_t s) {
  hd::PoissonArgs A = poisson_args(v, phases);
  void* args[] = {&A};
  return vcuda(cudaLaunchCooperativeKernel((void*)hd::poisson_kernel, dim3(v->cg_grid), dim3(hd::kCgThreads), args, 0,
                                           s),
               "Poisson launch");
}

// rho (from the moment partials), the right-hand side, CG from the chosen
// initial guess and the field; asynchronous (statistics stay on the device)
int solve_poisson(hd_vp* v, cudaStream_t s) {
  const long long nx = v->g.nx_dofs;
  if (v->d_ainv) {
    // direct: rho and rhs, phi = A^+ rhs, the field
    int rc = launch_poisson(v, 1, s);
    if (rc) return rc;
    hd::dense_gemv<<<unsigned((nx * 32 + 255) / 256), 256, 0, s>>>(nx, v->d_ainv, v->d_rhs, v->d_phi);
    rc = vcuda(cudaGetLastError(), "direct Poisson solve");
    if (rc) return rc;
    return launch_poisson(v, 4, s);
  }
  if (v->guess == HD_VP_GUESS_ZERO) {
    int rc = vcuda(cudaMemsetAsync(v->d_phi, 0, sizeof(double) * nx, s), "zero guess");
    if (rc) return rc;
  }
  if (v->guess == HD_VP_GUESS_LEARNED && v->d_ls) {
    // least-squares fit: one launch predicts, selects, solves and adds the pair
    v->ls_head = (v->ls_head + 1) % v->ls_kkeep;
    if (v->ls_nraw < v->ls_kkeep) ++v->ls_nraw;
    return launch_poisson(v, 3, s);
  }
  const bool learned = v->guess == HD_VP_GUESS_LEARNED && v->model;
  if (!learned) return launch_poisson(v, 3, s);
  // learned: the solution map is linear, so the model is trained on and
  // applied to differences to the previous solve: guess = phi_prev +
  // model(rho - rho_prev), weighed against phi_prev by the initial residual
  // (without a previous solve both differences are taken from zero)
  int rc = launch_poisson(v, 1, s);
  if (rc) return rc;
  const unsigned nb = unsigned((nx + 255) / 256);
  if (v->have_prev) {
    rc = vcuda(cudaMemcpyAsync(v->d_phi_prev, v->d_phi, sizeof(double) * nx, cudaMemcpyDeviceToDevice, s),
               "previous potential");
  } else {
    rc = vcuda(cudaMemsetAsync(v->d_phi_prev, 0, sizeof(double) * nx, s), "previous potential");
    if (!rc) rc = vcuda(cudaMemsetAsync(v->d_rho_prev, 0, sizeof(double) * nx, s), "previous density");
  }
  if (rc) return rc;
  hd::diff_kernel<<<nb, 256, 0, s>>>(nx, v->d_rho, v->d_rho_prev, v->d_dx);
  if (hd::vp_model_ready(v->model)) {
    rc = vcuda(hd::vp_model_predict(v->model, v->d_dx, v->d_guess, s), "learned guess");
    if (rc) return rc;
    hd::add_kernel<<<nb, 256, 0, s>>>(nx, v->d_phi_prev, v->d_guess);
    constexpr int kPickBlocks = 64;
    hd::residual_partials<<<kPickBlocks, 256, 0, s>>>(nx, v->ell_w, v->d_ell_col, v->d_ell_val, v->d_rhs, v->d_phi,
                                                       v->d_guess, v->d_pick);
    hd::choose_guess<<<1, 1024, 0, s>>>(nx, kPickBlocks, v->d_pick, v->d_phi, v->d_guess, v->d_stats);
  }
  rc = vcuda(cudaGetLastError(), "learned guess");
  if (rc) return rc;
  rc = launch_poisson(v, 2, s);
  if (rc) return rc;
  // the solver's own (rho - rho_prev, phi - phi_prev) pair trains the learned guess
  hd::diff_kernel<<<nb, 256, 0, s>>>(nx, v->d_phi, v->d_phi_prev, v->d_dy);
  const int every = v->desc.learn_every > 0 ? v->desc.learn_every : 1;
  rc = vcuda(hd::vp_model_observe(v->model, v->d_dx, v->d_dy, s, (v->observed++ % every) == 0),
             "learned guess update");
  if (!rc) rc = vcuda(cudaMemcpyAsync(v->d_rho_prev, v->d_rho, sizeof(double) * nx, cudaMemcpyDeviceToDevice, s),
                      "previous density");
  if (rc) return rc;
  v->have_prev = true;
  return HD_OK;
}

// the phase-space advection with the current field: apply, or a fused LSRK stage
// the FP32 advection kernel that runs (HD_KERNEL_PIPELINED where it applies, unless GENERIC is set)
int vp_kernel(const hd_vp* v) {
  return v->dtype == HD_F32 && v->kernel != HD_KERNEL_GENERIC && hd::vp_pipe_eligible(v->g) ? HD_KERNEL_PIPELINED
                                                                                           : HD_KERNEL_GENERIC;
}

int vp_advect(hd_vp* v, int mode, const void* src, const void* uin, void* dst, void* tout, double fb, double fa,
              cudaStream_t s) {
  cudaError_t e;
  if (v->dtype == HD_F32) {
    hd::VpAdvParams<float> P{(const float*)src, (float*)dst, (const float*)uin, (float*)tout, float(fb), float(fa),
                             (const float*)v->d_xs, (const float*)v->d_es, v->g};
    e = vp_kernel(v) == HD_KERNEL_PIPELINED
            ? hd::launch_vp_pipelined(P, mode, s, v->d_pipe, v->pipe_wait, v->pipe_skip)
            : hd::launch_vp_advection(P, mode, s);
  } else {
    hd::VpAdvParams<double> P{(const double*)src, (double*)dst, (const double*)uin, (double*)tout, fb, fa,
                              (const double*)v->d_xs, (const double*)v->d_es, v->g};
    e = hd::launch_vp_advection(P, mode, s, v->arith == HD_ARITH_FP32X2);
  }
  return vcuda(e, "vp advection");
}

}  // namespace

extern "C" {

int hd_vp_create(const hd_vp_desc* desc, hd_vp** out) {
  if (!desc || !out) return vfail(HD_ERR_INVALID, "hd_vp_create: null argument");
  *out = nullptr;
  const hd_vp_desc& d = *desc;
  if (d.dim_x < 1 || d.dim_x > 3 || d.dim_v != d.dim_x)
    return vfail(HD_ERR_INVALID, "hd_vp_create: dim_v must equal dim_x (1..3)");
  if (d.degree < 1 || d.degree + 1 > hd::kMaxN) return vfail(HD_ERR_UNSUPPORTED, "hd_vp_create: degree 1..5");
  if (d.dtype != HD_F64 && d.dtype != HD_F32) return vfail(HD_ERR_INVALID, "hd_vp_create: unknown dtype");
  if (!(d.cg_tol > 0.0) || d.cg_max_iter < 1) return vfail(HD_ERR_INVALID, "hd_vp_create: cg_tol > 0, cg_max_iter >= 1");
  if (d.guess < HD_VP_GUESS_ZERO || d.guess > HD_VP_GUESS_LEARNED)
    return vfail(HD_ERR_INVALID, "hd_vp_create: unknown guess");
  if (d.cg_precond != HD_VP_PRECOND_NONE && d.cg_precond != HD_VP_PRECOND_BLOCK_JACOBI)
    return vfail(HD_ERR_INVALID, "hd_vp_create: unknown preconditioner");
  if (d.learn_fit != HD_VP_FIT_LEAST_SQUARES && d.learn_fit != HD_VP_FIT_ADAM)
    return vfail(HD_ERR_INVALID, "hd_vp_create: unknown learned-guess fit");
  if (d.poisson_solver != HD_VP_SOLVER_CG && d.poisson_solver != HD_VP_SOLVER_DIRECT)
    return vfail(HD_ERR_INVALID, "hd_vp_create: unknown Poisson solver");
  if (d.learn_fit == HD_VP_FIT_LEAST_SQUARES &&
      (d.learn_rank < 0 || d.learn_rank > hd::kLsMax || d.learn_history < 0 ||
       (d.learn_rank > 0 && d.learn_history >= d.learn_rank)))
    return vfail(HD_ERR_INVALID, "hd_vp_create: least-squares guess needs learn_rank <= 16 and "
                                 "learn_history < learn_rank");
  if (d.quadrature != HD_QUAD_GAUSS_LOBATTO && d.quadrature != HD_QUAD_GAUSS)
    return vfail(HD_ERR_INVALID, "hd_vp_create: unknown quadrature");
  hd_vp* v = new (std::nothrow) hd_vp;
  if (!v) return vfail(HD_ERR_ALLOC, "out of host memory");
  std::memset(v, 0, sizeof(*v));
  v->desc = d;
  v->dtype = d.dtype;
  v->arith = HD_ARITH_NATIVE;
  v->kernel = HD_KERNEL_AUTO;
  v->pipe_skip = -1;
  v->guess = d.guess;
  hd::VpGeom& g = v->g;
  g.dx = d.dim_x;
  g.D = 2 * d.dim_x;
  g.N = d.degree + 1;
  g.NCx = hd::ipow(g.N, g.dx);
  g.NC = hd::ipow(g.N, g.D);
  g.ncx = 1;
  g.ncv = 1;
  long long st = 1;
  for (int i = 0; i < g.D; ++i) {
    const bool isx = i < g.dx;
    const int c = isx ? d.cells_x[i] : d.cells_v[i - g.dx];
    const double lo = isx ? d.lo_x[i] : d.lo_v[i - g.dx];
    const double hi = isx ? d.hi_x[i] : d.hi_v[i - g.dx];
    if (c < 1 || !(hi > lo)) { delete v; return vfail(HD_ERR_INVALID, "hd_vp_create: bad mesh"); }
    g.cells[i] = c;
    g.lo[i] = lo;
    g.h[i] = (hi - lo) / c;
    g.cstride[i] = st;
    st *= c;
    if (isx) g.ncx *= c;
    else g.ncv *= c;
  }
  g.cstride[g.D] = st;
  g.n_cells = st;
  g.nx_dofs = g.ncx * g.NCx;
  for (int i = 0; i < g.D; ++i) g.dcell[i] = hd::make_divu64((unsigned long long)g.cells[i]);
  g.dncx = hd::make_divu64((unsigned long long)g.ncx);
  vp_tables(g.N, g.gl, g.glw, g.Dm);
  const int N = g.N;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double k = 0.0;
      for (int q = 0; q < N; ++q) k += g.Dm[q * N + i] * g.glw[q] * g.Dm[q * N + j];
      g.K1[i * N + j] = k;
      g.G[i * N + j] = g.Dm[j * N + i] * g.glw[j] / g.glw[i];
    }
  g.pen = double(d.degree > 1 ? d.degree : 1) * (d.degree + 1.0);
  g.gauss = d.quadrature == HD_QUAD_GAUSS;
  if (g.gauss) {
    // Gauss points and the tables of the non-collocation path (hd_vp.cuh)
    hd::rules::gauss_rule(N, g.gq, g.gw);
    double Dg[hd::kMaxN * hd::kMaxN], f0[hd::kMaxN], f1[hd::kMaxN];
    hd::rules::lagrange_derivative_matrix(N, g.gq, Dg);  // Dg[q*N + j] = L_j'(gq_q), Gauss-point basis
    for (int q = 0; q < N; ++q) {
      f0[q] = hd::rules::lagrange_value(N, g.gq, q, 0.0);
      f1[q] = hd::rules::lagrange_value(N, g.gq, q, 1.0);
      for (int j = 0; j < N; ++j) g.S[q * N + j] = hd::rules::lagrange_value(N, g.gl, j, g.gq[q]);
    }
    for (int q = 0; q < N; ++q)
      for (int j = 0; j < N; ++j) {
        double a = 0.0, m = 0.0;
        for (int k = 0; k < N; ++k) {
          a += Dg[q * N + k] * g.S[k * N + j];
          m += g.gw[k] * g.S[k * N + q] * g.S[k * N + j];
        }
        g.GS[q * N + j] = a;
        g.M1[q * N + j] = m;
      }
    if (!invert_small(N, g.S, g.Si)) { delete v; return vfail(HD_ERR_INVALID, "hd_vp_create: singular basis change"); }
    // line operators in the Gauss-point basis (advection_operation.h:325-526 with
    // the flux 0.5((u- + u+) a.n + |a.n| (u- - u+)) on both faces, divided by the weights)
    for (int i = 0; i < N; ++i) {
      for (int q = 0; q < N; ++q) {
        const double vol = Dg[q * N + i] * g.gw[q];
        g.Ap[i * N + q] = (vol - f1[i] * f1[q]) / g.gw[i];
        g.Am[i * N + q] = (vol + f0[i] * f0[q]) / g.gw[i];
      }
      g.cp[i] = f0[i] / g.gw[i];
      g.cm[i] = -f1[i] / g.gw[i];
    }
    const size_t smem = size_t(d.dtype == HD_F64 ? 8 : 4) * (size_t(2) * g.NC + size_t(2) * g.D * (g.NC / N));
    if (smem > 220 * 1024) {
      delete v;
      return vfail(HD_ERR_UNSUPPORTED, "hd_vp_create: Gauss quadrature up to 3x+3v degree 3 (FP64)");
    }
  }
  // the advection kernel keeps two copies of CTA's cells in shared memory: 3x+3v up to degree 3
  if (g.D == 6 && N > 4) { delete v; return vfail(HD_ERR_UNSUPPORTED, "hd_vp_create: 3x+3v only for degree <= 3"); }
  for (int i = 0; i < g.dx; ++i)
    if (d.cells_v[i] > hd::kVpMaxCellsV) { delete v; return vfail(HD_ERR_UNSUPPORTED, "hd_vp_create: at most 64 v-cells per direction"); }
  // device buffers
  const int NCv = g.NC / g.NCx;
  v->nchunks = int((g.ncv + hd::kMomChunk * hd::kMomBlockChunks - 1) / (hd::kMomChunk * hd::kMomBlockChunks));
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hd::poisson_kernel, hd::kCgThreads, 0);
  long long want = (g.nx_dofs + hd::kCgThreads - 1) / hd::kCgThreads;
  long long cap = (long long)sms * (per_sm > 0 ? per_sm : 1);
  v->cg_grid = int(want < cap ? want : cap);
  if (v->cg_grid < 1) v->cg_grid = 1;
  const long long nx = g.nx_dofs;
  cudaError_t e = cudaSuccess;
  auto alloc = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  alloc((void**)&v->d_wv, sizeof(double) * NCv);
  alloc((void**)&v->d_partial, sizeof(double) * size_t(v->nchunks) * nx);
  alloc((void**)&v->d_rho, sizeof(double) * nx);
  alloc((void**)&v->d_rhs, sizeof(double) * nx);
  alloc((void**)&v->d_phi, sizeof(double) * nx);
  alloc((void**)&v->d_E, sizeof(double) * nx * g.dx);
  alloc(&v->d_es, sizeof(double) * nx * g.dx);
  alloc(&v->d_xs, sizeof(double) * g.dx * hd::kVpMaxCellsV * hd::kMaxN);
  alloc((void**)&v->d_cg, sizeof(double) * (5 * nx + 6 * v->cg_grid));
  v->ell_w = g.gauss ? g.NCx * (1 + 2 * g.dx) : 3 * N * g.dx;
  alloc((void**)&v->d_ell_col, sizeof(int) * size_t(v->ell_w) * nx);
  alloc((void**)&v->d_ell_val, sizeof(double) * size_t(v->ell_w) * nx);
  alloc((void**)&v->d_stats, sizeof(hd::VpStats));
  alloc((void**)&v->d_diag, sizeof(double) * (152 * 16 * 6 + 16));
  alloc((void**)&v->d_guess, sizeof(double) * nx);
  alloc((void**)&v->d_rho_prev, sizeof(double) * nx);
  alloc((void**)&v->d_phi_prev, sizeof(double) * nx);
  alloc((void**)&v->d_dx, sizeof(double) * nx);
  alloc((void**)&v->d_dy, sizeof(double) * nx);
  alloc((void**)&v->d_pick, sizeof(double) * 2 * 64);
  alloc((void**)&v->d_pipe, sizeof(int) * 2);
  if (e != cudaSuccess) { vp_free(v); return vcuda(e, "hd_vp_create: cudaMalloc"); }
  {
    double wv[4096];
    if (NCv > 4096) { vp_free(v); return vfail(HD_ERR_UNSUPPORTED, "hd_vp_create: v-cell too large"); }
    double jv = 1.0;
    for (int d2 = g.dx; d2 < g.D; ++d2) jv *= g.h[d2];
    for (int iv = 0; iv < NCv; ++iv) {
      double w = jv;
      int t = iv;
      for (int d2 = 0; d2 < g.dx; ++d2) { w *= g.glw[t % N]; t /= N; }
      wv[iv] = w;
    }
    e = cudaMemcpy(v->d_wv, wv, sizeof(double) * NCv, cudaMemcpyHostToDevice);
    // x-line velocity tables: v-coordinate of node i of v-cell c along v-direction dx + d, over h_{x_d}
    {
      double xs64[3 * hd::kVpMaxCellsV * hd::kMaxN];
      float xs32[3 * hd::kVpMaxCellsV * hd::kMaxN];
      // one block of kVpMaxCellsV v-cells per direction: entry (d * kVpMaxCellsV + c) * N + i
      const int k = g.dx * hd::kVpMaxCellsV * N;
      for (int t = 0; t < k; ++t) {
        xs64[t] = 0.0;
        xs32[t] = 0.f;
      }
      for (int d2 = 0; d2 < g.dx; ++d2) {
        const int e2 = g.dx + d2;
        for (int c = 0; c < g.cells[e2]; ++c)
          for (int i = 0; i < N; ++i) {
            const int t = (d2 * hd::kVpMaxCellsV + c) * N + i;
            xs64[t] = (g.lo[e2] + (c + (g.gauss ? g.gq[i] : g.gl[i])) * g.h[e2]) / g.h[d2];
            xs32[t] = float(xs64[t]);
          }
      }
      if (e == cudaSuccess)
        e = cudaMemcpy(v->d_xs, d.dtype == HD_F64 ? (const void*)xs64 : (const void*)xs32,
                       size_t(k) * (d.dtype == HD_F64 ? 8 : 4), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemset(v->d_es, 0, sizeof(double) * nx * g.dx);
    if (e == cudaSuccess) e = cudaMemset(v->d_stats, 0, sizeof(hd::VpStats));
    if (e == cudaSuccess) e = cudaMemset(v->d_pipe, 0, sizeof(int) * 2);
    if (e == cudaSuccess && g.gauss) {
      std::vector<int> col;
      std::vector<double> val;
      assemble_sipg_gauss(g, v->ell_w, col, val);
      e = cudaMemcpy(v->d_ell_col, col.data(), sizeof(int) * col.size(), cudaMemcpyHostToDevice);
      if (e == cudaSuccess) e = cudaMemcpy(v->d_ell_val, val.data(), sizeof(double) * val.size(), cudaMemcpyHostToDevice);
    } else if (e == cudaSuccess) {
      hd::assemble_sipg_ell<<<unsigned((nx + 127) / 128), 128>>>(g, v->ell_w, v->d_ell_col, v->d_ell_val);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemset(v->d_phi, 0, sizeof(double) * nx);
    if (e == cudaSuccess) e = cudaMemset(v->d_E, 0, sizeof(double) * nx * g.dx);
    if (e != cudaSuccess) { vp_free(v); return vcuda(e, "hd_vp_create: init"); }
  }
  if (d.poisson_solver == HD_VP_SOLVER_DIRECT) {
    const int rc = build_direct(v);
    if (rc) { vp_free(v); return rc; }
  } else if (d.cg_precond == HD_VP_PRECOND_BLOCK_JACOBI) {
    const int rc = build_block_jacobi(v);
    if (rc) { vp_free(v); return rc; }
  }
  if (d.learn_fit == HD_VP_FIT_LEAST_SQUARES) {
    v->ls_kmax = d.learn_rank > 0 ? d.learn_rank : 16;
    v->ls_kkeep = d.learn_history > 0 ? d.learn_history : (v->ls_kmax * 3 + 7) / 8;
    if (v->ls_kkeep >= v->ls_kmax) v->ls_kkeep = v->ls_kmax - 1;
    if (v->ls_kkeep < 1) { vp_free(v); return vfail(HD_ERR_INVALID, "hd_vp_create: learn_rank >= 2"); }
  }
  if (d.guess == HD_VP_GUESS_LEARNED) {
    const int rc = learned_create(v);
    if (rc) { vp_free(v); return rc; }
  }
  *out = v;
  return HD_OK;
}

int hd_vp_destroy(hd_vp* v) {
  vp_free(v);
  return HD_OK;
}

long long hd_vp_n_dofs(const hd_vp* v) { return v ? v->g.n_cells * v->g.NC : -1; }
long long hd_vp_n_dofs_x(const hd_vp* v) { return v ? v->g.nx_dofs : -1; }

int hd_vp_interpolate(hd_vp* v, const hd_function* f, double time, void* dst, void* stream) {
  if (!v || !f || !dst) return vfail(HD_ERR_INVALID, "hd_vp_interpolate: null argument");
  if (f->kind < 0 || f->kind > 3) return vfail(HD_ERR_INVALID, "hd_vp_interpolate: unknown function kind");
  hd::DevFunction df;
  std::memset(&df, 0, sizeof(df));
  df.kind = f->kind;
  df.amp = f->amp;
  for (int i = 0; i < HD_MAX_DIM; ++i) {
    df.omega[i] = f->omega[i];
    df.speed[i] = f->speed[i];
    df.phase[i] = f->phase[i];
    df.cosine[i] = f->cosine[i];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned grid = unsigned(v->g.n_cells < 152 * 32 ? v->g.n_cells : 152 * 32);
  if (v->dtype == HD_F32) hd::vp_interpolate_kernel<float><<<grid, 256, 0, s>>>(v->g, df, time, (float*)dst);
  else hd::vp_interpolate_kernel<double><<<grid, 256, 0, s>>>(v->g, df, time, (double*)dst);
  return vcuda(cudaGetLastError(), "vp interpolate");
}

int hd_vp_solve_field(hd_vp* v, const void* f, void* stream) {
  if (!v || !f) return vfail(HD_ERR_INVALID, "hd_vp_solve_field: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  hd::VpGeom& g = v->g;
  const dim3 grid(unsigned(g.ncx), unsigned(v->nchunks));
  const int threads = g.NC >= 256 ? 256 : ((g.NC + 31) / 32) * 32;
  const size_t sh = sizeof(double) * g.NC;
  if (v->dtype == HD_F32) hd::moment_partials<float><<<grid, threads, sh, s>>>(g, (const float*)f, v->d_wv, v->d_partial);
  else hd::moment_partials<double><<<grid, threads, sh, s>>>(g, (const double*)f, v->d_wv, v->d_partial);
  int rc = vcuda(cudaGetLastError(), "vp moments");
  if (rc) return rc;
  return solve_poisson(v, s);
}

int hd_vp_apply(hd_vp* v, void* dst, const void* src, double time, void* stream) {
  (void)time;
  if (!v || !dst || !src) return vfail(HD_ERR_INVALID, "hd_vp_apply: null argument");
  if (dst == src) return vfail(HD_ERR_INVALID, "hd_vp_apply: dst and src must differ");
  int rc = hd_vp_solve_field(v, src, stream);
  if (rc) return rc;
  return vp_advect(v, hd::kApply, src, nullptr, dst, nullptr, 0.0, 0.0, (cudaStream_t)stream);
}

int hd_vp_lsrk_step(hd_vp* v, const hd_lsrk* rk, void* sol, void* Ki, void* Ti, double time, double dt, void* stream) {
  if (!v || !rk || !sol || !Ki || !Ti) return vfail(HD_ERR_INVALID, "hd_vp_lsrk_step: null argument");
  const int ns = hd_lsrk_n_stages(rk);
  double ai[16], bi[16], ci[16];
  int rc = hd_lsrk_coefficients(rk, ai, bi, ci);
  if (rc) return rc;
  const long long n = hd_vp_n_dofs(v);
  cudaStream_t s = (cudaStream_t)stream;
  rc = vcuda(cudaMemcpyAsync(Ti, sol, size_t(n) * (v->dtype == HD_F64 ? 8 : 4), cudaMemcpyDeviceToDevice, s),
             "copy sol -> Ti");
  if (rc) return rc;
  for (int st = 0; st < ns; ++st) {
    rc = hd_vp_apply(v, Ki, Ti, time + ci[st] * dt, stream);
    if (rc) return rc;
    rc = hd_lsrk_stage_update(v->dtype, n, bi[st] * dt, st == ns - 1 ? 0.0 : ai[st] * dt, Ki, sol, Ti, stream);
    if (rc) return rc;
  }
  return HD_OK;
}

int hd_vp_lsrk_step_fused(hd_vp* v, const hd_lsrk* rk, void** sol, void** Ki, void** Ti, double time, double dt,
                          void* stream) {
  if (!v || !rk || !sol || !Ki || !Ti || !*sol || !*Ki || !*Ti)
    return vfail(HD_ERR_INVALID, "hd_vp_lsrk_step_fused: null argument");
  if (*sol == *Ki || *sol == *Ti || *Ki == *Ti) return vfail(HD_ERR_INVALID, "hd_vp_lsrk_step_fused: vectors must differ");
  const int ns = hd_lsrk_n_stages(rk);
  if (ns < 2) return vfail(HD_ERR_INVALID, "hd_vp_lsrk_step_fused: the scheme needs at least two stages");
  double ai[16], bi[16], ci[16];
  int rc = hd_lsrk_coefficients(rk, ai, bi, ci);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  // the rotation of hd_lsrk_step: X0 holds U and T_1, the new solution
  // accumulates in X1, the stage inputs alternate between X2 and X0; every
  // stage first solves for the field of its input
  void* X0 = *sol;
  void* X1 = *Ki;
  void* X2 = *Ti;
  void* t_in = X0;
  void* t_free = X2;
  for (int st = 0; st < ns; ++st) {
    const bool last = st == ns - 1;
    const int mode = st == 0 ? hd::kStageFirst : (last ? hd::kStageLast : hd::kStageMid);
    rc = hd_vp_solve_field(v, t_in, stream);
    if (rc) return rc;
    rc = vp_advect(v, mode, t_in, st == 0 ? t_in : X1, X1, last ? nullptr : t_free, bi[st] * dt,
                   last ? 0.0 : ai[st] * dt, s);
    if (rc) return rc;
    if (!last) {
      void* next = t_free;
      t_free = (st == 0) ? X0 : t_in;
      t_in = next;
    }
  }
  (void)time;
  *sol = X1;
  *Ki = X0;
  *Ti = X2;
  return HD_OK;
}

int hd_vp_diagnostics(hd_vp* v, const void* f, double* out, void* stream) {
  if (!v || !f || !out) return vfail(HD_ERR_INVALID, "hd_vp_diagnostics: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  hd::VpGeom& g = v->g;
  const int blocks = 152 * 16, dv = g.D - g.dx;
  double* part = v->d_diag;
  double* res = v->d_diag + blocks * 6;
  if (g.gauss) {
    const size_t sm = sizeof(double) * g.NC;
    if (v->dtype == HD_F32) {
      cudaFuncSetAttribute(hd::phase_diag_gauss_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      hd::phase_diag_gauss_kernel<float><<<blocks, 128, sm, s>>>(g, (const float*)f, part);
    } else {
      cudaFuncSetAttribute(hd::phase_diag_gauss_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
      hd::phase_diag_gauss_kernel<double><<<blocks, 128, sm, s>>>(g, (const double*)f, part);
    }
  } else if (v->dtype == HD_F32) {
    hd::phase_diag_kernel<float><<<blocks, 256, 0, s>>>(g, (const float*)f, part);
  } else {
    hd::phase_diag_kernel<double><<<blocks, 256, 0, s>>>(g, (const double*)f, part);
  }
  hd::diag_finish<<<1, 1024, 0, s>>>(blocks, 3 + dv, part, res);
  hd::energy_kernel<<<1, 1024, 0, s>>>(g, v->d_E, res + 8);
  int rc = vcuda(cudaGetLastError(), "vp diagnostics");
  if (rc) return rc;
  double h[16];
  rc = vcuda(cudaMemcpyAsync(h, res, sizeof(double) * 16, cudaMemcpyDeviceToHost, s), "diagnostics copy");
  if (rc) return rc;
  rc = vcuda(cudaStreamSynchronize(s), "diagnostics synchronize");
  if (rc) return rc;
  for (int d = 0; d < g.dx; ++d) out[d] = h[8 + d];
  for (int k = 0; k < 3 + dv; ++k) out[g.dx + k] = h[k];
  return HD_OK;
}

int hd_vp_fields(hd_vp* v, double* rho, double* phi, double* E, void* stream) {
  if (!v) return vfail(HD_ERR_INVALID, "hd_vp_fields: null handle");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t nx = size_t(v->g.nx_dofs);
  int rc = HD_OK;
  if (rho && !rc) rc = vcuda(cudaMemcpyAsync(rho, v->d_rho, sizeof(double) * nx, cudaMemcpyDeviceToDevice, s), "rho");
  if (phi && !rc) rc = vcuda(cudaMemcpyAsync(phi, v->d_phi, sizeof(double) * nx, cudaMemcpyDeviceToDevice, s), "phi");
  if (E && !rc)
    rc = vcuda(cudaMemcpyAsync(E, v->d_E, sizeof(double) * nx * v->g.dx, cudaMemcpyDeviceToDevice, s), "E");
  return rc;
}

int hd_vp_cg_stats(const hd_vp* v, int* last_iterations, long long* total_iterations, long long* solves,
                   double* last_residual, long long* learned_picked) {
  if (!v) return vfail(HD_ERR_INVALID, "hd_vp_cg_stats: null handle");
  hd::VpStats st;
  int rc = vcuda(cudaDeviceSynchronize(), "hd_vp_cg_stats: synchronize");
  if (!rc) rc = vcuda(cudaMemcpy(&st, v->d_stats, sizeof(st), cudaMemcpyDeviceToHost), "hd_vp_cg_stats: copy");
  if (rc) return rc;
  if (learned_picked) *learned_picked = st.learned_picked;
  if (last_iterations) *last_iterations = st.last_iters;
  if (total_iterations) *total_iterations = st.total_iters;
  if (solves) *solves = st.solves;
  if (last_residual) *last_residual = st.last_res;
  return HD_OK;
}

int hd_vp_set_arithmetic(hd_vp* v, int arithmetic) {
  if (!v) return vfail(HD_ERR_INVALID, "hd_vp_set_arithmetic: null handle");
  if (arithmetic != HD_ARITH_NATIVE && arithmetic != HD_ARITH_FP32X2)
    return vfail(HD_ERR_INVALID, "unknown arithmetic");
  if (arithmetic == HD_ARITH_FP32X2 && (v->dtype != HD_F64 || v->g.dx > 2 || v->g.gauss))
    return vfail(HD_ERR_UNSUPPORTED, "FP32x2 arithmetic needs FP64 storage, collocation and dim_x = dim_v <= 2");
  v->arith = arithmetic;
  return HD_OK;
}

int hd_vp_set_guess(hd_vp* v, int guess) {
  if (!v) return vfail(HD_ERR_INVALID, "hd_vp_set_guess: null handle");
  if (guess < HD_VP_GUESS_ZERO || guess > HD_VP_GUESS_LEARNED) return vfail(HD_ERR_INVALID, "unknown guess");
  if (guess == HD_VP_GUESS_LEARNED && guess != v->guess) {
    const int rc = learned_create(v);
    if (rc) return rc;
  }
  if (guess != v->guess) v->have_prev = false;
  v->guess = guess;
  return HD_OK;
}

}  // extern "C"

extern "C" int hd_vp_set_kernel(hd_vp* v, int variant) {
  if (!v) return vfail(HD_ERR_INVALID, "hd_vp_set_kernel: null handle");
  if (variant != HD_KERNEL_AUTO && variant != HD_KERNEL_GENERIC && variant != HD_KERNEL_PIPELINED)
    return vfail(HD_ERR_INVALID, "hd_vp_set_kernel: unknown kernel");
  if (variant == HD_KERNEL_PIPELINED && !(v->dtype == HD_F32 && hd::vp_pipe_eligible(v->g)))
    return vfail(HD_ERR_UNSUPPORTED, "hd_vp_set_kernel: the pipelined advection needs FP32, 2x+2v, degree 3, "
                                     "collocation and 16 cells along x0");
  v->kernel = variant;
  return HD_OK;
}

extern "C" int hd_vp_kernel(const hd_vp* v) { return v ? vp_kernel(v) : -1; }

extern "C" int hd_vp_device_status(hd_vp* v, int* status) {
  if (!v || !status) return vfail(HD_ERR_INVALID, "hd_vp_device_status: null argument");
  int rc = vcuda(cudaDeviceSynchronize(), "hd_vp_device_status: synchronize");
  if (!rc) rc = vcuda(cudaMemcpy(status, v->d_pipe, sizeof(int), cudaMemcpyDeviceToHost), "hd_vp_device_status");
  if (!rc) rc = vcuda(cudaMemset(v->d_pipe, 0, sizeof(int)), "hd_vp_device_status: reset");
  return rc;
}

extern "C" int hd_vp_set_wait_test(hd_vp* v, unsigned wait_limit, int skip_issue) {
  if (!v) return vfail(HD_ERR_INVALID, "hd_vp_set_wait_test: null handle");
  if (skip_issue != -1 && skip_issue != 0) return vfail(HD_ERR_INVALID, "hd_vp_set_wait_test: skip_issue -1 or 0");
  v->pipe_wait = wait_limit;
  v->pipe_skip = skip_issue;
  return HD_OK;
}

extern "C" int hd_vp_learn_loss_grad(long long n, int rank, int batch, const float* W1, const float* W2,
                                     const float* X, const float* Y, float* dW1, float* dW2, float* loss,
                                     void* stream) {
  if (n < 1 || rank < 1 || batch < 1 || !W1 || !W2 || !X || !Y || !dW1 || !dW2 || !loss)
    return vfail(HD_ERR_INVALID, "hd_vp_learn_loss_grad: bad argument");
  float* work = nullptr;
  cudaError_t e = cudaMalloc(&work, sizeof(float) * hd::vp_model_work_floats(n, rank, batch));
  if (e != cudaSuccess) return vcuda(e, "hd_vp_learn_loss_grad: cudaMalloc");
  cudaStream_t s = (cudaStream_t)stream;
  e = hd::vp_model_loss_grad(n, rank, batch, W1, W2, X, Y, dW1, dW2, loss, work, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(work);
  return vcuda(e, "hd_vp_learn_loss_grad");
}
